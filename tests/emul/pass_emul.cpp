// pass_emul.cpp -- thread-by-thread CPU emulation of the engine's in-CTA
// building blocks (the same template code the kernels instantiate):
//   * the runtime Stockham stage loop for every supported N (forward,
//     inverse and the forward -> transfer -> reversed inverse propagation);
//   * the TMA tile geometry of the screen gather and the separable bicubic,
//     against a direct periodic Keys bicubic in double;
//   * the FP32-only atan2 of the science unwrap against (float) of the
//     double atan2 (count of differing results and the largest difference
//     in units in the last place).
// Prints one line per check: "<name> <max error>"; exit code 0.
#include <array>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <vector>

#include "fft_core.cuh"
#include "gather_core.cuh"
#include "atan_ff.cuh"
#include "epi_math.cuh"

using namespace atmwfs;
using cd = std::complex<double>;

static unsigned long long g_rng = 88172645463325252ull;
static double urand()
{
    g_rng ^= g_rng << 13;
    g_rng ^= g_rng >> 7;
    g_rng ^= g_rng << 17;
    return (double)(g_rng >> 11) * (1.0 / 9007199254740992.0);
}

// The kernel's runtime stage loop, one thread after the other (the
// __syncthreads of the device loop separate the per-thread sweeps).
// The two-stage compile-time plan (fft2_ct), one thread after the other.
template <int N, int T, int E, int RA, int RB>
void emu_fft2_ct(std::vector<std::array<float2, E>>& V, float2* buf, const float2* tws1)
{
    for (int t = 0; t < T; t++) stage_dft<E, RA, -1>(V[t].data());
    for (int t = 0; t < T; t++) stage_store<N, T, E, RA, 1>(V[t].data(), buf, t);
    for (int t = 0; t < T; t++) {
        stage_load<N, T, E, RB>(V[t].data(), buf, t);
        stage_twiddle_rt<N, T, E, RB>(V[t].data(), t, tws1, RA);
        stage_dft<E, RB, -1>(V[t].data());
    }
}

// The three-stage compile-time plan of the alternative radix plans (fft3_ct).
template <int N, int T, int E, int RA, int RB, int RC>
void emu_fft3_ct(std::vector<std::array<float2, E>>& V, float2* buf, const float2* twsB, const float2* twsC)
{
    for (int t = 0; t < T; t++) stage_dft<E, RA, -1>(V[t].data());
    for (int t = 0; t < T; t++) stage_store<N, T, E, RA, 1>(V[t].data(), buf, t);
    for (int t = 0; t < T; t++) {
        stage_load<N, T, E, RB>(V[t].data(), buf, t);
        stage_twiddle_rt<N, T, E, RB>(V[t].data(), t, twsB, RA);
        stage_dft<E, RB, -1>(V[t].data());
    }
    for (int t = 0; t < T; t++) stage_store<N, T, E, RB, RA>(V[t].data(), buf, t);
    for (int t = 0; t < T; t++) {
        stage_load<N, T, E, RC>(V[t].data(), buf, t);
        stage_twiddle_rt<N, T, E, RC>(V[t].data(), t, twsC, RA * RB);
        stage_dft<E, RC, -1>(V[t].data());
    }
}

template <int N, int T, int E, int PV = 0>
void emu_fft_rt(std::vector<std::array<float2, E>>& V, float2* buf, const float2* tw, float ds, int rev)
{
    if (ds > 0.0f)
        for (int t = 0; t < T; t++) conj_all<E>(V[t].data());
    if constexpr (PV != 0 && Stages<N, PV>::S == 3) {
        constexpr int R0 = Stages<N, PV>::R0, R1 = Stages<N, PV>::R1, R2 = Stages<N, PV>::R2;
        if (rev) emu_fft3_ct<N, T, E, R2, R1, R0>(V, buf, tw + tw_offset<N, PV>(1, 1), tw + tw_offset<N, PV>(1, 2));
        else emu_fft3_ct<N, T, E, R0, R1, R2>(V, buf, tw + tw_offset<N, PV>(0, 1), tw + tw_offset<N, PV>(0, 2));
        if (ds > 0.0f)
            for (int t = 0; t < T; t++) conj_all<E>(V[t].data());
        return;
    }
    if constexpr (Stages<N>::S == 2) {
        constexpr int R0 = Stages<N>::R0, R1 = Stages<N>::R1;
        if (rev) emu_fft2_ct<N, T, E, R1, R0>(V, buf, tw + tw_offset<N>(1, 1));
        else emu_fft2_ct<N, T, E, R0, R1>(V, buf, tw + tw_offset<N>(0, 1));
        if (ds > 0.0f)
            for (int t = 0; t < T; t++) conj_all<E>(V[t].data());
        return;
    }
    int ns = 1, rp = 0, nsp = 1;
    for (int st = 0; st < Stages<N>::S; st++) {
        const int r = stage_radix<N>(st, rev);
        if (st > 0) {
            for (int t = 0; t < T; t++) stage_exchange_store<N, T, E>(V[t].data(), buf, t, rp, nsp);
            for (int t = 0; t < T; t++) stage_exchange_load<N, T, E>(V[t].data(), buf, t, r);
        }
        for (int t = 0; t < T; t++) stage_compute<N, T, E>(V[t].data(), t, tw + tw_offset<N>(rev, st), r, ns);
        rp = r;
        nsp = ns;
        ns *= r;
    }
    if (ds > 0.0f)
        for (int t = 0; t < T; t++) conj_all<E>(V[t].data());
}

static std::vector<cd> dft(const std::vector<cd>& x, int sign)
{
    const int n = (int)x.size();
    std::vector<cd> X(n);
    for (int k = 0; k < n; k++) {
        cd s = 0;
        for (int j = 0; j < n; j++) {
            const long m = ((long)j * k) % n;
            const double a = sign * 2.0 * M_PI * (double)m / n;
            s += x[j] * cd(cos(a), sin(a));
        }
        X[k] = s;
    }
    return X;
}

template <int N, int PV = 0>
void check_fft()
{
    constexpr int T = Plan<N, PV>::T, E = Plan<N, PV>::E;
    std::vector<float2> tw(tw_total<N, PV>() + 1);
    build_twiddles<N, PV>(tw.data());
    std::vector<float2> buf(padi(N) + 64);
    std::vector<cd> x(N);
    for (int i = 0; i < N; i++) x[i] = cd(urand() - 0.5, urand() - 0.5);
    constexpr int RL = last_radix<N, PV>();
    const char* sfx = PV == 0 ? "" : "v1";
    for (int D : {-1, +1}) {
        std::vector<std::array<float2, E>> V(T);
        for (int t = 0; t < T; t++)
            for (int e = 0; e < E; e++) V[t][e] = make_float2((float)x[t + e * T].real(), (float)x[t + e * T].imag());
        emu_fft_rt<N, T, E, PV>(V, buf.data(), tw.data(), (float)D, 0);
        std::vector<cd> X = dft(x, D);
        double err = 0, nrm = 0;
        std::vector<int> seen(N, 0);
        for (int t = 0; t < T; t++)
            for (int s = 0; s < E; s++) {
                const int k = last_index<N, T, RL>(t, s);
                seen[k]++;
                err = fmax(err, std::abs(cd(V[t][s].x, V[t][s].y) - X[k]));
                nrm = fmax(nrm, std::abs(X[k]));
            }
        for (int k = 0; k < N; k++)
            if (seen[k] != 1) { printf("fft%s_%d%s_coverage 1e9\n", D < 0 ? "fwd" : "inv", N, sfx); return; }
        printf("fft%s_%d%s %.3e\n", D < 0 ? "fwd" : "inv", N, sfx, err / nrm);
    }
    // propagation: forward, multiply by a unit-modulus table, inverse
    std::vector<float2> h(N);
    std::vector<cd> hd(N);
    for (int k = 0; k < N; k++) {
        const double a = 2 * M_PI * urand();
        hd[k] = cd(cos(a), sin(a)) / (double)N;
        h[k] = make_float2((float)hd[k].real(), (float)hd[k].imag());
    }
    std::vector<std::array<float2, E>> V(T);
    for (int t = 0; t < T; t++)
        for (int e = 0; e < E; e++) V[t][e] = make_float2((float)x[t + e * T].real(), (float)x[t + e * T].imag());
    emu_fft_rt<N, T, E, PV>(V, buf.data(), tw.data(), -1.0f, 0);
    for (int t = 0; t < T; t++)
        for (int s = 0; s < E; s++) V[t][s] = cmul(V[t][s], h[last_index<N, T, RL>(t, s)]);
    emu_fft_rt<N, T, E, PV>(V, buf.data(), tw.data(), 1.0f, 1);
    std::vector<cd> X = dft(x, -1);
    for (int k = 0; k < N; k++) X[k] *= hd[k];
    std::vector<cd> y = dft(X, +1);
    double err = 0, nrm = 0;
    for (int t = 0; t < T; t++)
        for (int e = 0; e < E; e++) {
            err = fmax(err, std::abs(cd(V[t][e].x, V[t][e].y) - y[t + e * T]));
            nrm = fmax(nrm, std::abs(y[t + e * T]));
        }
    printf("prop_%d%s %.3e\n", N, sfx, err / nrm);
}

// ---------------------------------------------------------------------------
// gather: padded periodic screen, TMA box layout, separable bicubic
// ---------------------------------------------------------------------------
static double keys(double t, int k)
{
    const double t2 = t * t, t3 = t2 * t;
    switch (k) {
        case 0: return 0.5 * (-t3 + 2 * t2 - t);
        case 1: return 0.5 * (3 * t3 - 5 * t2 + 2);
        case 2: return 0.5 * (-3 * t3 + 4 * t2 + t);
        default: return 0.5 * (t3 - t2);
    }
}

template <int N, int CFG = 0>
void check_gather(int M, int ix, int iy, float fx, float fy, int orient, int y0)
{
    constexpr int RR = tile_cfg(N, CFG).rr;
    constexpr int NT = Plan<N>::T * RR;
    constexpr int TROWS = RR + 3, NBOX = N / kBoxW + 1;
    std::vector<float> S((size_t)M * M);
    for (auto& v : S) v = (float)(urand() * 20 - 10);
    const int Wp = M + N + 64, Hp = M + N + 8;
    // padded copy, as k_pad_screen
    std::vector<float> P((size_t)Wp * Hp);
    for (int yp = 0; yp < Hp; yp++)
        for (int xp = 0; xp < Wp; xp++) {
            const int a = ((yp - kPadY) % M + M) % M, b = ((xp - kPadX) % M + M) % M;
            P[(size_t)yp * Wp + xp] = orient ? S[(size_t)b * M + a] : S[(size_t)a * M + b];
        }
    LayerPos p{ix, iy, fx, fy};
    const TileGeom g = tile_geom(p, orient, y0);
    std::vector<float> tile((size_t)NBOX * TROWS * kBoxW);
    bool inb = true;
    for (int k = 0; k < NBOX; k++)
        for (int r = 0; r < TROWS; r++)
            for (int c = 0; c < kBoxW; c++) {
                const int xp = g.xs + k * kBoxW + c, yp = g.ys + r;
                if (xp < 0 || yp < 0 || xp >= Wp || yp >= Hp) { inb = false; continue; }
                tile[((size_t)k * TROWS + r) * kBoxW + c] = P[(size_t)yp * Wp + xp];
            }
    std::vector<float> out((size_t)RR * N, NAN);
    for (int tid = 0; tid < NT; tid++)
        gather_tile<N, RR, NT>(tile.data(), g, 1.0f, tid, [&](int r, int x, float v) { out[(size_t)r * N + x] = v; });
    double err = 0;
    for (int r = 0; r < RR; r++)
        for (int x = 0; x < N; x++) {
            // pass coordinates (row y0 + r, column x) -> screen sample
            const int row = y0 + r;
            double X, Y;
            if (orient == 0) { X = ix + (double)fx + x; Y = iy + (double)fy + row; }
            else { X = ix + (double)fx + row; Y = iy + (double)fy + x; }
            const long xi = (long)floor(X), yi = (long)floor(Y);
            const double tx = X - xi, ty = Y - yi;
            double v = 0;
            for (int b = 0; b < 4; b++)
                for (int a = 0; a < 4; a++) {
                    const long sx = ((xi - 1 + a) % M + M) % M, sy = ((yi - 1 + b) % M + M) % M;
                    v += keys(tx, a) * keys(ty, b) * S[(size_t)sy * M + sx];
                }
            err = fmax(err, fabs(v - out[(size_t)r * N + x]));
        }
    printf("gather_%d_c%d_o%d_ix%d_iy%d %.3e\n", N, CFG, orient, ix, iy, inb ? err : 1e9);
}

static int ulp_distance(float a, float b)
{
    if (a == b) return 0;
    int32_t ia, ib;
    std::memcpy(&ia, &a, 4);
    std::memcpy(&ib, &b, 4);
    if ((ia < 0) != (ib < 0)) return 1 << 30;
    return std::abs(ia - ib);
}

// The FP32-only atan2 against (float)atan2 in double on five input families:
// uniform in the square, log-spread magnitudes (2^-60 .. 2^60) with random
// signs, near the diagonal |y| ~ |x|, ratios on and beside the table points,
// and signed zeros / the axes.
static void check_atan2()
{
    std::vector<float2> tab(kAtanTabN + 1);
    atan_table_host(tab.data());
    long n = 0, diff = 0;
    int maxulp = 0;
    auto one = [&](float y, float x) {
        const float a = atan2_ff(y, x, tab.data());
        const float b = (float)std::atan2((double)y, (double)x);
        const int d = ulp_distance(a, b);
        n++;
        if (d) diff++;
        if (d > maxulp) maxulp = d;
    };
    for (int i = 0; i < 1000000; i++) one((float)(2 * urand() - 1), (float)(2 * urand() - 1));
    for (int i = 0; i < 1000000; i++) {
        const float y = (float)std::ldexp(urand() + 0.5, (int)(urand() * 120) - 60) * (urand() < 0.5 ? -1.0f : 1.0f);
        const float x = (float)std::ldexp(urand() + 0.5, (int)(urand() * 120) - 60) * (urand() < 0.5 ? -1.0f : 1.0f);
        one(y, x);
    }
    for (int i = 0; i < 500000; i++) {
        const float x = (float)(urand() * 100 + 1e-3) * (urand() < 0.5 ? -1.0f : 1.0f);
        const float y = x * (float)(1.0 + (urand() - 0.5) * 1e-5) * (urand() < 0.5 ? -1.0f : 1.0f);
        one(y, x);
        one(x, y);
    }
    for (int k = 0; k <= kAtanTabN; k++)
        for (int j = -3; j <= 3; j++) {
            const float x = 1024.0f * (1.0f + (float)j * 1.1920929e-7f);
            const float y = (float)k;
            one(y, x);
            one(-y, -x);
            one(x, y);
            one(-x, y);
            one(y * (1.0f + 3e-4f * j), x);
        }
    const float zs[] = {0.0f, -0.0f, 1.0f, -1.0f, 1e-38f, -1e-45f, 3e38f, -3e38f};
    for (float y : zs)
        for (float x : zs) one(y, x);
    std::printf("atan2_diff %ld\n", diff);
    std::printf("atan2_maxulp %d\n", maxulp);
    std::printf("atan2_count %ld\n", n);
}

// The output epilogue's FP32 atan2 against the double atan2: the largest
// absolute difference in radians over every quadrant, the octant boundaries,
// the tan(pi/8) switch, magnitudes spread over many decades, and the axes.
static void check_atan2_out()
{
    double worst = 0;
    long n = 0;
    auto one = [&](float y, float x) {
        const double ref = atan2((double)y, (double)x);
        double d = fabs((double)atan2_out(y, x) - ref);
        if (d > M_PI) d = fabs(d - 2 * M_PI);  // +-pi on the negative x axis
        worst = fmax(worst, d);
        n++;
    };
    for (int i = 0; i < 2000000; i++) {
        const double ang = (urand() * 2 - 1) * M_PI, mag = pow(10.0, urand() * 12 - 6);
        one((float)(mag * sin(ang)), (float)(mag * cos(ang)));
    }
    const double t8 = tan(M_PI / 8);
    for (int i = -2000; i <= 2000; i++)
        for (int q = 0; q < 8; q++) {
            const double base = q * M_PI / 4, ang = base + i * 1e-7;
            one((float)sin(ang), (float)cos(ang));
            const double a2 = atan(t8) + q * M_PI / 2 + i * 1e-7;
            one((float)(3.0 * sin(a2)), (float)(3.0 * cos(a2)));
        }
    for (float v : {1.0f, -1.0f, 1e-30f, -1e30f}) {
        one(v, 0.0f);
        one(0.0f, v);
        one(v, v);
        one(-v, v);
    }
    std::printf("atan2out_count %ld\n", n);
    std::printf("atan2out_maxerr %.3e\n", worst);
}

int main()
{
    check_atan2();
    check_atan2_out();
    check_fft<64>();
    check_fft<128>();
    check_fft<256>();
    check_fft<512>();
    check_fft<1024>();
    check_fft<1024, 1>();  // alternative radix plan 16 x 8 x 8
    check_fft<2048>();
    check_fft<4096>();   // whole-row plans of the large 2-D transforms
    check_fft<8192>();
    const int M = 512;
    for (int orient = 0; orient < 2; orient++) {
        check_gather<64>(M, 0, 0, 0.25f, 0.75f, orient, 32);
        check_gather<128>(M, M - 1, M - 2, 0.5f, 0.125f, orient, 96);
        check_gather<256>(M, 7, M - 1, 0.9f, 0.01f, orient, 240);
        check_gather<512>(M, M - 3, 5, 0.3f, 0.6f, orient, 496);
        check_gather<1024>(M, 13, M - 7, 0.77f, 0.33f, orient, 1016);
        check_gather<2048>(M, M - 1, M - 1, 0.999f, 0.001f, orient, 2044);
        check_gather<1024>(M, 2, 3, 0.0f, 0.0f, orient, 0);
        check_gather<64, 1>(M, 1, 2, 0.4f, 0.2f, orient, 48);
        check_gather<256, 1>(M, M - 2, 9, 0.7f, 0.9f, orient, 248);
        check_gather<1024, 1>(M, 5, M - 1, 0.1f, 0.5f, orient, 1020);
        check_gather<2048, 1>(M, M - 4, 3, 0.6f, 0.3f, orient, 2046);
    }
    return 0;
}
