// aux_kernels.cu -- setup and per-step helper kernels of the engine.
#include <cstdlib>
#include <algorithm>

#include "aux_kernels.cuh"
#include "pass_impl.cuh"
#include "atan_ff.cuh"

namespace atmwfs {

// ---------------------------------------------------------------------------
// halo-padded periodic screen copies (one-time setup)
//   orient 0: P[yp][xp] = S[(yp - kPadY) mod M][(xp - kPadX) mod M]
//   orient 1: P[yp][xp] = S[(xp - kPadX) mod M][(yp - kPadY) mod M]
// ---------------------------------------------------------------------------
__global__ void k_pad_screen(const float* __restrict__ S, int M, float* __restrict__ P, int Wp, int Hp, int orient)
{
    __shared__ float tileT[32][33];
    const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
    if (orient == 0) {
        for (int r = threadIdx.y; r < 32; r += blockDim.y) {
            const int yp = by + r, xp = bx + threadIdx.x;
            if (yp < Hp && xp < Wp) {
                const int a = ((yp - kPadY) % M + M) % M, b = ((xp - kPadX) % M + M) % M;
                P[(size_t)yp * Wp + xp] = S[(size_t)a * M + b];
            }
        }
        return;
    }
    // transposed: read a 32 x 32 block of S coalesced, write it transposed
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int xp = bx + r, yp = by + threadIdx.x;  // element (yp, xp) = S[(xp-4)][(yp-1)]
        const int a = ((xp - kPadX) % M + M) % M, b = ((yp - kPadY) % M + M) % M;
        tileT[r][threadIdx.x] = S[(size_t)a * M + b];
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int yp = by + r, xp = bx + threadIdx.x;
        if (yp < Hp && xp < Wp) P[(size_t)yp * Wp + xp] = tileT[threadIdx.x][r];
    }
}

cudaError_t pad_screen(const float* S, int M, float* P, int Wp, int Hp, int orient, cudaStream_t st)
{
    dim3 grid((Wp + 31) / 32, (Hp + 31) / 32), block(32, 8);
    k_pad_screen<<<grid, block, 0, st>>>(S, M, P, Wp, Hp, orient);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// r0 measurement: sum over ii < M - dpix, all jj of (S[jj][ii] - S[jj][ii+dpix])^2
// (AtmosphericTurbulence.c:2246-2263); float per thread, double per block.
// ---------------------------------------------------------------------------
__global__ void k_lagsq(const float* __restrict__ S, int M, int dpix, double* acc)
{
    double local = 0.0;
    const long n = (long)M * M;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int ii = (int)(i % M);
        if (ii < M - dpix) {
            const double d = (double)S[i] - (double)S[i + dpix];
            local += d * d;
        }
    }
    __shared__ double red[32];
    for (int o = 16; o > 0; o >>= 1) local += __shfl_down_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = local;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (threadIdx.x == 0) atomicAdd(acc, v);
    }
}

cudaError_t lag_sumsq(const float* S, int M, int dpix, double* acc, cudaStream_t st)
{
    k_lagsq<<<4 * 152, 256, 0, st>>>(S, M, dpix, acc);
    return cudaGetLastError();
}

// S[i] = (float)((double)S[i] * f)  (the reference's float *= double)
__global__ void k_scale(float* __restrict__ S, long n, double f)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        S[i] = (float)((double)S[i] * f);
}

cudaError_t scale_screen(float* S, long n, double f, cudaStream_t st)
{
    k_scale<<<4 * 152, 256, 0, st>>>(S, n, f);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// science-output unwrap: bin relaxation (AtmosphericTurbulence.c:3629-3941
// float branch).  One CTA per science instance.  The twelve sweeps vote
// +-0.2 (8-neighbourhood) or +-0.15 (distance-2 ring) into a float change
// map; votes reach each bin in the reference's loop order so that the float
// rounding of the accumulation is reproduced.
// ---------------------------------------------------------------------------
struct Sweep {
    int dx, dy, ox, oy;
    double c;
};
__constant__ Sweep c_sweeps[12] = {
    {+1, 0, 0, 0, 0.2},   {0, +1, 0, 0, 0.2},   {+1, +1, 0, 0, 0.2},  {+1, -1, 0, 1, 0.2},
    {+2, 0, 0, 0, 0.15},  {0, -2, 0, 2, 0.15},  {-1, -2, 1, 2, 0.15}, {+1, -2, 0, 2, 0.15},
    {-2, -2, 2, 2, 0.15}, {+2, -2, 0, 2, 0.15}, {+2, -1, 0, 1, 0.15}, {-2, -1, 2, 1, 0.15},
};

__device__ __forceinline__ float vote_acc(float ch, double c) { return __double2float_rn((double)ch + c); }

// ppf[i] = (double)pb[i] + pi rounded toward -inf to float: for a float x,
// x > (double)pb[i] + pi  <=>  x > ppf[i], so the reference's double
// comparisons run as float comparisons with identical outcomes.
//
// The votes are found with float compares only and applied afterwards, in
// the same order, with the reference's double accumulation: most bins get
// none (a vote needs two neighbouring bins more than pi apart), so the
// FP64 additions -- slow on this part, and otherwise evaluated for all 48
// candidate votes of every bin -- run only where a vote fired.
__device__ float bin_votes(const float* pb, const float* ppf, int nb, int bx, int by)
{
    const float pv = pb[by * nb + bx];
    const float pvp = ppf[by * nb + bx];
    // bit 4 s + 2 k + m: vote m of role slot k of sweep s fired; the same bit
    // of neg: that vote is -c
    unsigned long long fired = 0ull, neg = 0ull;
#pragma unroll
    for (int s = 0; s < 12; s++) {
        const Sweep w = c_sweeps[s];
        // role A: this bin is index1, partner index2 = (bx + dx, by + dy)
        // role B: this bin is index2, partner index1 = (bx - dx, by - dy)
        const int ax = bx + w.dx, ay = by + w.dy;
        const int bxp = bx - w.dx, byp = by - w.dy;
        const bool va = ax >= 0 && ax < nb && ay >= 0 && ay < nb;
        const bool vb = bxp >= 0 && bxp < nb && byp >= 0 && byp < nb;
        const bool a_first = (w.dx < 0) || (w.dx == 0 && w.dy < 0);
#pragma unroll
        for (int k = 0; k < 2; k++) {
            const bool doA = (k == 0) == a_first;
            const unsigned long long b0 = 1ull << (4 * s + 2 * k), b1 = b0 << 1;
            if (doA && va) {
                const int j = ay * nb + ax;
                if (pb[j] > pvp) fired |= b0;                         // pv2 > pv + pi: +c
                if (pv > ppf[j]) { fired |= b1; neg |= b1; }          // pv > pv2 + pi: -c
            }
            if (!doA && vb) {
                const int j = byp * nb + bxp;
                if (pv > ppf[j]) { fired |= b0; neg |= b0; }          // pv > pv1 + pi: -c
                if (pb[j] > pvp) fired |= b1;                         // pv1 > pv + pi: +c
            }
        }
    }
    float ch = 0.0f;
    while (fired) {
        const int b = __ffsll((long long)fired) - 1;
        fired &= fired - 1ull;
        const double c = c_sweeps[b >> 2].c;
        ch = vote_acc(ch, ((neg >> b) & 1ull) ? -c : c);
    }
    return ch;
}

__global__ void k_unwrap(const InstDev* __restrict__ insts, const int* __restrict__ list, unsigned* status,
                         int* iters_out, const float2* __restrict__ atan_tab)
{
    pdl_gate();
    const InstDev& I = insts[list[blockIdx.x]];
    const int nb = I.nb;
    if (nb <= 0) return;
    const int n = nb * nb;
    extern __shared__ float sh[];
    float* pb = sh;
    float* ch = sh + n;
    float* ppf = sh + 2 * n;
    // vote maximum and flip count, double-buffered by iteration parity so
    // that one iteration needs two barriers: the counters of iteration it-1
    // are cleared in iteration it after its first barrier, when every thread
    // has read them, and are next written after its second barrier
    __shared__ unsigned s_max[2];
    __shared__ int s_cnt[2];
    const double kTwoPi = 2.0 * 3.14159265358979323846;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        // the fixed-point sums back to float (one rounding; the scaling by
        // 2^-kBinFrac is exact), then (float)atan2((double)im, (double)re)
        // without FP64 (atan_ff.cuh)
        const float q = 1.0f / (float)(1ull << kBinFrac);
        const float re = __ll2float_rn((long long)I.bins[i]) * q;
        const float im = __ll2float_rn((long long)I.bins[n + i]) * q;
        const float v = atan2_ff(im, re, atan_tab);
        pb[i] = v;
        ppf[i] = __double2float_rd((double)v + kTwoPi * 0.5);
        I.bins[i] = 0ull;
        I.bins[n + i] = 0ull;
    }
    if (threadIdx.x < 2) { s_max[threadIdx.x] = 0u; s_cnt[threadIdx.x] = 0; }
    __syncthreads();
    int chiter = 0, chcnt0cnt = 0, par = 0;
    double plim = 1.0;
    while (plim > 0.51 && chiter < 1000 && chcnt0cnt < 5) {
        chiter++;
        unsigned umax = 0u;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const float c = bin_votes(pb, ppf, nb, i % nb, i / nb);
            ch[i] = c;
            umax = max(umax, __float_as_uint(fabsf(c)));
        }
        // one shared atomic per warp (max is order-free)
        umax = __reduce_max_sync(0xffffffffu, umax);
        if ((threadIdx.x & 31) == 0) atomicMax(&s_max[par], umax);
        __syncthreads();
        plim = (double)__uint_as_float(s_max[par]) - 0.001;
        if (plim < 0.5) plim = 0.5;
        if (threadIdx.x == 0) { s_max[par ^ 1] = 0u; s_cnt[par ^ 1] = 0; }
        // for a float c: c > plim <=> c > rd(plim) (rd: round toward -inf to float)
        const float plimf = __double2float_rd(plim);
        int cnt = 0;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const int bx = i % nb, by = i / nb;
            const bool interior = bx > 1 && by > 1 && bx < nb - 2 && by < nb - 2;
            const float c = ch[i];
            const int dir = c > plimf ? 1 : (c < -plimf ? -1 : 0);
            if (dir != 0 && interior) cnt++;
            // the FP64 update only in warps where a bin flips (a plain
            // branch would be evaluated speculatively for every bin)
            if (__any_sync(__activemask(), dir != 0) && dir != 0) {
                const float v = (float)((double)pb[i] + (dir > 0 ? kTwoPi : -kTwoPi));
                pb[i] = v;
                ppf[i] = __double2float_rd((double)v + kTwoPi * 0.5);
            }
        }
        cnt = __reduce_add_sync(0xffffffffu, cnt);
        if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(&s_cnt[par], cnt);
        __syncthreads();
        if (s_cnt[par] == 0) chcnt0cnt++;
        else chcnt0cnt = 0;
        par ^= 1;
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) I.peak[i] = pb[i];
    if (threadIdx.x == 0 && iters_out) iters_out[list[blockIdx.x]] = chiter;
}

cudaError_t unwrap_bins(const InstDev* insts, const int* list, int nsci, int maxnb, unsigned* status, int* iters,
                        const float2* atan_tab, cudaStream_t st)
{
    if (nsci <= 0) return cudaSuccess;
    const size_t sm = (size_t)3 * maxnb * maxnb * sizeof(float);
    if (sm > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k_unwrap, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
    }
    return launch_gated(k_unwrap, dim3(nsci), dim3(512), sm, st, insts, list, status, iters, atan_tab);
}

// final science phase: pha + 2 pi round((phasum - pha - peak[bin]) / 2 pi)
// (AtmosphericTurbulence.c:3918-3941)
__global__ void k_sci_apply(const InstDev* __restrict__ insts, const int* __restrict__ list, const int* d_step)
{
    pdl_gate();
    const InstDev& I = insts[list[blockIdx.y]];
    const int Nout = I.Nout, nb = I.nb;
    const int step = d_step ? *d_step : 0;
    float* pha = I.out_pha + (size_t)(step % I.ring) * I.ostride;
    const short* __restrict__ binx = I.binx;
    const float* __restrict__ peakv = I.peak;
    const float* __restrict__ psum = I.phisum;
    // one row per block iteration; four columns per thread as 16-byte vectors
    // when the row length allows, else one column per thread
    const bool v4 = (Nout % 4 == 0) && ((reinterpret_cast<uintptr_t>(pha) & 15) == 0) &&
                    ((reinterpret_cast<uintptr_t>(psum) & 15) == 0);
    for (int jj = blockIdx.x; jj < Nout; jj += gridDim.x) {
        const int bj = nb > 0 ? binx[jj] * nb : 0;
        const size_t ro = (size_t)jj * Nout;
        const float2* __restrict__ gs = I.gsum ? I.gsum + (size_t)(jj + I.off) * I.wstride + I.off : nullptr;
        const float sc = I.scoeff[0];
        auto one = [&](float p, float s, int ii) {
            const float peak = nb > 0 ? peakv[bj + binx[ii]] : 0.0f;
            float d1, e1, d2, e2;
            two_sum(s, -p, d1, e1);
            two_sum(d1, -peak, d2, e2);
            return add_2pi_multiple(p, round_2pi(d2, e1 + e2));
        };
        if (v4) {
            for (int i4 = threadIdx.x; i4 < Nout / 4; i4 += blockDim.x) {
                const int ii = 4 * i4;
                const float4 p = *reinterpret_cast<const float4*>(pha + ro + ii);
                float4 s;
                if (gs) {
                    const float2 g0 = gs[ii], g1 = gs[ii + 1], g2 = gs[ii + 2], g3 = gs[ii + 3];
                    s = make_float4(fmaf(sc, g0.x, sc * g0.y), fmaf(sc, g1.x, sc * g1.y), fmaf(sc, g2.x, sc * g2.y),
                                    fmaf(sc, g3.x, sc * g3.y));
                } else {
                    s = *reinterpret_cast<const float4*>(psum + ro + ii);
                }
                *reinterpret_cast<float4*>(pha + ro + ii) =
                    make_float4(one(p.x, s.x, ii), one(p.y, s.y, ii + 1), one(p.z, s.z, ii + 2), one(p.w, s.w, ii + 3));
            }
        } else {
            for (int ii = threadIdx.x; ii < Nout; ii += blockDim.x)
                pha[ro + ii] = one(pha[ro + ii], gs ? fmaf(sc, gs[ii].x, sc * gs[ii].y) : psum[ro + ii], ii);
        }
    }
}

cudaError_t sci_apply(const InstDev* insts, const int* list, int nsci, int maxnout, const int* d_step, cudaStream_t st)
{
    if (nsci <= 0) return cudaSuccess;
    const int bx = maxnout < 256 ? maxnout : 256;
    return launch_gated(k_sci_apply, dim3(bx, nsci), dim3(256), 0, st, insts, list, d_step);
}

// Layer sum of one window group, from the top layer down with a two-sum
// (the order of the reference's accumulation, AtmosphericTurbulence.c:2909-2916,
// without the per-layer Scoeff that factors out of the sum): four pixels per
// thread as 16-byte vectors, every layer requested before the sums.
__global__ void __launch_bounds__(256) k_group_sum(const GroupSumJob* __restrict__ jobs, int L)
{
    pdl_gate();
    const GroupSumJob& J = jobs[blockIdx.y];
    const long n4 = (long)J.side * J.side / 4;
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n4; k += (long)gridDim.x * blockDim.x) {
        float hi[4] = {0.0f, 0.0f, 0.0f, 0.0f}, lo[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        float4 w[kMaxLayers];
#pragma unroll
        for (int l = 0; l < kMaxLayers; l++)
            if (l < L) w[l] = __ldg(reinterpret_cast<const float4*>(J.win[l]) + k);
#pragma unroll
        for (int l = kMaxLayers - 1; l >= 0; l--) {
            if (l >= L) continue;
            const float wv[4] = {w[l].x, w[l].y, w[l].z, w[l].w};
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const float s = __fadd_rn(hi[j], wv[j]);
                const float bp = __fsub_rn(s, hi[j]);
                const float e = __fadd_rn(__fsub_rn(hi[j], __fsub_rn(s, bp)), __fsub_rn(wv[j], bp));
                hi[j] = s;
                lo[j] = __fadd_rn(lo[j], e);
            }
        }
        float4* o = reinterpret_cast<float4*>(J.out) + 2 * k;
        o[0] = make_float4(hi[0], lo[0], hi[1], lo[1]);
        o[1] = make_float4(hi[2], lo[2], hi[3], lo[3]);
    }
}

cudaError_t group_sums(const GroupSumJob* jobs, int njobs, int L, int maxside, cudaStream_t st)
{
    if (njobs <= 0) return cudaSuccess;
    const long n4 = (long)maxside * maxside / 4;
    const long b = (n4 + 255) / 256;
    return launch_gated(k_group_sum, dim3((unsigned)(b < 1024 ? b : 1024), (unsigned)njobs), dim3(256), 0, st, jobs, L);
}

__global__ void k_step_advance(int* d_step)
{
    pdl_gate();
    *d_step += 1;
}

cudaError_t step_advance(int* d_step, cudaStream_t st)
{
    return launch_gated(k_step_advance, dim3(1), dim3(1), 0, st, d_step);
}

// ---------------------------------------------------------------------------
// master-screen synthesis (AtmosphericTurbulence.c:643-855)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1)
{
#pragma unroll
    for (int r = 0; r < 10; r++) {
        const uint32_t lo0 = 0xD2511F53u * c[0], hi0 = __umulhi(0xD2511F53u, c[0]);
        const uint32_t lo1 = 0xCD9E8D57u * c[2], hi1 = __umulhi(0xCD9E8D57u, c[2]);
        const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

// ---------------------------------------------------------------------------
// Frame copy-out into the caller's sink (pinned host or device memory).
// The host link, not the issuer, bounds a device-to-host copy (about 190
// GB/s here for the copy engine and for SM stores alike), and 8 CTAs of
// plain 16-byte stores reach 185 GB/s while holding 8 of the 152 SMs; the
// copy engine reading the frames meanwhile slows the passes more (measured
// on the batched series: 29,291 frames/s end to end with 8 copy CTAs, 29,153
// with 16, 27,811 with 32, 26,280 with the copy engine).
// ---------------------------------------------------------------------------
__global__ void k_copy_out(const float4* __restrict__ s0, float4* __restrict__ d0, long n0,
                           const float4* __restrict__ s1, float4* __restrict__ d1, long n1)
{
    const long stride = (long)gridDim.x * blockDim.x;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n0; i += stride) d0[i] = s0[i];
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n1; i += stride) d1[i] = s1[i];
}

cudaError_t copy_out(const float4* src0, float4* dst0, long n0, const float4* src1, float4* dst1, long n1,
                     cudaStream_t st)
{
    if (!dst0) n0 = 0;
    if (!dst1) n1 = 0;
    if (n0 + n1 == 0) return cudaSuccess;
    // CTAs of the copy (ATMWFS_COPY_CTAS overrides the measured default)
    static const int ctas = [] {
        const char* e = getenv("ATMWFS_COPY_CTAS");
        const int v = e ? atoi(e) : 0;
        return v >= 1 && v <= 152 ? v : 8;
    }();
    k_copy_out<<<ctas, 256, 0, st>>>(src0, dst0, n0, src1, dst1, n1);
    return cudaGetLastError();
}

// Spectrum A(k) exp(i 2 pi u), written at its fftshifted position (the
// reference applies permut() before the FFT, :782).
__global__ void k_screen_spectrum(uint64_t seed, uint32_t stream, int M, double fo, double fi, float2* __restrict__ C)
{
    const long n = (long)M * M;
    const int lg = __ffs(M) - 1;
    const float fo2 = (float)(fo * fo), fif = (float)fi;
    for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < n; p += (long)gridDim.x * blockDim.x) {
        uint32_t c[4] = {(uint32_t)p, stream, 0u, 0u};
        philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
        const float u = (float)(c[0] >> 8) * (1.0f / 16777216.0f);
        const float u1 = ((float)(c[1] >> 8) + 1.0f) * (1.0f / 16777216.0f);
        const float u2 = (float)(c[2] >> 8) * (1.0f / 16777216.0f);
        const float g = sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
        const int ii = (int)p & (M - 1), jj = (int)(p >> lg);  // M is a power of two
        const float dx = (float)(ii - M / 2), dy = (float)(jj - M / 2);
        const float r2 = dx * dx + dy * dy;
        const float d = sqrtf(r2 + fo2);
        const float gi = g * sqrtf(expf(-r2 / fif / fif));
        float a = gi / powf(d, 11.0f / 6.0f);
        if (ii == M / 2 && jj == M / 2) a = 0.0f;
        float s, co;
        sincospif(2.0f * u, &s, &co);
        const int io = (ii + M / 2) % M, jo = (jj + M / 2) % M;
        C[(size_t)jo * M + io] = make_float2(a * co, a * s);
    }
}

cudaError_t screen_spectrum(uint64_t seed, uint32_t stream, int M, double fo, double fi, float2* C, cudaStream_t st)
{
    k_screen_spectrum<<<8 * 152, 256, 0, st>>>(seed, stream, M, fo, fi, C);
    return cudaGetLastError();
}

// Structure function D(lx, ly) of the real and imaginary parts at lags
// (1..2)^2, circular (fft_structure_function, info.c:1670-1690, from its
// definition).  acc[8]: [part][lag] sums.  Each thread keeps its sums in
// float-float: the difference of two floats exactly (two-sum), its square
// as an exact product plus the cross term, accumulated by two-sums (about
// 46 bits, against the 53 of a double sum); the FP64 pipe, slow on this
// part, is used only for the per-warp totals.
__global__ void k_strf(const float2* __restrict__ F, int M, double* acc)
{
    float hi[8], lo[8];
#pragma unroll
    for (int q = 0; q < 8; q++) hi[q] = lo[q] = 0.0f;
    const long n = (long)M * M;
    const int lg = __ffs(M) - 1, mk = M - 1;  // M is a power of two
    auto add_sq = [&](int q, float a, float b) {
        float dh, dl;
        ff_two_sum(a, -b, dh, dl);
        const float p = ff_mul(dh, dh);
        const float pe = ff_fma(ff_add(dh, dh), dl, ff_fma(dh, dh, -p));
        float s, e;
        ff_two_sum(hi[q], p, s, e);
        hi[q] = s;
        lo[q] = ff_add(lo[q], ff_add(e, pe));
    };
    for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < n; p += (long)gridDim.x * blockDim.x) {
        const int x = (int)p & mk, y = (int)(p >> lg);
        const float2 a = F[p];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int lx = 1 + (q & 1), ly = 1 + (q >> 1);
            const float2 b = F[(size_t)((y + ly) & mk) * M + ((x + lx) & mk)];
            add_sq(q, a.x, b.x);
            add_sq(4 + q, a.y, b.y);
        }
    }
    // warp totals in float-float, then one double atomic per warp and sum
#pragma unroll
    for (int q = 0; q < 8; q++) {
        float h = hi[q], l = lo[q];
        for (int o = 16; o > 0; o >>= 1) {
            const float h2 = __shfl_down_sync(0xffffffffu, h, o), l2 = __shfl_down_sync(0xffffffffu, l, o);
            float s, e;
            ff_two_sum(h, h2, s, e);
            h = s;
            l = ff_add(l, ff_add(l2, e));
        }
        if ((threadIdx.x & 31) == 0) atomicAdd(&acc[q], (double)h + (double)l);
    }
}

cudaError_t strf_lags(const float2* F, int M, double* acc, cudaStream_t st)
{
    k_strf<<<4 * 152, 256, 0, st>>>(F, M, acc);
    return cudaGetLastError();
}

// o = v s with s = sh + sl (float pair of the double scale): the exact
// product v sh (two-product) plus v sl, rounded once -- the float of the
// double product except when that lies within about 2^-46 of a midpoint.
__device__ __forceinline__ float scale_ff(float v, float sh, float sl)
{
    const float p = ff_mul(v, sh);
    return ff_add(p, ff_fma(v, sl, ff_fma(v, sh, -p)));
}

__global__ void k_split_scale(const float2* __restrict__ F, long n, float s1h, float s1l, float s2h, float s2l,
                              float* o1, float* o2)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const float2 v = F[i];
        if (o1) o1[i] = scale_ff(v.x, s1h, s1l);
        if (o2) o2[i] = scale_ff(v.y, s2h, s2l);
    }
}

cudaError_t split_scale(const float2* F, long n, double s1, double s2, float* o1, float* o2, cudaStream_t st)
{
    const float s1h = (float)s1, s2h = (float)s2;
    k_split_scale<<<4 * 152, 256, 0, st>>>(F, n, s1h, (float)(s1 - (double)s1h), s2h, (float)(s2 - (double)s2h), o1, o2);
    return cudaGetLastError();
}

}  // namespace atmwfs

namespace atmwfs {

// ---------------------------------------------------------------------------
// per-layer phase windows of one instance at the last completed step: the
// same Keys bicubic samples the passes form (horizontal taps first, then
// the vertical ones), times the instance's Scoeff, in screen orientation
// ---------------------------------------------------------------------------
struct LayerScales {
    float s[kMaxLayers];
    const float* scr[kMaxLayers];
};

__global__ void k_windows(LayerScales ls, int M, const LayerPos* __restrict__ pos, int poscap, int ninst, int gidx,
                          int L, const int* __restrict__ d_step, int W, float* __restrict__ out)
{
    const int l = blockIdx.y;
    const int step = *d_step - 1;
    const LayerPos p = pos[((size_t)(step % poscap) * ninst + gidx) * L + l];
    float wx[4], wy[4];
    keys_weights(p.fx, wx);
    keys_weights(p.fy, wy);
    const float* S = ls.scr[l];
    const long n = (long)W * W;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int y = (int)(i / W), x = (int)(i % W);
        float h[4];
#pragma unroll
        for (int b = 0; b < 4; b++) {
            const int sy = ((p.iy + y - 1 + b) % M + M) % M;
            const float* r = S + (size_t)sy * M;
            const int c0 = p.ix + x - 1;
            h[b] = wx[0] * r[((c0) % M + M) % M] + wx[1] * r[((c0 + 1) % M + M) % M] +
                   wx[2] * r[((c0 + 2) % M + M) % M] + wx[3] * r[((c0 + 3) % M + M) % M];
        }
        out[(size_t)l * n + i] = (wy[0] * h[0] + wy[1] * h[1] + wy[2] * h[2] + wy[3] * h[3]) * ls.s[l];
    }
}

cudaError_t windows(const float* const* screens, const float* scoeff, int L, int M, const LayerPos* pos, int poscap,
                    int ninst, int gidx, const int* d_step, int W, float* out, cudaStream_t st)
{
    if (L > kMaxLayers) return cudaErrorInvalidValue;
    LayerScales ls;
    for (int l = 0; l < L; l++) {
        ls.s[l] = scoeff ? scoeff[l] : 1.0f;
        ls.scr[l] = screens[l];
    }
    const long n = (long)W * W;
    const unsigned bx = (unsigned)std::min<long>((n + 255) / 256, 1024);
    k_windows<<<dim3(bx, L), 256, 0, st>>>(ls, M, pos, poscap, ninst, gidx, L, d_step, W, out);
    return cudaGetLastError();
}

}  // namespace atmwfs
