// pass_impl.cuh -- the row-pass kernel of the wavefront-series engine.
//
// A 2-D Fresnel hop U' = IFFT2(H FFT2(U)) with the separable transfer
// function H(fx, fy) = Hx(fx) Hy(fy) (Fresnel_propagate_wavefront,
// src/WFpropagate/WFpropagate.c:68-152) is the product of a 1-D propagation
// along x and one along y.  Every pass below works on whole rows held by one
// CTA and stores its result transposed, so consecutive passes alternate
// between the two axes.  One pass does [1-D propagation, phase-screen
// gather + phasor, 1-D propagation]: a frame with P hops costs P + 1 passes.
#pragma once
#include "engine.cuh"
#include "epi_math.cuh"
#include "fft_half.cuh"
#include "gather_core.cuh"

namespace atmwfs {

// ---------------------------------------------------------------------------
// PTX helpers: mbarrier, TMA tile load, global timer
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t gtimer_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, int count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, int parity)
{
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

__device__ __forceinline__ void tma_load_2d(float* dst, const CUtensorMap* map, int x, int y, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// 16-byte asynchronous copy global -> shared (both addresses 16-byte aligned)
__device__ __forceinline__ void cp_async16(void* dst, const void* src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)),
                 "l"(static_cast<uint64_t>(__cvta_generic_to_global(src)))
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }
// every commit group but the most recent one has completed
__device__ __forceinline__ void cp_async_wait_group1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

// Every thread polls the barrier with the same time limit; the CTA agrees
// on the outcome through __syncthreads_or, so a timeout never splits it.
__device__ __forceinline__ bool cta_wait_tile(uint64_t* bar, int parity, unsigned* status)
{
    const uint64_t limit = 1000000000ull;  // 1 s
    const uint64_t t0 = gtimer_ns();
    int timed_out = 0;
    while (!mbar_try_wait(bar, parity)) {
        if (gtimer_ns() - t0 > limit) { timed_out = 1; break; }
    }
    if (__syncthreads_or(timed_out)) {
        if (threadIdx.x == 0 && status) atomicOr(status, kStatTmaTimeout);
        // let copies still in flight land before the CTA retires
        const uint64_t t1 = gtimer_ns();
        while (!mbar_try_wait(bar, parity)) {
            if (gtimer_ns() - t1 > limit) break;
        }
        __syncthreads();
        return false;
    }
    return true;
}

// ---------------------------------------------------------------------------
// geometry
// ---------------------------------------------------------------------------
template <int N, int RR, int V = 0>
struct PassGeom {
    static constexpr int T = Plan<N, V>::T;
    static constexpr int E = Plan<N, V>::E;
    static constexpr int NT = T * RR;
    static constexpr int RS = row_stride<N>();
    static constexpr int NBOX = N / kBoxW + 1;
    static constexpr int TROWS = RR + 3;
    static constexpr size_t XBYTES = size_t(RR) * RS * 8;
    static constexpr size_t TILE_BYTES = size_t(NBOX) * TROWS * kBoxW * 4;  // screen tile (window kernel)
    static constexpr size_t WIN_BYTES = size_t(RR) * N * 4;          // staged window rows, [RR][N]
    static constexpr int NJ = RR > 16 ? 3 : 2;                        // bin rows a tile can touch
    static constexpr size_t COLSUM_BYTES = size_t(NJ) * N * 8;        // epilogue column sums, [NJ][N]
    AW_HD static constexpr size_t round128(size_t b) { return (b + 127) / 128 * 128; }
    AW_HD static constexpr size_t mx(size_t a, size_t b) { return a > b ? a : b; }
    // Layout: [exchange rows | window rows of the plane's first layer |
    // (staged transfer tables)]; the epilogue's column sums reuse the window
    // rows once the phasor is applied.
    static constexpr size_t HBYTES = size_t(2) * N * 8;  // the pass's two hop tables
    AW_HD static constexpr size_t win_offset() { return round128(XBYTES); }
    AW_HD static constexpr size_t h_offset(int ops)
    {
        const bool gather = (ops & (OP_GATHER | OP_EPI)) != 0, epi = (ops & OP_EPI) != 0;
        if (!gather) return round128(XBYTES);
        return round128(win_offset() + mx(WIN_BYTES, epi ? COLSUM_BYTES : 0));
    }
    AW_HD static constexpr size_t smem(int ops, bool hs = false)
    {
        return h_offset(ops) + ((hs && (ops & (OP_PROP1 | OP_PROP2)) != 0) ? HBYTES : 0);
    }
    static_assert(N % (RR) == 0, "rows per CTA must divide N");
};

// One layer's tile as NBOX box copies, issued by lane 0 of every warp of the
// CTA (warp w takes boxes w, w + nwarps, ...): a single issuing thread would
// hold its warp, and with it the whole CTA at the next barrier, for the
// length of the issue sequence.  Warp 0 posts the tile's byte count with its
// arrival; boxes of other warps may land before that, which leaves the
// phase's transaction count negative until the arrival and is allowed.
// Called by every thread of the CTA (threads other than lane 0 return).
template <int N, int RR>
__device__ __forceinline__ void tma_issue_layer(const TmaSet& maps, int orient, int l, const TileGeom& g, float* tile,
                                                uint64_t* bar, int tid, int nthreads)
{
    using G = PassGeom<N, RR>;
    if (tid & 31) return;
    const int w = tid >> 5, nw = (nthreads + 31) >> 5;
    if (w == 0) mbar_expect_tx(bar, (uint32_t)G::TILE_BYTES);
    const CUtensorMap* m = &maps.m[orient][l];
#pragma unroll 1
    for (int k = w; k < G::NBOX; k += nw) tma_load_2d(tile + k * G::TROWS * kBoxW, m, g.xs + k * kBoxW, g.ys, bar);
}

// One 1-D transform of the row in v through a runtime stage loop: every
// stage of every transform of the kernel runs through the same code of its
// radix, which keeps the kernel inside the instruction cache.  ds = -1
// forward, +1 inverse; rev walks the radix sequence backwards (the inverse of
// a propagation, which starts from the forward's register layout and ends in
// the natural layout x[t + e T]).
// Two-stage plans (N <= 1024) with the radices, strides and exchange
// indices known at compile time: stage A (stride 1, no twiddles), the
// exchange, stage B (stride RA).
template <int N, int T, int E, int RA, int RB>
__device__ __forceinline__ void fft2_ct(float2* v, float2* xrow, int t, const float2* __restrict__ tws1)
{
    stage_dft<E, RA, -1>(v);
    row_sync<T>();
    stage_store<N, T, E, RA, 1>(v, xrow, t);
    row_sync<T>();
    stage_load<N, T, E, RB>(v, xrow, t);
    stage_twiddle_rt<N, T, E, RB>(v, t, tws1, RA);
    stage_dft<E, RB, -1>(v);
}

// Square two-stage plans with one work item per thread (64 = 8 x 8,
// 256 = 16 x 16, 1024 = 32 x 32): the second stage's twiddles of a thread,
// w^(t r) for r = 1 .. R - 1, are the same in every transform of every row the
// thread holds (forward and inverse alike), so a pass can load them once into
// registers instead of reading the table in each of its four transforms.
template <int N, int V = 0>
AW_HD constexpr bool reg_twiddles()
{
    return Stages<N, V>::S == 2 && Stages<N, V>::R0 == Stages<N, V>::R1 && Plan<N, V>::E == Stages<N, V>::R1;
}
template <int N, int V = 0>
AW_HD constexpr int reg_twiddle_count() { return reg_twiddles<N, V>() ? Stages<N, V>::R1 - 1 : 1; }

// The same transform with the second stage's twiddles in registers:
// twr[r - 1] = w^((t mod RA) r), RB = E (one work item per thread).
template <int N, int T, int E, int RA, int RB>
__device__ __forceinline__ void fft2_ct_r(float2* v, float2* xrow, int t, const float2* twr)
{
    static_assert(E == RB, "one work item per thread");
    stage_dft<E, RA, -1>(v);
    row_sync<T>();
    stage_store<N, T, E, RA, 1>(v, xrow, t);
    row_sync<T>();
    stage_load<N, T, E, RB>(v, xrow, t);
#pragma unroll
    for (int r = 1; r < RB; r++) v[r] = cmul(v[r], twr[r - 1]);
    stage_dft<E, RB, -1>(v);
}

// Three-stage plans with compile-time radices and strides (the alternative
// plans, see Plan): stage A (stride 1), exchange, stage B (stride RA),
// exchange, stage C (stride RA RB); twsB / twsC are the stage tables.
template <int N, int T, int E, int RA, int RB, int RC>
__device__ __forceinline__ void fft3_ct(float2* v, float2* xrow, int t, const float2* __restrict__ twsB,
                                        const float2* __restrict__ twsC)
{
    stage_dft<E, RA, -1>(v);
    row_sync<T>();
    stage_store<N, T, E, RA, 1>(v, xrow, t);
    row_sync<T>();
    stage_load<N, T, E, RB>(v, xrow, t);
    stage_twiddle_rt<N, T, E, RB>(v, t, twsB, RA);
    stage_dft<E, RB, -1>(v);
    row_sync<T>();
    stage_store<N, T, E, RB, RA>(v, xrow, t);
    row_sync<T>();
    stage_load<N, T, E, RC>(v, xrow, t);
    stage_twiddle_rt<N, T, E, RC>(v, t, twsC, RA * RB);
    stage_dft<E, RC, -1>(v);
}

template <int N, int T, int E, bool RT = false, int V = 0>
__device__ __forceinline__ void fft_rt(float2* v, float2* xrow, int t, const float2* __restrict__ tw, float ds, int rev,
                                       const float2* twr = nullptr)
{
    if (ds > 0.0f) conj_all<E>(v);     // inverse = conj(forward(conj))
    if constexpr (V != 0 && Stages<N, V>::S == 3) {
        constexpr int R0 = Stages<N, V>::R0, R1 = Stages<N, V>::R1, R2 = Stages<N, V>::R2;
        if (rev) fft3_ct<N, T, E, R2, R1, R0>(v, xrow, t, tw + tw_offset<N, V>(1, 1), tw + tw_offset<N, V>(1, 2));
        else fft3_ct<N, T, E, R0, R1, R2>(v, xrow, t, tw + tw_offset<N, V>(0, 1), tw + tw_offset<N, V>(0, 2));
        if (ds > 0.0f) conj_all<E>(v);
        return;
    }
    if constexpr (Stages<N>::S == 2) {
        constexpr int R0 = Stages<N>::R0, R1 = Stages<N>::R1;
        if constexpr (RT && reg_twiddles<N>()) {
            fft2_ct_r<N, T, E, R0, R1>(v, xrow, t, twr);
        } else if constexpr (R0 == R1) {
            fft2_ct<N, T, E, R0, R1>(v, xrow, t, tw + tw_offset<N>(rev, 1));
        } else {
            if (rev) fft2_ct<N, T, E, R1, R0>(v, xrow, t, tw + tw_offset<N>(1, 1));
            else fft2_ct<N, T, E, R0, R1>(v, xrow, t, tw + tw_offset<N>(0, 1));
        }
        if (ds > 0.0f) conj_all<E>(v);
        return;
    }
    int ns = 1, rp = 0, nsp = 1;
#pragma unroll 1
    for (int st = 0; st < Stages<N>::S; st++) {
        const int r = stage_radix<N>(st, rev);
        if (st > 0) {
            row_sync<T>();
            stage_exchange_store<N, T, E>(v, xrow, t, rp, nsp);
            row_sync<T>();
            stage_exchange_load<N, T, E>(v, xrow, t, r);
        }
        stage_compute<N, T, E>(v, t, tw + tw_offset<N>(rev, st), r, ns);
        rp = r;
        nsp = ns;
        ns *= r;
    }
    if (ds > 0.0f) conj_all<E>(v);
}

// 1-D Fresnel propagation (forward FFT, transfer table, inverse FFT) with a
// single copy of the transform code.
template <int N, int T, int E, bool RT = false, int V = 0, bool HSM = false>
__device__ __forceinline__ void prop_row_rt(float2* v, float2* xrow, int t, const float2* __restrict__ tw,
                                            const float2* __restrict__ h, const float2* twr = nullptr)
{
    constexpr int RL = last_radix<N, V>();
    // IFFT(H FFT(x)) = conj(FFT(conj(H FFT(x)))): the first conjugation is
    // folded into the transfer multiply, both transforms run the forward code
#pragma unroll 1
    for (int dir = 0; dir < 2; dir++) {
        fft_rt<N, T, E, RT, V>(v, xrow, t, tw, -1.0f, dir, twr);
        if (dir == 0) {
#pragma unroll
            for (int s = 0; s < E; s++) {
                const float2 a = v[s];
                const float2 b = HSM ? h[last_index<N, T, RL>(t, s)] : __ldg(h + last_index<N, T, RL>(t, s));
                v[s] = make_float2(a.x * b.x - a.y * b.y, -(a.x * b.y + a.y * b.x));
            }
        }
    }
    conj_all<E>(v);
}

// Nearest integer to (hi + lo) / 2 pi, halves rounded up, with the
// remainder evaluated against a two-term 2 pi so that the decision is exact
// to ~1e-7 rad (the reference rounds with (long)(x / 2 pi + 1000.5) - 1000).
__device__ __forceinline__ float round_2pi(float hi, float lo)
{
    const float kInv2Pi = 0.159154943091895336f;
    const float k2PiHi = 6.28125f;
    const float k2PiLo = 0.0019353071795864769f;
    const float kPi = 3.14159265358979323846f;
    float k = floorf(fmaf(hi, kInv2Pi, 0.5f));
    float r = fmaf(-k, k2PiHi, hi);
    r = fmaf(-k, k2PiLo, r) + lo;
    if (r >= kPi) k += 1.0f;
    else if (r < -kPi) k -= 1.0f;
    return k;
}

// exp(i phi) with phi reduced to [-pi, pi] against a two-term 2 pi, then the
// hardware sine/cosine (absolute error ~4e-7 on that range).
__device__ __forceinline__ float2 phasor(float phi)
{
    const float k = rintf(phi * 0.159154943091895336f);
    float r = fmaf(-k, 6.28125f, phi);
    r = fmaf(-k, 0.0019353071795864769f, r);
    float s, c;
    __sincosf(r, &s, &c);
    return make_float2(c, s);
}

__device__ __forceinline__ float add_2pi_multiple(float p, float k)
{
    return fmaf(k, 6.28125f, p) + k * 0.0019353071795864769f;
}

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
    s = a + b;
    const float bp = s - a;
    e = (a - (s - bp)) + (b - bp);
}

// ---------------------------------------------------------------------------
// the pass kernel
// ---------------------------------------------------------------------------
// series passes (as opposed to the unit operators, which have no instance)
#define I_SERIES(ops) (((ops) & (OP_GATHER | OP_EPI)) != 0)

template <int N, int RR, int MINB, int OPS, bool ALIAS, bool HP = false, int V = 0, bool HS = false>
__global__ void __launch_bounds__(Plan<N, V>::T* RR, MINB)
    k_pass(const __grid_constant__ PassArgs a, const __grid_constant__ TmaSet maps, const float2* __restrict__ tw)
{
    using G = PassGeom<N, RR, V>;
    static_assert(!HP || V == 0, "FP16 transforms use the default plan");
    static_assert(!HP || !HS, "FP16 transforms read their tables from global memory");
    constexpr int T = G::T, E = G::E, NT = G::NT, RS = G::RS;
    constexpr bool kEpi = (OPS & OP_EPI) != 0;
    constexpr bool kGather = (OPS & (OP_GATHER | OP_EPI)) != 0;
    extern __shared__ __align__(1024) unsigned char sm[];
    float2* xb = reinterpret_cast<float2*>(sm);
    float* wrows = reinterpret_cast<float*>(sm + G::win_offset());  // [RR][N]
    pdl_gate();

    const int tid = threadIdx.x;
    const int t = tid % T;
    const int rr = tid / T;
    const int y0 = a.row0 + blockIdx.x * RR;
    const int y = y0 + rr;
    const InstDev* I = a.inst ? a.inst + blockIdx.y : nullptr;
    const int step = a.d_step ? *a.d_step : 0;
    float2* xrow = xb + rr * RS;

    const int ltop = a.g_hi - 1;
    const int lbot = a.g_lo;
    // HS: the transfer tables of this pass's hops are copied into shared
    // memory (cp.async, their own commit group) while the field loads, and
    // the transfer multiplies read them there
    constexpr bool kHs = HS && I_SERIES(OPS) && (OPS & (OP_PROP1 | OP_PROP2)) != 0;
    float2* hsm = reinterpret_cast<float2*>(sm + G::h_offset(OPS));
    if constexpr (kHs) {
#pragma unroll
        for (int hp = 0; hp < 2; hp++) {
            if (!(hp == 0 ? (OPS & OP_PROP1) != 0 : (OPS & OP_PROP2) != 0)) continue;
            const float2* src = I->H + (size_t)(hp == 0 ? a.hop1 : a.hop2) * N;
#pragma unroll 4
            for (int k = tid; k < N / 2; k += NT) cp_async16(hsm + hp * N + 2 * k, src + 2 * k);
        }
        cp_async_commit();
    }
    const bool win_copy = kGather && ltop >= lbot;
    if constexpr (kGather) {
        // this CTA's rows of the window of the plane's first layer, copied
        // while the first propagation runs
        if (ltop >= lbot) {
            const float* src = I->win[a.orient][ltop] + (size_t)y0 * I->wstride;
            constexpr int C4 = N / 4;
#pragma unroll 4
            for (int k = tid; k < RR * C4; k += NT) {
                const int r = k / C4, c = k - r * C4;
                cp_async16(wrows + r * N + 4 * c, src + (size_t)r * I->wstride + 4 * c);
            }
            cp_async_commit();
        }
    }

    // second-stage twiddles of the square plans, kept in registers by the
    // series passes (FP32 transforms) without the output epilogue (whose
    // registers they would crowd: measured slower there) in the tile
    // configurations that leave room for them (at most three CTAs per SM)
    constexpr bool kRegTw = reg_twiddles<N, V>() && !HP && MINB <= 3 && I_SERIES(OPS) && (OPS & OP_EPI) == 0 &&
                            (OPS & (OP_PROP1 | OP_PROP2)) != 0;
    float2 twr[reg_twiddle_count<N, V>()];
    if constexpr (kRegTw) {
        constexpr int R = Stages<N>::R1;
#pragma unroll
        for (int r = 1; r < R; r++) twr[r - 1] = __ldg(tw + tw_offset<N>(0, 1) + r * Stages<N>::R0 + (t % Stages<N>::R0));
    }

    float2 v[E];
    if constexpr ((OPS & OP_LOAD) != 0) {
        const float2* src = (I ? I->fld[a.src] : a.ext_in) + (size_t)y * N + t;
#pragma unroll
        for (int e = 0; e < E; e++) v[e] = src[e * T];
    } else {
#pragma unroll
        for (int e = 0; e < E; e++) v[e] = make_float2(1.0f, 0.0f);
    }

    if constexpr ((OPS & (OP_FFT_FWD | OP_FFT_INV)) != 0) {
        fft_rt<N, T, E, false, V>(v, xrow, t, tw, (OPS & OP_FFT_FWD) ? -1.0f : 1.0f, 0);
    } else {
        // phase 0: propagation 1; phase 1: screens of this plane; phase 2:
        // propagation 2 -- a runtime loop, so the transform code appears once
#pragma unroll 1
        for (int ph = 0; ph < 3; ph++) {
            if (ph == 1) {
                if constexpr (kGather) {
                    if (ltop >= lbot) {
                        cp_async_wait_all();
                        __syncthreads();  // every thread's copies have landed
                        // phase of the plane: its layers from the top down,
                        // each window sample times the layer's Scoeff
                        const float* wr = wrows + rr * N + t;
                        const float sc0 = I->scoeff[ltop];
                        float phs[E];
#pragma unroll
                        for (int e = 0; e < E; e++) phs[e] = __fmul_rn(wr[e * T], sc0);
                        for (int l = ltop - 1; l >= lbot; l--) {
                            const float* g = I->win[a.orient][l] + (size_t)y * I->wstride + t;
                            const float sc = I->scoeff[l];
#pragma unroll
                            for (int e = 0; e < E; e++) phs[e] = __fadd_rn(phs[e], __fmul_rn(__ldg(g + e * T), sc));
                        }
#pragma unroll
                        for (int e = 0; e < E; e++) v[e] = cmul(v[e], phasor(phs[e]));
                    }
                }
                continue;
            }
            const bool run = ph == 0 ? ((OPS & OP_PROP1) != 0) : ((OPS & OP_PROP2) != 0);
            if (!run) continue;
            const int hop = ph == 0 ? a.hop1 : a.hop2;
            if constexpr (kHs) {
                if (ph == 0 || (OPS & OP_PROP1) == 0) {
                    // the tables' group is complete (the window copy may still run)
                    if (win_copy && ph == 0) cp_async_wait_group1();
                    else cp_async_wait_all();
                    __syncthreads();
                }
            }
            if constexpr (HP) {
                // FP16 transforms: tw is the FP16 twiddle table, Hh holds N H
                prop_row_h<N, T, E>(v, xrow, t, reinterpret_cast<const __half2*>(tw),
                                    reinterpret_cast<const __half2*>(I->Hh) + (size_t)hop * N);
            } else {
                if constexpr (kHs) {
                    const float2* h = hsm + (ph == 0 ? 0 : N);
                    if constexpr (kRegTw) prop_row_rt<N, T, E, true, V, true>(v, xrow, t, tw, h, twr);
                    else prop_row_rt<N, T, E, false, V, true>(v, xrow, t, tw, h);
                } else {
                    const float2* h = I ? I->H + (size_t)hop * N : (ph == 0 ? a.H1 : a.H2);
                    if constexpr (kRegTw) prop_row_rt<N, T, E, true, V>(v, xrow, t, tw, h, twr);
                    else prop_row_rt<N, T, E, false, V>(v, xrow, t, tw, h);
                }
            }
        }
    }

    if constexpr (kEpi) {
        // Outputs of the crop.  The geometric phase sum over all layers
        // (reference array1 / sarray1) comes from k_phasum.  The field is
        // staged in shared memory; each thread then owns whole columns of the
        // CTA's rows, so the science bin sums need no shared atomics.
        constexpr int CPT = (N + NT - 1) / NT;  // columns per thread
        const int off = I->off, Nout = I->Nout, mode = I->mode;
        const int slot = step % I->ring;
        float* __restrict__ opha = I->out_pha + (size_t)slot * I->ostride;
        float* __restrict__ oamp = I->out_amp + (size_t)slot * I->ostride;
        const float* __restrict__ psum = I->phisum;
        __syncthreads();  // phasor reads of the window rows are done
#pragma unroll
        for (int e = 0; e < E; e++) xrow[padi(t + e * T)] = v[e];
        const int ya = max(y0, off), yb = min(y0 + RR, off + Nout);
        if (ya >= yb) return;  // uniform: the CTA has no crop row
        // prefetch this thread's phase sums: every load issued before any
        // is used (one uniform branch between the two sources, predicated
        // loads inside)
        float ps[RR][CPT];
        if (const float2* __restrict__ gs = I->gsum) {
            const float sg = I->scoeff[0];
            const size_t ws = (size_t)I->wstride;
            float2 g[RR][CPT];
#pragma unroll
            for (int r = 0; r < RR; r++)
#pragma unroll
                for (int c = 0; c < CPT; c++) {
                    const int x = off + tid + c * NT, y = y0 + r;
                    const bool in = y >= ya && y < yb && x < off + Nout;
                    g[r][c] = in ? __ldg(gs + (size_t)y * ws + x) : make_float2(0.0f, 0.0f);
                }
#pragma unroll
            for (int r = 0; r < RR; r++)
#pragma unroll
                for (int c = 0; c < CPT; c++) ps[r][c] = fmaf(sg, g[r][c].x, sg * g[r][c].y);
        } else {
#pragma unroll
            for (int r = 0; r < RR; r++)
#pragma unroll
                for (int c = 0; c < CPT; c++) {
                    const int x = off + tid + c * NT, y = y0 + r;
                    const bool in = y >= ya && y < yb && x < off + Nout;
                    ps[r][c] = in ? psum[(size_t)(y - off) * Nout + (x - off)] : 0.0f;
                }
        }
        __syncthreads();
        const int nb = I->nb;
        const bool bins = (mode == kModeSci) && nb > 0;
        const short* __restrict__ binx = I->binx;
        const int jb0 = bins ? binx[ya - off] : 0;
        // bins are at least 20 rows tall: RR rows touch at most NJ bin rows
        constexpr int NJ = G::NJ;
        int jr[RR];  // bin row of each of the CTA's rows, relative to jb0
#pragma unroll
        for (int r = 0; r < RR; r++) {
            const int y = y0 + r;
            jr[r] = (bins && y >= ya && y < yb) ? binx[y - off] - jb0 : 0;
        }
        // [NJ][N]: per bin row, per column; clear of the staged rows in xb
        float2* colsum = reinterpret_cast<float2*>(wrows);
        // One loop per output mode with a branch-free body: every pixel of the
        // thread's columns is computed (rows and columns outside the crop read
        // a valid staged value) and only the stores and bin sums are
        // predicated, so the compiler can interleave the pixels.
        bool rin[RR];
#pragma unroll
        for (int r = 0; r < RR; r++) rin[r] = y0 + r >= ya && y0 + r < yb;
        if (mode == kModePhase) {
#pragma unroll
            for (int c = 0; c < CPT; c++) {
                const int x = off + tid + c * NT;
#pragma unroll
                for (int r = 0; r < RR; r++) {
                    if (!(rin[r] && x < off + Nout)) continue;
                    const size_t o = (size_t)(y0 + r - off) * Nout + (x - off);
                    opha[o] = ps[r][c];
                    oamp[o] = 1.0f;
                }
            }
        } else {
            const bool ref = mode == kModeRef;
#pragma unroll
            for (int c = 0; c < CPT; c++) {
                const int x = off + tid + c * NT;
                const bool xin = x < off + Nout;
                const int xl = xin ? x : off;
                float2 accr[RR];
#pragma unroll
                for (int r = 0; r < RR; r++) {
                    const bool in = xin && rin[r];
                    const size_t o = (size_t)(y0 + r - off) * Nout + (x - off);
                    const float2 u = xb[r * RS + padi(xl)];
                    const float amp = sqrt_approx(fmaf(u.x, u.x, u.y * u.y));
                    const float pha = atan2_out(u.y, u.x);
                    const float out = ref ? add_2pi_multiple(pha, round_2pi(ps[r][c], 0.0f)) : pha;
                    if (in) {
                        oamp[o] = amp;
                        opha[o] = out;
                    }
                    accr[r] = make_float2(0.0f, 0.0f);
                    if (bins) {
                        float d, de;
                        two_sum(ps[r][c], -pha, d, de);
                        const float2 z = phasor(d + de);  // exp(i (sum - pha))
                        accr[r] = in ? z : make_float2(0.0f, 0.0f);
                    }
                }
                if (bins && xin) {
#pragma unroll
                    for (int j = 0; j < NJ; j++) {
                        float2 acc = make_float2(0.0f, 0.0f);
#pragma unroll
                        for (int r = 0; r < RR; r++) {
                            const bool sel = NJ == 2 ? (j == 0) == (jr[r] == 0) : jr[r] == j;
                            if (sel) {
                                acc.x += accr[r].x;
                                acc.y += accr[r].y;
                            }
                        }
                        colsum[j * N + x - off] = acc;
                    }
                }
            }
        }
        if (bins) {
            // one thread per (bin row, bin): sum its contiguous columns in a
            // fixed order, one global atomic per bin and CTA
            __syncthreads();
            const int nj = binx[yb - 1 - off] - jb0 + 1;
            const short* __restrict__ bx0 = I->binx0;
            unsigned long long* __restrict__ gb = I->bins;
            for (int k = tid; k < nj * nb; k += NT) {
                const int j = k / nb, ib = k % nb;
                float sr = 0.0f, si = 0.0f;
                for (int x = bx0[ib]; x < bx0[ib + 1]; x++) {
                    const float2 z = colsum[j * N + x];
                    sr += z.x;
                    si += z.y;
                }
                // fixed point (exact scaling by 2^kBinFrac, then the nearest
                // integer): integer additions give the same totals in any order
                const float q = (float)(1ull << kBinFrac);
                atomicAdd(&gb[(jb0 + j) * nb + ib], (unsigned long long)__float2ll_rn(sr * q));
                atomicAdd(&gb[nb * nb + (jb0 + j) * nb + ib], (unsigned long long)__float2ll_rn(si * q));
            }
        }
        return;
    }

    if constexpr ((OPS & OP_STORE_T) != 0) {
        __syncthreads();
        constexpr bool kFreq = (OPS & (OP_FFT_FWD | OP_FFT_INV)) != 0;
        constexpr int RL = last_radix<N, V>();
#pragma unroll
        for (int s = 0; s < E; s++) {
            const int x = kFreq ? last_index<N, T, RL>(t, s) : t + s * T;
            xrow[padi(x)] = v[s];
        }
        __syncthreads();
        float2* dst = I ? I->fld[a.dst] : a.ext_out;
#pragma unroll 4
        for (int k = 0; k < E; k++) {
            const int idx = tid + NT * k;
            const int r2 = idx % RR, x = idx / RR;
            dst[(size_t)x * N + y0 + r2] = xb[r2 * RS + padi(x)];
        }
    }
}

// ---------------------------------------------------------------------------
// Per-step bicubic windows (the reference's window sampling,
// AtmosphericTurbulence.c:2806-2917 / :3133-3246, without the Scoeff factor):
// one job per (window group, layer, orientation); the CTA loads its screen
// tile (RR rows + 3 halo rows) by TMA and writes the RR window rows.  Every
// instance of a group (the wavelengths of one direction) then reads the same
// samples instead of interpolating the screen itself.
// ---------------------------------------------------------------------------
template <int N, int RR>
__global__ void __launch_bounds__(PassGeom<N, RR>::NT)
    k_layer_windows(const __grid_constant__ PassArgs a, const __grid_constant__ TmaSet maps)
{
    using G = PassGeom<N, RR>;
    constexpr int NT = G::NT;
    extern __shared__ __align__(1024) unsigned char sm[];
    float* tile = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(sm) + 127) & ~uintptr_t(127));
    __shared__ __align__(8) uint64_t bar;
    pdl_gate();
    const WinJob J = a.jobs[blockIdx.y];
    const int tid = threadIdx.x;
    const int y0 = blockIdx.x * RR;
    const int step = *a.d_step;
    const LayerPos p = a.pos[((size_t)(step % a.poscap) * a.ninst_total + J.gidx) * a.L + J.layer];
    const TileGeom g = tile_geom(p, J.orient, y0);
    if (tid == 0) mbar_init(&bar, 1);
    __syncthreads();
    tma_issue_layer<N, RR>(maps, J.orient, J.layer, g, tile, &bar, tid, NT);
    if (!cta_wait_tile(&bar, 0, a.d_status)) return;
    float* out = J.out + (size_t)y0 * J.stride;
    const int stride = J.stride;
    gather_tile<N, RR, NT>(tile, g, 1.0f, tid, [=](int r, int x, float val) { out[(size_t)r * stride + x] = val; });
}

// ---------------------------------------------------------------------------
// geometric phase sum over all layers for the crop (reference array1 /
// sarray1, AtmosphericTurbulence.c:2909-2916, 3237-3245) from the step's
// windows in the screen orientation: per pixel the layers from the top
// down, each window sample times the layer's Scoeff, accumulated with a
// two-sum (compensated FP32; the reference keeps a float sum).  Independent
// of the field, so it runs beside the propagation passes.
// ---------------------------------------------------------------------------
// Four pixels of one row per thread (one when the crop breaks 16-byte
// vectors); the samples of up to eight layers are requested together before
// their sums, which take the layers from the top down.  The kernel waits on
// the window reads (L2 hits: the instances of a direction run one after the
// other), so it keeps its registers low for four CTAs per SM.
template <int N>
__global__ void __launch_bounds__(kPhasumThreads, 4) k_phasum(const __grid_constant__ PassArgs a)
{
    constexpr int kChunk = 8;
    pdl_gate();
    const InstDev* I = a.inst + blockIdx.y;
    if (I->gsum) return;  // this instance's phase sum factors through its group's layer sum
    const int off = I->off, Nout = I->Nout, L = a.L;
    const size_t ws = (size_t)I->wstride;
    const bool v4 = (off % 4) == 0 && (Nout % 4) == 0;
    const int per = v4 ? 4 : 1;
    const long nitems = (long)Nout * Nout / per;
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < nitems; k += (long)gridDim.x * blockDim.x) {
        const long q = k * per;
        const int yy = (int)(q / Nout), xx = (int)(q - (long)yy * Nout);
        const size_t o = (size_t)(yy + off) * ws + (size_t)(xx + off);
        float hi[4] = {0.0f, 0.0f, 0.0f, 0.0f}, lo[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        for (int top = L - 1; top >= 0; top -= kChunk) {
            float4 w[kChunk];
#pragma unroll
            for (int c = 0; c < kChunk; c++) {
                if (top - c < 0) break;
                const float* src = I->win[0][top - c] + o;
                w[c] = v4 ? __ldg(reinterpret_cast<const float4*>(src)) : make_float4(__ldg(src), 0.0f, 0.0f, 0.0f);
            }
#pragma unroll
            for (int c = 0; c < kChunk; c++) {
                if (top - c < 0) break;
                const float sc = I->scoeff[top - c];
                const float wv[4] = {w[c].x, w[c].y, w[c].z, w[c].w};
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const float val = __fmul_rn(wv[j], sc);
                    float sum, err;
                    two_sum(hi[j], val, sum, err);
                    hi[j] = sum;
                    lo[j] = __fadd_rn(lo[j], err);
                }
            }
        }
        float* dst = I->phisum + q;
        if (v4) {
            *reinterpret_cast<float4*>(dst) = make_float4(__fadd_rn(hi[0], lo[0]), __fadd_rn(hi[1], lo[1]),
                                                          __fadd_rn(hi[2], lo[2]), __fadd_rn(hi[3], lo[3]));
        } else {
            dst[0] = __fadd_rn(hi[0], lo[0]);
        }
    }
}

// host launcher for one (N, configuration); SO: the series passes only (the
// unit operators, phase sums and windows launch in configuration 0)
template <int N, int RR, int MINB, bool ALIAS, bool HP = false, int V = 0, bool SO = false, bool HS = false>
cudaError_t launch_pass_t(int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const float2* tw, cudaStream_t st)
{
    using G = PassGeom<N, RR, V>;
    static TmaSet empty_maps;  // unit passes gather nothing
    const TmaSet& m = maps ? *maps : empty_maps;
    dim3 block(G::NT);
#define AW_CASE(VAR)                                                                                   \
    case VAR: {                                                                                        \
        constexpr size_t sm = G::smem(VAR, HS);                                                        \
        static bool attr = false;                                                                      \
        if (!attr) {                                                                                   \
            cudaError_t e = cudaFuncSetAttribute(k_pass<N, RR, MINB, VAR, ALIAS, HP, V, HS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm); \
            if (e != cudaSuccess) return e;                                                            \
            attr = true;                                                                               \
        }                                                                                              \
        return launch_gated(k_pass<N, RR, MINB, VAR, ALIAS, HP, V, HS>, grid, block, sm, st, a, m, tw); \
    }
    if constexpr (HP || V != 0 || SO || HS) {
        // FP16 transforms, the alternative radix plans and configurations
        // other than 0: the series passes only
        switch (var) {
            AW_CASE(kVarFirst)
            AW_CASE(kVarMid)
            AW_CASE(kVarLast)
            AW_CASE(kVarSingle)
            default: return cudaErrorInvalidValue;
        }
    } else {
    switch (var) {
        AW_CASE(kVarFirst)
        AW_CASE(kVarMid)
        AW_CASE(kVarLast)
        AW_CASE(kVarSingle)
        AW_CASE(kVarUnitProp)
        AW_CASE(kVarUnitFwd)
        AW_CASE(kVarUnitInv)
        case kVarPhasum: {
            return launch_gated(k_phasum<N>, grid, dim3(kPhasumThreads), 0, st, a);
        }
        case kVarWindows: {
            constexpr size_t sm = G::TILE_BYTES + 128;
            static bool attr = false;
            if (!attr) {
                cudaError_t e = cudaFuncSetAttribute(k_layer_windows<N, RR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
                if (e != cudaSuccess) return e;
                attr = true;
            }
            return launch_gated(k_layer_windows<N, RR>, grid, dim3(G::NT), sm, st, a, m);
        }
        default: return cudaErrorInvalidValue;
    }
    }
#undef AW_CASE
}

template <int N>
cudaError_t launch_pass_n(int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const float2* tw, cudaStream_t st)
{
    constexpr TileCfg c0 = tile_cfg(N, 0);
    return launch_pass_t<N, c0.rr, c0.minb, c0.alias>(var, grid, a, maps, tw, st);
}

// FP16-transform passes: tile configuration 2, tw = the FP16 twiddle table
template <int N>
cudaError_t launch_pass_hn(int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const void* tw, cudaStream_t st)
{
    constexpr TileCfg c2 = tile_cfg(N, 2);
    return launch_pass_t<N, c2.rr, c2.minb, c2.alias, true>(var, grid, a, maps, reinterpret_cast<const float2*>(tw), st);
}

template <int N>
cudaError_t launch_pass_nc(int cfg, int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const float2* tw,
                           cudaStream_t st)
{
    constexpr TileCfg c0 = tile_cfg(N, 0), c1 = tile_cfg(N, 1), c2 = tile_cfg(N, 2);
    constexpr TileCfg c3 = tile_cfg(N, 3), c4 = tile_cfg(N, 4), c5 = tile_cfg(N, 5);
    static_assert(kNumTileCfg == 6, "one branch per configuration");
    if constexpr (c5.rr > 0) if (cfg == 5) return launch_pass_t<N, c5.rr, c5.minb, c5.alias, false, c5.plan, true, c5.hsm>(var, grid, a, maps, tw, st);
    if constexpr (c3.rr > 0) if (cfg == 3) return launch_pass_t<N, c3.rr, c3.minb, c3.alias, false, c3.plan>(var, grid, a, maps, tw, st);
    if constexpr (c4.rr > 0) if (cfg == 4) return launch_pass_t<N, c4.rr, c4.minb, c4.alias, false, c4.plan>(var, grid, a, maps, tw, st);
    if (cfg >= 3) return cudaErrorInvalidValue;  // no such configuration at this size
    if (cfg == 2) return launch_pass_t<N, c2.rr, c2.minb, c2.alias, false, 0, true>(var, grid, a, maps, tw, st);
    if (cfg == 1) return launch_pass_t<N, c1.rr, c1.minb, c1.alias, false, 0, true>(var, grid, a, maps, tw, st);
    return launch_pass_t<N, c0.rr, c0.minb, c0.alias>(var, grid, a, maps, tw, st);
}

}  // namespace atmwfs
