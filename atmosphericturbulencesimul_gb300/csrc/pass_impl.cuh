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
template <int N, int RR>
struct PassGeom {
    static constexpr int T = Plan<N>::T;
    static constexpr int E = Plan<N>::E;
    static constexpr int NT = T * RR;
    static constexpr int RS = row_stride<N>();
    static constexpr int NBOX = N / kBoxW + 1;
    static constexpr int TROWS = RR + 3;
    static constexpr size_t XBYTES = size_t(RR) * RS * 8;
    static constexpr size_t PHI_EPI_BYTES = size_t(3) * RR * N * 4;
    static constexpr size_t TILE_BYTES = size_t(NBOX) * TROWS * kBoxW * 4;
    AW_HD static constexpr size_t round128(size_t b) { return (b + 127) / 128 * 128; }
    AW_HD static constexpr size_t region(bool epi) { return round128((epi && PHI_EPI_BYTES > XBYTES) ? PHI_EPI_BYTES : XBYTES); }
    AW_HD static constexpr size_t smem(int ops)
    {
        return region((ops & OP_EPI) != 0) + (((ops & (OP_GATHER | OP_EPI)) != 0) ? TILE_BYTES + 128 : 0);
    }
    static_assert(N % (RR) == 0, "rows per CTA must divide N");
};

template <int N, int RR>
__device__ __forceinline__ void tma_issue_layer(const TmaSet& maps, int orient, int l, const TileGeom& g, float* tile,
                                                uint64_t* bar)
{
    using G = PassGeom<N, RR>;
    mbar_expect_tx(bar, (uint32_t)G::TILE_BYTES);
    const CUtensorMap* m = &maps.m[orient][l];
#pragma unroll 1
    for (int k = 0; k < G::NBOX; k++) tma_load_2d(tile + k * G::TROWS * kBoxW, m, g.xs + k * kBoxW, g.ys, bar);
}

// ---------------------------------------------------------------------------
// FFT sequencing (device): stages exchange through one padded row of the
// shared exchange buffer: [sync, store, sync, load] between stages.
// ---------------------------------------------------------------------------
template <int N, int T, int E, int D, int NS, int R, int... Rest>
__device__ __forceinline__ void run_stages(float2* v, float2* xrow, int t, const float2* __restrict__ tw)
{
    stage_twiddle<N, T, E, R, NS, D>(v, t, tw);
    stage_dft<E, R, D>(v);
    if constexpr (sizeof...(Rest) > 0) {
        __syncthreads();
        stage_store<N, T, E, R, NS>(v, xrow, t);
        __syncthreads();
        stage_load<N, T, E, FirstRadix<Rest...>::value>(v, xrow, t);
        run_stages<N, T, E, D, NS * R, Rest...>(v, xrow, t, tw);
    }
}

template <int N, int T, int E, int D, int... Rs>
__device__ __forceinline__ void run_fft(float2* v, float2* xrow, int t, const float2* __restrict__ tw, Radices<Rs...>)
{
    run_stages<N, T, E, D, 1, Rs...>(v, xrow, t, tw);
}

template <int... Rs>
AW_HD constexpr int last_of(Radices<Rs...>) { return LastRadix<Rs...>::value; }

// 1-D Fresnel propagation of the row held in v (layout x[t + e T]):
// forward FFT, multiply by the transfer table h[k] (unshifted frequency
// index k, 1/N included), inverse FFT.  Ends in the same layout.
template <int N, int T, int E>
__device__ __forceinline__ void prop_row(float2* v, float2* xrow, int t, const float2* __restrict__ tw,
                                         const float2* __restrict__ h)
{
    using FR = typename FwdRadices<N>::type;
    using IR = typename InvRadices<N>::type;
    constexpr int RL = last_of(FR{});
    run_fft<N, T, E, -1>(v, xrow, t, tw, FR{});
#pragma unroll
    for (int s = 0; s < E; s++) v[s] = cmul(v[s], __ldg(h + last_index<N, T, RL>(t, s)));
    run_fft<N, T, E, +1>(v, xrow, t, tw, IR{});
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
template <int N, int RR, int OPS>
__global__ void __launch_bounds__(Plan<N>::T* RR, 1)
    k_pass(const __grid_constant__ PassArgs a, const __grid_constant__ TmaSet maps, const float2* __restrict__ tw)
{
    using G = PassGeom<N, RR>;
    constexpr int T = G::T, E = G::E, NT = G::NT, RS = G::RS, TROWS = G::TROWS;
    constexpr bool kEpi = (OPS & OP_EPI) != 0;
    constexpr bool kGather = (OPS & (OP_GATHER | OP_EPI)) != 0;
    extern __shared__ __align__(1024) unsigned char sm[];
    float2* xb = reinterpret_cast<float2*>(sm);
    // TMA destination: 128-byte aligned whatever the dynamic smem base
    float* tile = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(sm + G::region(kEpi)) + 127) & ~uintptr_t(127));
    __shared__ __align__(8) uint64_t bar;
    __shared__ float sbins[3 * 2 * 104];

    const int tid = threadIdx.x;
    const int t = tid % T;
    const int rr = tid / T;
    const int y0 = a.row0 + blockIdx.x * RR;
    const int y = y0 + rr;
    const InstDev* I = a.inst ? a.inst + blockIdx.y : nullptr;
    const int step = a.d_step ? *a.d_step : 0;
    const LayerPos* P = I ? a.pos + ((size_t)(step % a.poscap) * a.ninst_total + I->gidx) * a.L : nullptr;
    float2* xrow = xb + rr * RS;

    const int ltop = kEpi ? a.L - 1 : a.g_hi - 1;
    const int lbot = kEpi ? 0 : a.g_lo;
    int parity = 0;
    if constexpr (kGather) {
        if (tid == 0) mbar_init(&bar, 1);
        __syncthreads();
        if (tid == 0 && ltop >= lbot) tma_issue_layer<N, RR>(maps, a.orient, ltop, tile_geom(P[ltop], a.orient, y0), tile, &bar);
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

    if constexpr ((OPS & OP_PROP1) != 0) prop_row<N, T, E>(v, xrow, t, tw, I ? I->H + (size_t)a.hop1 * N : a.H1);
    if constexpr ((OPS & OP_FFT_FWD) != 0) run_fft<N, T, E, -1>(v, xrow, t, tw, typename FwdRadices<N>::type{});
    if constexpr ((OPS & OP_FFT_INV) != 0) run_fft<N, T, E, +1>(v, xrow, t, tw, typename FwdRadices<N>::type{});

    if constexpr (kGather && !kEpi) {
        float* phi = reinterpret_cast<float*>(xb);  // [RR][N]
        __syncthreads();
        for (int l = ltop; l >= lbot; l--) {
            if (!cta_wait_tile(&bar, parity, a.d_status)) return;
            parity ^= 1;
            const bool first = (l == ltop);
            gather_tile<N, RR, NT>(tile, tile_geom(P[l], a.orient, y0), I->scoeff[l], tid, [=](int r, int x, float val) {
                phi[r * N + x] = first ? val : phi[r * N + x] + val;
            });
            __syncthreads();
            if (tid == 0 && l > lbot) tma_issue_layer<N, RR>(maps, a.orient, l - 1, tile_geom(P[l - 1], a.orient, y0), tile, &bar);
        }
#pragma unroll
        for (int e = 0; e < E; e++) {
            float s, c;
            sincosf(phi[rr * N + t + e * T], &s, &c);
            v[e] = cmul(v[e], make_float2(c, s));
        }
    }

    if constexpr (kEpi) {
        // phi0: phase of the layers at the last plane; (hi, lo): compensated
        // geometric phase sum over all layers (reference array1 / sarray1).
        float* phi0 = reinterpret_cast<float*>(xb);
        float* shi = phi0 + RR * N;
        float* slo = shi + RR * N;
        __syncthreads();
        for (int i = tid; i < 3 * RR * N; i += NT) phi0[i] = 0.0f;
        for (int i = tid; i < 3 * 2 * 104; i += NT) sbins[i] = 0.0f;
        __syncthreads();
        for (int l = ltop; l >= lbot; l--) {
            if (!cta_wait_tile(&bar, parity, a.d_status)) return;
            parity ^= 1;
            const bool in0 = (l >= a.g_lo && l < a.g_hi);
            gather_tile<N, RR, NT>(tile, tile_geom(P[l], a.orient, y0), I->scoeff[l], tid, [=](int r, int x, float val) {
                const int i = r * N + x;
                if (in0) phi0[i] += val;
                float s, e;
                two_sum(shi[i], val, s, e);
                shi[i] = s;
                slo[i] += e;
            });
            __syncthreads();
            if (tid == 0 && l > lbot) tma_issue_layer<N, RR>(maps, a.orient, l - 1, tile_geom(P[l - 1], a.orient, y0), tile, &bar);
        }
        const int off = I->off, Nout = I->Nout, mode = I->mode;
        const int slot = step % I->ring;
        const bool rowin = (y >= off) && (y < off + Nout);
        const int yo = y - off;
        float* opha = I->out_pha + (size_t)slot * Nout * Nout;
        float* oamp = I->out_amp + (size_t)slot * Nout * Nout;
        const int nb = I->nb;
        const int yb = max(y0, off) - off;
        const int jb0 = (nb > 0 && yb < Nout) ? I->binx[yb] : 0;
#pragma unroll
        for (int e = 0; e < E; e++) {
            const int x = t + e * T;
            if (!rowin || x < off || x >= off + Nout) continue;
            const int i = rr * N + x;
            const float hi = shi[i], lo = slo[i];
            const size_t o = (size_t)yo * Nout + (x - off);
            if (mode == kModePhase) {
                opha[o] = hi + lo;
                oamp[o] = 1.0f;
                continue;
            }
            float s, c;
            sincosf(phi0[i], &s, &c);
            const float2 u = cmul(v[e], make_float2(c, s));
            const float amp = sqrtf(u.x * u.x + u.y * u.y);
            const float pha = atan2f(u.y, u.x);
            oamp[o] = amp;
            if (mode == kModeRef) {
                opha[o] = add_2pi_multiple(pha, round_2pi(hi, lo));
            } else {
                opha[o] = pha;
                I->phisum[o] = hi + lo;
                if (nb > 0) {
                    float d, de;
                    two_sum(hi, -pha, d, de);
                    float bs, bc;
                    sincosf(d + (de + lo), &bs, &bc);
                    const int ib = I->binx[x - off];
                    const int jb = I->binx[yo] - jb0;
                    atomicAdd(&sbins[(jb * nb + ib) * 2 + 0], bc);
                    atomicAdd(&sbins[(jb * nb + ib) * 2 + 1], bs);
                }
            }
        }
        if (mode == kModeSci && nb > 0) {
            __syncthreads();
            const int ylast = min(y0 + RR, off + Nout) - 1;
            if (ylast >= max(y0, off)) {
                const int nj = I->binx[ylast - off] - jb0 + 1;
                for (int k = tid; k < nj * nb; k += NT) {
                    const int jb = jb0 + k / nb, ib = k % nb;
                    atomicAdd(&I->bins[jb * nb + ib], sbins[k * 2 + 0]);
                    atomicAdd(&I->bins[nb * nb + jb * nb + ib], sbins[k * 2 + 1]);
                }
            }
        }
        return;
    }

    if constexpr ((OPS & OP_PROP2) != 0) prop_row<N, T, E>(v, xrow, t, tw, I ? I->H + (size_t)a.hop2 * N : a.H2);

    if constexpr ((OPS & OP_STORE_T) != 0) {
        __syncthreads();
        constexpr bool kFreq = (OPS & (OP_FFT_FWD | OP_FFT_INV)) != 0;
        constexpr int RL = last_of(typename FwdRadices<N>::type{});
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

// host launcher for one N
template <int N>
cudaError_t launch_pass_n(int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const float2* tw, cudaStream_t st)
{
    constexpr int RR = (N == 64 || N == 128) ? 32 : (N == 256 || N == 512) ? 16 : (N == 1024) ? 8 : 4;
    using G = PassGeom<N, RR>;
    static TmaSet empty_maps;  // unit passes gather nothing
    const TmaSet& m = maps ? *maps : empty_maps;
    dim3 block(G::NT);
#define AW_CASE(VAR)                                                                                   \
    case VAR: {                                                                                        \
        constexpr size_t sm = G::smem(VAR);                                                            \
        static bool attr = false;                                                                      \
        if (!attr) {                                                                                   \
            cudaError_t e = cudaFuncSetAttribute(k_pass<N, RR, VAR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm); \
            if (e != cudaSuccess) return e;                                                            \
            attr = true;                                                                               \
        }                                                                                              \
        k_pass<N, RR, VAR><<<grid, block, sm, st>>>(a, m, tw);                                         \
        return cudaGetLastError();                                                                     \
    }
    switch (var) {
        AW_CASE(kVarFirst)
        AW_CASE(kVarMid)
        AW_CASE(kVarLast)
        AW_CASE(kVarSingle)
        AW_CASE(kVarUnitProp)
        AW_CASE(kVarUnitFwd)
        AW_CASE(kVarUnitInv)
        default: return cudaErrorInvalidValue;
    }
#undef AW_CASE
}

}  // namespace atmwfs
