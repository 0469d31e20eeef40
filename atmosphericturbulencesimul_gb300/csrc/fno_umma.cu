// fno_umma.cu -- the surrogate's pointwise channel mixing on the 5th-generation
// tensor cores (tcgen05 / TMEM):
//
//   C[b] (o x P) = W (o x c) X[b] (c x P) + bias[o] (+ beta C[b]);  act = gelu(C)
//
// the product of every Fourier layer, the lift and the projection
// (u = W_l h + b_l in each layer of the network).  It is computed as the
// transposed product D = X[b]^T W^T, a tile of 128 pixels (the MMA's M) by
// the o output channels (N), K = c input channels:
//   * A (128 x c, BF16, K-major): the tile's pixels, read from the FP32
//     channel planes of X and rounded to BF16 by the CTA's threads while they
//     store it in the canonical no-swizzle layout (8 x 8 core matrices);
//   * B (o x c, BF16, K-major): the weights, staged once per CTA;
//   * D (128 x o, FP32) in tensor memory: lane = pixel, column = channel;
// one thread issues the c/16 MMAs and commits them to an mbarrier; the four
// warps read their 32 lanes back with tcgen05.ld and write C as coalesced
// rows of each channel plane, with the bias, the beta term and the GELU.
//
// Every wait is bounded (1 s on %globaltimer): a timeout sets a status bit,
// the CTA frees its tensor memory and returns.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "atmwfs_fno.h"
#include "fno_gemm.cuh"

namespace atmwfs {
void set_error_message(const char* msg);

namespace umma {

constexpr int kM = 128;      // pixels per tile (MMA M, one TMEM lane each)
constexpr int kThreads = 256;
constexpr uint64_t kWaitNs = 1000000000ull;

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t now_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Shared-memory matrix descriptor, no swizzle, K-major: core matrices of 8
// rows x 16 bytes; `lbo` = byte distance of core matrices along K, `sbo` =
// along M/N (8-row groups); bits 46-47 = 1 (descriptor version of sm_100).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFF);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;
    return d;  // base offset 0, layout type 0 (no swizzle)
}

// Instruction descriptor of kind::f16: D FP32, A and B BF16, both K-major,
// N = n, M = 128.
__host__ __device__ constexpr uint32_t instr_desc(int n)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kM >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 16 consecutive TMEM columns of this warp's 32 lanes: register j = column c0 + j.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&r)[16])
{
    uint32_t u[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
        : "=r"(u[0]), "=r"(u[1]), "=r"(u[2]), "=r"(u[3]), "=r"(u[4]), "=r"(u[5]), "=r"(u[6]), "=r"(u[7]),
          "=r"(u[8]), "=r"(u[9]), "=r"(u[10]), "=r"(u[11]), "=r"(u[12]), "=r"(u[13]), "=r"(u[14]), "=r"(u[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 16; j++) r[j] = __uint_as_float(u[j]);
}

// Byte offset of element (row, k) in a K-major no-swizzle tile with kc = K/8
// core matrices per 8-row group (LBO = 128 B, SBO = kc * 128 B).
__device__ __forceinline__ uint32_t kmajor_off(int row, int k, int kc)
{
    return (uint32_t)((row >> 3) * kc * 128 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ void cp_async16(void* dst, const void* src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)),
                 "l"(static_cast<uint64_t>(__cvta_generic_to_global(src)))
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// The pixels of one tile (C channel rows of 128 pixels, FP32 or BF16 as
// stored) copied into the staging buffer with 16-byte asynchronous copies;
// pixels past P are zeros, and so are the channel rows from CR on (X holds
// CR channels per sample; K is padded to the MMA's multiple of 16).
template <int C, int CR, typename TX>
__device__ __forceinline__ void stage_tile(TX* stage, const TX* X, long P, int tile, long tiles_per_sample, int tid)
{
    constexpr int EPC = 16 / sizeof(TX);  // elements per 16-byte chunk
    const long b = tile / tiles_per_sample;
    const long p0 = (tile - b * tiles_per_sample) * kM;
    const TX* xs = X + (size_t)b * CR * P + p0;
    constexpr int CH = kM / EPC;  // chunks per channel row
    for (int i = tid; i < C * CH; i += kThreads) {
        const int k = i / CH, ch = i - k * CH;
        TX* dst = stage + k * kM + EPC * ch;
        if (k < CR && p0 + EPC * ch < P) cp_async16(dst, xs + (size_t)k * P + EPC * ch);
        else *reinterpret_cast<uint4*>(dst) = make_uint4(0u, 0u, 0u, 0u);
    }
    cp_async_commit();
}

__device__ __forceinline__ float to_f(float x) { return x; }
__device__ __forceinline__ float to_f(__nv_bfloat16 x) { return __bfloat162float(x); }
__device__ __forceinline__ void put(float* p, float v) { *p = v; }
__device__ __forceinline__ void put(__nv_bfloat16* p, float v) { *p = __float2bfloat16_rn(v); }

// Pipeline per tile: the staged FP32 pixels are rounded into the BF16 A
// tile; the next tile's copies start; one thread issues the MMAs; all wait
// for their commit; the eight warps read D (warp w: lanes 32 (w % 4) ..,
// columns of half w / 4) and write C while the next tile's pixels arrive.
template <int O, int C, typename TX, typename TA, int CR = C>
__global__ void __launch_bounds__(kThreads, 3) k_pointwise(const __nv_bfloat16* __restrict__ W, const TX* __restrict__ X,
                                                           float* __restrict__ Cm, TA* __restrict__ act,
                                                           const float* __restrict__ bias, float beta, long P, int ntiles,
                                                           unsigned* status, int swap, int write_c)
{
    static_assert(O % 32 == 0 && O <= 256, "N of the MMA: a multiple of 32 (two halves of 16-column chunks)");
    static_assert(C % 16 == 0 && C >= 16, "K: a multiple of 16");
    constexpr int KC = C / 8;                         // core matrices along K
    constexpr uint32_t STAGE_BYTES = C * kM * sizeof(TX), A_BYTES = kM * C * 2;
    constexpr uint32_t kCols = O <= 64 ? 64 : O <= 128 ? 128 : 256;  // TMEM columns (power of 2)
    extern __shared__ __align__(1024) unsigned char sm[];
    TX* stage = reinterpret_cast<TX*>(sm);            // the tile's pixels [C][128]
    unsigned char* sa = sm + STAGE_BYTES;             // A tile
    unsigned char* sb = sa + A_BYTES;                 // B (weights)
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tmem_base;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const long tiles_per_sample = (P + kM - 1) / kM;
    if (blockIdx.x < ntiles) stage_tile<C, CR, TX>(stage, X, P, blockIdx.x, tiles_per_sample, tid);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_base)),
                     "r"(kCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) mbar_init(&bar);
    // weights: W is o x CR, row-major (K contiguous), element loads (the
    // parameter blocks carry no alignment guarantee); zeros for k >= CR
    for (int i = tid; i < O * C; i += kThreads) {
        const int n = i / C, k = i - n * C;
        *reinterpret_cast<__nv_bfloat16*>(sb + kmajor_off(n, k, KC)) =
            k < CR ? W[n * CR + k] : __float2bfloat16_rn(0.0f);
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = tmem_base;
    const uint32_t a_addr = smem_addr(sa), b_addr = smem_addr(sb);
    uint32_t parity = 0;

    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const long b = tile / tiles_per_sample;
        const long p0 = (tile - b * tiles_per_sample) * kM;
        cp_async_wait_all();
        __syncthreads();  // every thread's copies of this tile have landed
        // A: 8 channels of one pixel per 16-byte store
        for (int i = tid; i < kM * KC; i += kThreads) {
            const int kc = i / kM, m = i - kc * kM;
            const TX* f = stage + kc * 8 * kM + m;
            uint4 v;
            __nv_bfloat162 h0 = __floats2bfloat162_rn(to_f(f[0]), to_f(f[kM]));
            __nv_bfloat162 h1 = __floats2bfloat162_rn(to_f(f[2 * kM]), to_f(f[3 * kM]));
            __nv_bfloat162 h2 = __floats2bfloat162_rn(to_f(f[4 * kM]), to_f(f[5 * kM]));
            __nv_bfloat162 h3 = __floats2bfloat162_rn(to_f(f[6 * kM]), to_f(f[7 * kM]));
            v.x = *reinterpret_cast<uint32_t*>(&h0);
            v.y = *reinterpret_cast<uint32_t*>(&h1);
            v.z = *reinterpret_cast<uint32_t*>(&h2);
            v.w = *reinterpret_cast<uint32_t*>(&h3);
            *reinterpret_cast<uint4*>(sa + kmajor_off(m, kc * 8, KC)) = v;
        }
        // the tensor core reads shared memory through the async proxy
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        fence_before();
        __syncthreads();
        fence_after();
        // the staging buffer is free: the next tile's pixels come in now
        if (tile + (int)gridDim.x < ntiles) stage_tile<C, CR, TX>(stage, X, P, tile + gridDim.x, tiles_per_sample, tid);
        if (tid == 0) {
#pragma unroll
            for (int ks = 0; ks < C / 16; ks++) {
                // K step of 16 = two core matrices along K
                // LBO: core matrices along K (128 B apart), SBO: along M/N
                // (KC * 128 B apart); `swap` exchanges the two fields
                const uint32_t lbo = swap ? KC * 128 : 128, sbo = swap ? 128 : KC * 128;
                const uint64_t da = smem_desc(a_addr + ks * 256, lbo, sbo);
                const uint64_t db = smem_desc(b_addr + ks * 256, lbo, sbo);
                const uint32_t acc = ks > 0 ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "setp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                    ::"r"(tmem), "l"(da), "l"(db), "r"(instr_desc(O)), "r"(acc)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_addr(&bar))
                         : "memory");
        }
        // every thread waits for the products (bounded)
        const uint64_t t0 = now_ns();
        int timed_out = 0;
        while (!mbar_try_wait(&bar, parity)) {
            if (now_ns() - t0 > kWaitNs) {
                timed_out = 1;
                break;
            }
        }
        if (__syncthreads_or(timed_out)) {
            if (tid == 0 && status) atomicOr(status, 1u);
            break;
        }
        parity ^= 1;
        fence_after();
        // epilogue: warp w reads TMEM lanes 32 (w % 4) .. (its 32 pixels) and
        // the columns of half w / 4, 16 at a time
        const int g = warp & 3, half = warp >> 2;
        const long p = p0 + g * 32 + lane;
        const uint32_t trow = tmem + ((uint32_t)(g * 32) << 16);
        float* cs = Cm + (size_t)b * O * P;
        TA* as = act ? act + (size_t)b * O * P : nullptr;
#pragma unroll 1
        for (int c0 = half * (O / 2); c0 < (half + 1) * (O / 2); c0 += 16) {
            float r[16];
            tmem_ld16(trow + c0, r);
            if (p < P) {
                float old[16];
                if (beta != 0.0f) {
#pragma unroll
                    for (int j = 0; j < 16; j++) old[j] = cs[(size_t)(c0 + j) * P + p];
                }
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    const size_t o = (size_t)(c0 + j) * P + p;
                    float v = r[j] + (bias ? bias[c0 + j] : 0.0f);
                    if (beta != 0.0f) v = fmaf(beta, old[j], v);
                    if (write_c) cs[o] = v;
                    if (as) put(as + o, gelu_f(v));
                }
            }
        }
        // the next tile's MMAs overwrite D and its conversion overwrites A
        fence_before();
        __syncthreads();
        fence_after();
    }
    cp_async_wait_all();  // no copy may still target this CTA's shared memory
    __syncthreads();
    if (warp == 0) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols) : "memory");
    }
}

template <int O, int C, typename TX, typename TA, int CR = C>
cudaError_t launch(const __nv_bfloat16* W, const TX* X, float* Cm, TA* act, const float* bias, float beta, int B, long P,
                   unsigned* status, int swap, int write_c, cudaStream_t st)
{
    if (P % 8 != 0) return cudaErrorNotSupported;  // 16-byte copies of the channel rows
    // shared memory: the staging buffer, A and B; at most three CTAs per SM
    // (registers), whose TMEM allocations (at most 128 columns) fit the 512
    constexpr size_t smem = (size_t)C * kM * sizeof(TX) + (size_t)kM * C * 2 + (size_t)O * C * 2;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_pointwise<O, C, TX, TA, CR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    const long tiles = (long)B * ((P + kM - 1) / kM);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long grid = tiles < 3L * sms ? tiles : 3L * sms;
    k_pointwise<O, C, TX, TA, CR><<<(unsigned)grid, kThreads, smem, st>>>(W, X, Cm, act, bias, beta, P, (int)tiles,
                                                                            status, swap, write_c);
    return cudaGetLastError();
}

// Storage types of the input (x_bf16) and of the activation output (a_bf16).
template <int O, int C>
cudaError_t launch_t(const __nv_bfloat16* W, const void* X, int x_bf16, float* Cm, void* act, int a_bf16,
                     const float* bias, float beta, int B, long P, unsigned* status, int swap, int write_c,
                     cudaStream_t st)
{
    using bf = __nv_bfloat16;
    if (x_bf16) {
        if (a_bf16) return launch<O, C, bf, bf>(W, (const bf*)X, Cm, (bf*)act, bias, beta, B, P, status, swap, write_c, st);
        return launch<O, C, bf, float>(W, (const bf*)X, Cm, (float*)act, bias, beta, B, P, status, swap, write_c, st);
    }
    if (a_bf16)
        return launch<O, C, float, bf>(W, (const float*)X, Cm, (bf*)act, bias, beta, B, P, status, swap, write_c, st);
    return launch<O, C, float, float>(W, (const float*)X, Cm, (float*)act, bias, beta, B, P, status, swap, write_c, st);
}

// ---------------------------------------------------------------------------
// The spectral products of the Fourier layers along y, C (o x P) = W (o x c)
// X (c x P), with a long K or a wide N: the forward DFT z = [FyA | FyB] a
// (o = 2 modes, c = 2 grid) and its inverse bb = GyBig y (o = 2 grid,
// c = 2 modes), P = samples x width x modes columns.  The same transposed
// tile product as k_pointwise (128 columns of X per tile, one TMEM lane
// each), with K taken in chunks of 64: each chunk's FP32 rows are staged by
// cp.async while the previous chunk's MMAs run, rounded into the BF16 A tile
// and accumulated into the same tensor-memory columns; N above 256 is split
// over two MMAs per K step (tensor-memory columns 0.. and 256..).  The whole
// W is staged once per CTA.  No bias or activation: C is written.
// ---------------------------------------------------------------------------
constexpr int kKch = 64;  // K per staged chunk

// One chunk (kKch rows of 128 columns) of tile `tile` of X, rows [j kKch, ..).
__device__ __forceinline__ void stage_chunk(float* stage, const float* X, long P, int tile, int j, int tid)
{
    const long p0 = (long)tile * kM;
    const float* xs = X + (size_t)j * kKch * P + p0;
    constexpr int CH = kM / 4;  // 16-byte chunks per row
    for (int i = tid; i < kKch * CH; i += kThreads) {
        const int k = i / CH, ch = i - k * CH;
        float* dst = stage + k * kM + 4 * ch;
        if (p0 + 4 * ch < P) cp_async16(dst, xs + (size_t)k * P + 4 * ch);
        else *reinterpret_cast<uint4*>(dst) = make_uint4(0u, 0u, 0u, 0u);
    }
    cp_async_commit();
}

template <int O, int C>
__global__ void __launch_bounds__(kThreads, 1) k_chunked(const __nv_bfloat16* __restrict__ W, const float* __restrict__ X,
                                                         float* __restrict__ Cm, long P, int ntiles, unsigned* status,
                                                         int swap)
{
    constexpr int NKC = C / kKch;                    // K chunks
    constexpr int KCB = C / 8, KCA = kKch / 8;       // core matrices along K in B / in one A chunk
    constexpr int NMMA = O > 256 ? 2 : 1, NI = O / NMMA;
    constexpr uint32_t STAGE_BYTES = kKch * kM * 4, A_BYTES = kM * kKch * 2;
    constexpr uint32_t kCols = O <= 32 ? 32 : O <= 64 ? 64 : O <= 128 ? 128 : O <= 256 ? 256 : 512;
    static_assert(C % kKch == 0, "K: whole chunks");
    static_assert(O % 32 == 0 && O <= 512 && NI % 16 == 0 && NI <= 256, "N per MMA: 16..256");
    extern __shared__ __align__(1024) unsigned char sm[];
    float* stage = reinterpret_cast<float*>(sm);     // one chunk of the tile [kKch][128]
    unsigned char* sa = sm + STAGE_BYTES;            // A chunk (BF16, K-major)
    unsigned char* sb = sa + A_BYTES;                // W (BF16, K-major)
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tmem_base;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (blockIdx.x < ntiles) stage_chunk(stage, X, P, blockIdx.x, 0, tid);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_base)),
                     "r"(kCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) mbar_init(&bar);
    for (int i = tid; i < O * C; i += kThreads) {
        const int n = i / C, k = i - n * C;
        *reinterpret_cast<__nv_bfloat16*>(sb + kmajor_off(n, k, KCB)) = W[i];
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = tmem_base;
    const uint32_t a_addr = smem_addr(sa), b_addr = smem_addr(sb);
    uint32_t parity = 0;
    bool failed = false;

    for (int tile = blockIdx.x; tile < ntiles && !failed; tile += gridDim.x) {
        const long p0 = (long)tile * kM;
        for (int j = 0; j < NKC; j++) {
            cp_async_wait_all();
            __syncthreads();  // every thread's copies of this chunk have landed
            for (int i = tid; i < kM * KCA; i += kThreads) {
                const int kc = i / kM, m = i - kc * kM;
                const float* f = stage + kc * 8 * kM + m;
                uint4 v;
                __nv_bfloat162 h0 = __floats2bfloat162_rn(f[0], f[kM]);
                __nv_bfloat162 h1 = __floats2bfloat162_rn(f[2 * kM], f[3 * kM]);
                __nv_bfloat162 h2 = __floats2bfloat162_rn(f[4 * kM], f[5 * kM]);
                __nv_bfloat162 h3 = __floats2bfloat162_rn(f[6 * kM], f[7 * kM]);
                v.x = *reinterpret_cast<uint32_t*>(&h0);
                v.y = *reinterpret_cast<uint32_t*>(&h1);
                v.z = *reinterpret_cast<uint32_t*>(&h2);
                v.w = *reinterpret_cast<uint32_t*>(&h3);
                *reinterpret_cast<uint4*>(sa + kmajor_off(m, kc * 8, KCA)) = v;
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            fence_before();
            __syncthreads();
            fence_after();
            // the staging buffer is free: the next chunk (or the next tile's first) comes in
            if (j + 1 < NKC) stage_chunk(stage, X, P, tile, j + 1, tid);
            else if (tile + (int)gridDim.x < ntiles) stage_chunk(stage, X, P, tile + gridDim.x, 0, tid);
            if (tid == 0) {
                const uint32_t lbo = swap ? KCA * 128 : 128, sbo_a = swap ? 128 : KCA * 128;
                const uint32_t lbo_b = swap ? KCB * 128 : 128, sbo_b = swap ? 128 : KCB * 128;
#pragma unroll
                for (int ks = 0; ks < kKch / 16; ks++) {
                    const uint64_t da = smem_desc(a_addr + ks * 256, lbo, sbo_a);
#pragma unroll
                    for (int h = 0; h < NMMA; h++) {
                        // B rows h NI.. (8-row groups KCB * 128 B apart), K core
                        // matrices 8 j + 2 ks.. (128 B apart)
                        const uint64_t db =
                            smem_desc(b_addr + (uint32_t)(h * (NI / 8) * KCB * 128) + (uint32_t)((j * KCA + ks * 2) * 128),
                                      lbo_b, sbo_b);
                        const uint32_t acc = (j > 0 || ks > 0) ? 1u : 0u;
                        asm volatile(
                            "{\n\t.reg .pred p;\n\t"
                            "setp.ne.b32 p, %4, 0;\n\t"
                            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                            ::"r"(tmem + (uint32_t)(h * NI)), "l"(da), "l"(db), "r"(instr_desc(NI)), "r"(acc)
                            : "memory");
                    }
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 smem_addr(&bar))
                             : "memory");
            }
            // the chunk's products complete before A is overwritten (bounded wait)
            const uint64_t t0 = now_ns();
            int timed_out = 0;
            while (!mbar_try_wait(&bar, parity)) {
                if (now_ns() - t0 > kWaitNs) {
                    timed_out = 1;
                    break;
                }
            }
            if (__syncthreads_or(timed_out)) {
                if (tid == 0 && status) atomicOr(status, 1u);
                failed = true;
                break;
            }
            parity ^= 1;
            fence_after();
        }
        if (failed) break;
        // epilogue: warp w reads TMEM lanes 32 (w % 4) .. and the columns of half w / 4
        const int g = warp & 3, half = warp >> 2;
        const long p = p0 + g * 32 + lane;
        const uint32_t trow = tmem + ((uint32_t)(g * 32) << 16);
#pragma unroll 1
        for (int c0 = half * (O / 2); c0 < (half + 1) * (O / 2); c0 += 16) {
            float r[16];
            tmem_ld16(trow + c0, r);
            if (p < P) {
#pragma unroll
                for (int jj = 0; jj < 16; jj++) Cm[(size_t)(c0 + jj) * P + p] = r[jj];
            }
        }
        fence_before();
        __syncthreads();
        fence_after();
    }
    cp_async_wait_all();
    __syncthreads();
    if (warp == 0) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols) : "memory");
    }
}

template <int O, int C>
cudaError_t launch_chunked(const __nv_bfloat16* W, const float* X, float* Cm, long P, unsigned* status, int swap,
                           cudaStream_t st)
{
    if (P % 8 != 0) return cudaErrorNotSupported;
    constexpr size_t smem = (size_t)kKch * kM * 4 + (size_t)kM * kKch * 2 + (size_t)O * C * 2;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_chunked<O, C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    const long tiles = (P + kM - 1) / kM;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // CTAs per SM: two by shared memory; one when a CTA holds all 512 TMEM columns
    const long per = O > 256 ? 1 : 2;
    const long grid = tiles < per * sms ? tiles : per * sms;
    k_chunked<O, C><<<(unsigned)grid, kThreads, smem, st>>>(W, X, Cm, P, (int)tiles, status, swap);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// The spectral products along x, D = A B with the rows of A contiguous in K:
// the forward DFT a = h Fx (rows: every (sample, channel, y) line of x
// values, K = grid, N = 2 modes) and its inverse spec = bb Gx (K = 2 modes,
// N = grid).  The planar spectra are read and written through the index
// maps of the mma.sync product: row m of A at (m % a_div) a_lo + (m / a_div)
// a_hi (a_div = 0: m a_lo) and K index k at (k / a_kdiv) a_khi + k % a_kdiv;
// row m of C at (m % c_div) c_lo + (m / c_div) c_hi, column n at (n / c_ndiv)
// c_nhi + n % c_ndiv.  A tile is 128 rows (one TMEM lane each); each row's
// K chunk of 64 FP32 values is staged by cp.async (16-byte pieces: a_kdiv a
// multiple of 4), rounded into the BF16 K-major A tile and accumulated in
// tensor memory; B (N x K, BF16, K-major: the transposed DFT matrix) is
// staged once per CTA.  The epilogue writes 16 consecutive columns of a row
// per 16-byte-vector group (c_ndiv a multiple of 16).
// ---------------------------------------------------------------------------
struct RowMaps {
    const float* A;
    long a_div, a_lo, a_hi;
    int a_kdiv;
    long a_khi;
    float* C;
    long c_div, c_lo, c_hi;
    int c_ndiv;
    long c_nhi;
    long M;
};

__device__ __forceinline__ long row_off(long m, long div, long lo, long hi)
{
    return div ? (m % div) * lo + (m / div) * hi : m * lo;
}

template <int K>
__device__ __forceinline__ void stage_rows(float* stage, const RowMaps& g, long m0, int j, int tid)
{
    constexpr int PIECES = kKch / 4;  // 16-byte pieces per row of a chunk
    for (int i = tid; i < kM * PIECES; i += kThreads) {
        const int r = i / PIECES, q = i - r * PIECES;
        float* dst = stage + r * kKch + 4 * q;  // [128][64]
        const long m = m0 + r;
        if (m < g.M) {
            const int k = j * kKch + 4 * q;
            const long ko = (long)(k / g.a_kdiv) * g.a_khi + k % g.a_kdiv;
            cp_async16(dst, g.A + row_off(m, g.a_div, g.a_lo, g.a_hi) + ko);
        } else {
            *reinterpret_cast<uint4*>(dst) = make_uint4(0u, 0u, 0u, 0u);
        }
    }
    cp_async_commit();
}

template <int N, int K>
__global__ void __launch_bounds__(kThreads, 1) k_rowprod(const __nv_bfloat16* __restrict__ Bt, const RowMaps g,
                                                         int ntiles, unsigned* status, int swap)
{
    constexpr int NKC = K / kKch;
    constexpr int KCB = K / 8, KCA = kKch / 8;
    constexpr uint32_t STAGE_BYTES = kM * kKch * 4, A_BYTES = kM * kKch * 2;
    constexpr uint32_t kCols = N <= 32 ? 32 : N <= 64 ? 64 : N <= 128 ? 128 : 256;
    static_assert(K % kKch == 0 && N % 32 == 0 && N <= 256, "K in chunks of 64, N per MMA 32..256");
    extern __shared__ __align__(1024) unsigned char sm[];
    float* stage = reinterpret_cast<float*>(sm);   // [128][64] FP32
    unsigned char* sa = sm + STAGE_BYTES;
    unsigned char* sb = sa + A_BYTES;
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tmem_base;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (blockIdx.x < ntiles) stage_rows<K>(stage, g, (long)blockIdx.x * kM, 0, tid);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_base)),
                     "r"(kCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) mbar_init(&bar);
    for (int i = tid; i < N * K; i += kThreads) {
        const int n = i / K, k = i - n * K;
        *reinterpret_cast<__nv_bfloat16*>(sb + kmajor_off(n, k, KCB)) = Bt[i];
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = tmem_base;
    const uint32_t a_addr = smem_addr(sa), b_addr = smem_addr(sb);
    uint32_t parity = 0;
    bool failed = false;

    for (int tile = blockIdx.x; tile < ntiles && !failed; tile += gridDim.x) {
        const long m0 = (long)tile * kM;
        for (int j = 0; j < NKC; j++) {
            cp_async_wait_all();
            __syncthreads();
            // A: 8 consecutive K values of one row per 16-byte store
            for (int i = tid; i < kM * KCA; i += kThreads) {
                const int r = i / KCA, kc = i - r * KCA;
                const float4 f0 = *reinterpret_cast<const float4*>(stage + r * kKch + kc * 8);
                const float4 f1 = *reinterpret_cast<const float4*>(stage + r * kKch + kc * 8 + 4);
                uint4 v;
                __nv_bfloat162 h0 = __floats2bfloat162_rn(f0.x, f0.y);
                __nv_bfloat162 h1 = __floats2bfloat162_rn(f0.z, f0.w);
                __nv_bfloat162 h2 = __floats2bfloat162_rn(f1.x, f1.y);
                __nv_bfloat162 h3 = __floats2bfloat162_rn(f1.z, f1.w);
                v.x = *reinterpret_cast<uint32_t*>(&h0);
                v.y = *reinterpret_cast<uint32_t*>(&h1);
                v.z = *reinterpret_cast<uint32_t*>(&h2);
                v.w = *reinterpret_cast<uint32_t*>(&h3);
                *reinterpret_cast<uint4*>(sa + kmajor_off(r, kc * 8, KCA)) = v;
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            fence_before();
            __syncthreads();
            fence_after();
            if (j + 1 < NKC) stage_rows<K>(stage, g, m0, j + 1, tid);
            else if (tile + (int)gridDim.x < ntiles) stage_rows<K>(stage, g, (long)(tile + gridDim.x) * kM, 0, tid);
            if (tid == 0) {
                const uint32_t lbo = swap ? KCA * 128 : 128, sbo_a = swap ? 128 : KCA * 128;
                const uint32_t lbo_b = swap ? KCB * 128 : 128, sbo_b = swap ? 128 : KCB * 128;
#pragma unroll
                for (int ks = 0; ks < kKch / 16; ks++) {
                    const uint64_t da = smem_desc(a_addr + ks * 256, lbo, sbo_a);
                    const uint64_t db = smem_desc(b_addr + (uint32_t)((j * KCA + ks * 2) * 128), lbo_b, sbo_b);
                    const uint32_t acc = (j > 0 || ks > 0) ? 1u : 0u;
                    asm volatile(
                        "{\n\t.reg .pred p;\n\t"
                        "setp.ne.b32 p, %4, 0;\n\t"
                        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                        ::"r"(tmem), "l"(da), "l"(db), "r"(instr_desc(N)), "r"(acc)
                        : "memory");
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 smem_addr(&bar))
                             : "memory");
            }
            const uint64_t t0 = now_ns();
            int timed_out = 0;
            while (!mbar_try_wait(&bar, parity)) {
                if (now_ns() - t0 > kWaitNs) {
                    timed_out = 1;
                    break;
                }
            }
            if (__syncthreads_or(timed_out)) {
                if (tid == 0 && status) atomicOr(status, 1u);
                failed = true;
                break;
            }
            parity ^= 1;
            fence_after();
        }
        if (failed) break;
        // epilogue: warp w reads TMEM lanes 32 (w % 4) .. (its 32 rows) and the
        // columns of half w / 4; each lane writes 16 consecutive columns of its row
        const int gq = warp & 3, half = warp >> 2;
        const long m = m0 + gq * 32 + lane;
        const uint32_t trow = tmem + ((uint32_t)(gq * 32) << 16);
        float* crow = m < g.M ? g.C + row_off(m, g.c_div, g.c_lo, g.c_hi) : nullptr;
#pragma unroll 1
        for (int c0 = half * (N / 2); c0 < (half + 1) * (N / 2); c0 += 16) {
            float r[16];
            tmem_ld16(trow + c0, r);
            if (crow) {
                float4* o = reinterpret_cast<float4*>(crow + (long)(c0 / g.c_ndiv) * g.c_nhi + c0 % g.c_ndiv);
#pragma unroll
                for (int q = 0; q < 4; q++) o[q] = make_float4(r[4 * q], r[4 * q + 1], r[4 * q + 2], r[4 * q + 3]);
            }
        }
        fence_before();
        __syncthreads();
        fence_after();
    }
    cp_async_wait_all();
    __syncthreads();
    if (warp == 0) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols) : "memory");
    }
}

template <int N, int K>
cudaError_t launch_rowprod(const __nv_bfloat16* Bt, const RowMaps& g, unsigned* status, int swap, cudaStream_t st)
{
    if (g.a_kdiv % 4 || g.c_ndiv % 16 || g.a_lo % 4 || g.a_hi % 4 || g.a_khi % 4 || g.c_lo % 4 || g.c_hi % 4 ||
        g.c_nhi % 4 || (reinterpret_cast<uintptr_t>(g.A) & 15) || (reinterpret_cast<uintptr_t>(g.C) & 15))
        return cudaErrorNotSupported;  // 16-byte pieces of A rows and C rows
    constexpr size_t smem = (size_t)kM * kKch * 4 + (size_t)kM * kKch * 2 + (size_t)N * K * 2;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_rowprod<N, K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    const long tiles = (g.M + kM - 1) / kM;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long grid = tiles < 2L * sms ? tiles : 2L * sms;
    k_rowprod<N, K><<<(unsigned)grid, kThreads, smem, st>>>(Bt, g, (int)tiles, status, swap);
    return cudaGetLastError();
}

}  // namespace umma

// The spectral products along x compiled for tcgen05 (grid 256, 32 modes):
// N x K = 64 x 256 (the forward DFT) and 256 x 64 (its inverse).
bool xspectral_umma_supported(int n, int k) { return (n == 64 && k == 256) || (n == 256 && k == 64); }

cudaError_t xspectral_umma(const __nv_bfloat16* Bt, int n, int k, const float* A, long a_div, long a_lo, long a_hi,
                           int a_kdiv, long a_khi, float* C, long c_div, long c_lo, long c_hi, int c_ndiv, long c_nhi,
                           long M, unsigned* status, int swap, cudaStream_t st)
{
    const umma::RowMaps g{A, a_div, a_lo, a_hi, a_kdiv, a_khi, C, c_div, c_lo, c_hi, c_ndiv, c_nhi, M};
    if (n == 64 && k == 256) return umma::launch_rowprod<64, 256>(Bt, g, status, swap, st);
    if (n == 256 && k == 64) return umma::launch_rowprod<256, 64>(Bt, g, status, swap, st);
    return cudaErrorNotSupported;
}

// The spectral products compiled for tcgen05 (grid 256, 32 modes):
// o x c = 64 x 512 (the forward DFT along y) and 512 x 64 (its inverse).
bool spectral_umma_supported(int o, int c) { return (o == 64 && c == 512) || (o == 512 && c == 64); }

cudaError_t spectral_umma(const __nv_bfloat16* W, int o, int c, const float* X, float* C, long P, unsigned* status,
                          int swap, cudaStream_t st)
{
    if (o == 64 && c == 512) return umma::launch_chunked<64, 512>(W, X, C, P, status, swap, st);
    if (o == 512 && c == 64) return umma::launch_chunked<512, 64>(W, X, C, P, status, swap, st);
    return cudaErrorNotSupported;
}

// The shapes of the surrogate's pointwise products that run on tcgen05:
// o x c in {64 x 64 (Fourier layers), 128 x 64 (projection 1), 64 x 8 (the
// lift: K padded to 16 with zero channels)}.  Others (the 2-channel output)
// return cudaErrorNotSupported and stay on the mma.sync product.
bool pointwise_umma_supported(int o, int c) { return (o == 64 && c == 64) || (o == 128 && c == 64) || (o == 64 && c == 8); }

cudaError_t pointwise_umma(const __nv_bfloat16* W, int o, int c, const void* X, int x_bf16, float* C, int B, long P,
                           float beta, const float* bias, void* act, int a_bf16, unsigned* status, int swap, bool write_c,
                           cudaStream_t st)
{
    const int wc = write_c ? 1 : 0;
    if (o == 64 && c == 64)
        return umma::launch_t<64, 64>(W, X, x_bf16, C, act, a_bf16, bias, beta, B, P, status, swap, wc, st);
    if (o == 128 && c == 64)
        return umma::launch_t<128, 64>(W, X, x_bf16, C, act, a_bf16, bias, beta, B, P, status, swap, wc, st);
    if (o == 64 && c == 8 && !x_bf16 && !act)
        return umma::launch<64, 16, float, float, 8>(W, (const float*)X, C, nullptr, bias, beta, B, P, status, swap, wc,
                                                     st);
    return cudaErrorNotSupported;
}

}  // namespace atmwfs

namespace atmwfs {
// Status bits of the tcgen05 products (a bounded wait that ran out), shared
// by every launch of the library on this device; read and cleared by
// atmwfs_fno_umma_status.
__device__ unsigned g_umma_status;

// Device address of the status word on the current device (looked up per call:
// a process may use several devices).
unsigned* umma_status_ptr()
{
    unsigned* p = nullptr;
    return cudaGetSymbolAddress((void**)&p, g_umma_status) == cudaSuccess ? p : nullptr;
}
}  // namespace atmwfs

extern "C" atmwfs_status atmwfs_fno_pointwise_dev(const void* W, int o, int c, const float* X, float* C, int batch,
                                                  long P, float beta, const float* bias, float* act, int engine,
                                                  void* stream)
{
    using namespace atmwfs;
    if (!W || !X || !C || o < 1 || c < 1 || batch < 1 || P < 1 || engine < 1 || engine > 2) {
        set_error_message("atmwfs_fno_pointwise_dev: bad arguments");
        return ATMWFS_ERR_INVALID;
    }
    const cudaStream_t st = (cudaStream_t)stream;
    const __nv_bfloat16* w = reinterpret_cast<const __nv_bfloat16*>(W);
    if (!pointwise_umma_supported(o, c)) {
        set_error_message("atmwfs_fno_pointwise_dev: shape not compiled for the tcgen05 product");
        return ATMWFS_ERR_INVALID;
    }
    unsigned* status = umma_status_ptr();
    if (!status) {
        set_error_message("atmwfs_fno_pointwise_dev: status symbol");
        return ATMWFS_ERR_CUDA;
    }
    const cudaError_t e = pointwise_umma(w, o, c, X, 0, C, batch, P, beta, bias, act, 0, status, engine == 2, true, st);
    if (e != cudaSuccess) {
        set_error_message(cudaGetErrorString(e));
        return ATMWFS_ERR_CUDA;
    }
    return ATMWFS_OK;
}

extern "C" atmwfs_status atmwfs_fno_spectral_dev(const void* W, int o, int c, const float* X, float* C, long P,
                                                 int engine, void* stream)
{
    using namespace atmwfs;
    if (!W || !X || !C || o < 1 || c < 1 || P < 1 || engine < 1 || engine > 2) {
        set_error_message("atmwfs_fno_spectral_dev: bad arguments");
        return ATMWFS_ERR_INVALID;
    }
    if (!spectral_umma_supported(o, c) || P % 8 != 0) {
        set_error_message("atmwfs_fno_spectral_dev: shape not compiled for the tcgen05 product");
        return ATMWFS_ERR_INVALID;
    }
    unsigned* status = umma_status_ptr();
    if (!status) {
        set_error_message("atmwfs_fno_spectral_dev: status symbol");
        return ATMWFS_ERR_CUDA;
    }
    const cudaError_t e = spectral_umma(reinterpret_cast<const __nv_bfloat16*>(W), o, c, X, C, P, status, engine == 2,
                                        (cudaStream_t)stream);
    if (e != cudaSuccess) {
        set_error_message(cudaGetErrorString(e));
        return ATMWFS_ERR_CUDA;
    }
    return ATMWFS_OK;
}

extern "C" atmwfs_status atmwfs_fno_xspectral_dev(const void* Bt, int n, int k, const float* A, long a_div, long a_lo,
                                                  long a_hi, int a_kdiv, long a_khi, float* C, long c_div, long c_lo,
                                                  long c_hi, int c_ndiv, long c_nhi, long M, int engine, void* stream)
{
    using namespace atmwfs;
    if (!Bt || !A || !C || M < 1 || a_kdiv < 1 || c_ndiv < 1 || engine < 1 || engine > 2) {
        set_error_message("atmwfs_fno_xspectral_dev: bad arguments");
        return ATMWFS_ERR_INVALID;
    }
    if (!xspectral_umma_supported(n, k)) {
        set_error_message("atmwfs_fno_xspectral_dev: shape not compiled for the tcgen05 product");
        return ATMWFS_ERR_INVALID;
    }
    unsigned* status = umma_status_ptr();
    if (!status) {
        set_error_message("atmwfs_fno_xspectral_dev: status symbol");
        return ATMWFS_ERR_CUDA;
    }
    const cudaError_t e = xspectral_umma(reinterpret_cast<const __nv_bfloat16*>(Bt), n, k, A, a_div, a_lo, a_hi, a_kdiv,
                                         a_khi, C, c_div, c_lo, c_hi, c_ndiv, c_nhi, M, status, engine == 2,
                                         (cudaStream_t)stream);
    if (e != cudaSuccess) {
        set_error_message(e == cudaErrorNotSupported ? "atmwfs_fno_xspectral_dev: maps break 16-byte pieces"
                                                     : cudaGetErrorString(e));
        return e == cudaErrorNotSupported ? ATMWFS_ERR_INVALID : ATMWFS_ERR_CUDA;
    }
    return ATMWFS_OK;
}

extern "C" unsigned atmwfs_fno_umma_status(int clear)
{
    unsigned v = 0;
    if (cudaMemcpyFromSymbol(&v, atmwfs::g_umma_status, sizeof v) != cudaSuccess) return 0xFFFFFFFFu;
    if (clear) {
        const unsigned z = 0;
        cudaMemcpyToSymbol(atmwfs::g_umma_status, &z, sizeof z);
    }
    return v;
}
