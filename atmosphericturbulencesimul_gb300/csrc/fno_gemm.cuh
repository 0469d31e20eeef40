// fno_gemm.cuh -- batched GEMM for the neural-operator surrogate:
//   C[b] = alpha * op(A[b]) * op(B[b]) + beta * C[b] (+ bias[n])
// with BF16 tensor-core products (mma.sync m16n8k16) and FP32
// accumulation.  Operands are read as FP32 or BF16 from global memory and
// rounded to BF16 while they are staged in shared memory; C is FP32.
// The epilogue applies beta itself (C is read only when beta != 0), except
// for split-K over grid.z and batches summed into one C (batch stride 0
// for C, as weight gradients are): those accumulate with atomics into a C
// that gemm_launch has scaled by beta beforehand.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace atmwfs {

struct GemmArgs {
    int M, N, K;
    const void* A;  // op(A) is M x K
    const void* B;  // op(B) is K x N
    float* C;       // M x N, row stride ldc
    long lda, ldb, ldc;
    long sA, sB, sC;      // batch strides (elements)
    int ta, tb;           // 1: A stored K x M / B stored N x K
    int a_bf16, b_bf16;   // storage type of A / B (else FP32)
    float alpha;
    float beta;           // applied in the epilogue unless the C is shared (atomic accumulation)
    const float* bias;    // added once (first split) or NULL
    int bias_rows;        // 1: bias[m] per row, else bias[n] per column
    int splitk;           // K ranges over grid.z % splitk
    int batch;
    float* C2;            // optional: gelu of the final C value, same layout (not with shared accumulation)
    // Optional index maps (0 = off; private C only).  Row m of C at
    // (m % rdiv) c_lo + (m / rdiv) c_hi instead of m ldc; column n of C at
    // (n / cdiv) cc_hi + n % cdiv; column k of A (stored M x K) at
    // (k / kdiv) ka_hi + k % kdiv.  They let a product read or write planar
    // and transposed layouts directly (multiples of 4 keep 16-byte vectors).
    int rdiv;
    long c_lo, c_hi;
    int cdiv;
    long cc_hi;
    int kdiv;
    long ka_hi;
    int ardiv;            // row m of A (stored M x K) at (m % ardiv) a_lo + (m / ardiv) a_hi
    long a_lo, a_hi;
};

// GELU, tanh form (Hendrycks & Gimpel 2016): 0.5 x (1 + tanh(c (x + 0.044715 x^3))), c = sqrt(2 / pi)
__device__ __forceinline__ float gelu_f(float x)
{
    const float c = 0.7978845608028654f;
    return 0.5f * x * (1.0f + tanhf(c * (x + 0.044715f * x * x * x)));
}

namespace gemm {

constexpr int BK = 32;
constexpr int PADK = 8;   // smem row pad (bf16): 80-byte rows, conflict-free fragment loads

__device__ __forceinline__ float ld_elem(const void* p, long i, int bf)
{
    if (bf) return __bfloat162float(reinterpret_cast<const __nv_bfloat16*>(p)[i]);
    return reinterpret_cast<const float*>(p)[i];
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// Tile BM x BN x BK, 256 threads = WM x WN warps; each warp owns a
// (BM / WM) x (BN / WN) block of m16 x n8 products.
template <int BM, int BN>
struct Shape {
    static constexpr int WM = BM == 128 ? 2 : (BN == 128 ? 1 : 2);
    static constexpr int WN = 8 / WM;
    static constexpr int TM = BM / WM / 16;  // m16 tiles per warp
    static constexpr int TN = BN / WN / 8;   // n8 tiles per warp
    static_assert(TM >= 1 && TN >= 1 && WM * WN == 8, "256 threads");
};

// Four consecutive elements along the operand's contiguous dimension:
// one vector load when they are in range and aligned, else element loads
// with zero fill.
__device__ __forceinline__ float4 ld4(const char* base, long i, long lim, int bf, bool vec)
{
    if (vec && i + 3 < lim) {
        if (bf) {
            const uint2 u = *reinterpret_cast<const uint2*>(base + i * 2);
            const __nv_bfloat162 lo = *reinterpret_cast<const __nv_bfloat162*>(&u.x);
            const __nv_bfloat162 hi = *reinterpret_cast<const __nv_bfloat162*>(&u.y);
            return make_float4(__low2float(lo), __high2float(lo), __low2float(hi), __high2float(hi));
        }
        return *reinterpret_cast<const float4*>(base + i * 4);
    }
    float4 r;
    r.x = i + 0 < lim ? ld_elem(base, i + 0, bf) : 0.0f;
    r.y = i + 1 < lim ? ld_elem(base, i + 1, bf) : 0.0f;
    r.z = i + 2 < lim ? ld_elem(base, i + 2, bf) : 0.0f;
    r.w = i + 3 < lim ? ld_elem(base, i + 3, bf) : 0.0f;
    return r;
}

__device__ __forceinline__ uint2 pack4(float4 v)
{
    const __nv_bfloat162 lo = __floats2bfloat162_rn(v.x, v.y), hi = __floats2bfloat162_rn(v.z, v.w);
    uint2 u;
    u.x = *reinterpret_cast<const uint32_t*>(&lo);
    u.y = *reinterpret_cast<const uint32_t*>(&hi);
    return u;
}

template <int BM, int BN>
__global__ void __launch_bounds__(256, 2) k_gemm(const GemmArgs g)
{
    using S = Shape<BM, BN>;
    constexpr int NA = BM * BK / 1024, NB = BN * BK / 1024;  // 4-element groups per thread
    __shared__ __align__(16) __nv_bfloat16 As[BM][BK + PADK];
    __shared__ __align__(16) __nv_bfloat16 Bs[BN][BK + PADK];  // n-major: k contiguous
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = warp / S::WN, wn = warp % S::WN;
    const int gq = lane >> 2, tq = lane & 3;
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
    const int bz = blockIdx.z / g.splitk, sk = blockIdx.z % g.splitk;
    const int esa = g.a_bf16 ? 2 : 4, esb = g.b_bf16 ? 2 : 4;
    const char* Ab = reinterpret_cast<const char*>(g.A) + (size_t)bz * g.sA * esa;
    const char* Bb = reinterpret_cast<const char*>(g.B) + (size_t)bz * g.sB * esb;
    float* Cb = g.C + (size_t)bz * g.sC;
    // vector loads need the contiguous dimension's stride and the base aligned
    const bool va = (g.lda % 4 == 0) && ((reinterpret_cast<uintptr_t>(Ab) & (4 * esa - 1)) == 0) &&
                    (!g.ardiv || (g.a_lo % 4 == 0 && g.a_hi % 4 == 0));
    const bool vb = (g.ldb % 4 == 0) && ((reinterpret_cast<uintptr_t>(Bb) & (4 * esb - 1)) == 0);
    // K range of this split, a multiple of BK
    const int kchunks = (g.K + BK - 1) / BK;
    const int per = (kchunks + g.splitk - 1) / g.splitk;
    const int kc0 = sk * per, kc1 = min(kchunks, kc0 + per);

    float4 ra[NA], rb[NB];
    auto load = [&](int kc) {
        const int k0 = kc * BK;
#pragma unroll
        for (int j = 0; j < NA; j++) {
            const int e = (tid + 256 * j) * 4;
            if (g.ta) {  // stored K x M: 4 consecutive m
                const int kk = e / BM, mm = e % BM, k = k0 + kk;
                ra[j] = (k < g.K) ? ld4(Ab + (size_t)k * g.lda * esa, m0 + mm, g.M, g.a_bf16, va)
                                  : make_float4(0.f, 0.f, 0.f, 0.f);
            } else {     // stored M x K: 4 consecutive k (one block of a split never straddles 4)
                const int mm = e / BK, kk = e % BK, m = m0 + mm, k = k0 + kk;
                const long ksh = g.kdiv ? (long)(k / g.kdiv) * (g.ka_hi - g.kdiv) : 0;   // split offset of column k
                const size_t aro = g.ardiv ? (size_t)(m % g.ardiv) * g.a_lo + (size_t)(m / g.ardiv) * g.a_hi
                                           : (size_t)m * g.lda;
                ra[j] = (m < g.M) ? ld4(Ab + (aro + ksh) * esa, k, g.K, g.a_bf16, va)
                                  : make_float4(0.f, 0.f, 0.f, 0.f);
            }
        }
#pragma unroll
        for (int j = 0; j < NB; j++) {
            const int e = (tid + 256 * j) * 4;
            if (g.tb) {  // stored N x K: 4 consecutive k
                const int nn = e / BK, kk = e % BK, n = n0 + nn;
                rb[j] = (n < g.N) ? ld4(Bb + (size_t)n * g.ldb * esb, k0 + kk, g.K, g.b_bf16, vb)
                                  : make_float4(0.f, 0.f, 0.f, 0.f);
            } else {     // stored K x N: 4 consecutive n
                const int kk = e / BN, nn = e % BN, k = k0 + kk;
                rb[j] = (k < g.K) ? ld4(Bb + (size_t)k * g.ldb * esb, n0 + nn, g.N, g.b_bf16, vb)
                                  : make_float4(0.f, 0.f, 0.f, 0.f);
            }
        }
    };
    auto store = [&]() {
#pragma unroll
        for (int j = 0; j < NA; j++) {
            const int e = (tid + 256 * j) * 4;
            if (g.ta) {
                const int kk = e / BM, mm = e % BM;
                As[mm + 0][kk] = __float2bfloat16_rn(ra[j].x);
                As[mm + 1][kk] = __float2bfloat16_rn(ra[j].y);
                As[mm + 2][kk] = __float2bfloat16_rn(ra[j].z);
                As[mm + 3][kk] = __float2bfloat16_rn(ra[j].w);
            } else {
                const int mm = e / BK, kk = e % BK;
                *reinterpret_cast<uint2*>(&As[mm][kk]) = pack4(ra[j]);
            }
        }
#pragma unroll
        for (int j = 0; j < NB; j++) {
            const int e = (tid + 256 * j) * 4;
            if (g.tb) {
                const int nn = e / BK, kk = e % BK;
                *reinterpret_cast<uint2*>(&Bs[nn][kk]) = pack4(rb[j]);
            } else {
                const int kk = e / BN, nn = e % BN;
                Bs[nn + 0][kk] = __float2bfloat16_rn(rb[j].x);
                Bs[nn + 1][kk] = __float2bfloat16_rn(rb[j].y);
                Bs[nn + 2][kk] = __float2bfloat16_rn(rb[j].z);
                Bs[nn + 3][kk] = __float2bfloat16_rn(rb[j].w);
            }
        }
    };

    float acc[S::TM][S::TN][4];
#pragma unroll
    for (int i = 0; i < S::TM; i++)
#pragma unroll
        for (int j = 0; j < S::TN; j++)
#pragma unroll
            for (int q = 0; q < 4; q++) acc[i][j][q] = 0.0f;

    if (kc0 < kc1) load(kc0);
    for (int kc = kc0; kc < kc1; kc++) {
        __syncthreads();  // the previous chunk's fragments are read
        store();
        __syncthreads();
        if (kc + 1 < kc1) load(kc + 1);  // next chunk's global loads overlap this chunk's products
#pragma unroll
        for (int ks = 0; ks < BK; ks += 16) {
            uint32_t af[S::TM][4], bfr[S::TN][2];
#pragma unroll
            for (int i = 0; i < S::TM; i++) {
                const int r = wm * (BM / S::WM) + i * 16 + gq;
                af[i][0] = *reinterpret_cast<const uint32_t*>(&As[r][ks + 2 * tq]);
                af[i][1] = *reinterpret_cast<const uint32_t*>(&As[r + 8][ks + 2 * tq]);
                af[i][2] = *reinterpret_cast<const uint32_t*>(&As[r][ks + 2 * tq + 8]);
                af[i][3] = *reinterpret_cast<const uint32_t*>(&As[r + 8][ks + 2 * tq + 8]);
            }
#pragma unroll
            for (int j = 0; j < S::TN; j++) {
                const int c = wn * (BN / S::WN) + j * 8 + gq;
                bfr[j][0] = *reinterpret_cast<const uint32_t*>(&Bs[c][ks + 2 * tq]);
                bfr[j][1] = *reinterpret_cast<const uint32_t*>(&Bs[c][ks + 2 * tq + 8]);
            }
#pragma unroll
            for (int i = 0; i < S::TM; i++)
#pragma unroll
                for (int j = 0; j < S::TN; j++)
                    mma_bf16(acc[i][j], af[i][0], af[i][1], af[i][2], af[i][3], bfr[j][0], bfr[j][1]);
        }
    }
    // epilogue.  A private C (no split K, no batch summed into one C) goes
    // through a shared-memory stage so that C, its beta term and the
    // activation move as whole 16-byte vectors along rows; a shared C takes
    // atomics from the fragments (gemm_launch scaled it by beta beforehand).
    const bool shared = g.splitk > 1 || (g.batch > 1 && g.sC == 0);
    const bool add_bias = g.bias && sk == 0 && (bz == 0 || g.sC != 0);
    if (shared) {
#pragma unroll
        for (int i = 0; i < S::TM; i++)
#pragma unroll
            for (int j = 0; j < S::TN; j++)
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int m = m0 + wm * (BM / S::WM) + i * 16 + gq + (q >= 2 ? 8 : 0);
                    const int n = n0 + wn * (BN / S::WN) + j * 8 + 2 * tq + (q & 1);
                    if (m >= g.M || n >= g.N) continue;
                    float v = g.alpha * acc[i][j][q];
                    if (add_bias) v += g.bias_rows ? g.bias[m] : g.bias[n];
                    atomicAdd(Cb + (size_t)m * g.ldc + n, v);
                }
        return;
    }
    extern __shared__ float4 gemm_stage[];
    constexpr int LDS = BN + 4;                 // padded row of the stage (floats)
    float* Cs = reinterpret_cast<float*>(gemm_stage);
#pragma unroll
    for (int i = 0; i < S::TM; i++)
#pragma unroll
        for (int j = 0; j < S::TN; j++)
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int ml = wm * (BM / S::WM) + i * 16 + gq + (q >= 2 ? 8 : 0);
                const int nl = wn * (BN / S::WN) + j * 8 + 2 * tq + (q & 1);
                Cs[ml * LDS + nl] = g.alpha * acc[i][j][q];
            }
    __syncthreads();
    const bool v4 = (g.ldc % 4 == 0) && ((reinterpret_cast<uintptr_t>(Cb) & 15) == 0) &&
                    (!g.C2 || ((reinterpret_cast<uintptr_t>(g.C2 + (size_t)bz * g.sC) & 15) == 0)) &&
                    (!g.rdiv || (g.c_lo % 4 == 0 && g.c_hi % 4 == 0)) &&
                    (!g.cdiv || (g.cdiv % 4 == 0 && g.cc_hi % 4 == 0));
    float* C2b = g.C2 ? g.C2 + (size_t)bz * g.sC : nullptr;
    const bool loadc = g.beta != 0.0f;
    if (!loadc) {
        // plain stores, one vector at a time
        for (int idx = tid; idx < BM * BN / 4; idx += 256) {
            const int ml = idx / (BN / 4), nl = (idx % (BN / 4)) * 4;
            const int m = m0 + ml, n = n0 + nl;
            if (m >= g.M || n >= g.N) continue;
            float4 v = *reinterpret_cast<const float4*>(&Cs[ml * LDS + nl]);
            const size_t roff = g.rdiv ? (size_t)(m % g.rdiv) * g.c_lo + (size_t)(m / g.rdiv) * g.c_hi : (size_t)m * g.ldc;
            const long csh = g.cdiv ? (long)(n / g.cdiv) * (g.cc_hi - g.cdiv) : 0;   // split offset of column n
            float* c = Cb + roff + csh + n;
            float* c2 = C2b ? C2b + roff + csh + n : nullptr;
            if (v4 && n + 3 < g.N) {
                if (add_bias) {
                    if (g.bias_rows) {
                        const float b = g.bias[m];
                        v.x += b; v.y += b; v.z += b; v.w += b;
                    } else {
                        v.x += g.bias[n]; v.y += g.bias[n + 1]; v.z += g.bias[n + 2]; v.w += g.bias[n + 3];
                    }
                }
                *reinterpret_cast<float4*>(c) = v;
                if (c2) *reinterpret_cast<float4*>(c2) = make_float4(gelu_f(v.x), gelu_f(v.y), gelu_f(v.z), gelu_f(v.w));
            } else {
                const float vv[4] = {v.x, v.y, v.z, v.w};
                for (int e = 0; e < 4 && n + e < g.N; e++) {
                    float x = vv[e];
                    if (add_bias) x += g.bias_rows ? g.bias[m] : g.bias[n + e];
                    c[e] = x;
                    if (c2) c2[e] = gelu_f(x);
                }
            }
        }
        return;
    }
    // with a beta term: groups of four vectors per thread, the old values of
    // a group all requested before the group's first store (their loads overlap)
    constexpr int ITER = BM * BN / 4 / 256, GRP = 4;
    static_assert(ITER % GRP == 0, "whole groups");
#pragma unroll 1
    for (int g0 = 0; g0 < ITER; g0 += GRP) {
        float4 val[GRP], old[GRP];
        size_t off[GRP];
        int mq[GRP], nq[GRP];
#pragma unroll
        for (int q = 0; q < GRP; q++) {
            const int idx = tid + 256 * (g0 + q);
            const int ml = idx / (BN / 4), nl = (idx % (BN / 4)) * 4;
            const int m = m0 + ml, n = n0 + nl;
            mq[q] = m;
            nq[q] = n;
            val[q] = *reinterpret_cast<const float4*>(&Cs[ml * LDS + nl]);
            const size_t roff = g.rdiv ? (size_t)(m % g.rdiv) * g.c_lo + (size_t)(m / g.rdiv) * g.c_hi : (size_t)m * g.ldc;
            const long csh = g.cdiv ? (long)(n / g.cdiv) * (g.cc_hi - g.cdiv) : 0;   // split offset of column n
            off[q] = roff + csh + n;
            old[q] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (loadc && v4 && m < g.M && n + 3 < g.N) old[q] = *reinterpret_cast<const float4*>(Cb + off[q]);
        }
#pragma unroll
        for (int q = 0; q < GRP; q++) {
            const int m = mq[q], n = nq[q];
            if (m >= g.M || n >= g.N) continue;
            float4 v = val[q];
            float* c = Cb + off[q];
            float* c2 = C2b ? C2b + off[q] : nullptr;
            if (v4 && n + 3 < g.N) {
                if (add_bias) {
                    if (g.bias_rows) {
                        const float b = g.bias[m];
                        v.x += b; v.y += b; v.z += b; v.w += b;
                    } else {
                        v.x += g.bias[n]; v.y += g.bias[n + 1]; v.z += g.bias[n + 2]; v.w += g.bias[n + 3];
                    }
                }
                if (loadc) {
                    const float4 o = old[q];
                    v.x = fmaf(g.beta, o.x, v.x); v.y = fmaf(g.beta, o.y, v.y);
                    v.z = fmaf(g.beta, o.z, v.z); v.w = fmaf(g.beta, o.w, v.w);
                }
                *reinterpret_cast<float4*>(c) = v;
                if (c2) *reinterpret_cast<float4*>(c2) = make_float4(gelu_f(v.x), gelu_f(v.y), gelu_f(v.z), gelu_f(v.w));
            } else {
                const float vv[4] = {v.x, v.y, v.z, v.w};
                for (int e = 0; e < 4 && n + e < g.N; e++) {
                    float x = vv[e];
                    if (add_bias) x += g.bias_rows ? g.bias[m] : g.bias[n + e];
                    if (loadc) x = fmaf(g.beta, c[e], x);
                    c[e] = x;
                    if (c2) c2[e] = gelu_f(x);
                }
            }
        }
    }
}

// dynamic shared memory of the epilogue stage of a BM x BN tile
constexpr size_t stage_bytes(int BM, int BN) { return (size_t)BM * (BN + 4) * sizeof(float); }

}  // namespace gemm

// C = alpha op(A) op(B) + beta C (+ bias); beta 0 clears C first.
cudaError_t gemm_launch(const GemmArgs& g, float beta, cudaStream_t st);

}  // namespace atmwfs
