// fno_gemm.cuh -- batched GEMM for the neural-operator surrogate:
//   C[b] = alpha * op(A[b]) * op(B[b]) + beta * C[b] (+ bias[n])
// with BF16 tensor-core products (mma.sync m16n8k16) and FP32
// accumulation.  Operands are read as FP32 or BF16 from global memory and
// rounded to BF16 while they are staged in shared memory; C is FP32.
// Split-K over grid.z, and batches summed into one C (batch stride 0 for
// C, as weight gradients are), accumulate with atomics into a C that
// gemm_launch has prepared (beta applied once).
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
    const float* bias;    // added once (first split) or NULL
    int bias_rows;        // 1: bias[m] per row, else bias[n] per column
    int splitk;           // K ranges over grid.z % splitk
    int batch;
};

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

template <int BM, int BN>
__global__ void __launch_bounds__(256) k_gemm(const GemmArgs g)
{
    using S = Shape<BM, BN>;
    __shared__ __align__(16) __nv_bfloat16 As[BM][BK + PADK];
    __shared__ __align__(16) __nv_bfloat16 Bs[BN][BK + PADK];  // n-major: k contiguous
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = warp / S::WN, wn = warp % S::WN;
    const int gq = lane >> 2, tq = lane & 3;
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
    const int bz = blockIdx.z / g.splitk, sk = blockIdx.z % g.splitk;
    const char* Ab = reinterpret_cast<const char*>(g.A) + (size_t)bz * g.sA * (g.a_bf16 ? 2 : 4);
    const char* Bb = reinterpret_cast<const char*>(g.B) + (size_t)bz * g.sB * (g.b_bf16 ? 2 : 4);
    float* Cb = g.C + (size_t)bz * g.sC;
    // K range of this split, a multiple of BK
    const int kchunks = (g.K + BK - 1) / BK;
    const int per = (kchunks + g.splitk - 1) / g.splitk;
    const int kc0 = sk * per, kc1 = min(kchunks, kc0 + per);

    float acc[S::TM][S::TN][4];
#pragma unroll
    for (int i = 0; i < S::TM; i++)
#pragma unroll
        for (int j = 0; j < S::TN; j++)
#pragma unroll
            for (int q = 0; q < 4; q++) acc[i][j][q] = 0.0f;

    for (int kc = kc0; kc < kc1; kc++) {
        const int k0 = kc * BK;
        __syncthreads();
        // stage A: BM x BK elements, op(A)[m][k]
        for (int e = tid; e < BM * BK; e += 256) {
            int mm, kk;
            if (g.ta) { mm = e % BM; kk = e / BM; }   // stored K x M: m contiguous
            else { kk = e % BK; mm = e / BK; }        // stored M x K: k contiguous
            const int m = m0 + mm, k = k0 + kk;
            float v = 0.0f;
            if (m < g.M && k < g.K) v = ld_elem(Ab, g.ta ? (long)k * g.lda + m : (long)m * g.lda + k, g.a_bf16);
            As[mm][kk] = __float2bfloat16_rn(v);
        }
        // stage B: BK x BN elements, op(B)[k][n] stored n-major
        for (int e = tid; e < BN * BK; e += 256) {
            int nn, kk;
            if (g.tb) { kk = e % BK; nn = e / BK; }   // stored N x K: k contiguous
            else { nn = e % BN; kk = e / BN; }        // stored K x N: n contiguous
            const int n = n0 + nn, k = k0 + kk;
            float v = 0.0f;
            if (n < g.N && k < g.K) v = ld_elem(Bb, g.tb ? (long)n * g.ldb + k : (long)k * g.ldb + n, g.b_bf16);
            Bs[nn][kk] = __float2bfloat16_rn(v);
        }
        __syncthreads();
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
    // epilogue: C (already scaled by beta) += alpha * acc (+ bias once)
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
                if (g.bias && sk == 0 && (bz == 0 || g.sC != 0)) v += g.bias_rows ? g.bias[m] : g.bias[n];
                float* c = Cb + (size_t)m * g.ldc + n;
                // split K, or a batch summed into one C: several CTAs add here
                if (g.splitk > 1 || (g.batch > 1 && g.sC == 0)) atomicAdd(c, v);
                else *c += v;
            }
}

}  // namespace gemm

// C = alpha op(A) op(B) + beta C (+ bias); beta 0 clears C first.
cudaError_t gemm_launch(const GemmArgs& g, float beta, cudaStream_t st);

}  // namespace atmwfs
