// fno_gemm.cu -- tile choice, beta handling and the C-ABI test entry of the
// surrogate's BF16 GEMM.
#include <algorithm>

#include "atmwfs.h"
#include "atmwfs_fno.h"
#include "fno_gemm.cuh"

namespace atmwfs {

void set_error_message(const char* msg);

namespace {

__global__ void k_scale_rows(float* C, long ldc, long sC, int M, int N, float beta)
{
    float* c = C + (size_t)blockIdx.z * sC;
    for (int m = blockIdx.y; m < M; m += gridDim.y)
        for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
            float* p = c + (size_t)m * ldc + n;
            *p = beta == 0.0f ? 0.0f : *p * beta;
        }
}

}  // namespace

template <int BM, int BN>
cudaError_t launch_tile(dim3 grid, const GemmArgs& g, cudaStream_t st)
{
    constexpr size_t sm = gemm::stage_bytes(BM, BN);
    static bool attr = false;
    if (!attr) {
        const cudaError_t e = cudaFuncSetAttribute(gemm::k_gemm<BM, BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    gemm::k_gemm<BM, BN><<<grid, 256, sm, st>>>(g);
    return cudaGetLastError();
}

cudaError_t gemm_launch(const GemmArgs& g0, float beta, cudaStream_t st)
{
    GemmArgs g = g0;
    if (g.M <= 0 || g.N <= 0 || g.batch <= 0) return cudaSuccess;
    // a split block must hold whole 4-element vectors; A maps need A stored M x K
    if ((g.cdiv && (g.cdiv % 4 || g.cc_hi % 4)) || (g.kdiv && (g.kdiv % 4 || g.ka_hi % 4 || g.ta)) ||
        (g.ardiv && g.ta))
        return cudaErrorInvalidValue;
    const bool bm128 = g.M > 64, bn128 = g.N > 64;
    const int BM = bm128 ? 128 : 64, BN = bn128 ? 128 : 64;
    const long tiles = (long)((g.M + BM - 1) / BM) * ((g.N + BN - 1) / BN) * g.batch;
    // split K until the grid covers the GPU a few times over (long, thin products)
    const int kchunks = (g.K + gemm::BK - 1) / gemm::BK;
    int split = 1;
    while (split < 64 && tiles * split < 4 * 152 && kchunks / (split * 2) >= 4) split *= 2;
    if (g.splitk < 1) g.splitk = split;
    if (g.rdiv || g.cdiv) g.splitk = 1;   // index maps: private C only
    if ((long)g.batch * g.splitk > 65535) g.splitk = std::max(1, 65535 / g.batch);
    const bool atomic = g.splitk > 1 || (g.batch > 1 && g.sC == 0);
    g.beta = beta;
    if ((atomic || g.K <= 0) && beta != 1.0f) {
        // shared accumulation (or no product): scale or clear C once
        const int nb = g.sC == 0 ? 1 : g.batch;
        const dim3 grid((unsigned)std::min((g.N + 255) / 256, 64), (unsigned)std::min(g.M, 1024), (unsigned)nb);
        k_scale_rows<<<grid, 256, 0, st>>>(g.C, g.ldc, g.sC, g.M, g.N, beta);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    if (g.K <= 0) return cudaSuccess;
    const dim3 grid((unsigned)((g.M + BM - 1) / BM), (unsigned)((g.N + BN - 1) / BN), (unsigned)(g.batch * g.splitk));
    if (bm128 && bn128) return launch_tile<128, 128>(grid, g, st);
    if (!bm128 && bn128) return launch_tile<64, 128>(grid, g, st);
    if (bm128 && !bn128) return launch_tile<128, 64>(grid, g, st);
    return launch_tile<64, 64>(grid, g, st);
}

}  // namespace atmwfs

extern "C" atmwfs_status atmwfs_gemm_bf16(int M, int N, int K, const void* A, long lda, int ta, int a_bf16,
                                          const void* B, long ldb, int tb, int b_bf16, float* C, long ldc,
                                          float alpha, float beta, const float* bias, int batch, long sA, long sB,
                                          long sC, void* stream)
{
    using namespace atmwfs;
    if (!A || !B || !C || M < 0 || N < 0 || K < 0 || batch < 1) {
        set_error_message("atmwfs_gemm_bf16: bad arguments");
        return ATMWFS_ERR_INVALID;
    }
    GemmArgs g{};
    g.M = M; g.N = N; g.K = K;
    g.A = A; g.B = B; g.C = C;
    g.lda = lda; g.ldb = ldb; g.ldc = ldc;
    g.sA = sA; g.sB = sB; g.sC = sC;
    g.ta = ta; g.tb = tb; g.a_bf16 = a_bf16; g.b_bf16 = b_bf16;
    g.alpha = alpha; g.bias = bias; g.bias_rows = 0; g.splitk = 0; g.batch = batch;
    const cudaError_t e = gemm_launch(g, beta, (cudaStream_t)stream);
    if (e != cudaSuccess) {
        set_error_message(cudaGetErrorString(e));
        return ATMWFS_ERR_CUDA;
    }
    return ATMWFS_OK;
}
