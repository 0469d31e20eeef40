// fft_large.cu -- unnormalised 2-D DFT of 4096^2 and 8192^2 complex grids,
// the transform behind master screens of that size (the reference's
// make_master_turbulence_screen, AtmosphericTurbulence.c:643-855, calls
// do2dfft on the full M x M spectrum, :783).
//
// The in-CTA plans of the propagation engine stop at 2048 points per row.
// Here one CTA of 1024 threads owns one row: the row is loaded into shared
// memory (two ping-pong buffers, 2 * M * 8 bytes: 128 KB at 8192), run
// through radix-4 Stockham stages (plus one radix-2 stage when log2 M is
// odd) and stored back.  Columns are done as rows of the transposed grid:
//   rows(in -> out), transpose(out -> tmp), rows(tmp -> tmp), transpose(tmp -> out).
// Every pass streams the grid once through HBM (read + write), so the
// transform costs 4 x 2 x 8 M^2 bytes: 4.3 GB, about 0.7 ms, at 8192^2.
#include <cmath>
#include <map>
#include <mutex>
#include <vector>

#include "aux_kernels.cuh"

namespace atmwfs {

constexpr int kBigThreads = 1024;

// One row per CTA.  tw[m] = exp(-2 pi i m / M), m < M (evaluated in double
// on the host); the inverse transform uses its conjugate.  in may equal out:
// the whole row is in shared memory before the first store.
__global__ void __launch_bounds__(kBigThreads, 1)
k_fft_row_big(const float2* in, float2* out, const float2* __restrict__ tw, int M, int sign)
{
    extern __shared__ float4 big_smem[];
    float2* src = reinterpret_cast<float2*>(big_smem);
    float2* dst = src + M;
    const size_t row = (size_t)blockIdx.x * M;
    const float4* in4 = reinterpret_cast<const float4*>(in + row);
    for (int i = threadIdx.x; i < M / 2; i += kBigThreads) reinterpret_cast<float4*>(src)[i] = in4[i];
    __syncthreads();
    const float ws = sign < 0 ? 1.0f : -1.0f;     // conjugate the table for the inverse
    const int q = M / 4;
    int Ns = 1;
    for (; Ns * 4 <= M; Ns *= 4) {
        const int ts = M / (4 * Ns);
        for (int j = threadIdx.x; j < q; j += kBigThreads) {
            const int k = j & (Ns - 1);
            float2 a0 = src[j], a1 = src[j + q], a2 = src[j + 2 * q], a3 = src[j + 3 * q];
            if (Ns > 1) {
                float2 w1 = __ldg(&tw[k * ts]), w2 = __ldg(&tw[2 * k * ts]), w3 = __ldg(&tw[3 * k * ts]);
                w1.y *= ws;
                w2.y *= ws;
                w3.y *= ws;
                a1 = cmul(a1, w1);
                a2 = cmul(a2, w2);
                a3 = cmul(a3, w3);
            }
            // 4-point DFT; (sign i) * a = (-sign a.y, sign a.x)
            const float s = (float)sign;
            const float2 p = make_float2(a0.x + a2.x, a0.y + a2.y), m = make_float2(a0.x - a2.x, a0.y - a2.y);
            const float2 r = make_float2(a1.x + a3.x, a1.y + a3.y), d = make_float2(a1.x - a3.x, a1.y - a3.y);
            const float2 wd = make_float2(-s * d.y, s * d.x);
            const int o = (j - k) * 4 + k;
            dst[o] = make_float2(p.x + r.x, p.y + r.y);
            dst[o + Ns] = make_float2(m.x + wd.x, m.y + wd.y);
            dst[o + 2 * Ns] = make_float2(p.x - r.x, p.y - r.y);
            dst[o + 3 * Ns] = make_float2(m.x - wd.x, m.y - wd.y);
        }
        __syncthreads();
        float2* t = src;
        src = dst;
        dst = t;
    }
    if (Ns < M) {       // last radix-2 stage: Ns = M / 2, k = j
        const int h = M / 2;
        for (int j = threadIdx.x; j < h; j += kBigThreads) {
            float2 w = __ldg(&tw[j]);
            w.y *= ws;
            const float2 a0 = src[j], a1 = cmul(src[j + h], w);
            dst[j] = make_float2(a0.x + a1.x, a0.y + a1.y);
            dst[j + h] = make_float2(a0.x - a1.x, a0.y - a1.y);
        }
        __syncthreads();
        src = dst;
    }
    float4* out4 = reinterpret_cast<float4*>(out + row);
    for (int i = threadIdx.x; i < M / 2; i += kBigThreads) out4[i] = reinterpret_cast<const float4*>(src)[i];
}

// out[x][y] = in[y][x] through 32 x 32 tiles (padded against bank conflicts).
__global__ void k_transpose_c(const float2* __restrict__ in, float2* __restrict__ out, int M)
{
    __shared__ float2 tile[32][33];
    const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
    for (int r = threadIdx.y; r < 32; r += blockDim.y) tile[r][threadIdx.x] = in[(size_t)(by + r) * M + bx + threadIdx.x];
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += blockDim.y) out[(size_t)(bx + r) * M + by + threadIdx.x] = tile[threadIdx.x][r];
}

bool fft2d_large_supported(long M) { return M == 4096 || M == 8192; }

// tw[m] = exp(-2 pi i m / M) for m < M, one copy per (device, M).
static const float2* big_twiddles(int M)
{
    static std::mutex mu;
    static std::map<std::pair<int, int>, float2*> cache;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    const auto key = std::make_pair(dev, M);
    const auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    std::vector<float2> h(M);
    for (int m = 0; m < M; m++) {
        const double a = -2.0 * M_PI * (double)m / (double)M;
        h[m] = make_float2((float)cos(a), (float)sin(a));
    }
    float2* d = nullptr;
    if (cudaMalloc(&d, sizeof(float2) * M) != cudaSuccess) return nullptr;
    if (cudaMemcpy(d, h.data(), sizeof(float2) * M, cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(d);
        return nullptr;
    }
    cache[key] = d;
    return d;
}

cudaError_t fft2d_large(const float2* in, float2* out, float2* tmp, int M, int sign, cudaStream_t st)
{
    if (!fft2d_large_supported(M)) return cudaErrorInvalidValue;
    const float2* tw = big_twiddles(M);
    if (!tw) return cudaErrorMemoryAllocation;
    const int smem = 2 * M * (int)sizeof(float2);
    cudaError_t e = cudaFuncSetAttribute(k_fft_row_big, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    const dim3 tg(M / 32, M / 32), tb(32, 8);
    k_fft_row_big<<<M, kBigThreads, smem, st>>>(in, out, tw, M, sign);
    k_transpose_c<<<tg, tb, 0, st>>>(out, tmp, M);
    k_fft_row_big<<<M, kBigThreads, smem, st>>>(tmp, tmp, tw, M, sign);
    k_transpose_c<<<tg, tb, 0, st>>>(tmp, out, M);
    return cudaGetLastError();
}

}  // namespace atmwfs
