// fft_large.cu -- unnormalised 2-D DFT of 4096^2 and 8192^2 complex grids,
// the transform behind master screens of that size (the reference's
// make_master_turbulence_screen, AtmosphericTurbulence.c:643-855, calls
// do2dfft on the full M x M spectrum, :783).
//
// One CTA of 256 threads owns one row: each thread holds M / 256 values in
// registers and the engine's Stockham stages (fft_rt) run three in-register
// radix stages (16 x 16 x 16 for 4096, 32 x 16 x 16 for 8192) with two
// exchanges through one padded shared row (68 KB at 8192, two CTAs per SM).
// Columns are done as rows of the transposed grid:
//   rows(in -> out), transpose(out -> tmp), rows(tmp -> tmp), transpose(tmp -> out).
// Every pass streams the grid once through HBM (read + write), so the
// transform moves 4 x 2 x 8 M^2 bytes: 4.3 GB at 8192^2.
// The whole-row plans of 4096 and 8192 points run faster with scalar
// butterflies (0.97 against 1.07 ms for an 8192^2 transform).
#define AW_SCALAR_BUTTERFLY 1
#include "aux_kernels.cuh"
#include "pass_impl.cuh"

namespace atmwfs {

// One row per CTA; in may equal out (the whole row is in registers before
// the first store).  ds = -1 forward, +1 inverse.
template <int N>
__global__ void __launch_bounds__(Plan<N>::T) k_fft_row_plan(const float2* in, float2* out,
                                                             const float2* __restrict__ tw, float ds)
{
    constexpr int T = Plan<N>::T, E = Plan<N>::E, RL = last_radix<N>();
    extern __shared__ float4 big_smem[];
    float2* xrow = reinterpret_cast<float2*>(big_smem);
    const int t = threadIdx.x;
    const size_t row = (size_t)blockIdx.x * N;
    float2 v[E];
#pragma unroll
    for (int e = 0; e < E; e++) v[e] = in[row + t + e * T];
    fft_rt<N, T, E>(v, xrow, t, tw, ds, 0);
    __syncthreads();
#pragma unroll
    for (int s = 0; s < E; s++) xrow[padi(last_index<N, T, RL>(t, s))] = v[s];
    __syncthreads();
#pragma unroll
    for (int e = 0; e < E; e++) out[row + t + e * T] = xrow[padi(t + e * T)];
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

template <int M>
static cudaError_t fft2d_large_t(const float2* in, float2* out, float2* tmp, int sign, cudaStream_t st)
{
    const float2* tw = stage_twiddles(M);
    if (!tw) return cudaErrorMemoryAllocation;
    const int smem = row_stride<M>() * (int)sizeof(float2);
    cudaError_t e = cudaFuncSetAttribute(k_fft_row_plan<M>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    const float ds = sign < 0 ? -1.0f : 1.0f;
    const dim3 tg(M / 32, M / 32), tb(32, 8);
    k_fft_row_plan<M><<<M, Plan<M>::T, smem, st>>>(in, out, tw, ds);
    k_transpose_c<<<tg, tb, 0, st>>>(out, tmp, M);
    k_fft_row_plan<M><<<M, Plan<M>::T, smem, st>>>(tmp, tmp, tw, ds);
    k_transpose_c<<<tg, tb, 0, st>>>(tmp, out, M);
    return cudaGetLastError();
}

cudaError_t fft2d_large(const float2* in, float2* out, float2* tmp, int M, int sign, cudaStream_t st)
{
    if (M == 4096) return fft2d_large_t<4096>(in, out, tmp, sign, st);
    if (M == 8192) return fft2d_large_t<8192>(in, out, tmp, sign, st);
    return cudaErrorInvalidValue;
}

}  // namespace atmwfs
