// psf.cu -- PSF consumers of the wavefront series on the GPU.
//
// Exposure PSFs (measure_wavefront_series_expoframes,
// AtmosphericTurbulence.c:6700-6735): each W x W frame amp e^{i pha} is
// placed at offset W/2 of a zero 2W x 2W field, transformed, centred
// (permut) and |F|^2 is added to the exposure.  Chromatic PSF
// (PSF_makeChromatPSF, psf.c:54-136): |FFT(amp e^{i c pha})|^2 for a list
// of coefficients c, each zoomed by c about the centre (bilinear) and
// summed with the weight m(c) / c^2.
//
// Both are two row passes of the engine's in-CTA Stockham transform
// (fft_rt): the row pass transforms only the W non-zero rows of a field
// and stores the result transposed; the column pass transforms each column
// (only its W non-zero entries are read) and, for exposures, keeps |F|^2 of
// all the frames of a batch in registers before one read-modify-write of
// the exposure accumulator.  Per frame of an exposure that is 8 B/px of the
// frame (amplitude + phase) read, 2 x 16 W^2 B of intermediate written and
// read, and 8 (2W)^2 / batch B of accumulator update.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "atmwfs_psf.h"
#include "aux_kernels.cuh"
#include "pass_impl.cuh"

namespace atmwfs {

void set_error_message(const char* msg);

// rows per CTA: 128 threads per CTA at every size
template <int N> struct PsfRows { static constexpr int RR = N <= 128 ? 16 : N <= 512 ? 8 : N == 1024 ? 4 : 2; };

// Row pass.  Field b: rows [off, off + W) hold amp * exp(i c_b pha) at
// columns [off, off + W); zero elsewhere.  Writes G[b][kx][y] for the band
// rows y (the other entries of G are never read).
template <int N>
__global__ void __launch_bounds__(Plan<N>::T * PsfRows<N>::RR)
k_psf_rows(const float* __restrict__ amp, long amp_fstride, const float* __restrict__ pha, long pha_fstride,
           const float* __restrict__ cscale, int W, int off, float2* __restrict__ G, const float2* __restrict__ tw)
{
    constexpr int RR = PsfRows<N>::RR, T = Plan<N>::T, E = Plan<N>::E, NT = T * RR, RS = row_stride<N>();
    constexpr int RL = last_radix<N>();
    __shared__ __align__(16) float2 xb[RR * RS];
    const int tid = threadIdx.x, t = tid % T, rr = tid / T;
    const int b = blockIdx.y;
    const int yb = blockIdx.x * RR + rr;
    const float c = cscale ? cscale[b] : 1.0f;
    const float* A = amp + (size_t)b * amp_fstride + (size_t)yb * W;
    const float* P = pha + (size_t)b * pha_fstride + (size_t)yb * W;
    float2* xrow = xb + rr * RS;
    float2 v[E];
#pragma unroll
    for (int e = 0; e < E; e++) {
        const int xi = t + e * T - off;
        if (xi >= 0 && xi < W) {
            const float a = A[xi];
            const float2 z = phasor(__fmul_rn(c, P[xi]));     // c * pha: float, as the reference's image product
            v[e] = make_float2(a * z.x, a * z.y);
        } else {
            v[e] = make_float2(0.0f, 0.0f);
        }
    }
    fft_rt<N, T, E>(v, xrow, t, tw, -1.0f, 0);
    __syncthreads();
#pragma unroll
    for (int s = 0; s < E; s++) xrow[padi(last_index<N, T, RL>(t, s))] = v[s];
    __syncthreads();
    float2* dst = G + (size_t)b * N * N + off + blockIdx.x * RR;
#pragma unroll 4
    for (int k = 0; k < E; k++) {
        const int idx = tid + NT * k;
        const int r2 = idx % RR, x = idx / RR;
        dst[(size_t)x * N + r2] = xb[r2 * RS + padi(x)];
    }
}

// Column pass over the B fields of G: one column per CTA, the fields spread
// over F frame lanes of the CTA (lane f takes fields f, f + F, ...), so that
// a batch of fields keeps F transforms of the column in flight per CTA (a
// column per CTA with the fields in sequence left a 1024-column transform
// with 1.7 CTAs of four warps per SM).  mode 0 (exposure): acc[kx][ky] +=
// |F_b[ky][kx]|^2 for b = 0..B-1: each lane sums its fields in order, then
// the lanes' partial sums are added to the accumulator in lane order (the
// accumulator is kept transposed and uncentred so that these updates are
// coalesced).  mode 1 (chromatic): I[b][kx][ky] = |F_b[ky][kx]|^2.
template <int N> struct PsfLanes { static constexpr int F = Plan<N>::T >= 64 ? 2 : 4; };

template <int N>
__global__ void __launch_bounds__(Plan<N>::T * PsfLanes<N>::F, 4)
k_psf_cols(const float2* __restrict__ G, int B, int W, int off, int mode, float* __restrict__ out,
           const float2* __restrict__ tw)
{
    constexpr int F = PsfLanes<N>::F, T = Plan<N>::T, E = Plan<N>::E, RS = row_stride<N>();
    constexpr int RL = last_radix<N>();
    static_assert(F * RS * 2 >= F * N, "the lane sums fit the exchange rows");
    __shared__ __align__(16) float2 xb[F * RS];
    const int tid = threadIdx.x, t = tid % T, f = tid / T;
    const int kx = blockIdx.x;
    float2* xrow = xb + f * RS;
    float s2[E];
#pragma unroll
    for (int s = 0; s < E; s++) s2[s] = 0.0f;
    // the same trip count in every lane (lanes may share a warp when T < 32)
#pragma unroll 1
    for (int b0 = 0; b0 < B; b0 += F) {
        const int b = b0 + f;
        const bool have = b < B;
        const float2* src = G + (size_t)(have ? b : 0) * N * N + (size_t)kx * N;
        float2 v[E];
#pragma unroll
        for (int e = 0; e < E; e++) {
            const int yi = t + e * T - off;
            v[e] = (have && yi >= 0 && yi < W) ? src[t + e * T] : make_float2(0.0f, 0.0f);
        }
        fft_rt<N, T, E>(v, xrow, t, tw, -1.0f, 0);
        if (mode == 0) {
#pragma unroll
            for (int s = 0; s < E; s++)
                s2[s] = __fadd_rn(s2[s], __fadd_rn(__fmul_rn(v[s].x, v[s].x), __fmul_rn(v[s].y, v[s].y)));
        } else if (have) {
            float* I = out + (size_t)b * N * N + (size_t)kx * N;
#pragma unroll
            for (int s = 0; s < E; s++)
                I[last_index<N, T, RL>(t, s)] = __fadd_rn(__fmul_rn(v[s].x, v[s].x), __fmul_rn(v[s].y, v[s].y));
        }
    }
    if (mode == 0) {
        __syncthreads();  // every lane's last transform is done with its exchange row
        float* red = reinterpret_cast<float*>(xb);  // [F][N]
#pragma unroll
        for (int s = 0; s < E; s++) red[f * N + last_index<N, T, RL>(t, s)] = s2[s];
        __syncthreads();
        for (int k = tid; k < N; k += T * F) {
            float p = red[k];
#pragma unroll
            for (int g = 1; g < F; g++) p = __fadd_rn(p, red[g * N + k]);
            out[(size_t)kx * N + k] = __fadd_rn(out[(size_t)kx * N + k], p);
        }
    }
}

// Exposure accumulator <-> the reference's centred image:
// img[j][i] = acc[(i + h) % N][(j + h) % N]; the same formula maps the image
// back (the map is an involution since 2 h = N).
__global__ void k_expo_layout(const float* __restrict__ src, float* __restrict__ dst, int N)
{
    __shared__ float tile[32][33];
    const int h = N / 2;
    const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
    for (int r = threadIdx.y; r < 32; r += blockDim.y) tile[r][threadIdx.x] = src[(size_t)(by + r) * N + bx + threadIdx.x];
    __syncthreads();
    // dst[q][p] = src[(p + h) % N][(q + h) % N]: src row by + c, column bx + r
    // goes to dst row (bx + r + h) % N, column (by + c + h) % N
    for (int r = threadIdx.y; r < 32; r += blockDim.y)
        dst[(size_t)((bx + r + h) % N) * N + (by + threadIdx.x + h) % N] = tile[threadIdx.x][r];
}

// Chromatic sum (psf.c:104-131): out[jj][ii] += m_s * bilinear(I_s, x, y) /
// c_s / c_s for s = 0..S-1 in order.  x = (ii - n/2) c_s + n/2 is rounded
// once to float (fmaf: the product of a small integer and a float is exact,
// as in the reference's double expression), i = (long) x truncates, the
// weights follow the reference's double and float expressions, and the
// accumulation is in float.  I_s is centred on read: I(j, i) =
// I_s[(i + h) % n][(j + h) % n].
__global__ void k_chromat_sum(const float* __restrict__ I, int S, int n, const float* __restrict__ coeff,
                              const float* __restrict__ mcoeff, float* __restrict__ out)
{
    const long np = (long)n * n;
    const int h = n / 2;
    for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < np; p += (long)gridDim.x * blockDim.x) {
        const int ii = (int)(p % n), jj = (int)(p / n);
        float acc = out[p];
        for (int s = 0; s < S; s++) {
            const float c = coeff[s];
            const float x = fmaf((float)(ii - h), c, (float)h);
            const float y = fmaf((float)(jj - h), c, (float)h);
            const int i = (int)x, j = (int)y;
            const float u = x - (float)i, t = y - (float)j;
            if (i < n - 1 && j < n - 1 && i > -1 && j > -1) {
                const float* Is = I + (size_t)s * np;
                const float v00 = Is[(size_t)((i + h) % n) * n + (j + h) % n];
                const float v01 = Is[(size_t)((i + h) % n) * n + (j + 1 + h) % n];
                const float v10 = Is[(size_t)((i + 1 + h) % n) * n + (j + h) % n];
                const float v11 = Is[(size_t)((i + 1 + h) % n) * n + (j + 1 + h) % n];
                const double du = 1.0 - (double)u, dt = 1.0 - (double)t;
                float tmp = (float)(du * dt * (double)v00);
                tmp = (float)((double)tmp + du * (double)t * (double)v01);
                tmp = (float)((double)tmp + (double)u * dt * (double)v10);
                tmp = __fadd_rn(tmp, __fmul_rn(__fmul_rn(u, t), v11));   // u * t * F: float arithmetic
                acc = __fadd_rn(acc, __fdiv_rn(__fdiv_rn(__fmul_rn(mcoeff[s], tmp), c), c));
            }
        }
        out[p] = acc;
    }
}

template <int N>
static cudaError_t psf_rows_n(const float* amp, long as, const float* pha, long ps, const float* cs, int W, int off,
                              int B, float2* G, const float2* tw, cudaStream_t st)
{
    constexpr int RR = PsfRows<N>::RR;
    if (W % RR != 0 || W > N || off + W > N) return cudaErrorInvalidValue;
    k_psf_rows<N><<<dim3((unsigned)(W / RR), (unsigned)B), Plan<N>::T * RR, 0, st>>>(amp, as, pha, ps, cs, W, off, G, tw);
    return cudaGetLastError();
}

template <int N>
static cudaError_t psf_cols_n(const float2* G, int B, int W, int off, int mode, float* out, const float2* tw,
                              cudaStream_t st)
{
    k_psf_cols<N><<<N, Plan<N>::T * PsfLanes<N>::F, 0, st>>>(G, B, W, off, mode, out, tw);
    return cudaGetLastError();
}

cudaError_t psf_rows(int N, const float* amp, long as, const float* pha, long ps, const float* cs, int W, int off,
                     int B, float2* G, const float2* tw, cudaStream_t st)
{
    switch (N) {
        case 64: return psf_rows_n<64>(amp, as, pha, ps, cs, W, off, B, G, tw, st);
        case 128: return psf_rows_n<128>(amp, as, pha, ps, cs, W, off, B, G, tw, st);
        case 256: return psf_rows_n<256>(amp, as, pha, ps, cs, W, off, B, G, tw, st);
        case 512: return psf_rows_n<512>(amp, as, pha, ps, cs, W, off, B, G, tw, st);
        case 1024: return psf_rows_n<1024>(amp, as, pha, ps, cs, W, off, B, G, tw, st);
        case 2048: return psf_rows_n<2048>(amp, as, pha, ps, cs, W, off, B, G, tw, st);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t psf_cols(int N, const float2* G, int B, int W, int off, int mode, float* out, const float2* tw,
                     cudaStream_t st)
{
    switch (N) {
        case 64: return psf_cols_n<64>(G, B, W, off, mode, out, tw, st);
        case 128: return psf_cols_n<128>(G, B, W, off, mode, out, tw, st);
        case 256: return psf_cols_n<256>(G, B, W, off, mode, out, tw, st);
        case 512: return psf_cols_n<512>(G, B, W, off, mode, out, tw, st);
        case 1024: return psf_cols_n<1024>(G, B, W, off, mode, out, tw, st);
        case 2048: return psf_cols_n<2048>(G, B, W, off, mode, out, tw, st);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t chromat_sum(const float* I, int S, int n, const float* coeff, const float* mcoeff, float* out,
                        cudaStream_t st)
{
    k_chromat_sum<<<4 * 152, 256, 0, st>>>(I, S, n, coeff, mcoeff, out);
    return cudaGetLastError();
}

}  // namespace atmwfs

// ---------------------------------------------------------------------------
// C ABI (include/atmwfs_psf.h), device side
// ---------------------------------------------------------------------------
using namespace atmwfs;

namespace {

atmwfs_status psf_fail(atmwfs_status s, const char* msg)
{
    set_error_message(msg);
    return s;
}

atmwfs_status psf_cuda(cudaError_t e, const char* what)
{
    if (e == cudaSuccess) return ATMWFS_OK;
    char buf[256];
    snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
    set_error_message(buf);
    return e == cudaErrorMemoryAllocation ? ATMWFS_ERR_NOMEM : ATMWFS_ERR_CUDA;
}

bool pow2_between(long n, long lo, long hi) { return n >= lo && n <= hi && (n & (n - 1)) == 0; }

// Fields per launch: about 256 MB of intermediate, 1..64 fields.
long psf_batch(long N) { return std::max(1L, std::min(64L, (256L << 20) / (N * N * 8))); }

// Step coefficients and weights with the reference's types (psf.c:86-99):
// float coeff, x and mcoeff from double expressions.
void chromat_weights(float coeff1, float coeff2, long nbstep, float apo, std::vector<float>& c, std::vector<float>& m)
{
    const float eps = 1.0e-5f;
    c.resize(nbstep);
    m.resize(nbstep);
    for (long step = 0; step < nbstep; step++) {
        const float coeff = (float)(coeff1 * pow(pow((coeff2 / coeff1), 1.0 / (nbstep - 1)), (double)step));
        const float x = (float)((coeff - (coeff1 + coeff2) / 2.0) / ((coeff2 - coeff1) / 2.0));
        float mc;
        if (apo > eps)
            mc = (float)pow((1.0 - pow((fabs(x) - (1.0 - apo)) / apo, 2.0)), 4.0);
        else
            mc = 1.0f;
        if ((1.0 - x * x) < eps) mc = 0.0f;
        if (fabs(x) < apo) mc = 1.0f;
        c[step] = coeff;
        m[step] = mc;
    }
}

}  // namespace

extern "C" {

atmwfs_status atmwfs_psf_expo_accumulate_dev(const float* amp, long amp_fstride, const float* pha, long W,
                                             long nframes, float* acc, void* stream)
{
    if (!amp || !pha || !acc) return psf_fail(ATMWFS_ERR_INVALID, "null buffer");
    if (!pow2_between(W, 32, 1024)) return psf_fail(ATMWFS_ERR_INVALID, "frame size must be a power of two in 32..1024");
    if (nframes < 0 || amp_fstride < 0) return psf_fail(ATMWFS_ERR_INVALID, "negative frame count or stride");
    if (nframes == 0) return ATMWFS_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const long N = 2 * W;
    const float2* tw = stage_twiddles((int)N);
    if (!tw) return psf_fail(ATMWFS_ERR_NOMEM, "twiddle allocation failed");
    const long B = std::min(psf_batch(N), nframes);
    float2* G = nullptr;
    atmwfs_status s = psf_cuda(cudaMallocAsync((void**)&G, sizeof(float2) * B * N * N, st), "intermediate allocation");
    if (s != ATMWFS_OK) return s;
    for (long f0 = 0; f0 < nframes && s == ATMWFS_OK; f0 += B) {
        const long b = std::min(B, nframes - f0);
        s = psf_cuda(psf_rows((int)N, amp + f0 * amp_fstride, amp_fstride, pha + f0 * W * W, W * W, nullptr, (int)W,
                              (int)(W / 2), (int)b, G, tw, st), "row pass");
        if (s == ATMWFS_OK) s = psf_cuda(psf_cols((int)N, G, (int)b, (int)W, (int)(W / 2), 0, acc, tw, st), "column pass");
    }
    cudaFreeAsync(G, st);
    return s;
}

atmwfs_status atmwfs_psf_expo_image_dev(const float* acc, long W, float* img, void* stream)
{
    if (!acc || !img || acc == img) return psf_fail(ATMWFS_ERR_INVALID, "null or aliased buffer");
    if (!pow2_between(W, 32, 1024)) return psf_fail(ATMWFS_ERR_INVALID, "frame size must be a power of two in 32..1024");
    const int N = (int)(2 * W);
    k_expo_layout<<<dim3(N / 32, N / 32), dim3(32, 8), 0, (cudaStream_t)stream>>>(acc, img, N);
    return psf_cuda(cudaGetLastError(), "layout kernel");
}

atmwfs_status atmwfs_psf_expo_load_dev(const float* img, long W, float* acc, void* stream)
{
    return atmwfs_psf_expo_image_dev(img, W, acc, stream);   // the same involution
}

atmwfs_status atmwfs_psf_expo_accumulate(const float* amp, long amp_fstride, const float* pha, long W, long nframes,
                                         float* psf)
{
    if (!amp || !pha || !psf) return psf_fail(ATMWFS_ERR_INVALID, "null buffer");
    if (!pow2_between(W, 32, 1024)) return psf_fail(ATMWFS_ERR_INVALID, "frame size must be a power of two in 32..1024");
    if (nframes < 0 || amp_fstride < 0) return psf_fail(ATMWFS_ERR_INVALID, "negative frame count or stride");
    const long N = 2 * W;
    const long namp = (amp_fstride && nframes > 0) ? amp_fstride * (nframes - 1) + W * W : W * W;
    float *da = nullptr, *dp = nullptr, *dimg = nullptr, *dacc = nullptr;
    atmwfs_status s = psf_cuda(cudaMalloc(&da, sizeof(float) * namp), "allocation");
    if (s == ATMWFS_OK) s = psf_cuda(cudaMalloc(&dp, sizeof(float) * std::max(nframes, 1L) * W * W), "allocation");
    if (s == ATMWFS_OK) s = psf_cuda(cudaMalloc(&dimg, sizeof(float) * N * N), "allocation");
    if (s == ATMWFS_OK) s = psf_cuda(cudaMalloc(&dacc, sizeof(float) * N * N), "allocation");
    if (s == ATMWFS_OK) s = psf_cuda(cudaMemcpy(da, amp, sizeof(float) * namp, cudaMemcpyHostToDevice), "copy");
    if (s == ATMWFS_OK && nframes > 0)
        s = psf_cuda(cudaMemcpy(dp, pha, sizeof(float) * nframes * W * W, cudaMemcpyHostToDevice), "copy");
    if (s == ATMWFS_OK) s = psf_cuda(cudaMemcpy(dimg, psf, sizeof(float) * N * N, cudaMemcpyHostToDevice), "copy");
    if (s == ATMWFS_OK) s = atmwfs_psf_expo_load_dev(dimg, W, dacc, nullptr);
    if (s == ATMWFS_OK) s = atmwfs_psf_expo_accumulate_dev(da, amp_fstride, dp, W, nframes, dacc, nullptr);
    if (s == ATMWFS_OK) s = atmwfs_psf_expo_image_dev(dacc, W, dimg, nullptr);
    if (s == ATMWFS_OK) s = psf_cuda(cudaMemcpy(psf, dimg, sizeof(float) * N * N, cudaMemcpyDeviceToHost), "copy");
    cudaFree(da);
    cudaFree(dp);
    cudaFree(dimg);
    cudaFree(dacc);
    return s;
}

atmwfs_status atmwfs_chromat_psf(const float* amp, const float* pha, long n, float coeff1, float coeff2, long nbstep,
                                 float apo_coeff, float* out)
{
    if (!amp || !pha || !out) return psf_fail(ATMWFS_ERR_INVALID, "null buffer");
    if (!pow2_between(n, 64, 2048)) return psf_fail(ATMWFS_ERR_INVALID, "size must be a power of two in 64..2048");
    if (nbstep < 1 || !(coeff1 > 0) || !(coeff2 > 0)) return psf_fail(ATMWFS_ERR_INVALID, "bad coefficients");
    std::vector<float> c, m;
    chromat_weights(coeff1, coeff2, nbstep, apo_coeff, c, m);
    const float2* tw = stage_twiddles((int)n);
    if (!tw) return psf_fail(ATMWFS_ERR_NOMEM, "twiddle allocation failed");
    const long B = std::min(psf_batch(n), nbstep);
    float *da = nullptr, *dp = nullptr, *dI = nullptr, *dout = nullptr, *dc = nullptr, *dm = nullptr;
    float2* G = nullptr;
    atmwfs_status s = psf_cuda(cudaMalloc(&da, sizeof(float) * n * n), "allocation");
    if (s == ATMWFS_OK) s = psf_cuda(cudaMalloc(&dp, sizeof(float) * n * n), "allocation");
    if (s == ATMWFS_OK) s = psf_cuda(cudaMalloc(&dI, sizeof(float) * B * n * n), "allocation");
    if (s == ATMWFS_OK) s = psf_cuda(cudaMalloc(&G, sizeof(float2) * B * n * n), "allocation");
    if (s == ATMWFS_OK) s = psf_cuda(cudaMalloc(&dout, sizeof(float) * n * n), "allocation");
    if (s == ATMWFS_OK) s = psf_cuda(cudaMalloc(&dc, sizeof(float) * nbstep), "allocation");
    if (s == ATMWFS_OK) s = psf_cuda(cudaMalloc(&dm, sizeof(float) * nbstep), "allocation");
    if (s == ATMWFS_OK) s = psf_cuda(cudaMemcpy(da, amp, sizeof(float) * n * n, cudaMemcpyHostToDevice), "copy");
    if (s == ATMWFS_OK) s = psf_cuda(cudaMemcpy(dp, pha, sizeof(float) * n * n, cudaMemcpyHostToDevice), "copy");
    if (s == ATMWFS_OK) s = psf_cuda(cudaMemcpy(dc, c.data(), sizeof(float) * nbstep, cudaMemcpyHostToDevice), "copy");
    if (s == ATMWFS_OK) s = psf_cuda(cudaMemcpy(dm, m.data(), sizeof(float) * nbstep, cudaMemcpyHostToDevice), "copy");
    if (s == ATMWFS_OK) s = psf_cuda(cudaMemset(dout, 0, sizeof(float) * n * n), "memset");
    for (long s0 = 0; s0 < nbstep && s == ATMWFS_OK; s0 += B) {
        const long b = std::min(B, nbstep - s0);
        s = psf_cuda(psf_rows((int)n, da, 0, dp, 0, dc + s0, (int)n, 0, (int)b, G, tw, nullptr), "row pass");
        if (s == ATMWFS_OK) s = psf_cuda(psf_cols((int)n, G, (int)b, (int)n, 0, 1, dI, tw, nullptr), "column pass");
        if (s == ATMWFS_OK) s = psf_cuda(chromat_sum(dI, (int)b, (int)n, dc + s0, dm + s0, dout, nullptr), "zoom sum");
    }
    if (s == ATMWFS_OK) s = psf_cuda(cudaMemcpy(out, dout, sizeof(float) * n * n, cudaMemcpyDeviceToHost), "copy");
    cudaFree(da);
    cudaFree(dp);
    cudaFree(dI);
    cudaFree(G);
    cudaFree(dout);
    cudaFree(dc);
    cudaFree(dm);
    return s;
}

}  // extern "C"
