// fno.cu -- Fourier neural operator surrogate of the multi-layer Fresnel
// propagation: forward, backward and Adam on the GPU with the project's
// BF16 tensor-core GEMM (fno_gemm.cuh) and elementwise kernels.
//
// Model (channel-major activations [B][C][G][G], FP32 in HBM):
//   h0 = Wlift x + blift                          (pointwise, nin -> w)
//   for l < nl:  u = Wl h + bl + S_l(h);  h = gelu(u) (no activation after the last layer)
//   out = P2 gelu(P1 h + c1) + c2                 (pointwise, w -> p -> nout)
// with the spectral convolution on the modes ky in [-m/2, m/2), kx in [0, m):
//   a = h Fx            (real DFT along x, G -> m complex, as [re | im] columns)
//   z = Fy a            (DFT along y of the kept rows)
//   y[k] = R_l[k] z[k]  (complex w x w mixing per mode)
//   s = Re(Gx (Gy y))   (inverse DFTs, kx > 0 counted twice, 1 / G^2)
// Parameters are FP32 masters with a BF16 mirror that the products read.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "atmwfs.h"
#include "atmwfs_fno.h"
#include "fno_gemm.cuh"

namespace atmwfs {
void set_error_message(const char* msg);
}

using namespace atmwfs;

struct FnoLayout {
    int nin, w, m, nl, p, nout, G;
    long lift_W, lift_b, proj1_W, proj1_b, proj2_W, proj2_b, total;
    std::vector<long> R, W, b;
    void build()
    {
        long o = 0;
        lift_W = o; o += (long)w * nin;
        lift_b = o; o += w;
        R.resize(nl); W.resize(nl); b.resize(nl);
        for (int l = 0; l < nl; l++) {
            R[l] = o; o += (long)m * m * w * w * 2;
            W[l] = o; o += (long)w * w;
            b[l] = o; o += w;
        }
        proj1_W = o; o += (long)p * w;
        proj1_b = o; o += p;
        proj2_W = o; o += (long)nout * p;
        proj2_b = o; o += nout;
        total = o;
    }
};

namespace atmwfs {
// tcgen05 pointwise product (fno_umma.cu)
bool pointwise_umma_supported(int o, int c);
cudaError_t pointwise_umma(const __nv_bfloat16* W, int o, int c, const void* X, int x_bf16, float* C, int B, long P,
                           float beta, const float* bias, void* act, int a_bf16, unsigned* status, int swap, bool write_c,
                           cudaStream_t st);
unsigned* umma_status_ptr();
bool spectral_umma_supported(int o, int c);
bool xspectral_umma_supported(int n, int k);
cudaError_t xspectral_umma(const __nv_bfloat16* Bt, int n, int k, const float* A, long a_div, long a_lo, long a_hi,
                           int a_kdiv, long a_khi, float* C, long c_div, long c_lo, long c_hi, int c_ndiv, long c_nhi,
                           long M, unsigned* status, int swap, cudaStream_t st);
cudaError_t spectral_umma(const __nv_bfloat16* W, int o, int c, const float* X, float* C, long P, unsigned* status,
                          int swap, cudaStream_t st);
}  // namespace atmwfs

struct atmwfs_fno {
    atmwfs_fno_cfg cfg;
    FnoLayout L;
    float* params = nullptr;            // FP32 masters
    __nv_bfloat16* pbf = nullptr;       // BF16 mirror read by the products
    float* grads = nullptr;
    float* adam_m = nullptr;
    float* adam_v = nullptr;
    long step = 0;
    // DFT matrices (FP32, rounded to BF16 by the products), and BF16 copies
    // of the y transforms for the tcgen05 spectral products
    float *Fx = nullptr, *FyAB = nullptr, *GyBig = nullptr, *Gx = nullptr;
    __nv_bfloat16 *FyAB_bf = nullptr, *GyBig_bf = nullptr;
    __nv_bfloat16 *FxT_bf = nullptr, *GxT_bf = nullptr;  // the x transforms transposed (N x K)
    // activations for one batch size
    int cap = 0;
    std::vector<float*> h, u, a, z;     // h[0..nl], u[0..nl-1], a/z per layer
    float *y = nullptr, *bb = nullptr, *qpre = nullptr, *q = nullptr;
    float *dh = nullptr, *dh2 = nullptr, *du = nullptr, *dq = nullptr, *dz = nullptr, *dy = nullptr, *da = nullptr, *dbb = nullptr;
    float* dout = nullptr;               // gradient of the loss at the output, [B][nout][G][G]
    double* d_loss = nullptr;
    std::vector<void*> allocs;
};

namespace {

bool umma_enabled();

const double kPi = 3.14159265358979323846264338328;

atmwfs_status err(atmwfs_status s, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    set_error_message(buf);
    return s;
}

#define FN_CUDA(x)                                                                            \
    do {                                                                                      \
        const cudaError_t e_ = (x);                                                           \
        if (e_ != cudaSuccess) return err(ATMWFS_ERR_CUDA, "%s: %s", #x, cudaGetErrorString(e_)); \
    } while (0)

#define FN_TRY(x)                                   \
    do {                                            \
        const atmwfs_status s_ = (x);               \
        if (s_ != ATMWFS_OK) return s_;             \
    } while (0)

atmwfs_status dalloc(atmwfs_fno* f, void** p, size_t bytes)
{
    if (cudaMalloc(p, bytes) != cudaSuccess) return err(ATMWFS_ERR_NOMEM, "cudaMalloc(%zu) failed", bytes);
    f->allocs.push_back(*p);
    return ATMWFS_OK;
}

// ---------------------------------------------------------------------------
// elementwise kernels
// ---------------------------------------------------------------------------
// GELU (gelu_f, fno_gemm.cuh) and its derivative
__device__ __forceinline__ float gelu_d(float x)
{
    const float c = 0.7978845608028654f;
    const float t = tanhf(c * (x + 0.044715f * x * x * x));
    return 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * c * (1.0f + 3.0f * 0.044715f * x * x);
}

__global__ void k_gelu(const float* __restrict__ in, float* __restrict__ out, long n)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        out[i] = gelu_f(in[i]);
}

__global__ void k_gelu_bwd(const float* __restrict__ dy, const float* __restrict__ x, float* __restrict__ dx, long n)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        dx[i] = dy[i] * gelu_d(x[i]);
}

// db[c] += sum over b, pixels of d[b][c][:]
__global__ void k_rowsum(const float* __restrict__ d, float* __restrict__ db, int B, int C, long P)
{
    const int c = blockIdx.y;
    float s = 0.0f;
    for (int bq = 0; bq < B; bq++) {
        const float* r = d + ((size_t)bq * C + c) * P;
        for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < P; i += (long)gridDim.x * blockDim.x) s += r[i];
    }
    __shared__ float red[32];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0f;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) atomicAdd(&db[c], s);
    }
}

// mean squared error and its gradient: dout = 2 (out - t) / n
__global__ void k_mse(const float* __restrict__ out, const float* __restrict__ t, float* __restrict__ dout, long n,
                      double* loss)
{
    double s = 0.0;
    const float inv = 2.0f / (float)n;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const float d = out[i] - t[i];
        dout[i] = inv * d;
        s += (double)d * d;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, s / (double)n);
}

// Mode mixing y[b][o][k] = sum_c R[k][o][c] z[b][c][k] (complex), one block
// per mode k = (ky, kx).  z / y layout [2m][B w][m]: row ky holds the real
// parts, row m + ky the imaginary parts, then (sample, channel), then kx.
__global__ void k_modemix(const __nv_bfloat16* __restrict__ R, const float* __restrict__ z, float* __restrict__ y,
                          int B, int w, int m)
{
    const int k = blockIdx.x, ky = k / m, kx = k % m;
    const long plane = m;                                     // (sample, channel) stride
    const long Nc = (long)B * w * m;
    const long ore = (long)ky * Nc + kx, oim = (long)(m + ky) * Nc + kx;
    extern __shared__ float sh[];
    float* zs = sh;                  // [B][w][2]
    float2* rs = reinterpret_cast<float2*>(sh + 2 * B * w);  // [w][w + 1]: R[o][c], padded rows
    const __nv_bfloat16* Rk = R + (size_t)k * w * w * 2;
    for (int i = threadIdx.x; i < w * w; i += blockDim.x) {
        const __nv_bfloat162 v = reinterpret_cast<const __nv_bfloat162*>(Rk)[i];  // coalesced (re, im) pairs
        rs[(i / w) * (w + 1) + i % w] = make_float2(__low2float(v), __high2float(v));
    }
    for (int i = threadIdx.x; i < B * w; i += blockDim.x) {
        zs[2 * i] = z[i * plane + ore];
        zs[2 * i + 1] = z[i * plane + oim];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < B * w; i += blockDim.x) {
        const int bq = i / w, o = i % w;
        const float2* r = rs + o * (w + 1);
        const float* zb = zs + 2 * bq * w;
        float sr = 0.0f, si = 0.0f;
        for (int c = 0; c < w; c++) {
            const float2 rc = r[c];
            const float zr = zb[2 * c], zi = zb[2 * c + 1];
            sr += rc.x * zr - rc.y * zi;
            si += rc.x * zi + rc.y * zr;
        }
        y[i * plane + ore] = sr;
        y[i * plane + oim] = si;
    }
}

// Backward of the mode mixing: dz = R^H dy per mode, and dR += sum_b dy z^H.
__global__ void k_modemix_bwd(const __nv_bfloat16* __restrict__ R, const float* __restrict__ z,
                              const float* __restrict__ dy, float* __restrict__ dz, float* __restrict__ dR, int B, int w,
                              int m)
{
    const int k = blockIdx.x, ky = k / m, kx = k % m;
    const long plane = m;                                     // (sample, channel) stride
    const long Nc = (long)B * w * m;
    const long ore = (long)ky * Nc + kx, oim = (long)(m + ky) * Nc + kx;
    extern __shared__ float sh[];
    float* zs = sh;                  // [B][w][2]
    float* ds = sh + 2 * B * w;      // [B][w][2]
    float2* rs = reinterpret_cast<float2*>(sh + 4 * B * w);  // [w][w + 1]
    const __nv_bfloat16* Rk = R + (size_t)k * w * w * 2;
    float* dRk = dR + (size_t)k * w * w * 2;
    for (int i = threadIdx.x; i < w * w; i += blockDim.x) {
        const __nv_bfloat162 v = reinterpret_cast<const __nv_bfloat162*>(Rk)[i];
        rs[(i / w) * (w + 1) + i % w] = make_float2(__low2float(v), __high2float(v));
    }
    for (int i = threadIdx.x; i < B * w; i += blockDim.x) {
        zs[2 * i] = z[i * plane + ore];
        zs[2 * i + 1] = z[i * plane + oim];
        ds[2 * i] = dy[i * plane + ore];
        ds[2 * i + 1] = dy[i * plane + oim];
    }
    __syncthreads();
    // dz[b][c] = sum_o conj(R[o][c]) dy[b][o]
    for (int i = threadIdx.x; i < B * w; i += blockDim.x) {
        const int bq = i / w, c = i % w;
        const float* db = ds + 2 * bq * w;
        float sr = 0.0f, si = 0.0f;
        for (int o = 0; o < w; o++) {
            const float2 rc = rs[o * (w + 1) + c];
            const float dr = db[2 * o], di = db[2 * o + 1];
            sr += rc.x * dr + rc.y * di;
            si += rc.x * di - rc.y * dr;
        }
        dz[i * plane + ore] = sr;
        dz[i * plane + oim] = si;
    }
    // dR[o][c] += sum_b dy[b][o] conj(z[b][c]); consecutive threads walk c (coalesced)
    for (int i = threadIdx.x; i < w * w; i += blockDim.x) {
        const int o = i / w, c = i % w;
        float sr = 0.0f, si = 0.0f;
        for (int bq = 0; bq < B; bq++) {
            const float dr = ds[2 * (bq * w + o)], di = ds[2 * (bq * w + o) + 1];
            const float zr = zs[2 * (bq * w + c)], zi = zs[2 * (bq * w + c) + 1];
            sr += dr * zr + di * zi;
            si += di * zr - dr * zi;
        }
        dRk[i * 2] += sr;
        dRk[i * 2 + 1] += si;
    }
}

__global__ void k_to_bf16(const float* __restrict__ in, __nv_bfloat16* __restrict__ out, long n)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        out[i] = __float2bfloat16_rn(in[i]);
}

// Adam with bias correction; refreshes the BF16 mirror and clears the gradient.
__global__ void k_adam(float* __restrict__ p, __nv_bfloat16* __restrict__ pb, float* __restrict__ g,
                       float* __restrict__ mo, float* __restrict__ ve, long n, float lr, float b1, float b2, float eps,
                       float c1, float c2)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * mo[i] + (1.0f - b1) * gi;
        const float vi = b2 * ve[i] + (1.0f - b2) * gi * gi;
        mo[i] = mi;
        ve[i] = vi;
        const float pi = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        p[i] = pi;
        pb[i] = __float2bfloat16_rn(pi);
        g[i] = 0.0f;
    }
}

// Surrogate input and target conventions.  Input channels: the layer
// phases at the instance's wavelength (rad) times kPhaseScale, then one
// plane holding the normalised wavelength.  Target: the diffraction
// correction D = U exp(-i phi) - 1 of the propagated field U relative to the
// geometric phase phi = sum of the layer phases, as (re, im) planes.
constexpr float kPhaseScale = 0.1f;
constexpr float kLamMid = 1.35e-6f, kLamHalf = 0.5e-6f;

__global__ void k_fno_prepare(const float* __restrict__ win, const float* __restrict__ lam, int L, long P,
                              float* __restrict__ in, float* __restrict__ phi)
{
    const int b = blockIdx.y;
    const float lc = (lam[b] - kLamMid) / kLamHalf;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < P; i += (long)gridDim.x * blockDim.x) {
        float s = 0.0f;
        for (int l = 0; l < L; l++) {
            const float v = win[((size_t)b * L + l) * P + i];
            in[((size_t)b * (L + 1) + l) * P + i] = v * kPhaseScale;
            s += v;
        }
        in[((size_t)b * (L + 1) + L) * P + i] = lc;
        phi[(size_t)b * P + i] = s;
    }
}

__global__ void k_fno_target(const float* __restrict__ amp, const float* __restrict__ pha,
                             const float* __restrict__ phi, long P, float* __restrict__ tgt)
{
    const int b = blockIdx.y;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < P; i += (long)gridDim.x * blockDim.x) {
        const size_t o = (size_t)b * P + i;
        float sn, cs;
        sincosf(pha[o] - phi[o], &sn, &cs);
        tgt[(size_t)b * 2 * P + i] = amp[o] * cs - 1.0f;
        tgt[(size_t)b * 2 * P + P + i] = amp[o] * sn;
    }
}

// U = exp(i phi) (1 + D): amplitude |1 + D|, phase phi + arg(1 + D)
__global__ void k_fno_assemble(const float* __restrict__ out, const float* __restrict__ phi, long P,
                               float* __restrict__ amp, float* __restrict__ pha)
{
    const int b = blockIdx.y;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < P; i += (long)gridDim.x * blockDim.x) {
        const float re = 1.0f + out[(size_t)b * 2 * P + i], im = out[(size_t)b * 2 * P + P + i];
        const size_t o = (size_t)b * P + i;
        amp[o] = sqrtf(re * re + im * im);
        pha[o] = phi[o] + atan2f(im, re);
    }
}

unsigned grid_for(long n) { return (unsigned)std::min<long>((n + 255) / 256, 152L * 16); }

// ---------------------------------------------------------------------------
// products
// ---------------------------------------------------------------------------
cudaError_t gemm(int M, int N, int K, const void* A, long lda, int ta, int abf, const void* B, long ldb, int tb,
                 int bbf, float* C, long ldc, float beta, int batch = 1, long sA = 0, long sB = 0, long sC = 0,
                 const float* bias = nullptr, int bias_rows = 0, cudaStream_t st = 0, float* C2 = nullptr)
{
    GemmArgs g{};
    g.C2 = C2;
    g.M = M; g.N = N; g.K = K;
    g.A = A; g.B = B; g.C = C;
    g.lda = lda; g.ldb = ldb; g.ldc = ldc;
    g.sA = sA; g.sB = sB; g.sC = sC;
    g.ta = ta; g.tb = tb; g.a_bf16 = abf; g.b_bf16 = bbf;
    g.alpha = 1.0f; g.bias = bias; g.bias_rows = bias_rows; g.splitk = 0; g.batch = batch;
    return gemm_launch(g, beta, st);
}

// Pointwise channel mixing per sample: C[b] (o x P) = W (o x c) X[b] (c x P)
// (+ row bias, + beta C); act, if given, receives gelu(C) in the same pass.
cudaError_t pointwise(const __nv_bfloat16* W, int o, int c, const float* X, float* C, int B, long P, float beta,
                      const float* bias, cudaStream_t st, float* act = nullptr)
{
    return gemm(o, (int)P, c, W, c, 0, 1, X, P, 0, 0, C, P, beta, B, 0, (long)c * P, (long)o * P, bias, 1, st, act);
}

// dW (o x c) += sum_b dC[b] (o x P) X[b]^T
cudaError_t pointwise_dw(int o, int c, const float* dC, const float* X, float* dW, int B, long P, cudaStream_t st)
{
    return gemm(o, c, (int)P, dC, P, 0, 0, X, P, 1, 0, dW, c, 1.0f, B, (long)o * P, (long)c * P, 0, nullptr, 0, st);
}

// dX[b] (c x P) = W^T (c x o) dC[b] (o x P), beta into dX
cudaError_t pointwise_dx(const __nv_bfloat16* W, int o, int c, const float* dC, float* dX, int B, long P, float beta,
                         cudaStream_t st)
{
    return gemm(c, (int)P, o, W, c, 1, 1, dC, P, 0, 0, dX, P, beta, B, 0, (long)o * P, (long)c * P, nullptr, 0, st);
}

atmwfs_status build_dft(atmwfs_fno* f)
{
    const int G = f->cfg.grid, m = f->cfg.modes;
    std::vector<float> Fx((size_t)G * 2 * m), FyA((size_t)2 * m * G), FyB((size_t)2 * m * G), Gyr((size_t)G * m),
        Gyi((size_t)G * m), Gyin((size_t)G * m), Gx((size_t)2 * m * G);
    auto ang = [&](long k, long x) { return 2.0 * kPi * (double)((k * x) % G + G) / (double)G; };
    for (int x = 0; x < G; x++)
        for (int kx = 0; kx < m; kx++) {
            Fx[(size_t)x * 2 * m + kx] = (float)cos(ang(kx, x));
            Fx[(size_t)x * 2 * m + m + kx] = (float)-sin(ang(kx, x));
        }
    for (int j = 0; j < m; j++) {
        const long ky = j < m / 2 ? j : j - m;
        for (int yy = 0; yy < G; yy++) {
            const double c = cos(ang(ky, yy)), s = -sin(ang(ky, yy));  // exp(-i 2 pi ky y / G)
            FyA[(size_t)j * G + yy] = (float)c;
            FyA[(size_t)(m + j) * G + yy] = (float)s;
            FyB[(size_t)j * G + yy] = (float)-s;
            FyB[(size_t)(m + j) * G + yy] = (float)c;
            Gyr[(size_t)yy * m + j] = (float)c;     // exp(+i ...) = c - i s
            Gyi[(size_t)yy * m + j] = (float)-s;
            Gyin[(size_t)yy * m + j] = (float)s;
        }
    }
    const double norm = 1.0 / ((double)G * G);
    for (int kx = 0; kx < m; kx++) {
        const double ck = kx == 0 ? 1.0 : 2.0;
        for (int x = 0; x < G; x++) {
            Gx[(size_t)kx * G + x] = (float)(ck * norm * cos(ang(kx, x)));
            Gx[(size_t)(m + kx) * G + x] = (float)(-ck * norm * sin(ang(kx, x)));
        }
    }
    // the y transforms as single products over the planar spectra:
    // FyAB = [FyA | FyB] (2m x 2G) maps [a_re; a_im] to z;
    // GyBig = [[Gyr | Gyin]; [Gyi | Gyr]] (2G x 2m) maps [y_re; y_im] to [bb_re; bb_im]
    std::vector<float> FyAB((size_t)2 * m * 2 * G), GyBig((size_t)2 * G * 2 * m);
    for (int r = 0; r < 2 * m; r++)
        for (int yy = 0; yy < G; yy++) {
            FyAB[(size_t)r * 2 * G + yy] = FyA[(size_t)r * G + yy];
            FyAB[(size_t)r * 2 * G + G + yy] = FyB[(size_t)r * G + yy];
        }
    for (int yy = 0; yy < G; yy++)
        for (int j = 0; j < m; j++) {
            GyBig[(size_t)yy * 2 * m + j] = Gyr[(size_t)yy * m + j];
            GyBig[(size_t)yy * 2 * m + m + j] = Gyin[(size_t)yy * m + j];
            GyBig[(size_t)(G + yy) * 2 * m + j] = Gyi[(size_t)yy * m + j];
            GyBig[(size_t)(G + yy) * 2 * m + m + j] = Gyr[(size_t)yy * m + j];
        }
    struct M { float** d; std::vector<float>* h; } mats[] = {{&f->Fx, &Fx}, {&f->FyAB, &FyAB}, {&f->GyBig, &GyBig},
                                                            {&f->Gx, &Gx}};
    for (auto& mm : mats) {
        FN_TRY(dalloc(f, (void**)mm.d, mm.h->size() * sizeof(float)));
        FN_CUDA(cudaMemcpy(*mm.d, mm.h->data(), mm.h->size() * sizeof(float), cudaMemcpyHostToDevice));
    }
    // transposes of the x transforms: FxT (2m x G) = Fx^T, GxT (G x 2m) = Gx^T
    std::vector<float> FxT((size_t)2 * m * G), GxT((size_t)G * 2 * m);
    for (int x = 0; x < G; x++)
        for (int n = 0; n < 2 * m; n++) {
            FxT[(size_t)n * G + x] = Fx[(size_t)x * 2 * m + n];
            GxT[(size_t)x * 2 * m + n] = Gx[(size_t)n * G + x];
        }
    struct MB { __nv_bfloat16** d; std::vector<float>* h; } bmats[] = {
        {&f->FyAB_bf, &FyAB}, {&f->GyBig_bf, &GyBig}, {&f->FxT_bf, &FxT}, {&f->GxT_bf, &GxT}};
    for (auto& mm : bmats) {
        std::vector<__nv_bfloat16> hb(mm.h->size());
        for (size_t i = 0; i < hb.size(); i++) hb[i] = __float2bfloat16_rn((*mm.h)[i]);
        FN_TRY(dalloc(f, (void**)mm.d, hb.size() * sizeof(__nv_bfloat16)));
        FN_CUDA(cudaMemcpy(*mm.d, hb.data(), hb.size() * sizeof(__nv_bfloat16), cudaMemcpyHostToDevice));
    }
    return ATMWFS_OK;
}

atmwfs_status ensure_batch(atmwfs_fno* f, int B)
{
    if (B <= f->cap) return ATMWFS_OK;
    // free the previous activation set
    auto drop = [&](float*& p) {
        if (!p) return;
        for (auto& a : f->allocs)
            if (a == p) a = nullptr;
        cudaFree(p);
        p = nullptr;
    };
    for (auto& p : f->h) drop(p);
    for (auto& p : f->u) drop(p);
    for (auto& p : f->a) drop(p);
    for (auto& p : f->z) drop(p);
    for (float** p : {&f->y, &f->bb, &f->qpre, &f->q, &f->dh, &f->dh2, &f->du, &f->dq, &f->dz, &f->dy,
                      &f->da, &f->dbb, &f->dout})
        drop(*p);
    const atmwfs_fno_cfg& c = f->cfg;
    const size_t P = (size_t)c.grid * c.grid;
    const size_t act = (size_t)B * c.width * P * 4, spa = (size_t)B * c.width * c.grid * 2 * c.modes * 4,
                 mod = (size_t)B * c.width * 2 * c.modes * c.modes * 4, prj = (size_t)B * c.proj * P * 4;
    f->h.assign(c.layers + 1, nullptr);
    f->u.assign(c.layers, nullptr);
    f->a.assign(c.layers, nullptr);
    f->z.assign(c.layers, nullptr);
    for (auto& p : f->h) FN_TRY(dalloc(f, (void**)&p, act));
    for (auto& p : f->u) FN_TRY(dalloc(f, (void**)&p, act));
    for (auto& p : f->a) FN_TRY(dalloc(f, (void**)&p, spa));
    for (auto& p : f->z) FN_TRY(dalloc(f, (void**)&p, mod));
    FN_TRY(dalloc(f, (void**)&f->y, mod));
    FN_TRY(dalloc(f, (void**)&f->bb, spa));
    FN_TRY(dalloc(f, (void**)&f->qpre, prj));
    FN_TRY(dalloc(f, (void**)&f->q, prj));
    FN_TRY(dalloc(f, (void**)&f->dh, act));
    FN_TRY(dalloc(f, (void**)&f->dh2, act));
    FN_TRY(dalloc(f, (void**)&f->du, act));
    FN_TRY(dalloc(f, (void**)&f->dq, prj));
    FN_TRY(dalloc(f, (void**)&f->dz, mod));
    FN_TRY(dalloc(f, (void**)&f->dy, mod));
    FN_TRY(dalloc(f, (void**)&f->da, spa));
    FN_TRY(dalloc(f, (void**)&f->dbb, spa));
    FN_TRY(dalloc(f, (void**)&f->dout, (size_t)B * c.nout * P * 4));
    f->cap = B;
    return ATMWFS_OK;
}

// Spectral images are planar and channel-interleaved so that the DFTs along
// y are single wide products over every (sample, channel): with Nc = B w m,
//   a, bb : [2][G][B w][m]   (real plane, imaginary plane; row y, channel, kx)
//   z, y  : [2m][B w][m]     (rows: real parts of the m kept ky, then imaginary)
// The x-DFT writes a through the product's row / column maps, and the x
// inverse reads bb through its column map.
static cudaError_t gemm_args(GemmArgs& g, float beta, cudaStream_t st)
{
    g.alpha = 1.0f;
    g.batch = 1;
    return gemm_launch(g, beta, st);
}

// spectral convolution of layer l: spec = S_l(h)
atmwfs_status spectral_fwd(atmwfs_fno* f, int l, const void* h, int h_bf16, float* spec, int B, cudaStream_t st)
{
    const atmwfs_fno_cfg& c = f->cfg;
    const int G = c.grid, m = c.modes, w = c.width;
    const long BW = (long)B * w, Nc = BW * m;
    float* a = f->a[l];
    float* z = f->z[l];
    const bool tcx = umma_enabled() && xspectral_umma_supported(2 * m, G) && xspectral_umma_supported(G, 2 * m);
    {   // a[p][y][bc][kx] = sum_x h[bc][y][x] Fx[x][p m + kx]
        if (tcx && !h_bf16 &&
            xspectral_umma(f->FxT_bf, 2 * m, G, (const float*)h, 0, G, 0, G, 0, a, G, Nc, m, m, (long)G * Nc, BW * G,
                           umma_status_ptr(), 0, st) == cudaSuccess) {
        } else {
            cudaGetLastError();
            GemmArgs g{};
            g.M = (int)(BW * G); g.N = 2 * m; g.K = G;
            g.A = h; g.a_bf16 = h_bf16; g.lda = G; g.B = f->Fx; g.ldb = 2 * m; g.C = a; g.ldc = 2 * m;
            g.rdiv = G; g.c_lo = Nc; g.c_hi = m; g.cdiv = m; g.cc_hi = (long)G * Nc;
            FN_CUDA(gemm_args(g, 0.0f, st));
        }
    }
    // z = FyAB a: [2m, 2G] x [2G, Nc], on tcgen05 where compiled
    const bool tc = umma_enabled() && Nc % 8 == 0;
    if (tc && spectral_umma_supported(2 * m, 2 * G))
        FN_CUDA(spectral_umma(f->FyAB_bf, 2 * m, 2 * G, a, z, Nc, umma_status_ptr(), 0, st));
    else
        FN_CUDA(gemm(2 * m, (int)Nc, 2 * G, f->FyAB, 2 * G, 0, 0, a, Nc, 0, 0, z, Nc, 0.0f, 1, 0, 0, 0, nullptr, 0, st));
    // y = R z per mode
    const size_t smf = sizeof(float) * (2 * B * w + 2 * w * (w + 1));
    if (smf > 227 * 1024) return err(ATMWFS_ERR_INVALID, "batch %d x width %d exceeds the mode-mixing shared memory", B, w);
    if (smf > 48 * 1024) FN_CUDA(cudaFuncSetAttribute(k_modemix, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smf));
    k_modemix<<<m * m, 256, smf, st>>>(f->pbf + f->L.R[l], z, f->y, B, w, m);
    FN_CUDA(cudaGetLastError());
    // bb = GyBig y: [2G, 2m] x [2m, Nc], on tcgen05 where compiled
    if (tc && spectral_umma_supported(2 * G, 2 * m))
        FN_CUDA(spectral_umma(f->GyBig_bf, 2 * G, 2 * m, f->y, f->bb, Nc, umma_status_ptr(), 0, st));
    else
        FN_CUDA(gemm(2 * G, (int)Nc, 2 * m, f->GyBig, 2 * m, 0, 0, f->y, Nc, 0, 0, f->bb, Nc, 0.0f, 1, 0, 0, 0, nullptr, 0,
                     st));
    {   // spec[bo][y][x] = sum_{p,kx} bb[p][y][bo][kx] Gx[p m + kx][x]: rows (bo, y), A read through its maps
        if (tcx && xspectral_umma(f->GxT_bf, G, 2 * m, f->bb, G, Nc, m, m, (long)G * Nc, spec, 0, G, 0, G, 0, BW * G,
                                  umma_status_ptr(), 0, st) == cudaSuccess) {
        } else {
            cudaGetLastError();
            GemmArgs g{};
            g.M = (int)(BW * G); g.N = G; g.K = 2 * m;
            g.A = f->bb; g.lda = m; g.ardiv = G; g.a_lo = Nc; g.a_hi = m; g.kdiv = m; g.ka_hi = (long)G * Nc;
            g.B = f->Gx; g.ldb = G; g.C = spec; g.ldc = G;
            FN_CUDA(gemm_args(g, 0.0f, st));
        }
    }
    return ATMWFS_OK;
}

// backward of the spectral convolution: dh += S_l^T(ds); dR_l += ...
atmwfs_status spectral_bwd(atmwfs_fno* f, int l, const float* ds, float* dh, int B, cudaStream_t st)
{
    const atmwfs_fno_cfg& c = f->cfg;
    const int G = c.grid, m = c.modes, w = c.width;
    const long BW = (long)B * w, Nc = BW * m;
    {   // dbb[p][y][bo][kx] = sum_x ds[bo][y][x] Gx[p m + kx][x]
        GemmArgs g{};
        g.M = (int)(BW * G); g.N = 2 * m; g.K = G;
        g.A = ds; g.lda = G; g.B = f->Gx; g.ldb = G; g.tb = 1; g.C = f->dbb; g.ldc = 2 * m;
        g.rdiv = G; g.c_lo = Nc; g.c_hi = m; g.cdiv = m; g.cc_hi = (long)G * Nc;
        FN_CUDA(gemm_args(g, 0.0f, st));
    }
    // dy = GyBig^T dbb: [2m, 2G] x [2G, Nc]
    FN_CUDA(gemm(2 * m, (int)Nc, 2 * G, f->GyBig, 2 * m, 1, 0, f->dbb, Nc, 0, 0, f->dy, Nc, 0.0f, 1, 0, 0, 0, nullptr, 0,
                 st));
    // dz, dR
    const size_t smb = sizeof(float) * (4 * B * w + 2 * w * (w + 1));
    if (smb > 227 * 1024) return err(ATMWFS_ERR_INVALID, "batch %d x width %d exceeds the mode-mixing shared memory", B, w);
    if (smb > 48 * 1024) FN_CUDA(cudaFuncSetAttribute(k_modemix_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smb));
    k_modemix_bwd<<<m * m, 256, smb, st>>>(f->pbf + f->L.R[l], f->z[l], f->dy, f->dz, f->grads + f->L.R[l], B, w, m);
    FN_CUDA(cudaGetLastError());
    // da = FyAB^T dz: [2G, 2m] x [2m, Nc]
    FN_CUDA(gemm(2 * G, (int)Nc, 2 * m, f->FyAB, 2 * G, 1, 0, f->dz, Nc, 0, 0, f->da, Nc, 0.0f, 1, 0, 0, 0, nullptr, 0,
                 st));
    {   // dh[bc][y][x] += sum_{p,kx} da[p][y][bc][kx] Fx[x][p m + kx]: rows (bc, y), A read through its maps
        GemmArgs g{};
        g.M = (int)(BW * G); g.N = G; g.K = 2 * m;
        g.A = f->da; g.lda = m; g.ardiv = G; g.a_lo = Nc; g.a_hi = m; g.kdiv = m; g.ka_hi = (long)G * Nc;
        g.B = f->Fx; g.ldb = 2 * m; g.tb = 1; g.C = dh; g.ldc = G;
        FN_CUDA(gemm_args(g, 1.0f, st));
    }
    return ATMWFS_OK;
}

// Input of the projection: the last Fourier layer's output, which has no
// activation, so it is that layer's u.
const float* last_h(const atmwfs_fno* f) { return f->u[f->cfg.layers - 1]; }

// The pointwise products of the forward pass run on the tcgen05 tensor cores
// for the shapes compiled there (the Fourier layers' width x width mixing and
// the first projection), unless ATMWFS_FNO_UMMA=0; on the mma.sync product
// otherwise.
bool umma_enabled()
{
    static const bool use = [] {
        const char* e = getenv("ATMWFS_FNO_UMMA");
        return !(e && e[0] == '0');
    }();
    return use;
}

// keep_c = false (inference with an activation output): the pre-activation C
// is not stored where only the backward pass would read it.  x_bf16 / a_bf16:
// the input and the activation output are stored as BF16 (tcgen05 path only).
cudaError_t pointwise_fwd(const __nv_bfloat16* W, int o, int c, const void* X, int x_bf16, float* C, int B, long P,
                          float beta, const float* bias, cudaStream_t st, void* act = nullptr, int a_bf16 = 0,
                          bool keep_c = true)
{
    if (umma_enabled() && pointwise_umma_supported(o, c) && P % 8 == 0) {
        unsigned* status = umma_status_ptr();
        if (!status) return cudaErrorUnknown;
        return pointwise_umma(W, o, c, X, x_bf16, C, B, P, beta, bias, act, a_bf16, status, 0, keep_c || !act, st);
    }
    if (x_bf16 || a_bf16) return cudaErrorNotSupported;
    return pointwise(W, o, c, (const float*)X, C, B, P, beta, bias, st, (float*)act);
}

// training = false (inference): pre-activations that only the backward pass
// reads are not stored.  With ATMWFS_FNO_BF16_ACT=1 (tcgen05 path) the
// activations between the Fourier layers (h[1..]) and of the projection (q)
// are also stored as BF16, which changes no value (every product that reads
// them rounds its operands to BF16) but measured slower (4,180 against
// 4,460 frames/s at 256^2: the spectral product reads its BF16 operand in
// 8-byte pieces), so FP32 storage is the default.
atmwfs_status forward(atmwfs_fno* f, const float* x, float* out, int B, cudaStream_t st, bool training)
{
    const atmwfs_fno_cfg& c = f->cfg;
    const long P = (long)c.grid * c.grid;
    FN_TRY(ensure_batch(f, B));
    const __nv_bfloat16* pb = f->pbf;
    const float* pf = f->params;
    const char* bf_var = getenv("ATMWFS_FNO_BF16_ACT");  // read per call: a test switches it
    const bool bf_env = bf_var && bf_var[0] == '1';
    const int bf = (!training && bf_env && umma_enabled() && P % 8 == 0 && pointwise_umma_supported(c.width, c.width) &&
                    pointwise_umma_supported(c.proj, c.width))
                       ? 1
                       : 0;
    FN_CUDA(pointwise_fwd(pb + f->L.lift_W, c.width, c.nin, x, 0, f->h[0], B, P, 0.0f, pf + f->L.lift_b, st));
    for (int l = 0; l < c.layers; l++) {
        // u = S_l(h) + W_l h + b_l; h' = gelu(u) from the same epilogue
        // (the last layer has no activation: its u is the projection's input)
        const int hb = l > 0 ? bf : 0;  // h[0] comes from the lift in FP32
        FN_TRY(spectral_fwd(f, l, f->h[l], hb, f->u[l], B, st));
        FN_CUDA(pointwise_fwd(pb + f->L.W[l], c.width, c.width, f->h[l], hb, f->u[l], B, P, 1.0f, pf + f->L.b[l], st,
                              l + 1 < c.layers ? f->h[l + 1] : nullptr, bf, training));
    }
    FN_CUDA(pointwise_fwd(pb + f->L.proj1_W, c.proj, c.width, last_h(f), 0, f->qpre, B, P, 0.0f, pf + f->L.proj1_b, st,
                          f->q, bf, training));
    FN_CUDA(gemm(c.nout, (int)P, c.proj, pb + f->L.proj2_W, c.proj, 0, 1, f->q, P, 0, bf, out, P, 0.0f, B, 0,
                 (long)c.proj * P, (long)c.nout * P, pf + f->L.proj2_b, 1, st));
    return ATMWFS_OK;
}

atmwfs_status backward(atmwfs_fno* f, const float* x, const float* dout, int B, cudaStream_t st)
{
    const atmwfs_fno_cfg& c = f->cfg;
    const long P = (long)c.grid * c.grid;
    const long nact = (long)B * c.width * P, nq = (long)B * c.proj * P;
    const __nv_bfloat16* pb = f->pbf;
    float* g = f->grads;
    const dim3 rs((unsigned)std::min<long>((P + 255) / 256, 64), 1);
    // projection
    FN_CUDA(pointwise_dw(c.nout, c.proj, dout, f->q, g + f->L.proj2_W, B, P, st));
    k_rowsum<<<dim3(rs.x, c.nout), 256, 0, st>>>(dout, g + f->L.proj2_b, B, c.nout, P);
    FN_CUDA(pointwise_dx(pb + f->L.proj2_W, c.nout, c.proj, dout, f->dq, B, P, 0.0f, st));
    k_gelu_bwd<<<grid_for(nq), 256, 0, st>>>(f->dq, f->qpre, f->dq, nq);
    FN_CUDA(pointwise_dw(c.proj, c.width, f->dq, last_h(f), g + f->L.proj1_W, B, P, st));
    k_rowsum<<<dim3(rs.x, c.proj), 256, 0, st>>>(f->dq, g + f->L.proj1_b, B, c.proj, P);
    FN_CUDA(pointwise_dx(pb + f->L.proj1_W, c.proj, c.width, f->dq, f->dh, B, P, 0.0f, st));
    // Fourier layers, last to first: dh holds dL/dh[l+1]
    for (int l = c.layers - 1; l >= 0; l--) {
        if (l + 1 < c.layers) k_gelu_bwd<<<grid_for(nact), 256, 0, st>>>(f->dh, f->u[l], f->du, nact);
        else FN_CUDA(cudaMemcpyAsync(f->du, f->dh, sizeof(float) * nact, cudaMemcpyDeviceToDevice, st));
        FN_CUDA(pointwise_dw(c.width, c.width, f->du, f->h[l], g + f->L.W[l], B, P, st));
        k_rowsum<<<dim3(rs.x, c.width), 256, 0, st>>>(f->du, g + f->L.b[l], B, c.width, P);
        FN_CUDA(pointwise_dx(pb + f->L.W[l], c.width, c.width, f->du, f->dh2, B, P, 0.0f, st));
        FN_TRY(spectral_bwd(f, l, f->du, f->dh2, B, st));
        std::swap(f->dh, f->dh2);
    }
    // lift
    FN_CUDA(pointwise_dw(c.width, c.nin, f->dh, x, g + f->L.lift_W, B, P, st));
    k_rowsum<<<dim3(rs.x, c.width), 256, 0, st>>>(f->dh, g + f->L.lift_b, B, c.width, P);
    FN_CUDA(cudaGetLastError());
    return ATMWFS_OK;
}

// Philox-free deterministic initialisation: uniform(-s, s) from a 64-bit LCG per tensor
void init_uniform(std::vector<float>& p, long off, long n, double s, uint64_t& st)
{
    for (long i = 0; i < n; i++) {
        st = st * 6364136223846793005ull + 1442695040888963407ull;
        const double u = (double)(st >> 11) * (1.0 / 9007199254740992.0);
        p[off + i] = (float)((2.0 * u - 1.0) * s);
    }
}

}  // namespace

extern "C" {

atmwfs_status atmwfs_fno_create(const atmwfs_fno_cfg* cfg, uint64_t seed, atmwfs_fno** out)
{
    if (!cfg || !out) return err(ATMWFS_ERR_INVALID, "null argument");
    *out = nullptr;
    const atmwfs_fno_cfg& c = *cfg;
    // an even width keeps every parameter tensor's offset even (paired BF16 loads)
    if (c.nin < 1 || c.width < 2 || (c.width & 1) || c.modes < 2 || (c.modes & 1) || c.layers < 1 || c.proj < 1 ||
        c.nout < 1 || c.grid < 8 || c.modes > c.grid / 2)
        return err(ATMWFS_ERR_INVALID, "bad FNO configuration");
    atmwfs_fno* f = new atmwfs_fno;
    f->cfg = c;
    f->L = FnoLayout{c.nin, c.width, c.modes, c.layers, c.proj, c.nout, c.grid, 0, 0, 0, 0, 0, 0, 0, {}, {}, {}};
    f->L.build();
    const long n = f->L.total;
    atmwfs_status s = ATMWFS_OK;
    auto fail = [&](atmwfs_status e) {
        atmwfs_fno_destroy(f);
        return e;
    };
    if ((s = dalloc(f, (void**)&f->params, sizeof(float) * n)) != ATMWFS_OK) return fail(s);
    if ((s = dalloc(f, (void**)&f->pbf, sizeof(__nv_bfloat16) * n)) != ATMWFS_OK) return fail(s);
    if ((s = dalloc(f, (void**)&f->grads, sizeof(float) * n)) != ATMWFS_OK) return fail(s);
    if ((s = dalloc(f, (void**)&f->adam_m, sizeof(float) * n)) != ATMWFS_OK) return fail(s);
    if ((s = dalloc(f, (void**)&f->adam_v, sizeof(float) * n)) != ATMWFS_OK) return fail(s);
    if ((s = dalloc(f, (void**)&f->d_loss, sizeof(double))) != ATMWFS_OK) return fail(s);
    if ((s = build_dft(f)) != ATMWFS_OK) return fail(s);
    // initialisation: pointwise weights U(+-1/sqrt(fan_in)), spectral weights U(+-1/w) scaled down
    std::vector<float> h(n, 0.0f);
    uint64_t st = seed * 0x9E3779B97F4A7C15ull + 1;
    init_uniform(h, f->L.lift_W, (long)c.width * c.nin, 1.0 / sqrt((double)c.nin), st);
    for (int l = 0; l < c.layers; l++) {
        init_uniform(h, f->L.R[l], (long)c.modes * c.modes * c.width * c.width * 2, 1.0 / ((double)c.width * c.width), st);
        init_uniform(h, f->L.W[l], (long)c.width * c.width, 1.0 / sqrt((double)c.width), st);
    }
    init_uniform(h, f->L.proj1_W, (long)c.proj * c.width, 1.0 / sqrt((double)c.width), st);
    init_uniform(h, f->L.proj2_W, (long)c.nout * c.proj, 1.0 / sqrt((double)c.proj), st);
    if ((s = atmwfs_fno_set_params(f, h.data())) != ATMWFS_OK) return fail(s);
    if (cudaMemset(f->grads, 0, sizeof(float) * n) != cudaSuccess || cudaMemset(f->adam_m, 0, sizeof(float) * n) != cudaSuccess ||
        cudaMemset(f->adam_v, 0, sizeof(float) * n) != cudaSuccess)
        return fail(err(ATMWFS_ERR_CUDA, "memset failed"));
    *out = f;
    return ATMWFS_OK;
}

void atmwfs_fno_destroy(atmwfs_fno* f)
{
    if (!f) return;
    for (void* p : f->allocs)
        if (p) cudaFree(p);
    delete f;
}

long atmwfs_fno_num_params(const atmwfs_fno* f) { return f ? f->L.total : 0; }

atmwfs_status atmwfs_fno_set_params(atmwfs_fno* f, const float* host)
{
    if (!f || !host) return err(ATMWFS_ERR_INVALID, "null argument");
    const long n = f->L.total;
    FN_CUDA(cudaMemcpy(f->params, host, sizeof(float) * n, cudaMemcpyHostToDevice));
    k_to_bf16<<<grid_for(n), 256>>>(f->params, f->pbf, n);
    FN_CUDA(cudaGetLastError());
    FN_CUDA(cudaDeviceSynchronize());
    return ATMWFS_OK;
}

atmwfs_status atmwfs_fno_get_params(const atmwfs_fno* f, float* host)
{
    if (!f || !host) return err(ATMWFS_ERR_INVALID, "null argument");
    FN_CUDA(cudaMemcpy(host, f->params, sizeof(float) * f->L.total, cudaMemcpyDeviceToHost));
    return ATMWFS_OK;
}

atmwfs_status atmwfs_fno_get_grads(const atmwfs_fno* f, float* host)
{
    if (!f || !host) return err(ATMWFS_ERR_INVALID, "null argument");
    FN_CUDA(cudaMemcpy(host, f->grads, sizeof(float) * f->L.total, cudaMemcpyDeviceToHost));
    return ATMWFS_OK;
}

atmwfs_status atmwfs_fno_zero_grads(atmwfs_fno* f, void* stream)
{
    if (!f) return err(ATMWFS_ERR_INVALID, "null model");
    FN_CUDA(cudaMemsetAsync(f->grads, 0, sizeof(float) * f->L.total, (cudaStream_t)stream));
    return ATMWFS_OK;
}

atmwfs_status atmwfs_fno_forward(atmwfs_fno* f, const float* in, float* out, int batch, void* stream)
{
    if (!f || !in || !out || batch < 1) return err(ATMWFS_ERR_INVALID, "bad arguments");
    return forward(f, in, out, batch, (cudaStream_t)stream, false);
}

atmwfs_status atmwfs_fno_loss_grad(atmwfs_fno* f, const float* in, const float* target, float* out, int batch,
                                   double* loss, void* stream)
{
    if (!f || !in || !target || !out || batch < 1) return err(ATMWFS_ERR_INVALID, "bad arguments");
    cudaStream_t st = (cudaStream_t)stream;
    FN_TRY(forward(f, in, out, batch, st, true));
    const long n = (long)batch * f->cfg.nout * f->cfg.grid * f->cfg.grid;
    FN_CUDA(cudaMemsetAsync(f->d_loss, 0, sizeof(double), st));
    k_mse<<<grid_for(n), 256, 0, st>>>(out, target, f->dout, n, f->d_loss);
    FN_CUDA(cudaGetLastError());
    FN_TRY(backward(f, in, f->dout, batch, st));
    if (loss) {
        FN_CUDA(cudaMemcpyAsync(loss, f->d_loss, sizeof(double), cudaMemcpyDeviceToHost, st));
        FN_CUDA(cudaStreamSynchronize(st));
    }
    return ATMWFS_OK;
}

atmwfs_status atmwfs_fno_adam(atmwfs_fno* f, float lr, float b1, float b2, float eps, void* stream)
{
    if (!f) return err(ATMWFS_ERR_INVALID, "null model");
    f->step++;
    const float c1 = 1.0f - powf(b1, (float)f->step), c2 = 1.0f - powf(b2, (float)f->step);
    const long n = f->L.total;
    k_adam<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(f->params, f->pbf, f->grads, f->adam_m, f->adam_v, n, lr, b1,
                                                          b2, eps, c1, c2);
    FN_CUDA(cudaGetLastError());
    return ATMWFS_OK;
}

atmwfs_status atmwfs_fno_prepare(const float* win, const float* lam, int batch, int nlayers, int grid, float* in,
                                 float* phi, void* stream)
{
    if (!win || !lam || !in || !phi || batch < 1 || nlayers < 1 || grid < 1) return err(ATMWFS_ERR_INVALID, "bad arguments");
    const long P = (long)grid * grid;
    k_fno_prepare<<<dim3((unsigned)std::min<long>((P + 255) / 256, 256), batch), 256, 0, (cudaStream_t)stream>>>(
        win, lam, nlayers, P, in, phi);
    FN_CUDA(cudaGetLastError());
    return ATMWFS_OK;
}

atmwfs_status atmwfs_fno_target(const float* amp, const float* pha, const float* phi, int batch, int grid, float* tgt,
                                void* stream)
{
    if (!amp || !pha || !phi || !tgt || batch < 1 || grid < 1) return err(ATMWFS_ERR_INVALID, "bad arguments");
    const long P = (long)grid * grid;
    k_fno_target<<<dim3((unsigned)std::min<long>((P + 255) / 256, 256), batch), 256, 0, (cudaStream_t)stream>>>(
        amp, pha, phi, P, tgt);
    FN_CUDA(cudaGetLastError());
    return ATMWFS_OK;
}

atmwfs_status atmwfs_fno_assemble(const float* out, const float* phi, int batch, int grid, float* amp, float* pha,
                                  void* stream)
{
    if (!out || !phi || !amp || !pha || batch < 1 || grid < 1) return err(ATMWFS_ERR_INVALID, "bad arguments");
    const long P = (long)grid * grid;
    k_fno_assemble<<<dim3((unsigned)std::min<long>((P + 255) / 256, 256), batch), 256, 0, (cudaStream_t)stream>>>(
        out, phi, P, amp, pha);
    FN_CUDA(cudaGetLastError());
    return ATMWFS_OK;
}

atmwfs_status atmwfs_fno_get_cfg(const atmwfs_fno* f, atmwfs_fno_cfg* cfg)
{
    if (!f || !cfg) return err(ATMWFS_ERR_INVALID, "null argument");
    *cfg = f->cfg;
    return ATMWFS_OK;
}

// File: "ATMFNO01", the configuration as seven int32, the parameter count
// as int64, then the FP32 parameters (little-endian hosts).
atmwfs_status atmwfs_fno_save(const atmwfs_fno* f, const char* path)
{
    if (!f || !path) return err(ATMWFS_ERR_INVALID, "null argument");
    std::vector<float> h(f->L.total);
    FN_TRY(atmwfs_fno_get_params(f, h.data()));
    FILE* fp = fopen(path, "wb");
    if (!fp) return err(ATMWFS_ERR_IO, "cannot create \"%s\"", path);
    const int32_t c[7] = {f->cfg.nin, f->cfg.width, f->cfg.modes, f->cfg.layers, f->cfg.proj, f->cfg.nout, f->cfg.grid};
    const int64_t n = f->L.total;
    bool ok = fwrite("ATMFNO01", 1, 8, fp) == 8 && fwrite(c, sizeof c, 1, fp) == 1 && fwrite(&n, sizeof n, 1, fp) == 1 &&
              fwrite(h.data(), sizeof(float), h.size(), fp) == h.size();
    ok = (fclose(fp) == 0) && ok;
    return ok ? ATMWFS_OK : err(ATMWFS_ERR_IO, "write to \"%s\" failed", path);
}

atmwfs_status atmwfs_fno_load(const char* path, atmwfs_fno** out)
{
    if (!path || !out) return err(ATMWFS_ERR_INVALID, "null argument");
    *out = nullptr;
    FILE* fp = fopen(path, "rb");
    if (!fp) return err(ATMWFS_ERR_IO, "cannot open \"%s\"", path);
    char magic[8];
    int32_t c[7];
    int64_t n = 0;
    if (fread(magic, 1, 8, fp) != 8 || memcmp(magic, "ATMFNO01", 8) != 0 || fread(c, sizeof c, 1, fp) != 1 ||
        fread(&n, sizeof n, 1, fp) != 1) {
        fclose(fp);
        return err(ATMWFS_ERR_IO, "\"%s\" is not a surrogate model file", path);
    }
    atmwfs_fno_cfg cfg{c[0], c[1], c[2], c[3], c[4], c[5], c[6]};
    atmwfs_fno* f = nullptr;
    atmwfs_status s = atmwfs_fno_create(&cfg, 0, &f);
    if (s != ATMWFS_OK) {
        fclose(fp);
        return s;
    }
    if (n != f->L.total) {
        fclose(fp);
        atmwfs_fno_destroy(f);
        return err(ATMWFS_ERR_IO, "\"%s\": %lld parameters, the configuration has %ld", path, (long long)n, f->L.total);
    }
    std::vector<float> h(n);
    const bool ok = fread(h.data(), sizeof(float), n, fp) == (size_t)n;
    fclose(fp);
    if (!ok) {
        atmwfs_fno_destroy(f);
        return err(ATMWFS_ERR_IO, "\"%s\": truncated", path);
    }
    s = atmwfs_fno_set_params(f, h.data());
    if (s != ATMWFS_OK) {
        atmwfs_fno_destroy(f);
        return s;
    }
    *out = f;
    return ATMWFS_OK;
}

}  // extern "C"
