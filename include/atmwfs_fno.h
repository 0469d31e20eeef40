/*
 * atmwfs_fno.h -- learned surrogate of the multi-layer Fresnel propagation:
 * a Fourier neural operator trained on pairs the plain path generates, with
 * the project's own BF16 tensor-core forward and backward kernels (FP32
 * accumulation, FP32 master weights, Adam).  The reference has no learned
 * path: this stands in for the per-frame propagation of the series in
 * real-time mode, with the plain Fresnel path as its fallback and judge.
 *
 * Data (device pointers, channel-major [batch][channel][grid][grid]):
 *   input   nin = nlayers + 1 planes: each layer's phase at the instance's
 *           wavelength (rad) x 0.1, then the wavelength as (lambda - 1.35 um) / 0.5 um;
 *   output  nout = 2 planes: the diffraction correction D = U exp(-i phi) - 1
 *           of the propagated field U relative to the geometric phase phi
 *           (the sum of the layer phases), real and imaginary parts.
 * atmwfs_fno_prepare / _target / _assemble convert between these and the
 * engine's per-layer windows (atmwfs_windows_dev) and amplitude / phase.
 */
#ifndef ATMWFS_FNO_H
#define ATMWFS_FNO_H

#include "atmwfs.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct atmwfs_fno_cfg {
    int nin;     /* input planes (layers + 1)                        */
    int width;   /* hidden channels                                  */
    int modes;   /* retained modes per axis: ky in [-modes/2, modes/2), kx in [0, modes) */
    int layers;  /* spectral layers                                  */
    int proj;    /* hidden channels of the projection                */
    int nout;    /* output planes (2)                                */
    int grid;    /* grid side                                        */
} atmwfs_fno_cfg;

typedef struct atmwfs_fno atmwfs_fno;

atmwfs_status atmwfs_fno_create(const atmwfs_fno_cfg* cfg, uint64_t seed, atmwfs_fno** out);
void atmwfs_fno_destroy(atmwfs_fno* f);
atmwfs_status atmwfs_fno_get_cfg(const atmwfs_fno* f, atmwfs_fno_cfg* cfg);

/* Flat FP32 parameter vector (host copies) and its gradient. */
long atmwfs_fno_num_params(const atmwfs_fno* f);
atmwfs_status atmwfs_fno_get_params(const atmwfs_fno* f, float* host);
atmwfs_status atmwfs_fno_set_params(atmwfs_fno* f, const float* host);
atmwfs_status atmwfs_fno_get_grads(const atmwfs_fno* f, float* host);
atmwfs_status atmwfs_fno_zero_grads(atmwfs_fno* f, void* stream);

/* Inference: out = f(in). */
atmwfs_status atmwfs_fno_forward(atmwfs_fno* f, const float* in, float* out, int batch, void* stream);

/* Training: forward, mean squared error against `target` (*loss, if not
 * NULL, after a stream synchronisation), backward; gradients accumulate
 * until atmwfs_fno_adam() applies and clears them. */
atmwfs_status atmwfs_fno_loss_grad(atmwfs_fno* f, const float* in, const float* target, float* out, int batch,
                                   double* loss, void* stream);
atmwfs_status atmwfs_fno_adam(atmwfs_fno* f, float lr, float beta1, float beta2, float eps, void* stream);

/* Conversions (device pointers): windows [batch][nlayers][grid^2] and
 * lambda [batch] -> input [batch][nlayers + 1][grid^2] and geometric phase
 * phi [batch][grid^2]; propagated amplitude / phase -> target D; model
 * output D -> amplitude |1 + D| and phase phi + arg(1 + D). */
atmwfs_status atmwfs_fno_prepare(const float* win, const float* lambda, int batch, int nlayers, int grid, float* in,
                                 float* phi, void* stream);
atmwfs_status atmwfs_fno_target(const float* amp, const float* pha, const float* phi, int batch, int grid, float* target,
                                void* stream);
atmwfs_status atmwfs_fno_assemble(const float* out, const float* phi, int batch, int grid, float* amp, float* pha,
                                  void* stream);

/* Model file: configuration and FP32 parameters. */
atmwfs_status atmwfs_fno_save(const atmwfs_fno* f, const char* path);
atmwfs_status atmwfs_fno_load(const char* path, atmwfs_fno** out);

/* The BF16 tensor-core product the surrogate runs on (device pointers):
 * C = alpha op(A) op(B) + beta C, op(A) M x K (ta: A stored K x M), op(B)
 * K x N (tb: B stored N x K), operands FP32 or BF16 (a_bf16 / b_bf16), FP32
 * accumulation and output; batch with element strides sA, sB, sC (sC = 0
 * sums the batch into one C). */
atmwfs_status atmwfs_gemm_bf16(int M, int N, int K, const void* A, long lda, int ta, int a_bf16, const void* B, long ldb,
                               int tb, int b_bf16, float* C, long ldc, float alpha, float beta, const float* bias,
                               int batch, long sA, long sB, long sC, void* stream);

/* The pointwise channel mixing of the network (device pointers; no
 * counterpart in the reference, whose path has no network):
 * C[b] (o x P) = W (o x c, BF16) X[b] (c x P, FP32) + bias[o] + beta C[b],
 * act[b] = gelu(C[b]) if act is not NULL, on the tcgen05 tensor cores
 * (accumulator in tensor memory), compiled for o x c = 64 x 64 and 128 x 64, and
 * 64 x 8 without act (the lift: K padded to 16 with zero channels).
 * engine 1: the product the network uses; 2: the same with the two
 * core-matrix strides of its shared-memory descriptors exchanged (a check
 * that only engine 1 matches the FP32 product). */
atmwfs_status atmwfs_fno_pointwise_dev(const void* W, int o, int c, const float* X, float* C, int batch, long P,
                                       float beta, const float* bias, float* act, int engine, void* stream);
/* The Fourier layers' spectral product along y on the tcgen05 tensor cores
 * (no counterpart in the reference): C (o x P) = W (o x c, BF16) X (c x P,
 * FP32, rounded to BF16), K taken in chunks of 64 accumulated in tensor
 * memory; compiled for o x c = 64 x 512 (the forward DFT of a 256 grid with
 * 32 modes) and 512 x 64 (its inverse); P a multiple of 8.  engine as for
 * atmwfs_fno_pointwise_dev. */
atmwfs_status atmwfs_fno_spectral_dev(const void* W, int o, int c, const float* X, float* C, long P, int engine,
                                      void* stream);
/* The Fourier layers' spectral products along x on the tcgen05 tensor cores
 * (no counterpart in the reference): C = A Bt^T with A (M x k, FP32, rounded
 * to BF16) and Bt (n x k, BF16, the transposed DFT matrix), K taken in
 * chunks of 64.  Row m of A starts at (m % a_div) a_lo + (m / a_div) a_hi
 * (a_div = 0: m a_lo) and its column j at (j / a_kdiv) a_khi + j % a_kdiv;
 * row m of C at (m % c_div) c_lo + (m / c_div) c_hi, column j at
 * (j / c_ndiv) c_nhi + j % c_ndiv (the planar spectrum layouts of the
 * network).  Compiled for n x k = 64 x 256 (forward DFT of a 256 grid with 32
 * modes) and 256 x 64 (its inverse); a_kdiv and the strides multiples of 4,
 * c_ndiv of 16.  engine as for atmwfs_fno_pointwise_dev. */
atmwfs_status atmwfs_fno_xspectral_dev(const void* Bt, int n, int k, const float* A, long a_div, long a_lo, long a_hi,
                                       int a_kdiv, long a_khi, float* C, long c_div, long c_lo, long c_hi, int c_ndiv,
                                       long c_nhi, long M, int engine, void* stream);
/* Status bits of the tcgen05 products since the last clear (1: a bounded
 * wait for the tensor cores ran out); clear != 0 resets them. */
unsigned atmwfs_fno_umma_status(int clear);

#ifdef __cplusplus
}
#endif

#endif /* ATMWFS_FNO_H */
