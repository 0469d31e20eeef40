// aux_kernels.cuh -- host launchers of the setup / per-step helper kernels.
#pragma once
#include "engine.cuh"

namespace atmwfs {

cudaError_t pad_screen(const float* S, int M, float* P, int Wp, int Hp, int orient, cudaStream_t st);
cudaError_t lag_sumsq(const float* S, int M, int dpix, double* acc, cudaStream_t st);
cudaError_t scale_screen(float* S, long n, double f, cudaStream_t st);
// atan_tab: atan(k / 1024), k = 0 .. 1024, as (hi, lo) pairs (atan_table_host)
cudaError_t unwrap_bins(const InstDev* insts, const int* list, int nsci, int maxnb, unsigned* status, int* iters,
                        const float2* atan_tab, cudaStream_t st);
cudaError_t sci_apply(const InstDev* insts, const int* list, int nsci, int maxnout, const int* d_step, cudaStream_t st);
cudaError_t step_advance(int* d_step, cudaStream_t st);
// Compensated layer sums of the window groups with a layer-independent
// Scoeff (one job per group, maxside the largest side).
cudaError_t group_sums(const GroupSumJob* jobs, int njobs, int L, int maxside, cudaStream_t st);
// Frame copy-out by a small grid of copy CTAs (16-byte aligned pointers,
// counts in float4): dst0 = src0, dst1 = src1 (either pair may be absent).
cudaError_t copy_out(const float4* src0, float4* dst0, long n0, const float4* src1, float4* dst1, long n1,
                     cudaStream_t st);
cudaError_t screen_spectrum(uint64_t seed, uint32_t stream, int M, double fo, double fi, float2* C, cudaStream_t st);
cudaError_t strf_lags(const float2* F, int M, double* acc, cudaStream_t st);
cudaError_t split_scale(const float2* F, long n, double s1, double s2, float* o1, float* o2, cudaStream_t st);

// Unnormalised 2-D DFT of an M x M grid for M = 4096 or 8192 (fft_large.cu);
// tmp holds M x M complex values; in may equal out.
bool fft2d_large_supported(long M);

// Concatenated stage twiddle tables of the in-CTA transform of size N
// (64..2048), device memory owned by the library.
const float2* stage_twiddles(int N);

// PSF consumers (psf.cu): row and column passes of zero-padded fields and
// the chromatic zoom sum.
cudaError_t psf_rows(int N, const float* amp, long amp_fstride, const float* pha, long pha_fstride, const float* cscale,
                     int W, int off, int B, float2* G, const float2* tw, cudaStream_t st);
cudaError_t psf_cols(int N, const float2* G, int B, int W, int off, int mode, float* out, const float2* tw,
                     cudaStream_t st);
cudaError_t chromat_sum(const float* I, int S, int n, const float* coeff, const float* mcoeff, float* out,
                        cudaStream_t st);
cudaError_t fft2d_large(const float2* in, float2* out, float2* tmp, int M, int sign, cudaStream_t st);

cudaError_t launch_pass_64(int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const float2* tw, cudaStream_t st);
cudaError_t launch_pass_128(int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const float2* tw, cudaStream_t st);
cudaError_t launch_pass_256(int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const float2* tw, cudaStream_t st);
cudaError_t launch_pass_512(int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const float2* tw, cudaStream_t st);
cudaError_t launch_pass_1024(int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const float2* tw, cudaStream_t st);
cudaError_t launch_pass_2048(int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const float2* tw, cudaStream_t st);

cudaError_t launch_pass_cfg_64(int cfg, int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const float2* tw,
                                cudaStream_t st);
cudaError_t launch_pass_cfg_128(int cfg, int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const float2* tw,
                                cudaStream_t st);
cudaError_t launch_pass_cfg_256(int cfg, int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const float2* tw,
                                cudaStream_t st);
cudaError_t launch_pass_cfg_512(int cfg, int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const float2* tw,
                                cudaStream_t st);
cudaError_t launch_pass_cfg_1024(int cfg, int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const float2* tw,
                                cudaStream_t st);
cudaError_t launch_pass_cfg_2048(int cfg, int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const float2* tw,
                                cudaStream_t st);

cudaError_t launch_pass_half_64(int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const void* tw, cudaStream_t st);
cudaError_t launch_pass_half_128(int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const void* tw, cudaStream_t st);
cudaError_t launch_pass_half_256(int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const void* tw, cudaStream_t st);
cudaError_t launch_pass_half_512(int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const void* tw, cudaStream_t st);
cudaError_t launch_pass_half_1024(int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const void* tw, cudaStream_t st);
cudaError_t launch_pass_half_2048(int var, dim3 grid, const PassArgs& a, const TmaSet* maps, const void* tw, cudaStream_t st);

// Per-layer phase windows (W x W, screen orientation) of global instance
// gidx at the last completed step, scaled by the instance's Scoeff.
cudaError_t windows(const float* const* screens, const float* scoeff, int L, int M, const LayerPos* pos, int poscap,
                    int ninst, int gidx, const int* d_step, int W, float* out, cudaStream_t st);

}  // namespace atmwfs
