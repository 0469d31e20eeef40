/* fftw3.h -- declarations of the FFTW3 API subset the reference calls
 * (src/fft/fft.c).  Implemented by oracle/ref/shim_fftw.c with the project's
 * own double-precision FFT; used only to build the reference as a checker. */
#ifndef ATMREF_FFTW3_SHIM_H
#define ATMREF_FFTW3_SHIM_H
#include <stddef.h>
#include <stdio.h>
typedef double fftw_complex[2];
typedef float fftwf_complex[2];
typedef struct atmref_plan* fftw_plan;
typedef struct atmref_plan* fftwf_plan;
#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_DESTROY_INPUT (1U << 0)
#define FFTW_UNALIGNED (1U << 1)
#define FFTW_EXHAUSTIVE (1U << 3)
#define FFTW_PRESERVE_INPUT (1U << 4)
#define FFTW_PATIENT (1U << 5)
#define FFTW_ESTIMATE (1U << 6)
void* fftw_malloc(size_t n);
void fftw_free(void* p);
void* fftwf_malloc(size_t n);
void fftwf_free(void* p);
fftw_plan fftw_plan_dft_1d(int n, fftw_complex* in, fftw_complex* out, int sign, unsigned flags);
fftw_plan fftw_plan_dft_2d(int n0, int n1, fftw_complex* in, fftw_complex* out, int sign, unsigned flags);
fftw_plan fftw_plan_dft_r2c_1d(int n, double* in, fftw_complex* out, unsigned flags);
fftw_plan fftw_plan_dft_r2c_2d(int n0, int n1, double* in, fftw_complex* out, unsigned flags);
fftw_plan fftw_plan_many_dft(int rank, const int* n, int howmany, fftw_complex* in, const int* inembed, int istride,
                             int idist, fftw_complex* out, const int* onembed, int ostride, int odist, int sign,
                             unsigned flags);
fftw_plan fftw_plan_many_dft_r2c(int rank, const int* n, int howmany, double* in, const int* inembed, int istride,
                                 int idist, fftw_complex* out, const int* onembed, int ostride, int odist,
                                 unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);
fftwf_plan fftwf_plan_dft_1d(int n, fftwf_complex* in, fftwf_complex* out, int sign, unsigned flags);
fftwf_plan fftwf_plan_dft_2d(int n0, int n1, fftwf_complex* in, fftwf_complex* out, int sign, unsigned flags);
fftwf_plan fftwf_plan_dft_r2c_1d(int n, float* in, fftwf_complex* out, unsigned flags);
fftwf_plan fftwf_plan_dft_r2c_2d(int n0, int n1, float* in, fftwf_complex* out, unsigned flags);
fftwf_plan fftwf_plan_many_dft(int rank, const int* n, int howmany, fftwf_complex* in, const int* inembed, int istride,
                               int idist, fftwf_complex* out, const int* onembed, int ostride, int odist, int sign,
                               unsigned flags);
fftwf_plan fftwf_plan_many_dft_r2c(int rank, const int* n, int howmany, float* in, const int* inembed, int istride,
                                   int idist, fftwf_complex* out, const int* onembed, int ostride, int odist,
                                   unsigned flags);
void fftwf_execute(const fftwf_plan p);
void fftwf_destroy_plan(fftwf_plan p);
int fftw_import_wisdom_from_file(FILE* f);
void fftw_export_wisdom_to_file(FILE* f);
int fftwf_import_wisdom_from_file(FILE* f);
void fftwf_export_wisdom_to_file(FILE* f);
int fftw_init_threads(void);
void fftw_plan_with_nthreads(int n);
void fftw_cleanup_threads(void);
void fftw_cleanup(void);
void fftw_set_timelimit(double t);
int fftwf_init_threads(void);
void fftwf_plan_with_nthreads(int n);
void fftwf_cleanup_threads(void);
void fftwf_cleanup(void);
void fftwf_set_timelimit(double t);
#endif
