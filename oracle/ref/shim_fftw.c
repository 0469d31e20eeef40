/*
 * shim_fftw.c -- the FFTW3 API subset used by the reference's src/fft/fft.c,
 * implemented with a plain double-precision FFT (radix-2 for powers of two,
 * direct DFT otherwise).  Part of the checker build of the reference
 * (oracle/ref): it stands in for the FFTW library, which is not installed.
 * Float plans are evaluated in double and rounded once on output.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "fftw3.h"

enum { K_C2C = 0, K_R2C = 1 };

struct atmref_plan {
    int kind, prec;   /* prec: 0 float, 1 double */
    int rank, n[2], howmany, sign;
    void *in, *out;
    long idist, odist;
};

/* Twiddles of every radix-2 level of a length-n transform, evaluated with the
 * same expression as inline (so the values are bit-identical): level len
 * keeps exp(sign 2 pi i k / len), k < len/2, at [len/2 + k]. */
static void twiddles(double *wr, double *wi, long n, int sign)
{
    for (long len = 2; len <= n; len <<= 1)
        for (long k = 0; k < len / 2; k++) {
            double a = sign * 2.0 * M_PI * (double)k / (double)len;
            wr[len / 2 + k] = cos(a);
            wi[len / 2 + k] = sin(a);
        }
}

static void fft1(double *re, double *im, long n, int sign, const double *twr, const double *twi)
{
    if (n <= 1) return;
    if ((n & (n - 1)) == 0) {
        for (long i = 1, j = 0; i < n; i++) {
            long bit = n >> 1;
            for (; j & bit; bit >>= 1) j ^= bit;
            j ^= bit;
            if (i < j) {
                double t = re[i]; re[i] = re[j]; re[j] = t;
                t = im[i]; im[i] = im[j]; im[j] = t;
            }
        }
        for (long len = 2; len <= n; len <<= 1) {
            for (long i = 0; i < n; i += len)
                for (long k = 0; k < len / 2; k++) {
                    double wr = twr[len / 2 + k], wi = twi[len / 2 + k];
                    long p = i + k, q = i + k + len / 2;
                    double tr = re[q] * wr - im[q] * wi, ti = re[q] * wi + im[q] * wr;
                    re[q] = re[p] - tr; im[q] = im[p] - ti;
                    re[p] += tr; im[p] += ti;
                }
        }
        return;
    }
    double *xr = malloc(sizeof(double) * n), *xi = malloc(sizeof(double) * n);
    for (long k = 0; k < n; k++) {
        double sr = 0, si = 0;
        for (long j = 0; j < n; j++) {
            double a = sign * 2.0 * M_PI * (double)((j * k) % n) / (double)n;
            sr += re[j] * cos(a) - im[j] * sin(a);
            si += re[j] * sin(a) + im[j] * cos(a);
        }
        xr[k] = sr; xi[k] = si;
    }
    memcpy(re, xr, sizeof(double) * n);
    memcpy(im, xi, sizeof(double) * n);
    free(xr); free(xi);
}

/* 2-D DFT of an n0 x n1 row-major array (n1 fastest) */
static void fft2(double *re, double *im, long n0, long n1, int sign)
{
    double *cr = malloc(sizeof(double) * n0), *ci = malloc(sizeof(double) * n0);
    double *t1r = malloc(sizeof(double) * (n1 + 1)), *t1i = malloc(sizeof(double) * (n1 + 1));
    double *t0r = malloc(sizeof(double) * (n0 + 1)), *t0i = malloc(sizeof(double) * (n0 + 1));
    if ((n1 & (n1 - 1)) == 0) twiddles(t1r, t1i, n1, sign);
    if ((n0 & (n0 - 1)) == 0) twiddles(t0r, t0i, n0, sign);
    for (long r = 0; r < n0; r++) fft1(re + r * n1, im + r * n1, n1, sign, t1r, t1i);
    for (long c = 0; c < n1; c++) {
        for (long r = 0; r < n0; r++) { cr[r] = re[r * n1 + c]; ci[r] = im[r * n1 + c]; }
        fft1(cr, ci, n0, sign, t0r, t0i);
        for (long r = 0; r < n0; r++) { re[r * n1 + c] = cr[r]; im[r * n1 + c] = ci[r]; }
    }
    free(cr); free(ci); free(t1r); free(t1i); free(t0r); free(t0i);
}

static struct atmref_plan *mk(int kind, int prec, int rank, const int *n, int howmany, void *in, void *out, int sign,
                             long idist, long odist)
{
    struct atmref_plan *p = calloc(1, sizeof *p);
    p->kind = kind; p->prec = prec; p->rank = rank; p->howmany = howmany; p->sign = sign;
    p->n[0] = n[0]; p->n[1] = rank > 1 ? n[1] : 1;
    p->in = in; p->out = out; p->idist = idist; p->odist = odist;
    return p;
}

static void run(const struct atmref_plan *p)
{
    const long n0 = p->rank > 1 ? p->n[0] : 1, n1 = p->rank > 1 ? p->n[1] : p->n[0];
    const long tot = n0 * n1;
    double *re = malloc(sizeof(double) * tot), *im = malloc(sizeof(double) * tot);
    for (int h = 0; h < p->howmany; h++) {
        for (long i = 0; i < tot; i++) {
            if (p->kind == K_C2C) {
                if (p->prec) { const double *x = (const double *)p->in + 2 * (h * p->idist + i); re[i] = x[0]; im[i] = x[1]; }
                else { const float *x = (const float *)p->in + 2 * (h * p->idist + i); re[i] = x[0]; im[i] = x[1]; }
            } else {
                re[i] = p->prec ? ((const double *)p->in)[h * p->idist + i] : ((const float *)p->in)[h * p->idist + i];
                im[i] = 0.0;
            }
        }
        fft2(re, im, n0, n1, p->kind == K_R2C ? -1 : p->sign);
        /* r2c keeps the n1/2 + 1 non-redundant columns */
        const long oc = p->kind == K_R2C ? n1 / 2 + 1 : n1;
        for (long r = 0; r < n0; r++)
            for (long c = 0; c < oc; c++) {
                const long o = h * p->odist + r * oc + c, i = r * n1 + c;
                if (p->prec) { double *y = (double *)p->out + 2 * o; y[0] = re[i]; y[1] = im[i]; }
                else { float *y = (float *)p->out + 2 * o; y[0] = (float)re[i]; y[1] = (float)im[i]; }
            }
    }
    free(re); free(im);
}

void *fftw_malloc(size_t n) { return malloc(n); }
void fftw_free(void *p) { free(p); }
void *fftwf_malloc(size_t n) { return malloc(n); }
void fftwf_free(void *p) { free(p); }

#define DEF_PLANS(PFX, CT, RT, PREC)                                                                          \
    PFX##_plan PFX##_plan_dft_1d(int n, CT *in, CT *out, int sign, unsigned f)                             \
    { (void)f; return mk(K_C2C, PREC, 1, &n, 1, in, out, sign, n, n); }                                    \
    PFX##_plan PFX##_plan_dft_2d(int n0, int n1, CT *in, CT *out, int sign, unsigned f)                    \
    { int n[2] = {n0, n1}; (void)f; return mk(K_C2C, PREC, 2, n, 1, in, out, sign, (long)n0 * n1, (long)n0 * n1); } \
    PFX##_plan PFX##_plan_dft_r2c_1d(int n, RT *in, CT *out, unsigned f)                                   \
    { (void)f; return mk(K_R2C, PREC, 1, &n, 1, in, out, -1, n, n / 2 + 1); }                              \
    PFX##_plan PFX##_plan_dft_r2c_2d(int n0, int n1, RT *in, CT *out, unsigned f)                          \
    { int n[2] = {n0, n1}; (void)f; return mk(K_R2C, PREC, 2, n, 1, in, out, -1, (long)n0 * n1, (long)n0 * (n1 / 2 + 1)); } \
    PFX##_plan PFX##_plan_many_dft(int rank, const int *n, int howmany, CT *in, const int *ie, int is, int idist, \
                                   CT *out, const int *oe, int os, int odist, int sign, unsigned f)        \
    { (void)ie; (void)is; (void)oe; (void)os; (void)f;                                                      \
      return mk(K_C2C, PREC, rank, n, howmany, in, out, sign, idist, odist); }                              \
    PFX##_plan PFX##_plan_many_dft_r2c(int rank, const int *n, int howmany, RT *in, const int *ie, int is,  \
                                       int idist, CT *out, const int *oe, int os, int odist, unsigned f)   \
    { (void)ie; (void)is; (void)oe; (void)os; (void)f;                                                      \
      return mk(K_R2C, PREC, rank, n, howmany, in, out, -1, idist, odist); }                                \
    void PFX##_execute(const PFX##_plan p) { run(p); }                                                      \
    void PFX##_destroy_plan(PFX##_plan p) { free(p); }                                                      \
    int PFX##_import_wisdom_from_file(FILE *f) { (void)f; return 1; }                                       \
    void PFX##_export_wisdom_to_file(FILE *f) { (void)f; }                                                  \
    int PFX##_init_threads(void) { return 1; }                                                              \
    void PFX##_plan_with_nthreads(int n) { (void)n; }                                                       \
    void PFX##_cleanup_threads(void) {}                                                                     \
    void PFX##_cleanup(void) {}                                                                             \
    void PFX##_set_timelimit(double t) { (void)t; }

DEF_PLANS(fftw, fftw_complex, double, 1)
DEF_PLANS(fftwf, fftwf_complex, float, 0)
