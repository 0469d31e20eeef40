/*
 * atmwfs_oracle.c -- CPU restatement of the wavefront-series hot path of
 * AtmosphericTurbulenceSimul 1.2.11 (AtmosphericTurbulence module).
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA engine and
 * the timed CPU baseline; no product code path links or calls it.
 *
 * It is compiled twice (see oracle/Makefile):
 *   -DOR_REAL=double  -> liboracle64.so : the FP64 oracle.  All images are
 *                        double, as in the reference's WFprecision=1 mode.
 *   -DOR_REAL=float   -> liboracle32.so : the float-storage port of the
 *                        reference's WFprecision=0 path (float images,
 *                        double per-pixel arithmetic, float FFT).  This is the
 *                        "port" CPU baseline.
 *
 * Every function cites the reference lines it restates (paths relative to the
 * reference project root).  The FFT is the project's own radix-2 transform
 * standing in for FFTW (the reference's FFT library, unpinned version).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef OR_REAL
#define OR_REAL double
#endif

#define OR_PI 3.14159265358979323846264338328

typedef OR_REAL real_t;
typedef struct { real_t re, im; } cplx_t;

#define OR_EXPORT __attribute__((visibility("default")))

/* ------------------------------------------------------------------------ */
/* threads                                                                  */
/* ------------------------------------------------------------------------ */
static int g_threads = 1;

OR_EXPORT void or_set_threads(int n)
{
    g_threads = n < 1 ? 1 : n;
#ifdef _OPENMP
    omp_set_num_threads(g_threads);
#endif
}

OR_EXPORT int or_real_bytes(void) { return (int)sizeof(real_t); }

/* ------------------------------------------------------------------------ */
/* 1-D / 2-D complex DFT (stand-in for FFTW's fftw[f]_plan_dft_2d, used by   */
/* FFT_do2dfft src/fft/fft.c:1145-1296).  Unnormalised; sign -1 forward,    */
/* +1 inverse, like FFTW.  Power-of-two sizes only.                          */
/* ------------------------------------------------------------------------ */
typedef struct { long n; real_t *wr, *wi; long *rev; } fftplan_t;

static int ilog2l(long n) { int k = 0; while ((1L << k) < n) k++; return k; }

static void plan_make(fftplan_t *p, long n)
{
    p->n = n;
    p->wr = (real_t *)malloc(sizeof(real_t) * (size_t)(n / 2 + 1));
    p->wi = (real_t *)malloc(sizeof(real_t) * (size_t)(n / 2 + 1));
    p->rev = (long *)malloc(sizeof(long) * (size_t)n);
    for (long k = 0; k <= n / 2; k++) {
        /* twiddles evaluated in double from the exact rational angle */
        double a = -2.0 * OR_PI * (double)k / (double)n;
        p->wr[k] = (real_t)cos(a);
        p->wi[k] = (real_t)sin(a);
    }
    int lg = ilog2l(n);
    for (long i = 0; i < n; i++) {
        long r = 0;
        for (int b = 0; b < lg; b++) if (i & (1L << b)) r |= 1L << (lg - 1 - b);
        p->rev[i] = r;
    }
}

static void plan_free(fftplan_t *p) { free(p->wr); free(p->wi); free(p->rev); }

static void fft1d(cplx_t *a, const fftplan_t *p, int sign)
{
    long n = p->n;
    for (long i = 0; i < n; i++) {
        long r = p->rev[i];
        if (r > i) { cplx_t t = a[i]; a[i] = a[r]; a[r] = t; }
    }
    for (long len = 2; len <= n; len <<= 1) {
        long half = len >> 1, step = n / len;
        for (long i = 0; i < n; i += len) {
            for (long k = 0; k < half; k++) {
                real_t wr = p->wr[k * step];
                real_t wi = sign < 0 ? p->wi[k * step] : -p->wi[k * step];
                cplx_t u = a[i + k], v = a[i + k + half];
                real_t tr = v.re * wr - v.im * wi;
                real_t ti = v.re * wi + v.im * wr;
                a[i + k].re = u.re + tr;        a[i + k].im = u.im + ti;
                a[i + k + half].re = u.re - tr; a[i + k + half].im = u.im - ti;
            }
        }
    }
}

/* 2-D DFT of a row-major ny x nx image a[y*nx + x] (x fastest), in place. */
OR_EXPORT void or_fft2d(cplx_t *a, long nx, long ny, int sign)
{
    fftplan_t px, py;
    plan_make(&px, nx);
    plan_make(&py, ny);
#pragma omp parallel for schedule(static)
    for (long y = 0; y < ny; y++) fft1d(a + y * nx, &px, sign);
    const long CB = 8;
#pragma omp parallel
    {
        cplx_t *col = (cplx_t *)malloc(sizeof(cplx_t) * (size_t)(ny * CB));
#pragma omp for schedule(static)
        for (long x0 = 0; x0 < nx; x0 += CB) {
            long cb = (x0 + CB <= nx) ? CB : nx - x0;
            for (long y = 0; y < ny; y++)
                for (long c = 0; c < cb; c++) col[c * ny + y] = a[y * nx + x0 + c];
            for (long c = 0; c < cb; c++) fft1d(col + c * ny, &py, sign);
            for (long y = 0; y < ny; y++)
                for (long c = 0; c < cb; c++) a[y * nx + x0 + c] = col[c * ny + y];
        }
        free(col);
    }
    plan_free(&px);
    plan_free(&py);
}

/* permut(): quadrant swap (fftshift) of a 2-D complex image,
 * src/fft/fft.c:570-794 (naxis==2 branch). */
OR_EXPORT void or_permut(cplx_t *a, long nx, long ny)
{
    long xh = nx / 2, yh = ny / 2;
    for (long y = 0; y < yh; y++)
        for (long x = 0; x < xh; x++) {
            cplx_t t = a[y * nx + x];
            a[y * nx + x] = a[(y + yh) * nx + x + xh];
            a[(y + yh) * nx + x + xh] = t;
        }
    for (long y = yh; y < ny; y++)
        for (long x = 0; x < xh; x++) {
            cplx_t t = a[y * nx + x];
            a[y * nx + x] = a[(y - yh) * nx + x + xh];
            a[(y - yh) * nx + x + xh] = t;
        }
}

/* ------------------------------------------------------------------------ */
/* Fresnel_propagate_wavefront, src/WFpropagate/WFpropagate.c:68-152        */
/* FFT -> permut -> multiply exp(-i coeff r^2)/N^2 -> permut -> inverse FFT  */
/* coeff = pi z lambda / (dx N)^2 (WFpropagate.c:91).  in and out may alias.*/
/* ------------------------------------------------------------------------ */
OR_EXPORT void or_fresnel(const cplx_t *in, cplx_t *out, long n, double dx, double z, double lambda)
{
    cplx_t *tmp = (cplx_t *)malloc(sizeof(cplx_t) * (size_t)(n * n));
    memcpy(tmp, in, sizeof(cplx_t) * (size_t)(n * n));
    or_fft2d(tmp, n, n, -1);
    or_permut(tmp, n, n);
    double coeff = OR_PI * z * lambda / (dx * (double)n) / (dx * (double)n);
    double co1 = (double)n * (double)n;
    long nh = n / 2;
#pragma omp parallel for schedule(static)
    for (long jj = 0; jj < n; jj++) {
        long dy2 = (jj - nh) * (jj - nh);
        for (long ii = 0; ii < n; ii++) {
            long dxi = ii - nh;
            double ang = -coeff * (double)(dxi * dxi + dy2);
            double re = (double)tmp[jj * n + ii].re / co1;
            double im = (double)tmp[jj * n + ii].im / co1;
            double c = cos(ang), s = sin(ang);
            tmp[jj * n + ii].re = (real_t)(re * c - im * s);
            tmp[jj * n + ii].im = (real_t)(re * s + im * c);
        }
    }
    or_permut(tmp, n, n);
    or_fft2d(tmp, n, n, +1);
    memcpy(out, tmp, sizeof(cplx_t) * (size_t)(n * n));
    free(tmp);
}

/* ------------------------------------------------------------------------ */
/* Keys (a = -1/2) bicubic sample of a periodic M x M screen at pixel        */
/* (xpos+ii, ypos+jj): AtmosphericTurbulence.c:2806-2903 (lambda_ref) and   */
/* :3133-3233 (lambda_sci).  The reference evaluates the 16-coefficient      */
/* polynomial form; this restatement uses the algebraically identical       */
/* separable weights.  Coordinates follow the reference: fmod of the        */
/* shifted pixel coordinate, truncation, x along ii, y along jj, wrap of    */
/* the four taps into [0, M).                                               */
/* ------------------------------------------------------------------------ */
static inline void keys_w(double t, double w[4])
{
    double t2 = t * t, t3 = t2 * t;
    w[0] = 0.5 * (-t3 + 2.0 * t2 - t);
    w[1] = 0.5 * (3.0 * t3 - 5.0 * t2 + 2.0);
    w[2] = 0.5 * (-3.0 * t3 + 4.0 * t2 + t);
    w[3] = 0.5 * (t3 - t2);
}

static inline double bicubic_at(const real_t *S, long M, double xpos, double ypos, long ii, long jj)
{
    double iimf = fmod(xpos + (double)ii, (double)M);
    double jjmf = fmod(ypos + (double)jj, (double)M);
    long iim = (long)iimf, jjm = (long)jjmf;
    double wx[4], wy[4];
    keys_w(iimf - (double)iim, wx);
    keys_w(jjmf - (double)jjm, wy);
    long xi[4], yj[4];
    for (int k = 0; k < 4; k++) {
        long a = iim - 1 + k, b = jjm - 1 + k;
        if (a > M - 1) a -= M;
        if (a < 0) a += M;
        if (b > M - 1) b -= M;
        if (b < 0) b += M;
        xi[k] = a; yj[k] = b;
    }
    double v = 0.0;
    for (int j = 0; j < 4; j++) {
        double h = 0.0;
        for (int i = 0; i < 4; i++) h += wx[i] * (double)S[yj[j] * M + xi[i]];
        v += wy[j] * h;
    }
    return v;
}

/* Bilinear alternative (BICUBIC = 0), AtmosphericTurbulence.c:2764-2797. */
static inline double bilinear_at(const real_t *S, long M, double xpos, double ypos, long ii, long jj)
{
    double iimf = fmod(xpos + (double)ii, (double)M);
    double jjmf = fmod(ypos + (double)jj, (double)M);
    long iim = (long)iimf, jjm = (long)jjmf;
    double fx = iimf - (double)iim, fy = jjmf - (double)jjm;
    long iim1 = iim + 1, jjm1 = jjm + 1;
    if (iim == M) iim = 0;
    if (jjm == M) jjm = 0;
    if (iim1 > M - 1) iim1 -= M;
    if (jjm1 > M - 1) jjm1 -= M;
    double v = (1.0 - fx) * (1.0 - fy) * (double)S[jjm * M + iim];
    v += (1.0 - fx) * fy * (double)S[jjm1 * M + iim];
    v += fx * fy * (double)S[jjm1 * M + iim1];
    v += fx * (1.0 - fy) * (double)S[jjm * M + iim1];
    return v;
}

/* Interpolated W x W window of one layer (value(ii,jj) at out[jj*W+ii]),
 * multiplied by scoeff when scoeff != 1 (reference :3235). */
OR_EXPORT void or_window(const real_t *S, long M, double xpos, double ypos, long W,
                         double scoeff, int bicubic, double *out)
{
#pragma omp parallel for schedule(static)
    for (long jj = 0; jj < W; jj++)
        for (long ii = 0; ii < W; ii++) {
            double v = bicubic ? bicubic_at(S, M, xpos, ypos, ii, jj) : bilinear_at(S, M, xpos, ypos, ii, jj);
            out[jj * W + ii] = v * scoeff;
        }
}

/* ------------------------------------------------------------------------ */
/* Super-layer grouping, AtmosphericTurbulence.c:2067-2132, and the layer ->*/
/* super-layer index, :2135-2147.  cn2 must already be normalised to sum 1  */
/* (:2009-2015).  Returns the number of super-layers; salt receives their   */
/* altitudes, sidx the index of each layer.                                 */
/* ------------------------------------------------------------------------ */
OR_EXPORT long or_superlayers(const double *alt, const double *cn2, long L, double bin,
                              double *salt, long *sidx)
{
    double *scn2 = (double *)malloc(sizeof(double) * (size_t)L);
    long S = L;
    for (long i = 0; i < L; i++) { salt[i] = alt[i]; scn2[i] = cn2[i]; }
    for (;;) {
        double mind = alt[L - 1];
        long idx = 0;
        for (long i = 0; i < S - 1; i++) {
            double v = salt[i + 1] - salt[i];
            if (v < mind) { mind = v; idx = i; }
        }
        if (mind > bin || S == 1) break;
        salt[idx] = (scn2[idx] * salt[idx] + scn2[idx + 1] * salt[idx + 1]) / (scn2[idx] + scn2[idx + 1]);
        scn2[idx] = scn2[idx] + scn2[idx + 1];
        for (long i = idx + 1; i < S - 1; i++) { salt[i] = salt[i + 1]; scn2[i] = scn2[i + 1]; }
        S--;
    }
    long nsep = S - 1;
    double *sep = (double *)malloc(sizeof(double) * (size_t)(nsep + 1));
    for (long i = 0; i < nsep; i++) sep[i] = 0.5 * (salt[i] + salt[i + 1]);
    sep[nsep] = INFINITY; /* the reference reads one element past the end here */
    for (long l = 0; l < L; l++) {
        long idx = 0;
        for (long i = 0; i < nsep; i++)
            if (sep[i] < alt[l] && sep[i + 1] > alt[l]) idx = i + 1;
        if (nsep > 0 && alt[l] > sep[nsep - 1]) idx = nsep;
        sidx[l] = idx;
    }
    free(sep);
    free(scn2);
    return S;
}

/* ------------------------------------------------------------------------ */
/* Frozen-flow position update, non-real-time branch,                       */
/* AtmosphericTurbulence.c:2700-2756: pos += v dt, then wrap into [0, M]    */
/* (strict comparisons, so pos == M survives) with wrap counters.           */
/* ------------------------------------------------------------------------ */
OR_EXPORT void or_position_step(double *pos, long *cnt, double v, float dt, long M)
{
    *pos += v * (double)dt;
    while (*pos < 0) { *pos += (double)M; (*cnt)++; }
    while (*pos > (double)M) { *pos -= (double)M; (*cnt)--; }
}

/* ------------------------------------------------------------------------ */
/* One frame for one wavelength: AtmosphericTurbulence.c:2566-2633 (reset), */
/* 2649-2692 (layer loop with Fresnel hops between super-layers) and the     */
/* per-pixel accumulation :2903-2916 / :3235-3245.                          */
/*   screens[l] : M x M screen of layer l (after renormalisation)           */
/*   xpos/ypos  : positions of every layer for this frame (already updated) */
/*   scoeff     : per-layer phase multiplier (NULL = none, lambda_ref path) */
/*   sidx/salt  : super-layer index of each layer and super-layer altitudes  */
/*   hop_n      : optional air index of each hop in the order they run (top */
/*                down): the hop uses lambda / hop_n[h] instead of the      */
/*                vacuum lambda of the reference (WFpropagate.c:91)         */
/* outputs: phase sum (W x W real) and complex field (W x W).               */
/* ------------------------------------------------------------------------ */
OR_EXPORT void or_frame_n(const real_t *const *screens, long M, long L,
                          const double *xpos, const double *ypos, const double *scoeff,
                          const long *sidx, const double *salt,
                          double dx, double zangle, double lambda, long W,
                          int amplitude, int fresnel, int bicubic, const double *hop_n,
                          real_t *phasum, cplx_t *field)
{
    long n = W * W;
    long hop = 0;
    for (long i = 0; i < n; i++) { phasum[i] = 0; field[i].re = 1; field[i].im = 0; }
    double *win = (double *)malloc(sizeof(double) * (size_t)n);
    for (long layer = L - 1; layer >= 0; layer--) {
        if (layer != L - 1 && sidx[layer + 1] != sidx[layer] && amplitude && fresnel) {
            double z = (salt[sidx[layer + 1]] - salt[sidx[layer]]) / cos(zangle);
            or_fresnel(field, field, W, dx, z, hop_n ? lambda / hop_n[hop] : lambda);
            hop++;
        }
        or_window(screens[layer], M, xpos[layer], ypos[layer], W, scoeff ? scoeff[layer] : 1.0, bicubic, win);
#pragma omp parallel for schedule(static)
        for (long i = 0; i < n; i++) {
            double v = win[i];
            phasum[i] = (real_t)((double)phasum[i] + v);
            if (amplitude) {
                double re = (double)field[i].re, im = (double)field[i].im;
                double c = cos(v), s = sin(v);
                field[i].re = (real_t)(re * c - im * s);
                field[i].im = (real_t)(re * s + im * c);
            }
        }
    }
    free(win);
}

OR_EXPORT void or_frame(const real_t *const *screens, long M, long L,
                        const double *xpos, const double *ypos, const double *scoeff,
                        const long *sidx, const double *salt,
                        double dx, double zangle, double lambda, long W,
                        int amplitude, int fresnel, int bicubic,
                        real_t *phasum, cplx_t *field)
{
    or_frame_n(screens, M, L, xpos, ypos, scoeff, sidx, salt, dx, zangle, lambda, W, amplitude, fresnel, bicubic, NULL,
               phasum, field);
}

/* reference's rounding idiom  (long)(x + 1000.5) - 1000  */
static inline double ref_round(double x) { return (double)((long)(x + 1000.5) - 1000); }

/* ------------------------------------------------------------------------ */
/* Reference-wavelength output, AtmosphericTurbulence.c:3418-3476: centre   */
/* crop; amp = |U|; pha = atan2(U) + 2 pi round(phasum / 2 pi).             */
/* ------------------------------------------------------------------------ */
OR_EXPORT void or_output_ref(const real_t *phasum, const cplx_t *field, long W, long Wout,
                             int amplitude, real_t *pha, real_t *amp)
{
    long off = (W - Wout) / 2;
    for (long jj = 0; jj < Wout; jj++)
        for (long ii = 0; ii < Wout; ii++) {
            long s = (jj + off) * W + ii + off, o = jj * Wout + ii;
            pha[o] = phasum[s];
            if (amplitude) {
                double re = (double)field[s].re, im = (double)field[s].im;
                amp[o] = (real_t)sqrt(re * re + im * im);
                double p = atan2(im, re);
                pha[o] = (real_t)(p + 2.0 * OR_PI * ref_round((double)pha[o] / 2.0 / OR_PI));
            } else {
                amp[o] = 1;
            }
        }
}

/* ------------------------------------------------------------------------ */
/* Science-wavelength output with bin-based phase unwrapping,               */
/* AtmosphericTurbulence.c:3522-3941 (float branch) / 3942-4215 (double).   */
/* nb = Wout/20 bins per axis; bins hold sum of exp(i(phasum - atan2 U));   */
/* the iterative 2 pi relaxation uses the 8-neighbourhood (vote 0.2) and    */
/* the ring at distance 2 (vote 0.15), in the reference's sweep order so    */
/* that the float accumulation of the votes is reproduced.                  */
/* Returns the number of relaxation iterations.                             */
/* ------------------------------------------------------------------------ */
typedef struct { int dx, dy; double c; } stencil_t;

/* the twelve sweeps: (offset of index2 relative to index1) and vote       */
static const stencil_t k_sweeps[12] = {
    {+1, 0, 0.2}, {0, +1, 0.2}, {+1, +1, 0.2}, {+1, -1, 0.2},
    {+2, 0, 0.15}, {0, -2, 0.15}, {-1, -2, 0.15}, {+1, -2, 0.15},
    {-2, -2, 0.15}, {+2, -2, 0.15}, {+2, -1, 0.15}, {-2, -1, 0.15},
};

/* Offsets of index1 relative to the loop variables (ii2, jj2) per sweep,  */
/* i.e. index1 = (ii2 + ox, jj2 + oy), index2 = index1 + (dx, dy).          */
static const int k_sweep_o1[12][2] = {
    {0, 0}, {0, 0}, {0, 0}, {0, 1},
    {0, 0}, {0, 2}, {1, 2}, {0, 2},
    {2, 2}, {0, 2}, {0, 1}, {2, 1},
};

static long unwrap_bins(real_t *pb, long nx, long ny)
{
    real_t *ch = (real_t *)malloc(sizeof(real_t) * (size_t)(nx * ny));
    long chiter = 0, chcnt0cnt = 0;
    double plim = 1.0;
    while (plim > 0.51 && chiter < 1000 && chcnt0cnt < 5) {
        chiter++;
        long chcnt = 0;
        for (long i = 0; i < nx * ny; i++) ch[i] = 0;
        for (int s = 0; s < 12; s++) {
            int dx = k_sweeps[s].dx, dy = k_sweeps[s].dy;
            int ox = k_sweep_o1[s][0], oy = k_sweep_o1[s][1];
            /* loop ranges: both endpoints inside the bin grid */
            long ilo = 0, ihi = nx, jlo = 0, jhi = ny;
            long x1min = ox, x2min = ox + dx, y1min = oy, y2min = oy + dy;
            long mnx = x1min < x2min ? x1min : x2min, mxx = x1min > x2min ? x1min : x2min;
            long mny = y1min < y2min ? y1min : y2min, mxy = y1min > y2min ? y1min : y2min;
            ilo = -mnx; ihi = nx - mxx; jlo = -mny; jhi = ny - mxy;
            if (ilo < 0) ilo = 0;
            if (jlo < 0) jlo = 0;
            double c = k_sweeps[s].c;
            for (long ii2 = ilo; ii2 < ihi; ii2++)
                for (long jj2 = jlo; jj2 < jhi; jj2++) {
                    long i1 = (jj2 + oy) * nx + ii2 + ox;
                    long i2 = (jj2 + oy + dy) * nx + ii2 + ox + dx;
                    double pv1 = (double)pb[i1], pv2 = (double)pb[i2];
                    if (pv2 > pv1 + OR_PI) { ch[i1] = (real_t)((double)ch[i1] + c); ch[i2] = (real_t)((double)ch[i2] - c); }
                    if (pv1 > pv2 + OR_PI) { ch[i1] = (real_t)((double)ch[i1] - c); ch[i2] = (real_t)((double)ch[i2] + c); }
                }
        }
        plim = 0.0;
        for (long i = 0; i < nx * ny; i++) if (fabs((double)ch[i]) > plim) plim = fabs((double)ch[i]);
        plim -= 0.001;
        if (plim < 0.5) plim = 0.5;
        for (long ii2 = 0; ii2 < nx; ii2++)
            for (long jj2 = 0; jj2 < ny; jj2++) {
                long i = jj2 * nx + ii2;
                int interior = (ii2 > 1) && (jj2 > 1) && (ii2 < nx - 2) && (jj2 < ny - 2);
                if ((double)ch[i] > plim) { if (interior) chcnt++; pb[i] = (real_t)((double)pb[i] + 2.0 * OR_PI); }
                if ((double)ch[i] < -plim) { if (interior) chcnt++; pb[i] = (real_t)((double)pb[i] - 2.0 * OR_PI); }
            }
        if (chcnt == 0) chcnt0cnt++; else chcnt0cnt = 0;
    }
    free(ch);
    return chiter;
}

OR_EXPORT long or_output_sci(const real_t *phasum, const cplx_t *field, long W, long Wout,
                             int amplitude, real_t *pha, real_t *amp, real_t *peakbins)
{
    long off = (W - Wout) / 2;
    if (!amplitude) {
        for (long jj = 0; jj < Wout; jj++)
            for (long ii = 0; ii < Wout; ii++) {
                pha[jj * Wout + ii] = phasum[(jj + off) * W + ii + off];
                amp[jj * Wout + ii] = 1;
            }
        return 0;
    }
    long nx = Wout / 20, ny = Wout / 20;
    real_t *bre = (real_t *)calloc((size_t)(nx * ny + 1), sizeof(real_t));
    real_t *bim = (real_t *)calloc((size_t)(nx * ny + 1), sizeof(real_t));
    real_t *pb = (real_t *)calloc((size_t)(nx * ny + 1), sizeof(real_t));
    for (long ii = 0; ii < Wout; ii++)
        for (long jj = 0; jj < Wout; jj++) {
            long s = (jj + off) * W + ii + off, o = jj * Wout + ii;
            double re = (double)field[s].re, im = (double)field[s].im;
            amp[o] = (real_t)sqrt(re * re + im * im);
            double p = atan2(im, re);
            pha[o] = (real_t)p;
            long i2 = (long)(1.0 * (double)ii / (double)Wout * (double)nx);
            long j2 = (long)(1.0 * (double)jj / (double)Wout * (double)ny);
            if (i2 < nx && j2 < ny) {
                bre[j2 * nx + i2] = (real_t)((double)bre[j2 * nx + i2] + cos((double)phasum[s] - p));
                bim[j2 * nx + i2] = (real_t)((double)bim[j2 * nx + i2] + sin((double)phasum[s] - p));
            }
        }
    for (long i = 0; i < nx * ny; i++) pb[i] = (real_t)atan2((double)bim[i], (double)bre[i]);
    long iters = unwrap_bins(pb, nx, ny);
    double peak = 0.0;
    for (long ii = 0; ii < Wout; ii++)
        for (long jj = 0; jj < Wout; jj++) {
            long i2 = (long)(1.0 * (double)ii / (double)Wout * (double)nx);
            long j2 = (long)(1.0 * (double)jj / (double)Wout * (double)ny);
            if (i2 < nx && j2 < ny) peak = (double)pb[j2 * nx + i2];
            long s = (jj + off) * W + ii + off, o = jj * Wout + ii;
            double p = (double)pha[o];
            pha[o] = (real_t)(p + 2.0 * OR_PI * ref_round(((double)phasum[s] - p - peak) / 2.0 / OR_PI));
        }
    if (peakbins) memcpy(peakbins, pb, sizeof(real_t) * (size_t)(nx * ny));
    free(bre); free(bim); free(pb);
    return iters;
}

/* ------------------------------------------------------------------------ */
/* r0 measurement, AtmosphericTurbulence.c:2241-2276: mean square phase     */
/* difference at a 50-pixel x lag, r0 = 50 (msd / 6.88)^(-3/5) pixels.      */
/* ------------------------------------------------------------------------ */
OR_EXPORT double or_measure_r0(const real_t *S, long M)
{
    const long dpix = 50;
    double tot = 0.0;
    long cnt = 0;
    for (long ii = 0; ii < M - dpix; ii++)
        for (long jj = 0; jj < M; jj++) {
            double p1 = (double)S[jj * M + ii], p2 = (double)S[jj * M + ii + dpix];
            tot += (p1 - p2) * (p1 - p2);
            cnt++;
        }
    return (double)dpix * pow((tot / (double)cnt) / 6.88, -3.0 / 5.0);
}

/* ------------------------------------------------------------------------ */
/* Master-screen synthesis given its noise, AtmosphericTurbulence.c:643-855 */
/*   upha : uniform [0,1) image (make_rnd, :683-689), scaled by 2 pi       */
/*   gau  : standard normal image (make_rnd -gauss, :742-745)               */
/* The amplitude is g sqrt(exp(-r^2/fi^2)) / (r^2 + fo^2)^(11/12) with      */
/* fo = M / L0pix, fi = (5.92/2pi) M / l0pix; DC set to 0; fftshift; FFT;   */
/* the real and imaginary parts are each scaled by 1/sqrt(C) where C is the */
/* geometric mean of D(r)/r^(5/3) over lags (1..2)^2 of the circular        */
/* structure function D (fft_structure_function, info.c:1670-1690, computed */
/* here directly from its definition).  Writes both screens.               */
/* ------------------------------------------------------------------------ */
static double strf_lag(const real_t *o, long M, long lx, long ly)
{
    double tot = 0.0;
    for (long y = 0; y < M; y++)
        for (long x = 0; x < M; x++) {
            double d = (double)o[y * M + x] - (double)o[((y + ly) % M) * M + (x + lx) % M];
            tot += d * d;
        }
    return tot / (double)(M * M);
}

OR_EXPORT void or_master_screen(const real_t *upha, const real_t *gau, long M, double L0pix,
                                double l0pix, real_t *out1, real_t *out2, double *cfit)
{
    double fo = (double)M / L0pix;
    double fi = (5.92 / (2.0 * OR_PI)) * (double)M / l0pix;
    cplx_t *c = (cplx_t *)malloc(sizeof(cplx_t) * (size_t)(M * M));
    for (long jj = 0; jj < M; jj++)
        for (long ii = 0; ii < M; ii++) {
            double dx = (double)ii - (double)(M / 2), dy = (double)jj - (double)(M / 2);
            real_t d = (real_t)sqrt(dx * dx + dy * dy + fo * fo);
            real_t g = (real_t)((double)gau[jj * M + ii] * sqrt(exp(-(dx * dx + dy * dy) / fi / fi)));
            real_t d1 = (real_t)pow((double)d, 11.0 / 6.0);
            real_t a = (real_t)((double)g / (double)d1);
            if (ii == M / 2 && jj == M / 2) a = 0;
            real_t ph = (real_t)((double)upha[jj * M + ii] * 2.0 * OR_PI);
            c[jj * M + ii].re = (real_t)((double)a * cos((double)ph));
            c[jj * M + ii].im = (real_t)((double)a * sin((double)ph));
        }
    or_permut(c, M, M);
    or_fft2d(c, M, M, -1);
    real_t *o1 = out1, *o2 = out2;
    for (long i = 0; i < M * M; i++) { o1[i] = c[i].re; o2[i] = c[i].im; }
    free(c);
    double C[2];
    for (int k = 0; k < 2; k++) {
        const real_t *o = k ? o2 : o1;
        double v = 0.0;
        long cnt = 0;
        for (long ii = 1; ii < 3; ii++)
            for (long jj = 1; jj < 3; jj++) {
                v += log10(strf_lag(o, M, ii, jj)) - 5.0 / 3.0 * log10(sqrt((double)(ii * ii + jj * jj)));
                cnt++;
            }
        C[k] = pow(10.0, v / (double)cnt);
    }
    double s1 = 1.0 / sqrt(C[0]), s2 = 1.0 / sqrt(C[1]);
    for (long i = 0; i < M * M; i++) { o1[i] = (real_t)((double)o1[i] * s1); o2[i] = (real_t)((double)o2[i] * s2); }
    if (cfit) { cfit[0] = C[0]; cfit[1] = C[1]; }
}

/* ------------------------------------------------------------------------ */
/* Philox4x32-10 counter-based generator (Salmon et al., SC'11), the noise  */
/* source of the seeded master screens.  For pixel p of stream s:           */
/* counter = (p, s, 0, 0), key = (seed lo, seed hi).  Uniform = top 24 bits */
/* of word 0 times 2^-24; Gaussian = Box-Muller on words 1 and 2.           */
/* ------------------------------------------------------------------------ */
static inline void philox_round(uint32_t c[4], const uint32_t k[2])
{
    uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c[1] ^ k[0];
    uint32_t n2 = hi0 ^ c[3] ^ k[1];
    c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
}

/* full-width form: 4-word counter, 2-word key (for the published known-answer vectors) */
OR_EXPORT void or_philox4(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
    uint32_t k[2] = {key[0], key[1]};
    for (int r = 0; r < 10; r++) {
        philox_round(c, k);
        if (r < 9) { k[0] += 0x9E3779B9u; k[1] += 0xBB67AE85u; }
    }
    memcpy(out, c, sizeof(c));
}

OR_EXPORT void or_philox(uint64_t seed, uint32_t ctr0, uint32_t ctr1, uint32_t out[4])
{
    const uint32_t c[4] = {ctr0, ctr1, 0u, 0u};
    const uint32_t k[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    or_philox4(c, k, out);
}

OR_EXPORT void or_screen_noise(uint64_t seed, uint32_t stream, long M, float *upha, float *gau)
{
    for (long p = 0; p < M * M; p++) {
        uint32_t r[4];
        or_philox(seed, (uint32_t)p, stream, r);
        float u = (float)(r[0] >> 8) * (1.0f / 16777216.0f);
        double u1 = ((double)(r[1] >> 8) + 1.0) * (1.0 / 16777216.0);
        double u2 = (double)(r[2] >> 8) * (1.0 / 16777216.0);
        upha[p] = u;
        gau[p] = (float)(sqrt(-2.0 * log(u1)) * cos(2.0 * OR_PI * u2));
    }
}
