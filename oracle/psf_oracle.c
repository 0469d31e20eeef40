/*
 * psf_oracle.c -- CPU restatement of the PSF consumers that follow the
 * wavefront series in AtmosphericTurbulenceSimul 1.2.11.
 *
 * TEST INFRASTRUCTURE ONLY: the checker of the GPU exposure and chromatic
 * PSFs and of the host image measures.  No product code path links it.
 *
 * Compiled with atmwfs_oracle.c into liboracle64.so (real_t = double) and
 * liboracle32.so (real_t = float); see oracle/Makefile.  Scalars of the
 * measures follow the reference's float / double types in both builds, the
 * images are real_t.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifndef OR_REAL
#define OR_REAL double
#endif
typedef OR_REAL real_t;
typedef struct { real_t re, im; } cplx_t;
#define OR_EXPORT __attribute__((visibility("default")))

void or_fft2d(cplx_t *a, long nx, long ny, int sign);

/* One frame of measure_wavefront_series_expoframes
 * (src/AtmosphericTurbulence/AtmosphericTurbulence.c:6700-6735): the W x W
 * field amp e^{i pha} at offset W/2 of a zero 2W x 2W array, do2dfft,
 * permut, psf += |.|^2.  psf is the centred 2W x 2W image. */
OR_EXPORT void or_psf_expo_add(const real_t *amp, const real_t *pha, long W, real_t *psf)
{
    const long N = 2 * W, off = W / 2, h = N / 2;
    cplx_t *a = (cplx_t *)calloc((size_t)(N * N), sizeof(cplx_t));
    for (long jj = 0; jj < W; jj++)
        for (long ii = 0; ii < W; ii++) {
            const double A = amp[jj * W + ii], P = pha[jj * W + ii];
            a[(jj + off) * N + ii + off].re = (real_t)(A * cos(P));
            a[(jj + off) * N + ii + off].im = (real_t)(A * sin(P));
        }
    or_fft2d(a, N, N, -1);
    for (long j = 0; j < N; j++)
        for (long i = 0; i < N; i++) {
            const cplx_t z = a[((j + h) % N) * N + (i + h) % N];
            psf[j * N + i] += z.re * z.re + z.im * z.im;
        }
    free(a);
}

/* PSF_makeChromatPSF (src/psf/psf.c:54-136). */
OR_EXPORT void or_chromat_psf(const real_t *amp, const real_t *pha, long n, float coeff1, float coeff2, long nbstep,
                              float apo, real_t *out)
{
    const float eps = 1.0e-5f;
    const long h = n / 2;
    cplx_t *a = (cplx_t *)malloc(sizeof(cplx_t) * (size_t)(n * n));
    real_t *I = (real_t *)malloc(sizeof(real_t) * (size_t)(n * n));
    memset(out, 0, sizeof(real_t) * (size_t)(n * n));
    for (long step = 0; step < nbstep; step++) {
        const float coeff = (float)(coeff1 * pow(pow((coeff2 / coeff1), 1.0 / (nbstep - 1)), (double)step));
        float x = (float)((coeff - (coeff1 + coeff2) / 2.0) / ((coeff2 - coeff1) / 2.0));
        float mc;
        if (apo > eps)
            mc = (float)pow((1.0 - pow((fabs(x) - (1.0 - apo)) / apo, 2.0)), 4.0);
        else
            mc = 1.0f;
        if ((1.0 - x * x) < eps) mc = 0.0f;
        if (fabs(x) < apo) mc = 1.0f;
        /* phase x coeff, complex field, permut, FFT, permut, |.|^2 (the
           first permut only multiplies the transform by (-1)^(kx+ky)) */
        for (long p = 0; p < n * n; p++) {
            const double P = (double)pha[p] * coeff;
            a[p].re = (real_t)(amp[p] * cos(P));
            a[p].im = (real_t)(amp[p] * sin(P));
        }
        or_fft2d(a, n, n, -1);
        for (long j = 0; j < n; j++)
            for (long i = 0; i < n; i++) {
                const cplx_t z = a[((j + h) % n) * n + (i + h) % n];
                I[j * n + i] = z.re * z.re + z.im * z.im;
            }
        for (long ii = 0; ii < n; ii++)
            for (long jj = 0; jj < n; jj++) {
                const float xx = (float)((1.0 * (ii - n / 2) * coeff) + n / 2);
                const float yy = (float)((1.0 * (jj - n / 2) * coeff) + n / 2);
                const long i = (long)xx, j = (long)yy;
                const double u = xx - i, t = yy - j;
                if ((i < n - 1) && (j < n - 1) && (i > -1) && (j > -1)) {
                    double tmp = (1.0 - u) * (1.0 - t) * I[j * n + i];
                    tmp += (1.0 - u) * t * I[(j + 1) * n + i];
                    tmp += u * (1.0 - t) * I[j * n + i + 1];
                    tmp += u * t * I[(j + 1) * n + i + 1];
                    out[jj * n + ii] += mc * tmp / coeff / coeff;
                }
            }
    }
    free(a);
    free(I);
}

/* gauss_filter (src/image_filter/image_filter.c:410-555) on one 2-D image. */
OR_EXPORT void or_gauss_filter(const real_t *in, long nx, long ny, float sigma, int filter_size, real_t *out)
{
    long fs = filter_size;
    if (fs > nx / 2 - 1) fs = nx / 2 - 1;
    if (fs > ny / 2 - 1) fs = ny / 2 - 1;
    const long K = 2 * fs + 1;
    double *a = (double *)malloc(sizeof(double) * (size_t)K), sum = 0.0;
    for (long i = 0; i < K; i++) {
        a[i] = exp(-(double)((i - fs) * (i - fs)) / sigma / sigma);
        sum += a[i];
    }
    for (long i = 0; i < K; i++) a[i] /= sum;
    real_t *tmp = (real_t *)calloc((size_t)(nx * ny), sizeof(real_t));
    memset(out, 0, sizeof(real_t) * (size_t)(nx * ny));
    for (long jj = 0; jj < ny; jj++) {
        const real_t *r = in + jj * nx;
        real_t *t = tmp + jj * nx;
        for (long ii = 0; ii < nx - K; ii++)
            for (long i = 0; i < K; i++) t[ii + fs] += a[i] * r[ii + i];
        for (long ii = 0; ii < fs; ii++) {
            double tot = 0.0;
            for (long i = fs - ii; i < K; i++) { t[ii] += a[i] * r[ii - fs + i]; tot += a[i]; }
            t[ii] /= tot;
        }
        for (long ii = nx - fs - 1; ii < nx; ii++) {
            double tot = 0.0;
            for (long i = 0; i < K - (ii - nx + fs + 1); i++) { t[ii] += a[i] * r[ii - fs + i]; tot += a[i]; }
            t[ii] /= tot;
        }
    }
    for (long ii = 0; ii < nx; ii++) {
        for (long jj = 0; jj < ny - K; jj++)
            for (long j = 0; j < K; j++) out[(jj + fs) * nx + ii] += a[j] * tmp[(jj + j) * nx + ii];
        for (long jj = 0; jj < fs; jj++) {
            double tot = 0.0;
            long jmax = K;
            if (jj - fs + jmax > ny) jmax = ny - jj + fs;
            for (long j = fs - jj; j < jmax; j++) { out[jj * nx + ii] += a[j] * tmp[(jj - fs + j) * nx + ii]; tot += a[j]; }
            out[jj * nx + ii] /= tot;
        }
        for (long jj = ny - fs - 1; jj < ny; jj++) {
            double tot = 0.0;
            for (long j = 0; j < K - (jj - ny + fs + 1); j++) { out[jj * nx + ii] += a[j] * tmp[(jj - fs + j) * nx + ii]; tot += a[j]; }
            out[jj * nx + ii] /= tot;
        }
    }
    free(a);
    free(tmp);
}

static int cmp_real(const void *x, const void *y)
{
    const real_t a = *(const real_t *)x, b = *(const real_t *)y;
    return a < b ? -1 : a > b ? 1 : 0;
}

/* center_PSF (src/psf/psf.c:442-530): background from arith_image_median
 * (COREMOD_arith.c:1207 -> arith_image_percentile :1150-1161, whose float
 * branch leaves its copy unsorted: the pixel at index (long)(0.5 n)), 3 x 3
 * median filter (image_filter.c:100-140), ten shrinking-box barycentres. */
OR_EXPORT void or_center_psf(const real_t *img, long nx, long ny, double *xc, double *yc)
{
    const long n = nx * ny;
    real_t *m = (real_t *)malloc(sizeof(real_t) * (size_t)n);
    const double back = img[(long)(0.5 * n)];
    memcpy(m, img, sizeof(real_t) * (size_t)n);
    real_t w[9];
    for (long jj = 1; jj < ny - 1; jj++)
        for (long ii = 1; ii < nx - 1; ii++) {
            int k = 0;
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) w[k++] = img[(jj - 1 + j) * nx + ii - 1 + i];
            qsort(w, 9, sizeof(real_t), cmp_real);
            m[jj * nx + ii] = w[4];
        }
    const int nbiter = 10;
    double cx = (double)(nx / 2), cy = (double)(ny / 2), ocx = cx, ocy = cy;
    for (int k = 0; k < nbiter; k++) {
        const long n3 = (long)(1.0 * nx / 2 / (1.0 + (0.1 * nx / 2 * k / (4 * nbiter))));
        long is = (long)(0.5 + ocx - n3), ie = (long)(0.5 + ocx + n3);
        long js = (long)(0.5 + ocy - n3), je = (long)(0.5 + ocy + n3);
        if (is < 0) is = 0;
        if (ie > nx - 1) ie = nx - 1;
        if (js < 0) js = 0;
        if (je > ny - 1) je = ny - 1;
        double tot = 0.0;
        cx = cy = 0.0;
        for (long jj = js; jj < je; jj++)
            for (long ii = is; ii < ie; ii++) {
                const double v = m[jj * nx + ii];
                if (v > back) {
                    cx += ii * (v - back);
                    cy += jj * (v - back);
                    tot += v - back;
                }
            }
        cx /= tot;
        cy /= tot;
        ocx = cx;
        ocy = cy;
    }
    *xc = cx;
    *yc = cy;
    free(m);
}

/* measure_FWHM (src/psf/psf.c:373-440), rings of width step; the last ring
 * is not tested (the reference reads past its arrays there). */
OR_EXPORT double or_measure_fwhm(const real_t *img, long nx, long ny, double xc, double yc, double step, long nb)
{
    double *dist = (double *)calloc((size_t)nb, sizeof(double)), *mean = (double *)calloc((size_t)nb, sizeof(double));
    long *cnt = (long *)calloc((size_t)nb, sizeof(long));
    for (long jj = 0; jj < ny; jj++)
        for (long ii = 0; ii < nx; ii++) {
            const double d = sqrt((ii - xc) * (ii - xc) + (jj - yc) * (jj - yc));
            const long i = (long)((long)d / step);
            if (i < nb) { dist[i] += d; mean[i] += img[jj * nx + ii]; cnt[i]++; }
        }
    for (long i = 0; i < nb; i++) { dist[i] /= cnt[i]; mean[i] /= cnt[i]; }
    double F = 0.0;
    for (long i = 0; i + 1 < nb; i++)
        if (mean[i + 1] < mean[0] / 2 && mean[i] > mean[0] / 2)
            F = 2.0 * dist[i] + (dist[i + 1] - dist[i]) * (mean[i] - mean[0] / 2) / (mean[i] - mean[i + 1]);
    free(dist);
    free(mean);
    free(cnt);
    return F;
}

/* measure_enc_NRJ (src/psf/psf.c:256-305). */
OR_EXPORT double or_measure_enc_nrj(const real_t *img, long nx, long ny, double xc, double yc, double fraction)
{
    const long asz = (long)(sqrt(2) * nx);
    double *tot = (double *)calloc((size_t)asz, sizeof(double)), all = 0.0, sum = 0.0;
    for (long jj = 0; jj < ny; jj++)
        for (long ii = 0; ii < nx; ii++) {
            const long idx = (long)(float)sqrt((ii - xc) * (ii - xc) + (jj - yc) * (jj - yc));
            if (idx < asz) tot[idx] += img[jj * nx + ii];
        }
    for (long i = 0; i < asz; i++) all += tot[i];
    all *= fraction;
    long ii = 0;
    while (sum < all && ii < asz) sum += tot[ii++];
    const double v = (ii - 2) + (all - (sum - tot[ii - 1])) / tot[ii - 1];
    free(tot);
    return v;
}
