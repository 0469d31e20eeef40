// host_psf.cpp -- host side of the PSF consumers: the image measures the
// reference's exposure loop prints (gauss_filter, center_PSF, measure_FWHM,
// measure_enc_NRJ) with the reference's float and double types, and the
// exposure driver measure_wavefront_series_expoframes
// (src/AtmosphericTurbulence/AtmosphericTurbulence.c:6592-6771) on top of
// the GPU accumulation of psf.cu.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "atmwfs.h"
#include "atmwfs_mkwfs.h"
#include "atmwfs_psf.h"

namespace atmwfs {
void set_error_message(const char* msg);
}

namespace {

atmwfs_status err(atmwfs_status s, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    atmwfs::set_error_message(buf);
    return s;
}

#define PSF_TRY(x)                                     \
    do {                                               \
        const atmwfs_status s_ = (x);                  \
        if (s_ != ATMWFS_OK) return s_;                \
    } while (0)

constexpr double kPI = 3.14159265358979323846264338328;

// arith_image_median of a float image (COREMOD_arith.c:1207 ->
// arith_image_percentile :1150-1161): the reference's float branch copies the
// image but does not sort the copy, so its "median" is the pixel at index
// (long)(0.5 n) -- reproduced, since it sets center_PSF's background level.
double image_median(const float* a, long n) { return (double)a[(long)(0.5 * n)]; }

// median_filter(in, out, 1) (image_filter.c:100-140): 3 x 3 medians of the
// interior, border pixels copied.  (The reference also writes the debug
// files mf_in.fits and mf_out.fits; they are not written here.)
void median3(const float* in, long nx, long ny, float* out)
{
    memcpy(out, in, sizeof(float) * nx * ny);
    float w[9];
    for (long jj = 1; jj < ny - 1; jj++)
        for (long ii = 1; ii < nx - 1; ii++) {
            int k = 0;
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) w[k++] = in[(jj - 1 + j) * nx + (ii - 1 + i)];
            std::nth_element(w, w + 4, w + 9);
            out[jj * nx + ii] = w[4];
        }
}

}  // namespace

extern "C" {

// gauss_filter (image_filter.c:410-555), one 2-D image: separable Gaussian
// of 2 fs + 1 taps, exp(-d^2 / sigma^2) normalised in float; rows then
// columns; border outputs renormalised by the taps that fall inside.
atmwfs_status atmwfs_gauss_filter(const float* in, long nx, long ny, float sigma, int filter_size, float* out)
{
    if (!in || !out || nx < 4 || ny < 4) return err(ATMWFS_ERR_INVALID, "gauss_filter: bad image");
    long fs = filter_size;
    if (fs > nx / 2 - 1) fs = nx / 2 - 1;
    if (fs > ny / 2 - 1) fs = ny / 2 - 1;
    const long K = 2 * fs + 1;
    std::vector<float> a(K);
    float sum = 0.0f;
    for (long i = 0; i < K; i++) {
        const float e = (float)(-((i - fs) * (i - fs))) / sigma / sigma;
        a[i] = (float)exp((double)e);
        sum += a[i];
    }
    for (long i = 0; i < K; i++) a[i] /= sum;
    std::vector<float> tmp((size_t)nx * ny, 0.0f);
    std::fill(out, out + nx * ny, 0.0f);
    for (long jj = 0; jj < ny; jj++) {
        const float* r = in + jj * nx;
        float* t = tmp.data() + jj * nx;
        for (long ii = 0; ii < nx - K; ii++)
            for (long i = 0; i < K; i++) t[ii + fs] += a[i] * r[ii + i];
        for (long ii = 0; ii < fs; ii++) {
            double tot = 0.0;
            for (long i = fs - ii; i < K; i++) {
                t[ii] += a[i] * r[ii - fs + i];
                tot += a[i];
            }
            t[ii] = (float)(t[ii] / tot);
        }
        for (long ii = nx - fs - 1; ii < nx; ii++) {
            double tot = 0.0;
            for (long i = 0; i < K - (ii - nx + fs + 1); i++) {
                t[ii] += a[i] * r[ii - fs + i];
                tot += a[i];
            }
            t[ii] = (float)(t[ii] / tot);
        }
    }
    for (long ii = 0; ii < nx; ii++) {
        for (long jj = 0; jj < ny - K; jj++)
            for (long j = 0; j < K; j++) out[(jj + fs) * nx + ii] += a[j] * tmp[(jj + j) * nx + ii];
        for (long jj = 0; jj < fs; jj++) {
            double tot = 0.0;
            long jmax = K;
            if (jj - fs + jmax > ny) jmax = ny - jj + fs;
            for (long j = fs - jj; j < jmax; j++) {
                out[jj * nx + ii] += a[j] * tmp[(jj - fs + j) * nx + ii];
                tot += a[j];
            }
            out[jj * nx + ii] = (float)(out[jj * nx + ii] / tot);
        }
        for (long jj = ny - fs - 1; jj < ny; jj++) {
            double tot = 0.0;
            for (long j = 0; j < K - (jj - ny + fs + 1); j++) {
                out[jj * nx + ii] += a[j] * tmp[(jj - fs + j) * nx + ii];
                tot += a[j];
            }
            out[jj * nx + ii] = (float)(out[jj * nx + ii] / tot);
        }
    }
    return ATMWFS_OK;
}

// center_PSF (psf.c:442-530): background = image_median above; a 3 x 3
// median-filtered copy; ten barycentres of the pixels above the background
// in a shrinking box around the previous centre, starting at the image
// centre.
atmwfs_status atmwfs_center_psf(const float* img, long nx, long ny, double* xcenter, double* ycenter)
{
    if (!img || nx < 3 || ny < 3) return err(ATMWFS_ERR_INVALID, "center_PSF: bad image");
    const int nbiter = 10;
    const double back = image_median(img, nx * ny);
    std::vector<float> m((size_t)nx * ny);
    median3(img, nx, ny, m.data());
    double cx = (double)(nx / 2), cy = (double)(ny / 2);
    double ocx = cx, ocy = cy;
    for (int k = 0; k < nbiter; k++) {
        const long n3 = (long)(1.0 * nx / 2 / (1.0 + (0.1 * nx / 2 * k / (4 * nbiter))));
        long is = (long)(0.5 + ocx - n3), ie = (long)(0.5 + ocx + n3);
        long js = (long)(0.5 + ocy - n3), je = (long)(0.5 + ocy + n3);
        if (is < 0) is = 0;
        if (ie > nx - 1) ie = nx - 1;
        if (js < 0) js = 0;
        if (je > ny - 1) je = ny - 1;
        cx = 0.0;
        cy = 0.0;
        double tot = 0.0;
        for (long jj = js; jj < je; jj++)
            for (long ii = is; ii < ie; ii++) {
                const float v = m[jj * nx + ii];
                if (v > back) {
                    cx += 1.0 * ii * (v - 1.0 * back);
                    cy += 1.0 * jj * (v - 1.0 * back);
                    tot += v - 1.0 * back;
                }
            }
        cx /= tot;
        cy /= tot;
        ocx = cx;
        ocy = cy;
    }
    if (xcenter) *xcenter = cx;
    if (ycenter) *ycenter = cy;
    return ATMWFS_OK;
}

// measure_FWHM (psf.c:373-440): radial mean profile in rings of width step;
// the last ring i whose mean is above half the central ring's mean while
// ring i + 1 is below gives 2 dist_i + (dist_{i+1} - dist_i)(mean_i - m0/2) /
// (mean_i - mean_{i+1}) (the interpolation term is not doubled, as in the
// reference).  The reference also reads ring nb_step, past its arrays; the
// last ring is not tested here.
atmwfs_status atmwfs_measure_fwhm(const float* img, long nx, long ny, float xcenter, float ycenter, float step,
                                  long nb_step, float* fwhm)
{
    if (!img || nb_step < 2 || !(step > 0)) return err(ATMWFS_ERR_INVALID, "measure_FWHM: bad arguments");
    std::vector<float> dist(nb_step, 0.0f), mean(nb_step, 0.0f);
    std::vector<long> counts(nb_step, 0);
    for (long jj = 0; jj < ny; jj++)
        for (long ii = 0; ii < nx; ii++) {
            const float d = (float)sqrt((1.0 * ii - xcenter) * (1.0 * ii - xcenter) +
                                        (1.0 * jj - ycenter) * (1.0 * jj - ycenter));
            const long i = (long)((float)(long)d / step);
            if (i < nb_step) {
                dist[i] += d;
                mean[i] += img[jj * nx + ii];
                counts[i] += 1;
            }
        }
    for (long i = 0; i < nb_step; i++) {
        dist[i] /= (float)counts[i];
        mean[i] /= (float)counts[i];
    }
    float F = 0.0f;
    for (long i = 0; i + 1 < nb_step; i++)
        if ((mean[i + 1] < mean[0] / 2) && (mean[i] > mean[0] / 2))
            F = (float)(2.0 * dist[i] + (dist[i + 1] - dist[i]) * (mean[i] - mean[0] / 2) / (mean[i] - mean[i + 1]));
    if (fwhm) *fwhm = F;
    return ATMWFS_OK;
}

// measure_enc_NRJ (psf.c:256-305): ring sums of width 1 out to sqrt(2) nx;
// the radius where the cumulative sum reaches `fraction` of the total, with
// the reference's offset of (ii - 2) + the fractional part of the last ring.
atmwfs_status atmwfs_measure_enc_nrj(const float* img, long nx, long ny, float xcenter, float ycenter, float fraction,
                                     float* radius)
{
    if (!img || nx < 2) return err(ATMWFS_ERR_INVALID, "measure_enc_NRJ: bad image");
    const long asz = (long)(sqrt(2) * nx);
    std::vector<float> total(asz, 0.0f);
    for (long jj = 0; jj < ny; jj++)
        for (long ii = 0; ii < nx; ii++) {
            const float d = (float)sqrt((1.0 * ii - xcenter) * (1.0 * ii - xcenter) +
                                        (1.0 * jj - ycenter) * (1.0 * jj - ycenter));
            const long index = (long)d;
            if (index < asz) total[index] += img[jj * nx + ii];
        }
    float sum_all = 0.0f;
    for (long i = 0; i < asz; i++) sum_all += total[i];
    float sum = 0.0f;
    sum_all *= fraction;
    long ii = 0;
    while (sum < sum_all && ii < asz) {      // the reference has no bound on ii
        sum += total[ii];
        ii++;
    }
    if (ii < 1) return err(ATMWFS_ERR_INVALID, "measure_enc_NRJ: empty image");
    const float v = (float)(1.0 * (ii - 2) + (sum_all - (sum - total[ii - 1])) / (total[ii - 1]));
    if (radius) *radius = v;
    return ATMWFS_OK;
}

atmwfs_status atmwfs_psf_measure(const float* psf, long n, double* fwhm_pix, double* ee50_pix, double* xcenter,
                                 double* ycenter)
{
    if (!psf || n < 8) return err(ATMWFS_ERR_INVALID, "psf_measure: bad image");
    std::vector<float> g((size_t)n * n);
    PSF_TRY(atmwfs_gauss_filter(psf, n, n, 3.0f, 10, g.data()));
    double xc = 0.0, yc = 0.0;
    PSF_TRY(atmwfs_center_psf(g.data(), n, n, &xc, &yc));
    float fw = 0.0f, ee = 0.0f;
    PSF_TRY(atmwfs_measure_fwhm(g.data(), n, n, (float)xc, (float)yc, 1.0f, n / 2, &fw));
    PSF_TRY(atmwfs_measure_enc_nrj(psf, n, n, (float)xc, (float)yc, 0.5f, &ee));
    if (fwhm_pix) *fwhm_pix = fw;
    if (ee50_pix) *ee50_pix = ee;
    if (xcenter) *xcenter = xc;
    if (ycenter) *ycenter = yc;
    return ATMWFS_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// the exposure driver
// ---------------------------------------------------------------------------
namespace {

struct DevBuf {
    void* p = nullptr;
    ~DevBuf() { if (p) cudaFree(p); }
    atmwfs_status alloc(size_t bytes)
    {
        if (p) cudaFree(p);
        p = nullptr;
        if (cudaMalloc(&p, bytes) != cudaSuccess) return err(ATMWFS_ERR_NOMEM, "cudaMalloc of %zu bytes failed", bytes);
        return ATMWFS_OK;
    }
    float* f() const { return (float*)p; }
};

atmwfs_status cuda_ok(cudaError_t e, const char* what)
{
    return e == cudaSuccess ? ATMWFS_OK : err(ATMWFS_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

std::string cube(const char* prefix, long tspan, long lam_pm, const char* q)
{
    char buf[512];
    snprintf(buf, sizeof buf, "%s%08ld.%09ld.%s.fits", prefix, tspan, lam_pm, q);
    return buf;
}

atmwfs_status read_cube(const std::string& name, long W, long nframes, std::vector<float>& out)
{
    int naxis = 0;
    long ax[3] = {1, 1, 1};
    out.resize((size_t)W * W * std::max(nframes, 1L));
    PSF_TRY(atmwfs_fits_read_f32(name.c_str(), nullptr, 0, &naxis, ax));   // sizes only
    if (ax[0] != W || ax[1] != W || ax[2] < nframes)
        return err(ATMWFS_ERR_INVALID, "%s: %ld x %ld x %ld, expected %ld x %ld x >= %ld frames", name.c_str(), ax[0],
                   ax[1], ax[2], W, W, nframes);
    std::vector<float> all((size_t)W * W * ax[2]);
    PSF_TRY(atmwfs_fits_read_f32(name.c_str(), all.data(), (long)all.size(), &naxis, ax));
    std::copy(all.begin(), all.begin() + (size_t)W * W * nframes, out.begin());
    return ATMWFS_OK;
}

}  // namespace

extern "C" atmwfs_status atmwfs_expoframes(const char* conf_file, float etime, const char* outfile, const float* pupil,
                                           long pupil_n, int amplitude_on, double* final_fwhm)
{
    if (!conf_file || !outfile) return err(ATMWFS_ERR_INVALID, "null argument");
    atmwfs_conf cf;
    PSF_TRY(atmwfs_conf_load(conf_file, &cf));
    // pupil amplitude: the caller's, or PUPIL_AMPL_FILE (ReadConf :1410-1415)
    std::vector<float> pup;
    long W = pupil_n;
    if (pupil) {
        pup.assign(pupil, pupil + W * W);
    } else {
        char path[512];
        if (atmwfs_conf_exists(conf_file, "PUPIL_AMPL_FILE") != 1 ||
            atmwfs_conf_read(conf_file, "PUPIL_AMPL_FILE", path, sizeof path) != 1)
            return err(ATMWFS_ERR_INVALID, "pupil amplitude map not loaded (no PUPIL_AMPL_FILE)");
        int naxis = 0;
        long ax[3] = {1, 1, 1};
        PSF_TRY(atmwfs_fits_read_f32(path, nullptr, 0, &naxis, ax));
        if (naxis != 2 || ax[0] != ax[1]) return err(ATMWFS_ERR_INVALID, "%s: not a square 2-D image", path);
        W = ax[0];
        pup.resize((size_t)W * W);
        PSF_TRY(atmwfs_fits_read_f32(path, pup.data(), (long)pup.size(), &naxis, ax));
    }
    if (W < 32 || W > 1024 || (W & (W - 1)))
        return err(ATMWFS_ERR_INVALID, "frame size %ld unsupported (power of two 32..1024)", W);
    const long N = 2 * W;
    // FOCAL_SCALE (:6632) with the reference's float / double mix; zoom 2
    const float focal_scale = (float)((double)(cf.lambda / (float)cf.wfsize / cf.pupil_scale) / kPI * 180.0 * 3600.0 * 2);
    const long nbframes = (long)(cf.time_span / cf.wftime_step);
    const long lam_pm = (long)(1.0e12 * 1.65e-6 + 0.5);   // the reference's fixed SLAMBDA (:6625)

    FILE* fp = fopen(outfile, "w");
    if (!fp) return err(ATMWFS_ERR_IO, "cannot create file %s", outfile);
    fclose(fp);

    DevBuf dpup, dpha, damp, dacc, dimg;
    PSF_TRY(dpup.alloc(sizeof(float) * W * W));
    PSF_TRY(dacc.alloc(sizeof(float) * N * N));
    PSF_TRY(dimg.alloc(sizeof(float) * N * N));
    PSF_TRY(dpha.alloc(sizeof(float) * W * W * std::max(nbframes, 1L)));
    if (amplitude_on == 1) PSF_TRY(damp.alloc(sizeof(float) * W * W * std::max(nbframes, 1L)));
    PSF_TRY(cuda_ok(cudaMemcpy(dpup.p, pup.data(), sizeof(float) * W * W, cudaMemcpyHostToDevice), "copy"));
    PSF_TRY(cuda_ok(cudaMemset(dacc.p, 0, sizeof(float) * N * N), "memset"));
    std::vector<float> img((size_t)N * N), pha, amp;

    float etime_left = etime;
    long frame_number = 0;
    for (long tspan = 0; tspan < cf.nb_tspan; tspan++) {
        PSF_TRY(read_cube(cube(cf.swf_file_prefix, tspan, lam_pm, "pha"), W, nbframes, pha));
        PSF_TRY(cuda_ok(cudaMemcpy(dpha.p, pha.data(), sizeof(float) * W * W * nbframes, cudaMemcpyHostToDevice), "copy"));
        if (amplitude_on == 1) {
            PSF_TRY(read_cube(cube(cf.swf_file_prefix, tspan, lam_pm, "amp"), W, nbframes, amp));
            PSF_TRY(cuda_ok(cudaMemcpy(damp.p, amp.data(), sizeof(float) * W * W * nbframes, cudaMemcpyHostToDevice), "copy"));
        }
        long f0 = 0;    // first frame not yet accumulated
        for (long frame = 0; frame < nbframes; frame++) {
            etime_left -= cf.wftime_step;
            if (etime_left < 0 || frame == nbframes - 1) {
                // frames f0..frame join the exposure in one launch sequence
                const float* a = amplitude_on == 1 ? damp.f() + f0 * W * W : dpup.f();
                PSF_TRY(atmwfs_psf_expo_accumulate_dev(a, amplitude_on == 1 ? W * W : 0, dpha.f() + f0 * W * W, W,
                                                       frame - f0 + 1, dacc.f(), nullptr));
                f0 = frame + 1;
            }
            if (etime_left < 0) {
                PSF_TRY(atmwfs_psf_expo_image_dev(dacc.f(), W, dimg.f(), nullptr));
                PSF_TRY(cuda_ok(cudaMemcpy(img.data(), dimg.p, sizeof(float) * N * N, cudaMemcpyDeviceToHost), "copy"));
                char name[64];
                snprintf(name, sizeof name, "!PSF%04ld.fits", frame_number);
                const long ax[2] = {N, N};
                PSF_TRY(atmwfs_fits_write(name, img.data(), -32, 2, ax));
                double fw = 0, ee = 0, xc = 0, yc = 0;
                PSF_TRY(atmwfs_psf_measure(img.data(), N, &fw, &ee, &xc, &yc));
                fp = fopen(outfile, "a");
                if (!fp) return err(ATMWFS_ERR_IO, "cannot open file %s", outfile);
                fprintf(fp, "%ld %f %f %f %f\n", frame_number, (double)(focal_scale * (float)fw),
                        2.0 * focal_scale * (float)ee, xc, yc);
                fclose(fp);
                PSF_TRY(cuda_ok(cudaMemset(dacc.p, 0, sizeof(float) * N * N), "memset"));
                etime_left = etime;
                frame_number++;
            }
        }
    }
    // the last, partial exposure (:6760-6766)
    PSF_TRY(atmwfs_psf_expo_image_dev(dacc.f(), W, dimg.f(), nullptr));
    PSF_TRY(cuda_ok(cudaMemcpy(img.data(), dimg.p, sizeof(float) * N * N, cudaMemcpyDeviceToHost), "copy"));
    const long ax[2] = {N, N};
    PSF_TRY(atmwfs_fits_write("!PSF", img.data(), -32, 2, ax));
    float fw = 0.0f;
    PSF_TRY(atmwfs_measure_fwhm(img.data(), N, N, (float)(1.0 * N / 2), (float)(1.0 * N / 2), 1.0f, N / 2, &fw));
    if (final_fwhm) *final_fwhm = (double)(focal_scale * fw);
    return ATMWFS_OK;
}
