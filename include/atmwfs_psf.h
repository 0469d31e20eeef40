/* atmwfs_psf.h -- the PSF consumers that follow the wavefront series:
 * exposure PSFs of a series (measure_wavefront_series_expoframes,
 * src/AtmosphericTurbulence/AtmosphericTurbulence.c:6592-6771) and the
 * chromatic PSF of a pupil (PSF_makeChromatPSF, src/psf/psf.c:54-136),
 * with the image measures the exposure loop prints (gauss_filter,
 * src/image_filter/image_filter.c:410-555; center_PSF, measure_FWHM,
 * measure_enc_NRJ, src/psf/psf.c:256-305, 373-440, 442-530).
 *
 * The transforms run on the GPU (one CTA per row group, rows and columns of
 * the zero-padded field, |F|^2 accumulated in registers across the frames
 * of a batch); the measures run on the host once per exposure.
 *
 * Sizes: the exposure field is 2W x 2W for W x W frames, W a power of two
 * in 32..1024; the chromatic PSF works on n x n with n a power of two in
 * 64..2048.  Every entry point returns an atmwfs_status.
 */
#ifndef ATMWFS_PSF_H
#define ATMWFS_PSF_H

#include "atmwfs.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Device accumulation into an exposure accumulator acc (2W x 2W floats):
 * acc += sum over the nframes frames of |FFT(pad(amp e^{i pha}))|^2, the
 * W x W frame placed at offset W/2 of the zero field
 * (AtmosphericTurbulence.c:6700-6735).  Frame f reads amp + f * amp_fstride
 * (amp_fstride 0: one pupil amplitude for every frame, the reference's ST_pa
 * branch) and pha + f * W * W.  Frames are summed in their order.  The
 * accumulator is kept transposed and uncentred (acc[kx][ky] = |F[ky][kx]|^2)
 * so that the updates are coalesced: zero it to start an exposure, and read
 * the reference's image (row-major, centred by permut()) with
 * atmwfs_psf_expo_image_dev.  All pointers are device memory; the calls are
 * asynchronous on stream. */
atmwfs_status atmwfs_psf_expo_accumulate_dev(const float* amp, long amp_fstride, const float* pha, long W,
                                             long nframes, float* acc, void* stream);
atmwfs_status atmwfs_psf_expo_image_dev(const float* acc, long W, float* img, void* stream);
/* The inverse: an exposure image back into the accumulator layout. */
atmwfs_status atmwfs_psf_expo_load_dev(const float* img, long W, float* acc, void* stream);

/* The same accumulation on host buffers (amp: nframes frames, or one when
 * amp_fstride is 0; pha: nframes frames; psf: the 2W x 2W centred image,
 * accumulated into). */
atmwfs_status atmwfs_psf_expo_accumulate(const float* amp, long amp_fstride, const float* pha, long W, long nframes,
                                         float* psf);

/* PSF_makeChromatPSF (psf.c:54-136): out (n x n, host, zeroed first) =
 * sum over nbstep log-spaced coefficients c from coeff1 to coeff2 of
 * m(c) / c^2 * bilinear zoom by c about n/2 of |FFT(amp e^{i c pha})|^2,
 * centred; m(c) is the reference's apodisation weight. */
atmwfs_status atmwfs_chromat_psf(const float* amp, const float* pha, long n, float coeff1, float coeff2, long nbstep,
                                 float apo_coeff, float* out);

/* The exposure measures (psf.c, image_filter.c) on a host n x n image, as
 * the exposure loop applies them: gauss_filter(psf, sigma 3, size 10),
 * center_PSF(filtered, n/2), measure_FWHM(filtered, centre, step 1, n/2
 * steps), measure_enc_NRJ(psf, centre, 0.5).  Outputs in pixels; any may
 * be NULL. */
atmwfs_status atmwfs_psf_measure(const float* psf, long n, double* fwhm_pix, double* ee50_pix, double* xcenter,
                                 double* ycenter);

/* Building blocks of the measures (single images, float as the reference). */
atmwfs_status atmwfs_gauss_filter(const float* in, long nx, long ny, float sigma, int filter_size, float* out);
atmwfs_status atmwfs_center_psf(const float* img, long nx, long ny, double* xcenter, double* ycenter);
atmwfs_status atmwfs_measure_fwhm(const float* img, long nx, long ny, float xcenter, float ycenter, float step,
                                  long nb_step, float* fwhm);
atmwfs_status atmwfs_measure_enc_nrj(const float* img, long nx, long ny, float xcenter, float ycenter, float fraction,
                                     float* radius);

/* measure_wavefront_series_expoframes(etime, outfile): reads the
 * configuration file conf (WFsim.conf keywords), the science cubes
 * <SWF_FILE_PREFIX>%08ld.%09ld.pha.fits (and .amp.fits when amplitude_on)
 * of every time span under the reference's fixed 1.65 um name, accumulates
 * one PSF per exposure of etime seconds on the GPU, writes PSF%04ld.fits per
 * exposure and the final partial exposure as "PSF", and writes one line
 * per exposure to outfile: exposure index, FWHM (arcsec), 2 x EE50 radius
 * (arcsec), centre x, centre y.  pupil (pupil_n x pupil_n) replaces the
 * reference's ST_pa image; NULL reads PUPIL_AMPL_FILE of the configuration.
 * The frames must have the pupil's size.  amplitude_on selects the
 * amplitude cubes instead of the pupil (the reference leaves this variable
 * uninitialised).  final_fwhm (may be NULL) receives the FWHM of the last,
 * partial exposure about the image centre, in arcsec. */
atmwfs_status atmwfs_expoframes(const char* conf, float etime, const char* outfile, const float* pupil, long pupil_n,
                                int amplitude_on, double* final_fwhm);

#ifdef __cplusplus
}
#endif

#endif
