/*
 * atmwfs_mkwfs.h -- host side of the wavefront-series command: the
 * configuration file, the turbulence profile, FITS cubes, shared-memory
 * images, and the driver that replaces the reference's
 * make_AtmosphericTurbulence_wavefront_series()
 * (src/AtmosphericTurbulence/AtmosphericTurbulence.c:1433-4455) on top of
 * the GPU engine of atmwfs.h.
 *
 * Everything here runs on the host; only atmwfs_mkwfs() touches the GPU.
 * Every function returns a status code (never exits), and the message of
 * the last failure on the calling thread is atmwfs_last_error().
 */
#ifndef ATMWFS_MKWFS_H
#define ATMWFS_MKWFS_H

#include "atmwfs.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ */
/* Configuration file                                                  */
/* ------------------------------------------------------------------ */

/* Replaces read_config_parameter (src/COREMOD_tools/COREMOD_tools.c:629-666).
 * Each line is split into its first two whitespace-separated tokens; the
 * last line whose first token equals `keyword` wins.  A line with fewer
 * tokens keeps the tokens of the line before it (the reference's sscanf
 * leaves them unchanged), so a bare keyword line repeats the previous
 * line's value.  Absent keyword: `content` = "-" and the return is 0;
 * found: 1.  Unreadable file: -1 (the reference exits).  `content` holds
 * at most cap-1 characters. */
int atmwfs_conf_read(const char* conf_file, const char* keyword, char* content, long cap);

/* Replaces read_config_parameter_exists (COREMOD_tools.c:596-626): 1 if a
 * line's first token equals `keyword`, 0 if not, -1 if unreadable. */
int atmwfs_conf_exists(const char* conf_file, const char* keyword);

/* The CONF_* globals of AtmosphericTurbulence.c:104-160, with their C
 * types, plus SITE_ALT of the atmosphere model (AtmosphereModel.c reads it
 * into a float).  Missing keywords read as "-", i.e. 0, exactly as in the
 * reference, except where it guards the read with an existence test
 * (WFOUTPUT = 1, SHM_OUTPUT = 0, SHM_SOUTPUT = 0, SKIP_EXISTING = 0). */
typedef struct atmwfs_conf {
    float lambda;                   /* TURBULENCE_REF_WAVEL [m] (file value in um x 1e-6) */
    float seeing;                   /* TURBULENCE_SEEING [arcsec] */
    char prof_file[200];            /* TURBULENCE_PROF_FILE */
    float zangle;                   /* ZENITH_ANGLE [rad] */
    float source_xpos, source_ypos; /* SOURCE_XPOS / SOURCE_YPOS [rad] */
    int wfoutput;                   /* WFOUTPUT */
    char wf_file_prefix[200];       /* WF_FILE_PREFIX */
    int shm_output;                 /* SHM_OUTPUT */
    int make_swavefront;            /* MAKE_SWAVEFRONT */
    int swf_write2disk;             /* SWF_WRITE2DISK */
    char swf_file_prefix[200];      /* SWF_FILE_PREFIX */
    int shm_soutput;                /* SHM_SOUTPUT */
    char shm_sprefix[100];          /* SHM_SPREFIX */
    int shm_soutputm;               /* SHM_SOUTPUTM: 0 rad, 1 m, 2 um */
    float pupil_scale;              /* PUPIL_SCALE [m/pixel] */
    long wfsize;                    /* WFsize (output crop) */
    int realtime;                   /* REALTIME */
    double realtime_factor;         /* REALTIMEFACTOR */
    float wftime_step;              /* WFTIME_STEP [s] */
    float time_span;                /* TIME_SPAN [s] */
    long nb_tspan;                  /* NB_TSPAN */
    long simtdelay;                 /* SIMTDELAY [us] */
    int waitforsem;                 /* WAITFORSEM */
    char waitsemimname[100];        /* WAITSEMIMNAME */
    int skip_existing;              /* SKIP_EXISTING (keyword present) */
    long wf_raw_size;               /* WF_RAW_SIZE (propagation grid) */
    long master_size;               /* MASTER_SIZE */
    int wavefront_amplitude;        /* WAVEFRONT_AMPLITUDE */
    int fresnel_propagation;        /* FRESNEL_PROPAGATION (0 unless amplitude) */
    float fresnel_propagation_bin;  /* FRESNEL_PROPAGATION_BIN [m] */
    float site_alt;                 /* SITE_ALT [m] */
} atmwfs_conf;

/* Replaces AtmosphericTurbulence_ReadConf (AtmosphericTurbulence.c:1233-1427)
 * and the SITE_ALT read of AtmosphereModel_Create_from_CONF.  The pupil
 * amplitude/phase files it also loads are not used by the series. */
atmwfs_status atmwfs_conf_load(const char* conf_file, atmwfs_conf* conf);

/* ------------------------------------------------------------------ */
/* Turbulence profile                                                  */
/* ------------------------------------------------------------------ */

/* Replaces the profile reader of AtmosphericTurbulence.c:1940-2015.  A line
 * is a layer when its first token starts with a digit; its first eight
 * numbers are altitude [m], Cn2 (relative), wind speed [m/s], direction
 * [rad], outer scale [m], inner scale [m], wind sigma [m/s], wind outer
 * scale [m].  As in the reference, a blank line keeps the previous line's
 * first token and values (so a blank line after a layer line repeats that
 * layer), and a line with fewer than eight numbers keeps the missing ones
 * from the line before.  Layers at or below site_alt - 0.1 m are refused
 * (ATMWFS_ERR_INVALID): the reference leaves them uninitialised.  Writes
 * min(n, cap) rows of 8 doubles to `layers` and n to *nlayers; Cn2 is
 * returned as read (atmwfs_create normalises it). */
atmwfs_status atmwfs_profile_read(const char* path, double site_alt, double* layers, long cap, long* nlayers);

/* Replaces AtmosphericTurbulence_makeHV_CN2prof (the mkHVturbprof command,
 * AtmosphericTurbulence.c:7841-7940): a Hufnagel-Valley profile of
 * `nlayers` layers from the site altitude to 30 km whose ground-layer
 * strength is tuned so that r0 at 550 nm is r0 [m], for wind speed wspeed
 * [m/s].  Writes `outfile` in the profile format above and, as the
 * reference does, the seeing [arcsec] to conf_turb.txt in the current
 * directory (also returned in *seeing if not NULL). */
atmwfs_status atmwfs_make_hv_profile(double wspeed, double r0, double sitealt, long nlayers, const char* outfile,
                                     double* seeing);

/* ------------------------------------------------------------------ */
/* FITS images                                                          */
/* ------------------------------------------------------------------ */

/* Primary-HDU FITS image with BITPIX -32 (float) or -64 (double), NAXIS 1-3,
 * naxes[0] varying fastest: the files of save_fl_fits / save_db_fits
 * (src/COREMOD_iofits/COREMOD_iofits.c:929-1060).  A leading '!' in `name`
 * overwrites an existing file (cfitsio's convention); without it an
 * existing file is an error. */
atmwfs_status atmwfs_fits_write(const char* name, const void* data, int bitpix, int naxis, const long* naxes);

/* Reads a primary-HDU image (BITPIX 8/16/32/64/-32/-64, BSCALE/BZERO
 * applied) into `out` as float.  naxes[0..2] receive the sizes (1 for
 * missing axes), *naxis the axis count.  At most `cap` values are stored;
 * ATMWFS_ERR_INVALID if the image holds more. */
atmwfs_status atmwfs_fits_read_f32(const char* name, float* out, long cap, int* naxis, long* naxes);

/* ------------------------------------------------------------------ */
/* Shared-memory images                                                */
/* ------------------------------------------------------------------ */

/* The stream image files of create_image_ID(..., shared = 1, NBkw = 0)
 * (src/COREMOD_memory/COREMOD_memory.c:1519-1730): /tmp/<name>.im.shm holds
 * an IMAGE_METADATA header (src/CLIcore.h:179-203, this platform's LP64
 * layout) followed by the pixels; the named semaphore <name>_semlog is
 * created as the reference does.  dtype 3 = float, 4 = double. */
typedef struct atmwfs_shm atmwfs_shm;
atmwfs_status atmwfs_shm_create(const char* name, long nx, long ny, int dtype, atmwfs_shm** out);

/* Copy one frame (nx*ny values of the image's type).  bump != 0 marks the
 * image as being written during the copy and increments cnt0 after it (the
 * science-wavelength stream, AtmosphericTurbulence.c:4283-4345); bump = 0
 * copies only (the reference-wavelength stream, :3478-3518). */
atmwfs_status atmwfs_shm_write(atmwfs_shm* shm, const void* frame, int bump);
void atmwfs_shm_close(atmwfs_shm* shm);

/* Wait on semaphore `index` of the stream image `name` (named semaphore
 * <name>_semNN), as COREMOD_MEMORY_image_set_semwait (COREMOD_memory.c:4246)
 * does for WAITFORSEM.  timeout_s > 0 bounds the wait (ATMWFS_ERR_TIMEOUT);
 * a missing semaphore is ATMWFS_ERR_INVALID (the reference prints an error
 * and continues). */
atmwfs_status atmwfs_shm_semwait(const char* name, long index, double timeout_s);

/* ------------------------------------------------------------------ */
/* The series command                                                  */
/* ------------------------------------------------------------------ */

/* Refractivity N = n - 1 of air at altitude alt [m] and vacuum wavelength
 * lambda [m]: the signature of the reference's AtmosphereModel_stdAtmModel_N
 * (src/AtmosphereModel/AtmosphereModel.c:3212, mode 0), float in and out. */
typedef float (*atmwfs_refractivity_fn)(float alt, float lambda, void* user);

typedef struct atmwfs_mkwfs_opts {
    /* Refractivity model for Scoeff (:2661-2663) and the refraction offsets
     * (:2159-2183).  NULL: a dry standard-air model (Ciddor 1996 with an
     * 8 km exponential density scale height), which differs from the
     * reference's atmosphere model by up to ~1 % of N near the ground. */
    atmwfs_refractivity_fn refractivity;
    void* refractivity_user;
    /* Per-layer overrides (length = number of layers, NULL = computed). */
    const double* scoeff;   /* science-wavelength phase multipliers */
    const double* roffset;  /* refraction offsets RoffsetS - Roffset [m] */
    /* Philox seed for master screens that have to be synthesised (the
     * reference seeds its generators from the clock). */
    unsigned long long seed;
    int verbose;            /* progress lines on stdout */
    /* Seconds a WAITFORSEM wait may take before the run stops with
     * ATMWFS_ERR_TIMEOUT; <= 0 waits without limit, as the reference. */
    double semwait_timeout;
    /* 1: every Fresnel hop propagates with lambda / n, n the air index of
     * the refractivity model at the middle of the hop (atmwfs_instance.hop_n);
     * 0 (default): the vacuum wavelength, as the reference (WFpropagate.c:91). */
    int fresnel_air_index;
} atmwfs_mkwfs_opts;

/* Replaces make_AtmosphericTurbulence_wavefront_series(slambdaum,
 * WFprecision) (AtmosphericTurbulence.c:1433): reads `conf_file` (NULL =
 * "WFsim.conf") and its profile, loads the master screens
 * t%03ld_%ld_{f,d}.fits of the current directory (synthesising and saving
 * missing ones), renormalises them, runs NB_TSPAN x NBFRAMES frames on the
 * GPU at TURBULENCE_REF_WAVEL and at slambda_um [um], and writes the cubes
 * <prefix>%08ld.%09ld.{pha,amp}.fits (time span, science wavelength in pm)
 * and the shared-memory streams the configuration asks for.  precision 1
 * reads/writes double files (the engine computes in float with FP64 range
 * reduction either way).  opts may be NULL. */
atmwfs_status atmwfs_mkwfs(const char* conf_file, float slambda_um, long precision, const atmwfs_mkwfs_opts* opts);

/* ------------------------------------------------------------------ */
/* Atmospheric refraction                                              */
/* ------------------------------------------------------------------ */

/* Absorption coefficient [1/m] of air at altitude alt [m] and wavelength
 * lambda [m]: the value the reference's AtmosphereModel_stdAtmModel_N
 * leaves in v_ABSCOEFF (AtmosphereModel.c:3210, 3293). */
typedef double (*atmwfs_absorption_fn)(float alt, float lambda, void* user);

/* Replaces AtmosphereModel_RefractionPath (AtmosphereModel.c:4215-4291):
 * traces a ray from the site altitude upward in 20 m steps over a
 * spherical Earth (R = 6371 km) with Snell's law between consecutive steps,
 * until 99 km, and iterates the launch angle (at most 20 times, until the
 * exit angle matches zangle to 1e-5 arcsec).  Returns the refraction
 * [arcsec] and the transmission of the last pass (absorption NULL: 1).
 * path_file (may be NULL) receives the reference's refractpath.txt lines
 * of the last pass.  N and K receive the same float arguments as the
 * reference's model calls.  A ray that has not reached 99 km after 10^6
 * steps is ATMWFS_ERR_INVALID. */
atmwfs_status atmwfs_refraction_path(double lambda, double zangle, double site_alt, atmwfs_refractivity_fn N,
                                     atmwfs_absorption_fn K, void* user, const char* path_file,
                                     double* refraction_arcsec, double* transmission);

/* The same for every (wavelength, zenith angle) pair on the GPU, one ray
 * per thread in FP64, from tabulated models: Ntab[i][k] and Ktab[i][k]
 * (Ktab may be NULL) are N and the absorption coefficient of wavelength i
 * at altitude k * dh, k < ntab, read with the reference's interpolation
 * (index (long)(alt / dh), float fraction clamped to [0, 1], the last
 * interval repeated above the table, as stdAtmModel_N reads its 10 m
 * density tables, AtmosphereModel.c:3240-3250).  Outputs
 * [nlambda][nzangle]; host buffers. */
atmwfs_status atmwfs_refraction_table(const double* lambdas, long nlambda, const double* zangles, long nzangle,
                                      double site_alt, const float* Ntab, const double* Ktab, long ntab, double dh,
                                      double* refraction_arcsec, double* transmission);

/* The same table model traced on the host, `threads` threads (<= 0: all
 * hardware threads): for hosts that keep the trace on the CPU, and the CPU
 * side of a comparison with the GPU form. */
atmwfs_status atmwfs_refraction_table_host(const double* lambdas, long nlambda, const double* zangles, long nzangle,
                                           double site_alt, const float* Ntab, const double* Ktab, long ntab, double dh,
                                           int threads, double* refraction_arcsec, double* transmission);

#ifdef __cplusplus
}
#endif

#endif /* ATMWFS_MKWFS_H */
