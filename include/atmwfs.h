/*
 * atmwfs.h -- C ABI of the GB300 wavefront-series engine (libatmwfs.so).
 *
 * Drop-in for the hot path of AtmosphericTurbulenceSimul's `mkwfs` command:
 * make_AtmosphericTurbulence_wavefront_series()
 * (src/AtmosphericTurbulence/AtmosphericTurbulence.c:1433-4455) and the
 * operators it calls.  Plain pointers and sizes only; every entry point
 * returns a status code instead of calling exit() as the reference does.
 *
 * Threading: a context is not re-entrant; use one context per host thread.
 * Images are row-major with x fastest, a[y*n + x], like the reference.
 * Complex images are interleaved (re, im) float pairs, like complex_float.
 */
#ifndef ATMWFS_H
#define ATMWFS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum atmwfs_status {
    ATMWFS_OK = 0,
    ATMWFS_ERR_INVALID = 1,   /* bad argument or unsupported size            */
    ATMWFS_ERR_NOMEM = 2,     /* host or device allocation failed            */
    ATMWFS_ERR_CUDA = 3,      /* CUDA runtime error (see atmwfs_last_error)  */
    ATMWFS_ERR_IO = 4,        /* file missing, short or malformed            */
    ATMWFS_ERR_TIMEOUT = 5,   /* a bounded wait expired (device or host)     */
    ATMWFS_ERR_STATE = 6,     /* call out of order (e.g. run before screens) */
    ATMWFS_ERR_NODEVICE = 7   /* no CUDA device                              */
} atmwfs_status;

/* Output mode of an instance. */
enum {
    ATMWFS_MODE_REF = 0,   /* reference-wavelength output: pha = atan2(U) + 2 pi round(sum/2 pi)
                              (AtmosphericTurbulence.c:3418-3476)                                   */
    ATMWFS_MODE_SCI = 1,   /* science output with the bin-relaxation unwrap (:3522-4260)          */
    ATMWFS_MODE_PHASE = 2  /* phase only (WAVEFRONT_AMPLITUDE = 0): pha = geometric phase sum     */
};

/* One (wavelength, direction, output mode) instance of the series. */
typedef struct atmwfs_instance {
    double lambda;          /* propagation wavelength in vacuum [m] (WFpropagate.c:91)             */
    int mode;               /* ATMWFS_MODE_*                                                        */
    float src_x, src_y;     /* source offset [rad] (SOURCE_XPOS / SOURCE_YPOS, :2187-2188)          */
    long wf_raw_size;       /* propagation grid N: power of two, 64..2048 (WF_RAW_SIZE)             */
    long wf_size;           /* output crop, <= wf_raw_size (WFsize)                                 */
    const float* scoeff;    /* [nlayers] phase multiplier (Scoeff, :2661-2663); NULL = 1            */
    const double* roffset;  /* [nlayers] refraction offset [m] added to y (:2163-2183); NULL = 0    */
    const double* hop_n;    /* [hops] optional refractive index of the air along each hop, in the
                               engine's hop order (top plane down, atmwfs_plane_info): the hop's
                               transfer function then uses lambda / n.  NULL = the vacuum lambda
                               of the reference's hops (WFpropagate.c:91, quirk of its :2672/:2685
                               calls: the air index enters only through Scoeff)               */
} atmwfs_instance;

/* Parsed configuration (the WFsim.conf keywords the path reads) and the
 * layer profile (TURBULENCE_PROF_FILE, in file order). */
typedef struct atmwfs_params {
    int nlayers;
    const double* alt;        /* [m]                                        */
    const double* cn2;        /* relative Cn2 (normalised to 1 internally)  */
    const double* speed;      /* [m/s]                                      */
    const double* dir;        /* [rad]                                      */
    double fresnel_bin;       /* FRESNEL_PROPAGATION_BIN [m]                */
    float zangle;             /* ZENITH_ANGLE [rad]                         */
    float pupil_scale;        /* PUPIL_SCALE [m/pixel]                      */
    float time_step;          /* WFTIME_STEP [s]                            */
    long master_size;         /* MASTER_SIZE (power of two, >= 64)          */
    int amplitude;            /* WAVEFRONT_AMPLITUDE                        */
    int fresnel;              /* FRESNEL_PROPAGATION                        */
    int realtime;             /* REALTIME                                   */
    double realtime_factor;   /* REALTIMEFACTOR                             */
    int ninst;
    const atmwfs_instance* inst;
    int ring;                 /* output frames kept on the device per instance (>= 1) */
    int fft_fp16;             /* 1: FFT stages of the propagation in FP16 with per-stage power-of-two
                                 scaling (precision study); 0: FP32                               */
} atmwfs_params;

typedef struct atmwfs_ctx atmwfs_ctx;

/* Where atmwfs_run() delivers frames: buffers of nslots *
 * atmwfs_frame_floats() floats (NULL = not copied), in host memory (pinned
 * buffers keep the copies asynchronous) or device memory.  Step s of the
 * call goes to slot s % nslots (nslots <= 0 means nslots = nsteps).  The
 * frames of one step are contiguous; instance i starts at
 * atmwfs_frame_offset(i). */
typedef struct atmwfs_sink {
    float* pha;
    float* amp;
    long nslots;
} atmwfs_sink;

/* Context life cycle.  Replaces the setup of make_AtmosphericTurbulence_
 * wavefront_series (:1654-2560): super-layer grouping (:2067-2147), start
 * positions and wind (:2152-2197), transfer tables, device buffers. */
atmwfs_status atmwfs_create(const atmwfs_params* p, atmwfs_ctx** out);
void atmwfs_destroy(atmwfs_ctx* ctx);

/* Master screen of layer `layer` (M x M floats, the t%03ld_%ld_f.fits image
 * loaded at :2204-2226).  The data are copied; the caller keeps ownership. */
atmwfs_status atmwfs_load_screen(atmwfs_ctx* ctx, int layer, const float* host, long M);
atmwfs_status atmwfs_load_screen_dev(atmwfs_ctx* ctx, int layer, const float* dev, long M);

/* Copy of the screen of layer `layer` as the frames use it (M x M floats
 * into `host`): after atmwfs_normalize_screens it carries the r0 scale and
 * the Cn2 weight, as the reference's image of that layer does after :2363. */
atmwfs_status atmwfs_read_screen(atmwfs_ctx* ctx, int layer, float* host);

/* r0 measurement and renormalisation of the loaded screens, then the
 * per-layer sqrt(Cn2 / cos(zenith)) weights (:2240-2363).  lambda_ref [m]
 * and seeing [arcsec] are TURBULENCE_REF_WAVEL and TURBULENCE_SEEING.
 * r0_pix[0..1] receives the mean r0 before and after renormalisation. */
atmwfs_status atmwfs_normalize_screens(atmwfs_ctx* ctx, float lambda_ref, float seeing, double* r0_pix);

/* The same with further M x M host screens that enter the mean r0 but are
 * not layers: the reference averages r0 over every master file present in
 * the directory (:2246-2285), also files beyond the number of layers. */
atmwfs_status atmwfs_normalize_screens_ext(atmwfs_ctx* ctx, float lambda_ref, float seeing, const float* const* extra,
                                           long nextra, double* r0_pix);

/* Run nsteps time steps (the frame loop, :2561-4345).  Frames of step s of
 * this call are written at offset s * wf_size^2 of the sink buffers.  The
 * copies into the sink run on a stream of their own: with ring >= 2 the
 * copy of step s overlaps the computation of step s + 1 (with ring = 1 they
 * alternate).  Every frame is in the sink when the call returns. */
atmwfs_status atmwfs_run(atmwfs_ctx* ctx, long nsteps, const atmwfs_sink* sink);

/* Advance nsteps time steps (window positions and the step counter) without
 * propagating: for callers that compute the frames another way, such as
 * the learned surrogate, from atmwfs_windows_dev(). */
atmwfs_status atmwfs_advance(atmwfs_ctx* ctx, long nsteps);

/* Device pointers of the most recent frame of instance i (valid until the
 * next run call). */
atmwfs_status atmwfs_frame_dev(atmwfs_ctx* ctx, int i, const float** pha, const float** amp);

/* Per-layer phase windows of instance i at the last completed step: the
 * bicubic screen samples the propagation uses (:2806-2917), times the
 * instance's Scoeff, in screen orientation: nlayers x W x W floats into the
 * device buffer `out` (W = wf_raw_size), on `stream` (NULL: the engine's). */
atmwfs_status atmwfs_windows_dev(atmwfs_ctx* ctx, int i, float* out, void* stream);

/* Layout of one step's frames: total floats, and the offset of instance i. */
size_t atmwfs_frame_floats(const atmwfs_ctx* ctx);
size_t atmwfs_frame_offset(const atmwfs_ctx* ctx, int i);

/* Relaxation iterations of the last science unwrap of instance i (-1 if none). */
int atmwfs_last_iters(atmwfs_ctx* ctx, int i);

/* Steps completed so far; number of propagation planes (runs of layers in
 * one super-layer, top first); layer range [lo, hi) of each plane and the
 * hop distance [m] from plane k to plane k + 1. */
long atmwfs_steps_done(const atmwfs_ctx* ctx);
int atmwfs_num_planes(const atmwfs_ctx* ctx);
atmwfs_status atmwfs_plane_info(const atmwfs_ctx* ctx, int* layer_lo, int* layer_hi, double* hop_z);

/* Host-only (no GPU needed): super-layer grouping of a profile
 * (AtmosphericTurbulence.c:2067-2147) and the propagation planes the engine
 * derives from it.  cn2 is normalised internally.  Arrays have room for L
 * entries (hop_z: L - 1). */
atmwfs_status atmwfs_layer_planes(const double* alt, const double* cn2, int L, double fresnel_bin, int amplitude,
                                  int fresnel, float zangle, int* nsuper, double* salt, int* sidx, int* nplanes,
                                  int* plane_lo, int* plane_hi, double* hop_z);

/* CUDA stream (cudaStream_t) on which the context runs. */
void* atmwfs_stream(atmwfs_ctx* ctx);

/* Diagnostics: launch pass k (1-based, of atmwfs_num_planes passes; k = 0 is
 * the geometric phase-sum kernel, k = atmwfs_num_planes + 1 the kernel that
 * computes the step's screen windows of the window groups of this grid size,
 * k = atmwfs_num_planes + 2 the science unwrap and apply of the whole context)
 * for the instances of grid class c `reps` times, timed with CUDA events on
 * the context stream.  Returns the mean duration [ms], the algorithmic bytes
 * of one launch (field in/out, window rows, outputs), and the class's grid
 * size and instance count.  Does not advance the simulation. */
atmwfs_status atmwfs_time_pass(atmwfs_ctx* ctx, int k, int c, int reps, double* ms, double* bytes, int* n,
                               int* count);
int atmwfs_num_classes(const atmwfs_ctx* ctx);

/* Pass configurations (radix plan x tile shape x table staging) the engine
 * can compile per grid size: 0-2 the default radix plan in three tile
 * shapes, 3-4 the size's alternative radix plan where it has one (1024:
 * 16 x 8 x 8 against the default 32 x 32), 5 configuration 1 with the hop
 * transfer tables staged in shared memory (512 and 1024).  The autotuner
 * times every configuration compiled for a grid class and keeps the
 * fastest. */
#define ATMWFS_NUM_TILE_CFG 6

/* Grid class ci (instances sharing wf_raw_size and wf_size): sizes, member
 * count, the rows per CTA the autotuner chose, and the mean time [ms] of the
 * tuned pass in each of the ATMWFS_NUM_TILE_CFG tile configurations (0 if
 * forced). */
atmwfs_status atmwfs_class_info(const atmwfs_ctx* ctx, int ci, int* n, int* nout, int* count, int* rows_per_cta,
                                double* tuned_ms);

/* Kernel launches of one time step (the kernel nodes of the step's CUDA
 * graph, captured at the first run; 0 before it). */
int atmwfs_step_kernels(const atmwfs_ctx* ctx);

/* The configuration the autotuner chose for grid class ci (0 ..
 * ATMWFS_NUM_TILE_CFG - 1, see above) and the radix sequence of its
 * forward transform (radices[0..2], 0 after the last stage). */
atmwfs_status atmwfs_class_plan(const atmwfs_ctx* ctx, int ci, int* cfg, int* radices);

/* Current layer positions (pixels) of instance i, after the last step. */
atmwfs_status atmwfs_positions(const atmwfs_ctx* ctx, int i, double* xpos, double* ypos);

/* Unit-level drop-ins.  Fresnel_propagate_wavefront(in, out, dx, z, lambda)
 * (src/WFpropagate/WFpropagate.c:68-152) on an n x n complex image. */
atmwfs_status atmwfs_fresnel(const float* in, float* out, long n, double dx, double z, double lambda);
atmwfs_status atmwfs_fresnel_dev(const void* in, void* out, long n, double dx, double z, double lambda,
                                 void* stream);

/* Allocation-free variant of atmwfs_fresnel_dev (no counterpart in the
 * reference).  For callers that must not allocate device memory while they
 * run: a real-time loop feeding an adaptive-optics controller cannot call the
 * CUDA allocator per frame (an allocation or free may wait on the whole
 * device and takes unbounded time), and a host that gives all device memory
 * to its own pool at start-up has nothing left to allocate from.  The
 * intermediate field and tables live in static device arrays of the library
 * sized for n <= ATMWFS_NOALLOC_MAX_N (2 MiB per GPU that loads the library,
 * kept until exit); larger n is rejected with ATMWFS_ERR_INVALID.  The first
 * call on a device looks the arrays up on that device, so make it before any
 * stream capture.  The call's transfer table and twiddles are written into
 * the arrays by a kernel on `stream`; nothing is copied from host memory.
 * Every call shares the arrays, which keep the last call's contents (the
 * first pass overwrites the whole region the second reads): calls that
 * overlap on the GPU race, so issue them on one stream. */
#define ATMWFS_NOALLOC_MAX_N 512
atmwfs_status atmwfs_fresnel_noalloc(const void* in, void* out, long n, double dx, double z, double lambda,
                                     void* stream);

/* do2dfft / do2dffti (src/fft/fft.c:1298-1315): unnormalised 2-D complex
 * DFT, sign -1 forward, +1 inverse.  n is a power of two in 64..2048, or
 * 4096 / 8192 (rows in shared memory, columns through a transpose). */
atmwfs_status atmwfs_fft2d(const float* in, float* out, long n, int sign);
atmwfs_status atmwfs_fft2d_dev(const void* in, void* out, long n, int sign, void* stream);

/* make_master_turbulence_screen (AtmosphericTurbulence.c:643-855) with a
 * seeded Philox4x32-10 noise source instead of the clock-seeded libc/GSL
 * generators.  Writes two M x M screens (either may be NULL) and the two
 * structure-function constants C1, C2 (may be NULL).  M is a power of two
 * in 64..8192. */
atmwfs_status atmwfs_master_screen(uint64_t seed, uint32_t stream, long M, double outer_pix, double inner_pix,
                                   float* out1, float* out2, double* cfit);

/* Last error message of this thread. */
const char* atmwfs_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* ATMWFS_H */
