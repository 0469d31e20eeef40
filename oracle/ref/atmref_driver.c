/*
 * atmref_driver.c -- command-line driver of the reference's own code, built
 * against the shims of this directory (checker build, never shipped).
 *
 * It sets up the global image/variable tables the way the reference's
 * main_init() does (src/CLIcore.c:992-1100) and calls reference functions
 * directly:
 *
 *   atmref fresnel <n> <dx> <z> <lambda> <in.c64> <out.c64>
 *       Fresnel_propagate_wavefront (src/WFpropagate/WFpropagate.c:68) on an
 *       n x n complex_float image read from / written to raw files.
 *   atmref mkwfs <lambda_um> <precision>
 *       make_AtmosphericTurbulence_wavefront_series
 *       (src/AtmosphericTurbulence/AtmosphericTurbulence.c:1433) in the
 *       current directory (WFsim.conf, profile, t%03ld_%ld_f.fits).
 *   atmref stdN <conf> <lambda_model> <alt> <lambda> [<alt> <lambda> ...]
 *       AtmosphereModel_Create_from_CONF then AtmosphereModel_stdAtmModel_N
 *       (src/AtmosphereModel/AtmosphereModel.c:3212) for each pair.
 *   atmref conf <conf> <keyword>...
 *       read_config_parameter_exists and read_config_parameter
 *       (src/COREMOD_tools/COREMOD_tools.c:596-666) for each keyword; one
 *       line "CONF <keyword> <exists> <found> [<content>]" each.
 *   atmref hv <wspeed> <r0> <sitealt> <nlayers> <outfile>
 *       AtmosphericTurbulence_makeHV_CN2prof (AtmosphericTurbulence.c:7841),
 *       which also writes conf_turb.txt in the current directory.
 *   atmref expo <etime> <outfile>
 *       measure_wavefront_series_expoframes (AtmosphericTurbulence.c:6592)
 *       in the current directory (WFsim.conf with PUPIL_AMPL_FILE, the
 *       science cubes under the fixed 1.65 um name).
 *   atmref chromat <n> <amp.f32> <pha.f32> <coeff1> <coeff2> <nbstep> <apo> <out.f32>
 *       PSF_makeChromatPSF (src/psf/psf.c:54) on raw n x n float images.
 *   atmref measure <n> <in.f32> <gauss.f32>
 *       the exposure loop's measures of a raw n x n float image:
 *       gauss_filter(in, 3, 10) (written out), center_PSF, measure_FWHM on
 *       the filtered image, measure_enc_NRJ(in, 0.5); one line
 *       "MEAS <xc> <yc> <fwhm> <ee50>".
 *   atmref refract <conf> <lambda_model> <lambda> <zangle> <writepath>
 *       AtmosphereModel_RefractionPath (src/AtmosphereModel/AtmosphereModel.c:4215);
 *       one line "REFR <refraction arcsec> <v_TRANSM> <SiteAlt>"; writepath 1
 *       leaves refractpath.txt in the current directory.
 *   atmref ntable <conf> <lambda_model> <lambda> <dh> <n> <out.bin>
 *       AtmosphereModel_stdAtmModel_N at altitudes k * dh, k < n: n floats
 *       (N) then n doubles (v_ABSCOEFF after each call).
 *   atmref roffset <conf> <lambda_model> <lambda_ref> <slambda> <zangle> <alt>...
 *       the per-layer refraction offset RoffsetS - Roffset [m] that
 *       make_AtmosphericTurbulence_wavefront_series adds to the start row
 *       (src/AtmosphericTurbulence/AtmosphericTurbulence.c:2159-2183): the
 *       same 1 m altitude steps from the site altitude over the reference's
 *       stdAtmModel_N, with its float/double operand types.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "CLIcore.h"
#include "AtmosphereModel/AtmosphereModel.h"
#include "AtmosphericTurbulence/AtmosphericTurbulence.h"
#include "COREMOD_memory/COREMOD_memory.h"
#include "WFpropagate/WFpropagate.h"
#include "image_filter/image_filter.h"
#include "psf/psf.h"

DATA data;
pid_t CLIPID;
int C_ERRNO;     /* globals of src/CLIcore.c:102-104 */
int TYPESIZE[9];

int init_AtmosphericTurbulence(void), init_AtmosphereModel(void), init_OpticsMaterials(void),
    init_WFpropagate(void), init_image_gen(void), init_statistic(void), init_fft(void), init_info(void),
    init_COREMOD_arith(void), init_COREMOD_iofits(void), init_COREMOD_memory(void), init_COREMOD_tools(void),
    init_00CORE(void);

static void init_data(void)
{
    memset(&data, 0, sizeof data);
    data.quiet = 1;
    data.NB_MAX_IMAGE = 5000;
    data.NB_MAX_VARIABLE = 5000 + NB_VARIABLES_BUFFER_REALLOC;
    data.INVRANDMAX = 1.0 / RAND_MAX;
    data.NB_MAX_MODULE = 100;
    data.module = (MODULE *)calloc(data.NB_MAX_MODULE, sizeof(MODULE));
    data.NB_MAX_COMMAND = 5000;
    data.cmd = (CMD *)calloc(data.NB_MAX_COMMAND, sizeof(CMD));
    data.image = (IMAGE *)calloc(data.NB_MAX_IMAGE, sizeof(IMAGE));
    data.variable = (VARIABLE *)calloc(data.NB_MAX_VARIABLE, sizeof(VARIABLE));
    data.image[0].used = 0;
    data.image[0].shmfd = -1;
    data.rndgen = gsl_rng_alloc(gsl_rng_mt19937);
    data.SHARED_DFT = 0;
    data.NBKEWORD_DFT = 10;
    /* element sizes as src/CLIcore.c:588-596 */
    TYPESIZE[0] = 0;
    TYPESIZE[1] = sizeof(char);
    TYPESIZE[2] = sizeof(int);
    TYPESIZE[3] = sizeof(float);
    TYPESIZE[4] = sizeof(double);
    TYPESIZE[5] = 2 * sizeof(float);
    TYPESIZE[6] = 2 * sizeof(double);
    TYPESIZE[7] = sizeof(unsigned short);
    TYPESIZE[8] = sizeof(long);
    C_ERRNO = 0;
    /* the module set-up of src/initmodules.c:27-51, for the compiled modules
       (the atmosphere model allocates its profile tables here) */
    init_AtmosphericTurbulence();
    init_AtmosphereModel();
    init_OpticsMaterials();
    init_WFpropagate();
    init_image_gen();
    init_statistic();
    init_fft();
    init_info();
    init_COREMOD_arith();
    init_COREMOD_iofits();
    init_COREMOD_memory();
    init_COREMOD_tools();
    init_00CORE();
}

static int cmd_fresnel(int argc, char **argv)
{
    if (argc < 8) return 2;
    long n = atol(argv[2]);
    double dx = atof(argv[3]), z = atof(argv[4]), lambda = atof(argv[5]);
    long ID = create_2DCimage_ID("wfin", n, n);
    FILE *f = fopen(argv[6], "rb");
    if (!f) return 3;
    size_t got = fread(data.image[ID].array.CF, sizeof(float) * 2, (size_t)(n * n), f);
    fclose(f);
    if (got != (size_t)(n * n)) return 3;
    Fresnel_propagate_wavefront("wfin", "wfout", dx, z, lambda);
    long IDo = image_ID("wfout");
    f = fopen(argv[7], "wb");
    if (!f) return 4;
    fwrite(data.image[IDo].array.CF, sizeof(float) * 2, (size_t)(n * n), f);
    fclose(f);
    return 0;
}

static int cmd_stdn(int argc, char **argv)
{
    if (argc < 6) return 2;
    AtmosphereModel_Create_from_CONF(argv[2], (float)atof(argv[3]));
    for (int i = 4; i + 1 < argc; i += 2)
        printf("STDN %.17g %.17g %.9g\n", atof(argv[i]), atof(argv[i + 1]),
               (double)AtmosphereModel_stdAtmModel_N((float)atof(argv[i]), (float)atof(argv[i + 1]), 0));
    return 0;
}

int read_config_parameter_exists(char *config_file, char *keyword);
int read_config_parameter(char *config_file, char *keyword, char *content);

static int cmd_conf(int argc, char **argv)
{
    if (argc < 4) return 2;
    for (int i = 3; i < argc; i++) {
        char content[1000];
        const int ex = read_config_parameter_exists(argv[2], argv[i]);
        const int rd = read_config_parameter(argv[2], argv[i], content);
        printf("CONF\t%s\t%d\t%d\t%s\n", argv[i], ex, rd, content);
    }
    return 0;
}

extern float SiteAlt;

static int cmd_roffset(int argc, char **argv)
{
    if (argc < 8) return 2;
    AtmosphereModel_Create_from_CONF(argv[2], (float)atof(argv[3]));
    const float lam_ref = (float)atof(argv[4]);
    const double slam = atof(argv[5]);
    const float za = (float)atof(argv[6]);
    for (int i = 7; i < argc; i++) {
        const double alt = atof(argv[i]);
        double off[2] = {0.0, 0.0};
        for (int w = 0; w < 2; w++) {
            for (double h = SiteAlt; h < alt; h += 1.0) {
                const double n = 1.0 + AtmosphereModel_stdAtmModel_N(h, w == 0 ? lam_ref : slam, 0);
                double t = sin(za) / sqrt(n * n - sin(za) * sin(za));
                t -= sin(za) / sqrt(1.0 - sin(za) * sin(za));
                off[w] += t;
            }
        }
        printf("ROFF %.17g %.17g\n", alt, off[1] - off[0]);
    }
    return 0;
}

static long read_raw(const char *path, const char *name, long n)
{
    long ID = create_2Dimage_ID(name, n, n);
    FILE *f = fopen(path, "rb");
    if (!f) return -1;
    size_t got = fread(data.image[ID].array.F, sizeof(float), (size_t)(n * n), f);
    fclose(f);
    return got == (size_t)(n * n) ? ID : -1;
}

static int write_raw(const char *path, const char *name, long n)
{
    long ID = image_ID(name);
    FILE *f = fopen(path, "wb");
    if (!f || ID < 0) return 4;
    fwrite(data.image[ID].array.F, sizeof(float), (size_t)(n * n), f);
    fclose(f);
    return 0;
}

static int cmd_chromat(int argc, char **argv)
{
    if (argc < 10) return 2;
    long n = atol(argv[2]);
    if (read_raw(argv[3], "amp", n) < 0 || read_raw(argv[4], "pha", n) < 0) return 3;
    PSF_makeChromatPSF("amp", "pha", (float)atof(argv[5]), (float)atof(argv[6]), atol(argv[7]), (float)atof(argv[8]),
                       "cpsf");
    return write_raw(argv[9], "cpsf", n);
}

static int cmd_measure(int argc, char **argv)
{
    if (argc < 5) return 2;
    long n = atol(argv[2]);
    double xc = 0.0, yc = 0.0;
    if (read_raw(argv[3], "PSF", n) < 0) return 3;
    gauss_filter("PSF", "PSFg", 3, 10);
    center_PSF("PSFg", &xc, &yc, n / 2);
    float fw = measure_FWHM("PSFg", xc, yc, 1.0, n / 2);
    float ee = measure_enc_NRJ("PSF", xc, yc, 0.5);
    printf("MEAS %.17g %.17g %.9g %.9g\n", xc, yc, fw, ee);
    return write_raw(argv[4], "PSFg", n);
}

extern double v_TRANSM, v_ABSCOEFF;

static int cmd_refract(int argc, char **argv)
{
    if (argc < 7) return 2;
    AtmosphereModel_Create_from_CONF(argv[2], (float)atof(argv[3]));
    const double r = AtmosphereModel_RefractionPath(atof(argv[4]), atof(argv[5]), atoi(argv[6]));
    printf("\nREFR %.17g %.17g %.9g\n", r, v_TRANSM, (double)SiteAlt);
    return 0;
}

static int cmd_ntable(int argc, char **argv)
{
    if (argc < 8) return 2;
    AtmosphereModel_Create_from_CONF(argv[2], (float)atof(argv[3]));
    const float lam = (float)atof(argv[4]);
    const double dh = atof(argv[5]);
    const long n = atol(argv[6]);
    float *N = (float *)malloc(sizeof(float) * n);
    double *K = (double *)malloc(sizeof(double) * n);
    for (long k = 0; k < n; k++) {
        N[k] = AtmosphereModel_stdAtmModel_N((float)(k * dh), lam, 0);
        K[k] = v_ABSCOEFF;
    }
    FILE *f = fopen(argv[7], "wb");
    if (!f) return 4;
    fwrite(N, sizeof(float), (size_t)n, f);
    fwrite(K, sizeof(double), (size_t)n, f);
    fclose(f);
    free(N);
    free(K);
    return 0;
}

int main(int argc, char **argv)
{
    if (argc < 2) {
        fprintf(stderr, "usage: atmref fresnel|mkwfs|stdN ...\n");
        return 2;
    }
    init_data();
    if (strcmp(argv[1], "fresnel") == 0) return cmd_fresnel(argc, argv);
    if (strcmp(argv[1], "mkwfs") == 0 && argc >= 4) {
        make_AtmosphericTurbulence_wavefront_series((float)atof(argv[2]), atol(argv[3]));
        return 0;
    }
    if (strcmp(argv[1], "stdN") == 0) return cmd_stdn(argc, argv);
    if (strcmp(argv[1], "roffset") == 0) return cmd_roffset(argc, argv);
    if (strcmp(argv[1], "conf") == 0) return cmd_conf(argc, argv);
    if (strcmp(argv[1], "expo") == 0 && argc >= 4) return measure_wavefront_series_expoframes((float)atof(argv[2]), argv[3]);
    if (strcmp(argv[1], "chromat") == 0) return cmd_chromat(argc, argv);
    if (strcmp(argv[1], "refract") == 0) return cmd_refract(argc, argv);
    if (strcmp(argv[1], "ntable") == 0) return cmd_ntable(argc, argv);
    if (strcmp(argv[1], "measure") == 0) return cmd_measure(argc, argv);
    if (strcmp(argv[1], "hv") == 0 && argc >= 7)
        return AtmosphericTurbulence_makeHV_CN2prof(atof(argv[2]), atof(argv[3]), atof(argv[4]), atol(argv[5]), argv[6]);
    return 2;
}
