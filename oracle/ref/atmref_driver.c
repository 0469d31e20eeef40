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
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "CLIcore.h"
#include "AtmosphereModel/AtmosphereModel.h"
#include "AtmosphericTurbulence/AtmosphericTurbulence.h"
#include "COREMOD_memory/COREMOD_memory.h"
#include "WFpropagate/WFpropagate.h"

DATA data;
pid_t CLIPID;

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
    return 2;
}
