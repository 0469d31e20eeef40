/*
 * shim_rng_stubs.c -- noise injection and inert stand-ins for the checker
 * build of the reference (oracle/ref).
 *
 * The reference draws master-screen noise from libc rand() (ran1,
 * src/statistic/statistic.c:91-97) and GSL gsl_ran_gaussian (gauss,
 * statistic.c:101), seeded from the clock.  Here both read seeded noise
 * streams from the file named by ATMREF_NOISE (float32: for every screen M^2
 * uniform values followed by M^2 Gaussian values), so the reference's own
 * make_rnd / make_master_turbulence_screen run on the same noise as the
 * engine.  When the streams run out a fixed-seed generator takes over.
 * ncurses display calls (interactive monitors, not on the path) are no-ops.
 */
#include <math.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include "gsl/gsl_randist.h"
#include "gsl/gsl_rng.h"
#include "ncurses.h"

static float *g_noise;
static long g_len, g_screen_len, g_upos, g_gpos, g_nscreens;
static uint64_t g_lcg = 0x9E3779B97F4A7C15ull;

static void noise_init(void)
{
    static int done;
    if (done) return;
    done = 1;
    const char *fn = getenv("ATMREF_NOISE");
    const char *ms = getenv("ATMREF_NOISE_M");
    if (!fn || !ms) return;
    long M = atol(ms);
    FILE *f = fopen(fn, "rb");
    if (!f) return;
    fseek(f, 0, SEEK_END);
    long bytes = ftell(f);
    fseek(f, 0, SEEK_SET);
    g_len = bytes / 4;
    g_noise = malloc((size_t)bytes);
    if (fread(g_noise, 4, (size_t)g_len, f) != (size_t)g_len) g_len = 0;
    fclose(f);
    g_screen_len = M * M;
    g_nscreens = g_len / (2 * g_screen_len);
}

static double lcg_uniform(void)
{
    g_lcg = g_lcg * 6364136223846793005ull + 1442695040888963407ull;
    return (double)(g_lcg >> 11) * (1.0 / 9007199254740992.0);
}

/* uniform stream: screen k occupies [2 k M^2, 2 k M^2 + M^2) */
int rand(void)
{
    noise_init();
    long s = g_upos / (g_screen_len ? g_screen_len : 1), i = g_upos % (g_screen_len ? g_screen_len : 1);
    double u;
    if (g_noise && s < g_nscreens) {
        u = g_noise[2 * s * g_screen_len + i];
        g_upos++;
    } else {
        u = lcg_uniform();
    }
    return (int)(u * (double)RAND_MAX + 0.5);
}

void srand(unsigned s) { (void)s; }

static const gsl_rng_type k_type = {"atmref"};
const gsl_rng_type *gsl_rng_default = &k_type;
const gsl_rng_type *gsl_rng_mt19937 = &k_type;
gsl_rng *gsl_rng_alloc(const gsl_rng_type *T) { (void)T; return calloc(1, sizeof(gsl_rng)); }
void gsl_rng_free(gsl_rng *r) { free(r); }
void gsl_rng_set(const gsl_rng *r, unsigned long seed) { (void)r; (void)seed; }
double gsl_rng_uniform(const gsl_rng *r) { (void)r; return lcg_uniform(); }
unsigned long gsl_rng_get(const gsl_rng *r) { (void)r; return (unsigned long)(lcg_uniform() * 4294967296.0); }
const gsl_rng_type *gsl_rng_env_setup(void) { return &k_type; }

/* Gaussian stream: screen k occupies [2 k M^2 + M^2, 2 (k + 1) M^2) */
double gsl_ran_gaussian(const gsl_rng *r, double sigma)
{
    (void)r;
    noise_init();
    long s = g_gpos / (g_screen_len ? g_screen_len : 1), i = g_gpos % (g_screen_len ? g_screen_len : 1);
    if (g_noise && s < g_nscreens) {
        g_gpos++;
        return sigma * g_noise[(2 * s + 1) * g_screen_len + i];
    }
    double u1 = lcg_uniform() + 1e-300, u2 = lcg_uniform();
    return sigma * sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}
double gsl_ran_gaussian_ziggurat(const gsl_rng *r, double sigma) { return gsl_ran_gaussian(r, sigma); }
double gsl_ran_ugaussian(const gsl_rng *r) { return gsl_ran_gaussian(r, 1.0); }
unsigned int gsl_ran_poisson(const gsl_rng *r, double mu) { (void)r; return (unsigned int)(mu + 0.5); }

/* ncurses no-ops */
WINDOW *stdscr;
WINDOW *initscr(void) { return NULL; }
int endwin(void) { return 0; }
int printw(const char *fmt, ...) { (void)fmt; return 0; }
int mvprintw(int y, int x, const char *fmt, ...) { (void)y; (void)x; (void)fmt; return 0; }
int attron(int a) { (void)a; return 0; }
int attroff(int a) { (void)a; return 0; }
int refresh(void) { return 0; }
int clear(void) { return 0; }
int start_color(void) { return 0; }
int init_pair(short p, short f, short b) { (void)p; (void)f; (void)b; return 0; }
SCREEN *newterm(const char *t, FILE *o, FILE *i) { (void)t; (void)o; (void)i; return NULL; }
SCREEN *set_term(SCREEN *s) { return s; }
