/* gsl_rng.h -- the GSL random-number declarations the reference uses; the
 * checker build replaces the generator (shim_gsl.c). */
#ifndef ATMREF_GSL_RNG_SHIM_H
#define ATMREF_GSL_RNG_SHIM_H
typedef struct atmref_rng_type { const char* name; } gsl_rng_type;
typedef struct atmref_rng { unsigned long long s; } gsl_rng;
extern const gsl_rng_type* gsl_rng_default;
extern const gsl_rng_type* gsl_rng_mt19937;
gsl_rng* gsl_rng_alloc(const gsl_rng_type* T);
void gsl_rng_free(gsl_rng* r);
void gsl_rng_set(const gsl_rng* r, unsigned long seed);
double gsl_rng_uniform(const gsl_rng* r);
unsigned long gsl_rng_get(const gsl_rng* r);
const gsl_rng_type* gsl_rng_env_setup(void);
#endif
