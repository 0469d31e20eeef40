#ifndef ATMREF_GSL_RANDIST_SHIM_H
#define ATMREF_GSL_RANDIST_SHIM_H
#include "gsl/gsl_rng.h"
double gsl_ran_gaussian(const gsl_rng* r, double sigma);
double gsl_ran_gaussian_ziggurat(const gsl_rng* r, double sigma);
double gsl_ran_ugaussian(const gsl_rng* r);
unsigned int gsl_ran_poisson(const gsl_rng* r, double mu);
#endif
