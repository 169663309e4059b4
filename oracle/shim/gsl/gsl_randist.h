/* Test-only GSL declarations (random distributions) for the oracle pin build;
 * not on the pinned path. */
#ifndef GWO_SHIM_GSL_RANDIST_H
#define GWO_SHIM_GSL_RANDIST_H
#include "gsl_rng.h"
double gsl_ran_gaussian(const gsl_rng *r, double sigma);
double gsl_ran_flat(const gsl_rng *r, double a, double b);
#endif
