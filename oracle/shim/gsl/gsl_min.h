/* Test-only GSL declarations (1-D minimisation) for the oracle pin build;
 * not on the pinned path. */
#ifndef GWO_SHIM_GSL_MIN_H
#define GWO_SHIM_GSL_MIN_H
#include "gsl_math.h"
typedef struct { int unused; } gsl_min_fminimizer_type;
typedef struct gwo_gsl_min_fminimizer gsl_min_fminimizer;
extern const gsl_min_fminimizer_type *gsl_min_fminimizer_brent;
gsl_min_fminimizer *gsl_min_fminimizer_alloc(const gsl_min_fminimizer_type *T);
void gsl_min_fminimizer_free(gsl_min_fminimizer *s);
int gsl_min_fminimizer_set(gsl_min_fminimizer *s, gsl_function *f, double x_minimum, double x_lower, double x_upper);
int gsl_min_fminimizer_iterate(gsl_min_fminimizer *s);
double gsl_min_fminimizer_x_minimum(const gsl_min_fminimizer *s);
double gsl_min_fminimizer_x_lower(const gsl_min_fminimizer *s);
double gsl_min_fminimizer_x_upper(const gsl_min_fminimizer *s);
int gsl_min_test_interval(double x_lower, double x_upper, double epsabs, double epsrel);
#define GSL_CONTINUE (-2)
#endif
