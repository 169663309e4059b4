/* Test-only GSL declarations (quadrature) so that the reference translation
 * units compile for the oracle pin build; not on the pinned path. */
#ifndef GWO_SHIM_GSL_INTEGRATION_H
#define GWO_SHIM_GSL_INTEGRATION_H
#include <stddef.h>
#include "gsl_math.h"
typedef struct gwo_gsl_integration_workspace gsl_integration_workspace;
enum { GSL_INTEG_GAUSS15 = 1, GSL_INTEG_GAUSS21, GSL_INTEG_GAUSS31, GSL_INTEG_GAUSS41, GSL_INTEG_GAUSS51,
       GSL_INTEG_GAUSS61 };
gsl_integration_workspace *gsl_integration_workspace_alloc(size_t n);
void gsl_integration_workspace_free(gsl_integration_workspace *w);
int gsl_integration_qag(const gsl_function *f, double a, double b, double epsabs, double epsrel, size_t limit, int key,
                        gsl_integration_workspace *workspace, double *result, double *abserr);
int gsl_integration_qags(const gsl_function *f, double a, double b, double epsabs, double epsrel, size_t limit,
                         gsl_integration_workspace *workspace, double *result, double *abserr);
#endif
