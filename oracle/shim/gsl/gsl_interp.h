/* Test-only GSL stand-in: natural cubic spline ("cspline") with the GSL
 * boundary conditions and evaluation formulas, for the oracle pin build only. */
#ifndef GWO_SHIM_GSL_INTERP_H
#define GWO_SHIM_GSL_INTERP_H
#include <stddef.h>
#include <stdlib.h>
#include <math.h>
typedef struct { int kind; } gsl_interp_type;
static const gsl_interp_type gwo_cspline_type = {1};
static const gsl_interp_type gwo_linear_type = {0};
#define gsl_interp_cspline (&gwo_cspline_type)
#define gsl_interp_linear (&gwo_linear_type)
#define gsl_interp_akima (&gwo_cspline_type)
typedef struct { size_t cache; } gsl_interp_accel;
static inline gsl_interp_accel *gsl_interp_accel_alloc(void) { return (gsl_interp_accel *)calloc(1, sizeof(gsl_interp_accel)); }
static inline void gsl_interp_accel_free(gsl_interp_accel *a) { free(a); }
static inline int gsl_interp_accel_reset(gsl_interp_accel *a) { a->cache = 0; return 0; }
#endif
