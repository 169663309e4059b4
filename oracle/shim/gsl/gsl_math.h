/* Test-only GSL declarations (function objects) for the oracle pin build. */
#ifndef GWO_SHIM_GSL_MATH_H
#define GWO_SHIM_GSL_MATH_H
#include <math.h>
typedef struct {
  double (*function)(double x, void *params);
  void *params;
} gsl_function;
#define GSL_FN_EVAL(F, x) (*((F)->function))(x, (F)->params)
int gsl_fcmp(double x1, double x2, double epsilon);
#endif
