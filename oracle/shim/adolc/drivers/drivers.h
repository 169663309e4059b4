#ifndef GWO_SHIM_DRIVERS_H
#define GWO_SHIM_DRIVERS_H
#include "../taping.h"
inline int gradient(short, int, const double *, double *) { return -1; }
inline int jacobian(short, int, int, const double *, double **) { return -1; }
inline int hessian(short, int, double *, double **) { return -1; }
#endif
