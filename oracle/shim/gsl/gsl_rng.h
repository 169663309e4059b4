#ifndef GWO_SHIM_GSL_RNG_H
#define GWO_SHIM_GSL_RNG_H
typedef struct { int unused; } gsl_rng_type;
typedef struct { int unused; } gsl_rng;
#endif
