/* Test-only GSL declarations (random numbers) for the oracle pin build; not
 * on the pinned path. */
#ifndef GWO_SHIM_GSL_RNG_H
#define GWO_SHIM_GSL_RNG_H
typedef struct { int unused; } gsl_rng_type;
typedef struct { int unused; } gsl_rng;
extern const gsl_rng_type *gsl_rng_default;
const gsl_rng_type *gsl_rng_env_setup(void);
gsl_rng *gsl_rng_alloc(const gsl_rng_type *T);
void gsl_rng_free(gsl_rng *r);
void gsl_rng_set(const gsl_rng *r, unsigned long seed);
double gsl_rng_uniform(const gsl_rng *r);
#endif
