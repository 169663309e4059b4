/* Test-only GSL declarations (special functions) for the oracle pin build;
 * used only by models off the pinned path. */
#ifndef GWO_SHIM_GSL_SF_H
#define GWO_SHIM_GSL_SF_H
typedef struct { double val, err; } gsl_sf_result;
typedef unsigned int gsl_mode_t;
#define GSL_PREC_DOUBLE 0
int gsl_sf_elljac_e(double u, double m, double *sn, double *cn, double *dn);
double gsl_sf_ellint_F(double phi, double k, gsl_mode_t mode);
double gsl_sf_ellint_Kcomp(double k, gsl_mode_t mode);
double gsl_sf_ellint_Ecomp(double k, gsl_mode_t mode);
double gsl_sf_ellint_E(double phi, double k, gsl_mode_t mode);
#endif
