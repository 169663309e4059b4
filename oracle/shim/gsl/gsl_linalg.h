/* Test-only GSL declarations (factorisations) for the oracle pin build.  The
 * pivoted Cholesky inverse of the reference goes through these; they are not
 * defined for the pin, so that step stays unpinned. */
#ifndef GWO_SHIM_GSL_LINALG_H
#define GWO_SHIM_GSL_LINALG_H
#include "gsl_matrix_double.h"
typedef struct { size_t size; size_t *data; } gsl_permutation;
gsl_permutation *gsl_permutation_alloc(size_t n);
void gsl_permutation_free(gsl_permutation *p);
int gsl_linalg_pcholesky_decomp(gsl_matrix *A, gsl_permutation *p);
int gsl_linalg_pcholesky_invert(const gsl_matrix *LDLT, const gsl_permutation *p, gsl_matrix *Ainv);
int gsl_linalg_cholesky_decomp1(gsl_matrix *A);
int gsl_linalg_cholesky_decomp(gsl_matrix *A);
int gsl_linalg_cholesky_invert(gsl_matrix *A);
int gsl_linalg_LU_decomp(gsl_matrix *A, gsl_permutation *p, int *signum);
int gsl_linalg_LU_invert(const gsl_matrix *LU, const gsl_permutation *p, gsl_matrix *inverse);
double gsl_linalg_LU_lndet(gsl_matrix *LU);
#endif
