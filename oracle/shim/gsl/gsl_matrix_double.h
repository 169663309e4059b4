/* Test-only GSL declarations (dense matrices) for the oracle pin build. */
#ifndef GWO_SHIM_GSL_MATRIX_DOUBLE_H
#define GWO_SHIM_GSL_MATRIX_DOUBLE_H
#include <stddef.h>
typedef struct {
  size_t size1, size2, tda;
  double *data;
} gsl_matrix;
gsl_matrix *gsl_matrix_alloc(size_t n1, size_t n2);
void gsl_matrix_free(gsl_matrix *m);
double gsl_matrix_get(const gsl_matrix *m, size_t i, size_t j);
void gsl_matrix_set(gsl_matrix *m, size_t i, size_t j, double x);
#endif
