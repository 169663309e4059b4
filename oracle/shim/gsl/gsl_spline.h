#ifndef GWO_SHIM_GSL_SPLINE_H
#define GWO_SHIM_GSL_SPLINE_H
#include "gsl_interp.h"
#include <string.h>
typedef struct {
  const gsl_interp_type *T;
  double *x, *y, *c;
  size_t size;
} gsl_spline;
static inline gsl_spline *gsl_spline_alloc(const gsl_interp_type *T, size_t n) {
  gsl_spline *s = (gsl_spline *)calloc(1, sizeof(gsl_spline));
  s->T = T; s->size = n;
  s->x = (double *)calloc(n, sizeof(double)); s->y = (double *)calloc(n, sizeof(double)); s->c = (double *)calloc(n, sizeof(double));
  return s;
}
static inline void gsl_spline_free(gsl_spline *s) { if (!s) return; free(s->x); free(s->y); free(s->c); free(s); }
/* Natural cubic spline (Burden & Faires, Numerical Analysis, sec. 3.5):
 * c[i] = S''(x_i)/2 with c[0] = c[n-1] = 0 from the symmetric tridiagonal
 * system of the interior knots, h_{i-1} c_{i-1} + 2 (h_{i-1} + h_i) c_i +
 * h_i c_{i+1} = 3 (s_i - s_{i-1}), solved by L D L^T: a forward sweep, then
 * back substitution.  The same arithmetic, in the same order, as
 * gwo_cspline_coeffs in oracle/gwat_oracle.c. */
static inline int gsl_spline_init(gsl_spline *s, const double *xa, const double *ya, size_t n) {
  memcpy(s->x, xa, n * sizeof(double));
  memcpy(s->y, ya, n * sizeof(double));
  if (s->T->kind == 0) return 0;
  double *c = s->c;
  const long m = (long)n - 2;
  c[0] = 0.0;
  c[n - 1] = 0.0;
  if (m < 1) return 0;
  double *piv = (double *)calloc(3 * (size_t)m, sizeof(double));
  double *mul = piv + m, *rhs = mul + m;
  double h_left = xa[1] - xa[0];
  double s_left = (ya[1] - ya[0]) * (h_left != 0.0 ? 1.0 / h_left : 0.0);
  for (long k = 0; k < m; k++) {
    const double h_right = xa[k + 2] - xa[k + 1];
    const double s_right = (ya[k + 2] - ya[k + 1]) * (h_right != 0.0 ? 1.0 / h_right : 0.0);
    const double diag = 2.0 * (h_right + h_left), load = 3.0 * (s_right - s_left);
    if (k == 0) {
      piv[0] = diag;
      rhs[0] = load;
    } else {
      piv[k] = diag - h_left * mul[k - 1];
      rhs[k] = load - mul[k - 1] * rhs[k - 1];
    }
    if (k < m - 1) mul[k] = h_right / piv[k];
    h_left = h_right;
    s_left = s_right;
  }
  c[m] = rhs[m - 1] / piv[m - 1];
  for (long k = m - 2; k >= 0; k--) c[k + 1] = rhs[k] / piv[k] - mul[k] * c[k + 2];
  free(piv);
  return 0;
}
static inline size_t gwo_bsearch(const double *x, double xv, size_t lo, size_t hi) {
  while (hi > lo + 1) { size_t i = (hi + lo) / 2; if (x[i] > xv) hi = i; else lo = i; }
  return lo;
}
static inline double gwo_spline_eval_impl(const gsl_spline *s, double xv, int deriv) {
  if (!(xv >= s->x[0] && xv <= s->x[s->size - 1])) return NAN;
  size_t i = gwo_bsearch(s->x, xv, 0, s->size - 1);
  double x_lo = s->x[i], x_hi = s->x[i + 1], dx = x_hi - x_lo, y_lo = s->y[i], dy = s->y[i + 1] - y_lo, delx = xv - x_lo;
  if (s->T->kind == 0) return deriv ? dy / dx : y_lo + delx * (dy / dx);
  double c_i = s->c[i], c_ip1 = s->c[i + 1];
  double b_i = (dy / dx) - dx * (c_ip1 + 2.0 * c_i) / 3.0, d_i = (c_ip1 - c_i) / (3.0 * dx);
  if (deriv) return b_i + delx * (2.0 * c_i + 3.0 * d_i * delx);
  return y_lo + delx * (b_i + delx * (c_i + delx * d_i));
}
static inline double gsl_spline_eval(const gsl_spline *s, double x, gsl_interp_accel *a) { (void)a; return gwo_spline_eval_impl(s, x, 0); }
static inline double gsl_spline_eval_deriv(const gsl_spline *s, double x, gsl_interp_accel *a) { (void)a; return gwo_spline_eval_impl(s, x, 1); }
#endif
