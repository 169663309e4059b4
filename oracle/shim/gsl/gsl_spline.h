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
/* natural spline: symmetric tridiagonal system, LDL^T recurrence */
static inline int gsl_spline_init(gsl_spline *s, const double *xa, const double *ya, size_t n) {
  memcpy(s->x, xa, n * sizeof(double)); memcpy(s->y, ya, n * sizeof(double));
  if (s->T->kind == 0) return 0;
  size_t max_index = n - 1, sys = max_index - 1;
  double *w = (double *)calloc(6 * (sys > 0 ? sys : 1), sizeof(double));
  double *diag = w, *off = w + sys, *g = w + 2 * sys, *gam = w + 3 * sys, *alp = w + 4 * sys, *z = w + 5 * sys;
  double *c = s->c;
  c[0] = 0.0; c[max_index] = 0.0;
  for (size_t i = 0; i < sys; i++) {
    double h_i = xa[i + 1] - xa[i], h_ip1 = xa[i + 2] - xa[i + 1];
    double yd_i = ya[i + 1] - ya[i], yd_ip1 = ya[i + 2] - ya[i + 1];
    double g_i = (h_i != 0.0) ? 1.0 / h_i : 0.0, g_ip1 = (h_ip1 != 0.0) ? 1.0 / h_ip1 : 0.0;
    off[i] = h_ip1; diag[i] = 2.0 * (h_ip1 + h_i); g[i] = 3.0 * (yd_ip1 * g_ip1 - yd_i * g_i);
  }
  if (sys == 1) { c[1] = g[0] / diag[0]; }
  else if (sys > 1) {
    size_t N = sys;
    alp[0] = diag[0]; gam[0] = off[0] / alp[0];
    for (size_t i = 1; i < N - 1; i++) { alp[i] = diag[i] - off[i - 1] * gam[i - 1]; gam[i] = off[i] / alp[i]; }
    alp[N - 1] = diag[N - 1] - off[N - 2] * gam[N - 2];
    z[0] = g[0];
    for (size_t i = 1; i < N; i++) z[i] = g[i] - gam[i - 1] * z[i - 1];
    for (size_t i = 0; i < N; i++) z[i] = z[i] / alp[i];
    c[N] = z[N - 1];
    for (long i = (long)N - 2; i >= 0; i--) c[1 + i] = z[i] - gam[i] * c[1 + i + 1];
  }
  free(w);
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
