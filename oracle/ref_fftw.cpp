// ref_fftw.cpp -- TEST INFRASTRUCTURE ONLY.
//
// The FFTW functions the reference's maximised likelihoods call
// (mcmc_gw.cpp:595-800 through fftw_outline, util.cpp:964-969), defined for
// the reference pin library oracle/_ref/libgwatref_full.so.  A plan records
// its length, arrays and sign; executing it evaluates the discrete Fourier
// transform by its definition,
//   out[k] = sum_n in[n] exp(sign * 2 pi i n k / N),
// with the twiddle index n*k reduced modulo N in integers, so every twiddle is
// one correctly reduced angle.  FFTW's sign convention: FFTW_FORWARD = -1.
// O(N^2): meant for the short grids of the pin tests.
#include <fftw3.h>

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

struct gwo_fftw_plan_s {
  int n;
  fftw_complex *in, *out;
  int sign;
};

extern "C" {

void *fftw_malloc(size_t n) { return std::malloc(n ? n : 1); }
void fftw_free(void *p) { std::free(p); }

fftw_plan fftw_plan_dft_1d(int n, fftw_complex *in, fftw_complex *out, int sign, unsigned flags) {
  (void)flags;
  gwo_fftw_plan_s *p = new gwo_fftw_plan_s;
  p->n = n;
  p->in = in;
  p->out = out;
  p->sign = sign;
  return p;
}

void fftw_execute_dft(const fftw_plan p, fftw_complex *in, fftw_complex *out) {
  const long n = p->n;
  std::vector<double> c(n), s(n);
  for (long m = 0; m < n; m++) {
    const double a = 2.0 * M_PI * (double)m / (double)n;
    c[m] = std::cos(a);
    s[m] = p->sign * std::sin(a);
  }
  std::vector<double> re(n), im(n);
  for (long k = 0; k < n; k++) {
    double sr = 0, si = 0;
    long idx = 0;  // n*k mod N, advanced by k each step
    for (long j = 0; j < n; j++) {
      const double xr = in[j][0], xi = in[j][1];
      sr += xr * c[idx] - xi * s[idx];
      si += xr * s[idx] + xi * c[idx];
      idx += k;
      if (idx >= n) idx -= n;
    }
    re[k] = sr;
    im[k] = si;
  }
  for (long k = 0; k < n; k++) {
    out[k][0] = re[k];
    out[k][1] = im[k];
  }
}

void fftw_execute(const fftw_plan p) { fftw_execute_dft(p, p->in, p->out); }
void fftw_destroy_plan(fftw_plan p) { delete p; }
void fftw_cleanup(void) {}

}  // extern "C"
