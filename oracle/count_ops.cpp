// Algorithmic-work counter (test infrastructure, not shipped).
//
// Built only with -DGWO_COUNT_OPS against the reference's own model sources
// (IMRPhenomD.cpp, IMRPhenomP.cpp, compiled unmodified over oracle/shim), it
// runs the adouble instantiation of the reference's waveform construction on a
// grid and reports how many additions, multiplications, divisions and
// elementary functions of each kind the reference algorithm performs.  Per-bin
// work follows from two runs that differ by one bin.
//
// The detector-bin work is the reference's projection, time-of-arrival shift
// and Simpson inner-product loops, restated here over adouble:
//   projection     waveform_util.cpp:865-873   r = F+ h+ + Fx hx
//   arrival shift  waveform_util.cpp:172-180   r *= exp(i (-2 pi dt) f)
//   integrands     mcmc_gw.cpp:814-816, 838-840  Re(r r*)/S, Re(d r*)/S
//   Simpson sums   util.h:844-856               two weighted sums
#include <complex>
#include <cstring>

#include "IMRPhenomD.h"
#include "IMRPhenomP.h"
#include "gwat_oracle.h"
#include "util.h"

long long gwo_opcount[GWO_NKINDS];

static void to_gen_params_a(const gwo_gen_params *p, gen_params_base<adouble> *g) {
  g->mass1 = p->mass1;
  g->mass2 = p->mass2;
  for (int i = 0; i < 3; i++) {
    g->spin1[i] = p->spin1[i];
    g->spin2[i] = p->spin2[i];
  }
  g->Luminosity_Distance = p->Luminosity_Distance;
  g->incl_angle = p->incl_angle;
  g->phiRef = p->phiRef;
  g->f_ref = p->f_ref;
  g->tc = p->tc;
  g->RA = p->RA;
  g->DEC = p->DEC;
  g->psi = p->psi;
  g->gmst = p->gmst;
  g->chip = p->chip;
  g->phip = p->phip;
  g->shift_time = p->shift_time != 0;
  g->shift_phase = p->shift_phase != 0;
  g->sky_average = p->sky_average != 0;
  g->dep_postmerger = p->dep_postmerger != 0;
}

// Counts (GWO_NKINDS values) of one waveform on n bins: the adouble form of
// the glue in oracle/ref_driver.cpp (waveform_generator.cpp:104-273).
extern "C" int count_waveform(const gwo_gen_params *p, int approximant, const double *freqs, int n,
                              long long *out) {
  std::memset(gwo_opcount, 0, sizeof(gwo_opcount));
  gen_params_base<adouble> in;
  to_gen_params_a(p, &in);
  source_parameters<adouble> params;
  params.populate_source_parameters(&in);
  params.phi = in.phi;
  params.theta = in.theta;
  params.incl_angle = in.incl_angle;
  params.f_ref = in.f_ref;
  params.phiRef = in.phiRef;
  params.shift_time = in.shift_time;
  params.sky_average = in.sky_average;
  params.shift_phase = in.shift_phase;
  params.dep_postmerger = in.dep_postmerger;
  std::vector<adouble> f(freqs, freqs + n);
  std::vector<std::complex<adouble>> hp(n), hc(n);
  if (approximant == GWO_IMRPHENOMD) {
    std::complex<adouble> ci = std::complex<adouble>(cos(params.incl_angle), 0);
    IMRPhenomD<adouble> model;
    model.construct_waveform(f.data(), n, hp.data(), &params);
    for (int i = 0; i < n; i++) hc[i] = std::complex<adouble>(0, -1) * hp[i];
    for (int i = 0; i < n; i++) {
      hc[i] *= ci;
      hp[i] *= std::complex<adouble>(.5, 0) * (std::complex<adouble>(1, 0) + ci * ci);
    }
  } else if (approximant == GWO_IMRPHENOMPV2) {
    IMRPhenomPv2<adouble> model;
    model.PhenomPv2_Param_Transform(&params);
    model.construct_waveform(f.data(), n, hp.data(), hc.data(), &params);
    std::complex<adouble> c2z = std::complex<adouble>(cos(2. * params.zeta_polariz));
    std::complex<adouble> s2z = std::complex<adouble>(sin(2. * params.zeta_polariz));
    for (int i = 0; i < n; i++) {
      std::complex<adouble> tp = hp[i], tx = hc[i];
      hp[i] = c2z * tp + s2z * tx;
      hc[i] = c2z * tx - s2z * tp;
    }
  } else {
    return 0;
  }
  std::memcpy(out, gwo_opcount, sizeof(gwo_opcount));
  return GWO_NKINDS;
}

// Counts of the detector-bin loops for n bins of one detector.
extern "C" int count_detector_bins(int n, long long *out) {
  std::vector<std::complex<adouble>> hp(n, std::complex<adouble>(1e-22, 2e-22)), hc(n, hp[0]), r(n), d(n, hp[0]);
  std::vector<adouble> f(n), psd(n, adouble(1e-46)), integrand(n);
  for (int i = 0; i < n; i++) f[i] = 20. + i / 32.;
  adouble fplus = 0.3, fcross = -0.4, dtoa = 0.01;
  std::memset(gwo_opcount, 0, sizeof(gwo_opcount));
  for (int i = 0; i < n; i++) r[i] = fplus * hp[i] + fcross * hc[i];
  adouble tc = -dtoa;
  tc *= 2 * M_PI;
  for (int j = 0; j < n; j++) r[j] *= exp(std::complex<adouble>(0, tc * f[j]));
  adouble hh = 0, dh = 0;
  for (int i = 0; i < n; i++) integrand[i] = real(r[i] * std::conj(r[i])) / psd[i];
  for (int i = 1; i < n - 1; i++) hh += (i % 2 == 0 ? 2. : 4.) * integrand[i];
  for (int i = 0; i < n; i++) integrand[i] = real(d[i] * std::conj(r[i])) / psd[i];
  for (int i = 1; i < n - 1; i++) dh += (i % 2 == 0 ? 2. : 4.) * integrand[i];
  std::memcpy(out, gwo_opcount, sizeof(gwo_opcount));
  return GWO_NKINDS;
}
