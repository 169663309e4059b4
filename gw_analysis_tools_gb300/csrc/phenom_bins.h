// phenom_bins.h -- FP64 per-bin evaluation (the plain form and the waveform /
// detector-response outputs).  Host and device.
//
// d_bin: one bin of IMRPhenomD::construct_waveform (IMRPhenomD.cpp:476-501)
// followed by the inclination factors of fourier_waveform
// (waveform_generator.cpp:191-200).  p_bin: one bin of
// IMRPhenomPv2::construct_waveform (IMRPhenomP.cpp:290-340 and 354-362)
// followed by the 2-zeta polarisation rotation (waveform_generator.cpp:257-266).
#pragma once

#include "phenom_model.h"

namespace gwt {

struct cd {
  double re, im;
};
GW_HD cd cmul(cd a, cd b) { return cd{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
GW_HD cd cadd(cd a, cd b) { return cd{a.re + b.re, a.im + b.im}; }
GW_HD cd csub(cd a, cd b) { return cd{a.re - b.re, a.im - b.im}; }
GW_HD cd cscale(cd a, double s) { return cd{a.re * s, a.im * s}; }

// build_phase with the per-bin PN coefficients 5 and 6 held locally instead
// of written into the shared coefficient array (IMRPhenomD.cpp:1040-1060, 1365-1399).
GW_HD double build_phase_bin(double f, const ModelD &m, const Pows &p) {
  const Source &s = m.s;
  if (f < s.f1_phase) {
    const double *pn = m.pn_phase;
    double M = s.M;
    double logF = log(kPi * (s.mass1 + s.mass2) * f);
    double c5 = pn[8] + logF * pn[9];
    double c6 = pn[10] - pn[11] * (logF);
    double pn_phase = pn[0] + pn[1] * m.pi.PIthird * p.MFthird + pn[2] * m.pi.PI2third * p.MF2third +
                      pn[3] * kPi * M * f + pn[4] * m.pi.PI4third * p.MF4third + c5 * m.pi.PI5third * p.MF5third +
                      c6 * m.pi.PIsquare * p.MFsquare + pn[7] * m.pi.PI7third * p.MF7third;
    double phase_TF2 = -kPi / 4. + s.k_tf2 * m.pi.PIminus_5third * p.MFminus_5third * pn_phase;
    return phase_TF2 + s.inv_eta * (0 + m.l.sigma[1] * M * f + (3. / 4.) * m.l.sigma[2] * p.MF4third +
                                     (3. / 5) * m.l.sigma[3] * p.MF5third + (1. / 2.) * m.l.sigma[4] * p.MFsquare);
  }
  if (f > s.f2_phase) return phase_mr(f, s, m.l);
  return phase_int(f, s, m.l);
}

// IMRPhenomD: h+ and hx at one frequency.
GW_HD void d_bin(const ModelD &m, double f, cd &hp, cd &hc) {
  if (f > m.fcut) {
    hp = cd{0., 0.};
    hc = cd{0., 0.};
    return;
  }
  double M = m.s.M;
  Pows p;
  if (f < m.s.f1_phase) {
    precalc_powers_ins(f, M, p);
  } else {
    p.MFsixth = sqrt(cbrt(M * f));
    p.MF7sixth = pow_int(p.MFsixth, 7);
  }
  double amp = (m.A0eff * build_amp(f, m, p));
  double phase = build_phase_bin(f, m, p);
  phase -= (m.tcl * (f - m.fref) + m.phic);
  double sn, cs;
  sincos(phase, &sn, &cs);
  cd h{amp * cs, -(amp * sn)};
  const double ci = m.s.cos_incl;
  hc = cd{h.im * ci, -h.re * ci};  // (-i h) cos(iota)
  const double fac = m.s.fac_incl;
  hp = cd{h.re * fac, h.im * fac};
}

// Twist-up factors (IMRPhenomP.cpp:696-715) with the harmonics real (phi = 0).
GW_HD void pv2_twist(double alpha, const double d2[5], const double dm2[5], const double Y[5], cd &hpf, cd &hcf) {
  double sa, ca;
  sincos(alpha, &sa, &ca);
  cd ea{ca, sa}, ema{ca, -sa};
  cd e2a = cmul(ea, ea), em2a = cmul(ema, ema);
  cd ev[5] = {em2a, ema, cd{1., 0.}, ea, e2a};
  hpf = cd{0., 0.};
  hcf = cd{0., 0.};
  for (int m = -2; m <= 2; m++) {
    cd T2m = cscale(ev[-m + 2], dm2[m + 2] * Y[m + 2]);
    cd Tm2m = cscale(ev[m + 2], d2[m + 2] * Y[m + 2]);
    hpf = cadd(hpf, cadd(T2m, Tm2m));
    cd dlt = csub(T2m, Tm2m);
    hcf = cadd(hcf, cd{-dlt.im, dlt.re});
  }
}
GW_HD void pv2_wignerd(double L, const Source &s, double d2[5], double dm2[5]) {  // IMRPhenomP.cpp:665-693
  double sv = s.SP / (L + s.SL);
  double cos_beta = 1. / sqrt(1.0 + sv * sv);
  double cbh = sqrt((1.0 + cos_beta) / 2.0), sbh = sqrt((1.0 - cos_beta) / 2.0);
  double c2 = cbh * cbh, s2 = sbh * sbh, c3 = c2 * cbh, s3 = s2 * sbh, c4 = c3 * cbh, s4 = s3 * sbh;
  d2[0] = s4;
  d2[1] = 2 * cbh * s3;
  d2[2] = kSqrt6 * s2 * c2;
  d2[3] = 2 * c3 * sbh;
  d2[4] = c4;
  dm2[0] = d2[4];
  dm2[1] = -d2[3];
  dm2[2] = d2[2];
  dm2[3] = -d2[1];
  dm2[4] = d2[0];
}

// IMRPhenomPv2: h+ and hx at one frequency, after the 2-zeta rotation.
GW_HD void p_bin(const ModelD &m, const ModelP &pm, double f, cd &hp, cd &hc) {
  if (f > m.fcut) {
    hp = cd{0., 0.};
    hc = cd{0., 0.};
    return;
  }
  const Source &s = m.s;
  Pows p;
  precalc_powers_ins(f, s.M, p);
  double amp = (m.A0eff * build_amp(f, m, p));
  double phase = build_phase_bin(f, m, p);
  double d2[5], dm2[5];
  pv2_wignerd(L2PN(s.eta, p.MF2third, m.pi.PI2third), s, d2, dm2);
  double alpha, eps;
  pv2_euler_angles(alpha, eps, p.MFthird, m.pi.PIthird, pm.ac, pm.ec);
  alpha = alpha + pm.alpha_shift;
  eps = eps - pm.eps_off;
  cd hpf, hcf;
  pv2_twist(alpha, d2, dm2, pm.Y, hpf, hcf);
  phase = phase + (2. * eps);
  double ampv = amp / 2.;
  double X = ((phase - m.tcl * (f - m.fref)) - m.phic) + (2 * kPi * pm.t_corr * f);
  double sn, cs;
  sincos(X, &sn, &cs);
  cd e{cs, -sn};
  cd tp = cmul(cscale(hpf, ampv), e), tx = cmul(cscale(hcf, ampv), e);
  hp = cd{pm.c2z * tp.re + pm.s2z * tx.re, pm.c2z * tp.im + pm.s2z * tx.im};
  hc = cd{pm.c2z * tx.re - pm.s2z * tp.re, pm.c2z * tx.im - pm.s2z * tp.im};
}

GW_HD void wave_bin(const Request &r, double f, cd &hp, cd &hc) {
  if (r.approximant == kPhenomPv2) p_bin(r.m, r.p, f, hp, hc);
  else d_bin(r.m, f, hp, hc);
}

// Detector response of detector d at one frequency:
// (F+ h+ + Fx hx) exp(i tau_d f)  (waveform_util.cpp:172-179, 865-873).
GW_HD cd response_bin(const DetProj &dp, cd hp, cd hc, double f, bool apply_shift) {
  cd r{dp.fp * hp.re + dp.fc * hc.re, dp.fp * hp.im + dp.fc * hc.im};
  if (!apply_shift) return r;
  double sn, cs;
  sincos(dp.tau * f, &sn, &cs);
  return cmul(r, cd{cs, sn});
}

// Simpson weight of bin k of n (util.h:844-856): 1, 4, 2, 4, ..., 2/4, 1.
GW_HD double simpson_weight(int k, int n) {
  if (k == 0 || k == n - 1) return 1.0;
  return (k & 1) ? 4.0 : 2.0;
}

}  // namespace gwt
