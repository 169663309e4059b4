// phenom_prologue.h -- per-request FP64 prologue (included by phenom_model.h).
//
// Computes every per-request constant of IMRPhenomD / IMRPhenomPv2 and of the
// detector projection once, so that per-bin work is only the bin loop of
// IMRPhenomD::construct_waveform (IMRPhenomD.cpp:476-501) or
// IMRPhenomPv2::construct_waveform (IMRPhenomP.cpp:290-362).
#pragma once

namespace gwt {

// (pi M)^(i/3) f^(i/3 - 1) = (pi M f)^(i/3) / f and M^((7+i)/3) f^((7+i)/3 - 1)
// = (M f)^((7+i)/3) / f: one cube root each instead of a pow per term.
GW_HD double Damp_ins(double f, const ModelD &m) {  // IMRPhenomD.cpp:1407-1419
  const double *pn = m.pn_amp;
  double pn_amp = 0, M = m.s.M;
  const double x = cbrt(kPi * M * f), y = cbrt(M * f), inv_f = 1. / f;
  double xi = 1.0;
  for (int i = 0; i < 7; i++, xi *= x) pn_amp += pn[i] * xi * inv_f * (i / 3.);
  double nr_amp = 0, yi = y * y;
  yi = yi * yi * yi * y;  // y^7
  for (int i = 0; i < 3; i++, yi *= y) nr_amp += (m.l.rho[i]) * yi * inv_f * (7. + i) / 3.;
  return pn_amp + nr_amp;
}
GW_HD double Damp_mr(double f, const Source &s, const Lambda &l) {  // IMRPhenomD.cpp:1514-1532
  double g1 = l.gamma[0], g2 = l.gamma[1], g3 = l.gamma[2], fdamp = s.fdamp, fRD = s.fRD, M = s.M;
  double d = f - fRD, den = d * d + fdamp * fdamp * g3 * g3;
  return -((exp(((-f + fRD) * g2) / (fdamp * g3)) * g1 * (d * d * g2 + 2 * fdamp * d * g3 + fdamp * fdamp * g2 * g3 * g3)) /
           (den * den * M));
}
GW_HD double Dphase_ins(double f, const Source &s, double *pn, const Lambda &l) {  // IMRPhenomD.cpp:1427-1460
  double M = s.M, eta = s.eta;
  pn_phase_coeff_nonstatic(s, pn, f);
  double d0 = (1. / f) * (38645. * kPi / 756 - 65 * kPi * eta / 9 +
                          s.delta_mass * (-732985. / 2268 - 140 * eta / 9) * s.chi_a +
                          (-732985. / 2268 + 24260 * eta / 81 + 340 * eta * eta / 9) * s.chi_s);  // :1067-1081
  double d1 = (-6848. * (1. / f) / 63);
  // powers of v = (pi M f)^(1/3) and w = (M f)^(1/3) by products
  const double v = cbrt(kPi * M * f), w = cbrt(M * f), inv_f = 1. / f;
  double vp[9];
  vp[0] = 1.0;
  for (int i = 1; i < 9; i++) vp[i] = vp[i - 1] * v;
  const double vm5 = 1. / (vp[5]);  // (pi M f)^(-5/3)
  double pn_phase = 0;
  for (int i = 0; i < 8; i++) pn_phase += pn[i] * vp[i];
  double phase_TF2 = +s.k_tf2 * vm5 * (-5. / 3.) * inv_f * pn_phase;
  double pn_phase_deriv = 0;
  for (int i = 0; i < 8; i++) pn_phase_deriv += pn[i] * vp[i] * (i / 3.) * inv_f;
  pn_phase_deriv += d0 * vp[5] + d1 * vp[6];
  phase_TF2 += pn_phase_deriv * (s.k_tf2 * vm5);
  return phase_TF2 + s.inv_eta * (l.sigma[1] * M + l.sigma[2] * M * w + l.sigma[3] * M * w * w + l.sigma[4] * M * M * f);
}
// Integer powers of the three matching frequencies and of M used by the
// intermediate-amplitude coefficients (products instead of pow calls).
struct DeltaPowers {
  double f1[6], f2[6], f3[6], m[5], d12_2, d13_3, d23_2;
  GW_HD DeltaPowers(double a, double b, double c, double M) {
    f1[0] = f2[0] = f3[0] = m[0] = 1.0;
    for (int k = 1; k < 6; k++) {
      f1[k] = f1[k - 1] * a;
      f2[k] = f2[k - 1] * b;
      f3[k] = f3[k - 1] * c;
    }
    for (int k = 1; k < 5; k++) m[k] = m[k - 1] * M;
    d12_2 = (a - b) * (a - b);
    d13_3 = (a - c) * (a - c) * (a - c);
    d23_2 = (b - c) * (b - c);
  }
};
/* calculate_delta_parameter_0..4 (IMRPhenomD.cpp:1709-1785) */
GW_HD double delta0(double f1, double f2, double f3, double v1, double v2, double v3, double dd1, double dd3, double M) {
  const DeltaPowers P(f1, f2, f3, M);
  (void)M;
  return (-(dd3 * P.f1[2] * P.d12_2 * f2 * (f1 - f3) * (f2 - f3) * f3) +
          dd1 * f1 * (f1 - f2) * f2 * (f1 - f3) * P.d23_2 * P.f3[2] - 4 * P.f1[2] * P.f2[3] * P.f3[2] * v1 +
          3 * f1 * P.f2[4] * P.f3[2] * v1 + 8 * P.f1[2] * P.f2[2] * P.f3[3] * v1 -
          4 * f1 * P.f2[3] * P.f3[3] * v1 - P.f2[4] * P.f3[3] * v1 - 4 * P.f1[2] * f2 * P.f3[4] * v1 -
          f1 * P.f2[2] * P.f3[4] * v1 + 2 * P.f2[3] * P.f3[4] * v1 + 2 * f1 * f2 * P.f3[5] * v1 -
          P.f2[2] * P.f3[5] * v1 + P.f1[5] * P.f3[2] * v2 - 3 * P.f1[4] * P.f3[3] * v2 +
          3 * P.f1[3] * P.f3[4] * v2 - P.f1[2] * P.f3[5] * v2 + P.f1[5] * P.f2[2] * v3 -
          2 * P.f1[4] * P.f2[3] * v3 + P.f1[3] * P.f2[4] * v3 - 2 * P.f1[5] * f2 * f3 * v3 +
          P.f1[4] * P.f2[2] * f3 * v3 + 4 * P.f1[3] * P.f2[3] * f3 * v3 - 3 * P.f1[2] * P.f2[4] * f3 * v3 +
          4 * P.f1[4] * f2 * P.f3[2] * v3 - 8 * P.f1[3] * P.f2[2] * P.f3[2] * v3 +
          4 * P.f1[2] * P.f2[3] * P.f3[2] * v3) /
         (P.d12_2 * P.d13_3 * P.d23_2);
}
GW_HD double delta1(double f1, double f2, double f3, double v1, double v2, double v3, double dd1, double dd3, double M) {
  const DeltaPowers P(f1, f2, f3, M);
  return (dd3 * f1 * P.d12_2 * (f1 - f3) * (f2 - f3) * (2 * f2 * f3 + f1 * (f2 + f3)) +
          f3 * (-(dd1 * (f1 - f2) * (f1 - f3) * P.d23_2 * (f2 * f3 + f1 * (2 * f2 + f3))) -
                2 * f1 *
                    (P.f3[4] * (v1 - v2) +
                     f1 * (2 * P.f3[3] * (-v1 + v2) - 4 * P.f2[3] * (v1 - v3) + 6 * P.f2[2] * f3 * (v1 - v3)) +
                     3 * P.f2[4] * (v1 - v3) + P.f1[4] * (v2 - v3) + 4 * P.f2[3] * f3 * (-v1 + v3) +
                     2 * P.f1[3] * f3 * (-v2 + v3)))) /
         (P.d12_2 * P.d13_3 * P.d23_2 * M);
}
GW_HD double delta2(double f1, double f2, double f3, double v1, double v2, double v3, double dd1, double dd3, double M) {
  const DeltaPowers P(f1, f2, f3, M);
  return (-(dd3 * P.d12_2 * (f1 - f3) * (f2 - f3) * (P.f1[2] + f2 * f3 + 2. * f1 * (f2 + f3))) +
          dd1 * (f1 - f3) * P.d23_2 * (-(f2 * f3 * (2 * f2 + f3)) + P.f1[2] * (f2 + 2 * f3) + f1 * (-P.f2[2] + P.f3[2])) -
          4 * P.f1[2] * P.f2[3] * v1 + 3 * f1 * P.f2[4] * v1 - 4 * f1 * P.f2[3] * f3 * v1 + 3 * P.f2[4] * f3 * v1 +
          12 * P.f1[2] * f2 * P.f3[2] * v1 - 4 * P.f2[3] * P.f3[2] * v1 - 8 * P.f1[2] * P.f3[3] * v1 +
          f1 * P.f3[4] * v1 + P.f3[5] * v1 + P.f1[5] * v2 + P.f1[4] * f3 * v2 - 8 * P.f1[3] * P.f3[2] * v2 +
          8 * P.f1[2] * P.f3[3] * v2 - f1 * P.f3[4] * v2 - P.f3[5] * v2 - P.f1[5] * v3 +
          4 * P.f1[2] * P.f2[3] * v3 - 3 * f1 * P.f2[4] * v3 - P.f1[4] * f3 * v3 + 4 * f1 * P.f2[3] * f3 * v3 -
          3 * P.f2[4] * f3 * v3 + 8 * P.f1[3] * P.f3[2] * v3 - 12 * P.f1[2] * f2 * P.f3[2] * v3 +
          4 * P.f2[3] * P.f3[2] * v3) /
         (P.d12_2 * P.d13_3 * P.d23_2 * P.m[2]);
}
GW_HD double delta3(double f1, double f2, double f3, double v1, double v2, double v3, double dd1, double dd3, double M) {
  const DeltaPowers P(f1, f2, f3, M);
  return (dd3 * P.d12_2 * (f1 - f3) * (f2 - f3) * (2 * f1 + f2 + f3) -
          dd1 * (f1 - f2) * (f1 - f3) * P.d23_2 * (f1 + f2 + 2 * f3) +
          2 * (P.f3[4] * (-v1 + v2) + 2 * P.f1[2] * P.d23_2 * (v1 - v3) + 2 * P.f2[2] * P.f3[2] * (v1 - v3) +
               2 * P.f1[3] * f3 * (v2 - v3) + P.f2[4] * (-v1 + v3) + P.f1[4] * (-v2 + v3) +
               2 * f1 * f3 * (P.f3[2] * (v1 - v2) + P.f2[2] * (v1 - v3) + 2 * f2 * f3 * (-v1 + v3)))) /
         (P.d12_2 * P.d13_3 * P.d23_2 * P.m[3]);
}
GW_HD double delta4(double f1, double f2, double f3, double v1, double v2, double v3, double dd1, double dd3, double M) {
  const DeltaPowers P(f1, f2, f3, M);
  return (-(dd3 * P.d12_2 * (f1 - f3) * (f2 - f3)) + dd1 * (f1 - f2) * (f1 - f3) * P.d23_2 -
          3 * f1 * P.f2[2] * v1 + 2 * P.f2[3] * v1 + 6 * f1 * f2 * f3 * v1 - 3 * P.f2[2] * f3 * v1 -
          3 * f1 * P.f3[2] * v1 + P.f3[3] * v1 + P.f1[3] * v2 - 3 * P.f1[2] * f3 * v2 + 3 * f1 * P.f3[2] * v2 -
          P.f3[3] * v2 - P.f1[3] * v3 + 3 * f1 * P.f2[2] * v3 - 2 * P.f2[3] * v3 + 3 * P.f1[2] * f3 * v3 -
          6 * f1 * f2 * f3 * v3 + 3 * P.f2[2] * f3 * v3) /
         (P.d12_2 * P.d13_3 * P.d23_2 * P.m[4]);
}

// amp_connection_coeffs (IMRPhenomD.cpp:1679-1702), in three parts so that the
// cooperative prologue can run them on different warps: the inspiral side
// (v1, dd1 at f1), the ringdown side (v3, dd3 at f3), then the deltas.
struct AmpConn {
  double v1, v3, dd1, dd3;
};
GW_HD void d_amp_conn_low(const ModelD &m, AmpConn &a) {
  Pows pw;
  precalc_powers_ins(m.s.f1, m.s.M, pw);
  a.v1 = amp_ins(m.s.f1, m, pw);
  a.dd1 = Damp_ins(m.s.f1, m);
}
GW_HD void d_amp_conn_high(const ModelD &m, AmpConn &a) {
  a.v3 = amp_mr(m.s.f3, m.s, m.l);
  a.dd3 = Damp_mr(m.s.f3, m.s, m.l);
}
GW_HD void d_deltas(ModelD &m, const AmpConn &a, int j0, int j1) {
  const Source &s = m.s;
  const double M = s.M, f1 = s.f1, f3 = s.f3, f2 = (f1 + f3) / 2., v2 = m.l.v2;
  for (int j = j0; j < j1; j++) {
    double d;
    switch (j) {
      case 0: d = delta0(f1, f2, f3, a.v1, v2, a.v3, a.dd1, a.dd3, M); break;
      case 1: d = delta1(f1, f2, f3, a.v1, v2, a.v3, a.dd1, a.dd3, M); break;
      case 2: d = delta2(f1, f2, f3, a.v1, v2, a.v3, a.dd1, a.dd3, M); break;
      case 3: d = delta3(f1, f2, f3, a.v1, v2, a.v3, a.dd1, a.dd3, M); break;
      default: d = delta4(f1, f2, f3, a.v1, v2, a.v3, a.dd1, a.dd3, M); break;
    }
    m.deltas[j] = d;
  }
}
// phase_connection_coefficients (IMRPhenomD.cpp:1614-1674)
// The C1 phase connection (IMRPhenomD.cpp: the beta0/beta1 and alpha0/alpha1
// constants) in parts: the inspiral values at f1, and the intermediate and
// merger-ringdown terms that do not involve the connection constants.  The
// two parts are independent (the cooperative prologue runs them at once);
// phase_conn_combine then forms the constants:
//   beta1  = eta/M (Dins(f1) - Dint(f1)|beta0=beta1=0)
//   beta0  = eta (ins(f1) - int(f1)|beta0=0)
//   alpha1 = eta/M (Dint(f2) - Dmr(f2)|alpha0=alpha1=0)
//   alpha0 = eta (int(f2) - mr(f2)|alpha0=0)
struct PhaseConnParts {
  double Dins1, ins1;      // inspiral derivative and phase at f1
  double Dint1, P1, Q1;    // at f1: Dint with beta1 = 0; beta2 ln Mf1; beta3 / 3 / Mf1^3
  double R2, S2, P2, Q2;   // at f2: beta2 / f2; beta3 / M^3 / f2^4; beta2 ln Mf2; beta3 / 3 / Mf2^3
  double Dmr2, T1, T2, T3; // at f2: Dmr with alpha1 = 0; alpha2 / Mf2; 4/3 alpha3 Mf2^(3/4); alpha4 atan(..)
  // model_d_finish: the phase at f_ref when it lies in the inspiral (have_phi),
  // the alpha1 fit, and the alpha1-free terms of Dphase_mr at f3
  double phi_fref, a1fit, A3, B3;
  int have_phi;
};
// The inspiral part in two halves (derivative, value), and the rest in two
// (terms at f1, terms at f2): four pieces that can run on four warps.
GW_HD void phase_conn_dins(const ModelD &m, PhaseConnParts &c) {
  double pn[12];  // coefficients 5 and 6 are set at f1 by the call
  for (int j = 0; j < 12; j++) pn[j] = m.pn_phase[j];
  c.Dins1 = Dphase_ins(m.s.f1_phase, m.s, pn, m.l);
}
GW_HD void phase_conn_phins(const ModelD &m, PhaseConnParts &c) {
  const Source &s = m.s;
  const double f1 = s.f1_phase;
  double pn[12];
  for (int j = 0; j < 12; j++) pn[j] = m.pn_phase[j];
  Pows pw;
  precalc_powers_ins(f1, s.M, pw);
  c.ins1 = phase_ins(f1, s, pn, m.l, m.pi, pw);
}
GW_HD void phase_conn_ins(const ModelD &m, PhaseConnParts &c) {
  phase_conn_dins(m, c);
  phase_conn_phins(m, c);
}
// Dphase_mr(f3) (IMRPhenomD.cpp:1539-1554) = (A3 + M (alpha1 + B3)) / eta;
// f3 = fpeak as model_d_freqs sets it (passed, so that this can run beside it).
GW_HD void finish_f3_terms(const ModelD &m, double f3, PhaseConnParts &c) {
  const Source &s = m.s;
  const Lambda &l = m.l;
  const double f = f3, M = s.M, u = f - l.alpha[5] * s.fRD;
  c.A3 = l.alpha[4] / (s.fdamp * (1. + (u * u) / (s.fdamp * s.fdamp))) + l.alpha[2] / ((f * f) * M);
  c.B3 = l.alpha[3] / sqrt(sqrt(f * M));
}
// The phase at f_ref when f_ref is in the inspiral part (the common case: it
// needs neither the matching frequencies nor the connection constants).
GW_HD void finish_fref_phase(const ModelD &m, PhaseConnParts &c) {
  const Source &s = m.s;
  c.have_phi = 0;
  if (!s.shift_phase || !(s.f_ref < 0.018 / (s.M))) return;  // f1_phase = 0.018 / M
  Pows pw;
  precalc_powers_ins(s.f_ref, s.M, pw);
  double pn[12];
  for (int j = 0; j < 12; j++) pn[j] = m.pn_phase[j];
  c.phi_fref = phase_ins(s.f_ref, s, pn, m.l, m.pi, pw);
  c.have_phi = 1;
}
GW_HD void phase_conn_imr1(const ModelD &m, PhaseConnParts &c) {
  const Source &s = m.s;
  const Lambda &l = m.l;
  const double M = s.M, M3 = M * M * M;
  c.a1fit = l.alpha[1];  // still the fit: the connection replaces it
  {
    const double f = s.f1_phase, ff = f * f, Mf = M * f, Mf3 = Mf * Mf * Mf;
    c.Dint1 = s.inv_eta * (l.beta[2] / f + l.beta[3] / M3 / (ff * ff));
    c.P1 = l.beta[2] * log(Mf);
    c.Q1 = l.beta[3] / 3. * 1. / Mf3;
  }
}
GW_HD void phase_conn_imr2(const ModelD &m, PhaseConnParts &c) {
  const Source &s = m.s;
  const Lambda &l = m.l;
  const double M = s.M, eta = s.eta, M3 = M * M * M;
  {
    const double f = s.f2_phase, ff = f * f, Mf = M * f, Mf3 = Mf * Mf * Mf;
    c.R2 = l.beta[2] / f;
    c.S2 = l.beta[3] / M3 / (ff * ff);
    c.P2 = l.beta[2] * log(Mf);
    c.Q2 = l.beta[3] / 3. * 1. / Mf3;
    const double u = f - l.alpha[5] * s.fRD;
    c.Dmr2 = (l.alpha[4] / (s.fdamp * (1. + (u * u) / (s.fdamp * s.fdamp))) + l.alpha[2] / ((f * f) * M) +
              M * (l.alpha[3] / sqrt(sqrt(f * M)))) /
             eta;
    c.T1 = l.alpha[2] * (1. / (Mf));
    c.T2 = (4. / 3) * l.alpha[3] * sqrt(sqrt(Mf * Mf * Mf));
    c.T3 = l.alpha[4] * atan((f - l.alpha[5] * s.fRD) / s.fdamp);
  }
}
GW_HD void phase_conn_imr(const ModelD &m, PhaseConnParts &c) {
  phase_conn_imr1(m, c);
  phase_conn_imr2(m, c);
}
GW_HD void phase_conn_combine(ModelD &m, const PhaseConnParts &c) {
  const Source &s = m.s;
  Lambda &l = m.l;
  const double M = s.M, eta = s.eta;
  l.beta[1] = (eta / M) * c.Dins1 - (eta / M) * c.Dint1;
  {
    const double Mf = M * s.f1_phase;
    const double intval = s.inv_eta * (l.beta[1] * Mf + c.P1 - c.Q1);
    l.beta[0] = (eta)*c.ins1 - eta * intval;
  }
  {
    const double Dint = s.inv_eta * (l.beta[1] * M + c.R2 + c.S2);
    l.alpha[1] = (eta / M) * Dint - eta / M * c.Dmr2;
  }
  {
    const double Mf = M * s.f2_phase;
    const double intval = s.inv_eta * (l.beta[0] + l.beta[1] * Mf + c.P2 - c.Q2);
    const double mr = s.inv_eta * (l.alpha[1] * Mf - c.T1 + c.T2 + c.T3);
    l.alpha[0] = (eta)*intval - eta * mr;
  }
}
GW_HD void d_phase_conn(ModelD &m) {
  PhaseConnParts c;
  phase_conn_ins(m, c);
  phase_conn_imr(m, c);
  phase_conn_combine(m, c);
}
GW_HDNI void d_connections(ModelD &m) {
  AmpConn a;
  d_amp_conn_low(m, a);
  d_amp_conn_high(m, a);
  d_deltas(m, a, 0, 5);
  d_phase_conn(m);
}

// Model setup shared by D and Pv2 (IMRPhenomD.cpp:410-432), in stages:
// calibration fits, ringdown frequencies (post_merger), matching frequencies,
// PN coefficients, connection coefficients.
// The fits in two independent halves (amplitude and inspiral; intermediate
// and merger-ringdown phase), and the powers of pi.
GW_HD void model_d_lambdas_a(ModelD &m) {
  const Source &s = m.s;
  Lambda &l = m.l;
  for (int i = 0; i < 4; i++) l.rho[i] = 0, l.gamma[i] = 0;
  for (int i = 0; i < 5; i++) l.sigma[i] = 0;
  for (int i = 0; i < 3; i++) l.rho[i] = lambda_elem(s, i);  // IMRPhenomD.cpp:833-852
  l.v2 = lambda_elem(s, 3);
  for (int i = 0; i < 3; i++) l.gamma[i] = lambda_elem(s, i + 4);
  for (int i = 0; i < 4; i++) l.sigma[i + 1] = lambda_elem(s, i + 7);
  precalc_powers_PI(m.pi);
}
GW_HD void model_d_lambdas_b(ModelD &m) {
  const Source &s = m.s;
  Lambda &l = m.l;
  for (int i = 0; i < 5; i++) l.beta[i] = 0;
  for (int i = 0; i < 7; i++) l.alpha[i] = 0;
  for (int i = 0; i < 3; i++) l.beta[i + 1] = lambda_elem(s, i + 11);
  for (int i = 0; i < 5; i++) l.alpha[i + 1] = lambda_elem(s, i + 14);
}
GW_HD void model_d_lambdas(ModelD &m) {
  model_d_lambdas_a(m);
  model_d_lambdas_b(m);
}
// The same fits in kLambdaSlots interleaved slots (fit i in slot i % 4), for
// slots running the same instructions on different lanes: slot 0 also clears
// the entries no fit sets and fills the powers of pi.
constexpr int kLambdaFits = 19, kLambdaSlots = 4;
GW_HD void model_d_lambdas_slot(ModelD &m, int slot) {
  const Source &s = m.s;
  Lambda &l = m.l;
  if (slot == 0) {
    l.rho[3] = l.gamma[3] = l.sigma[0] = l.beta[0] = l.beta[4] = l.alpha[0] = l.alpha[6] = 0;
    precalc_powers_PI(m.pi);
  }
  for (int i = slot; i < kLambdaFits; i += kLambdaSlots) {
    const double v = lambda_elem(s, i);  // IMRPhenomD.cpp:833-852
    double *dst = i < 3 ? &l.rho[i] : i == 3 ? &l.v2 : i < 7 ? &l.gamma[i - 4] : i < 11 ? &l.sigma[i - 6]
                : i < 14 ? &l.beta[i - 10] : &l.alpha[i - 13];
    *dst = v;
  }
}
// needs the fits and post_merger
GW_HD void model_d_freqs(ModelD &m) {
  Source &s = m.s;
  s.f1_phase = 0.018 / (s.M);
  s.f2_phase = s.fRD / 2.;
  s.f1 = 0.014 / (s.M);
  s.f3 = fpeak(s, m.l);
  for (int i = 0; i < 5; i++) m.deltas[i] = 0;
  m.fcut = .2 / s.M;
  m.status = kModelOK;
  if (!(s.eta > 0 && s.eta <= 0.25 + 1e-12) || !(s.fRD > 0) || !(s.fdamp > 0) || !(s.M > 0)) m.status |= kModelQnmRange;
}
GW_HD void model_d_pn(ModelD &m) {
  pn_amp_coeff(m.s, m.pn_amp);
  pn_phase_coeff_static(m.s, m.pn_phase);
}
GW_HDNI int model_d_prologue(ModelD &m, const double *qnm) {
  model_d_lambdas(m);
  post_merger(m.s, qnm);
  model_d_freqs(m);
  model_d_pn(m);
  d_connections(m);
  return m.status;
}

// D-specific phase/time shift and amplitude scale (IMRPhenomD.cpp:434-470)
GW_HD void model_d_finish_parts(ModelD &m, const PhaseConnParts &c) {
  Source &s = m.s;
  double M = s.M;
  if (s.shift_phase) {
    m.fref = s.f_ref;
    double phi_shift;
    if (c.have_phi) {
      phi_shift = c.phi_fref;
    } else {
      Pows pw;
      precalc_powers_ins(m.fref, M, pw);
      double pn[12];
      for (int j = 0; j < 12; j++) pn[j] = m.pn_phase[j];
      phi_shift = build_phase(m.fref, m, pn, pw);
    }
    m.phic = 2 * s.phiRef + phi_shift;
  } else {
    m.fref = 0;
    m.phic = s.phiRef;
  }
  double tc_shift = 0;
  if (s.shift_time) {
    const double Dmr = (c.A3 + M * (m.l.alpha[1] + c.B3)) / s.eta;
    tc_shift = Dmr + (-m.l.alpha[1] + c.a1fit) * s.M / s.eta;
  }
  m.tcl = 2 * kPi * s.tc + tc_shift;
  m.A0eff = s.A0 * pow_7_6(M);
}
GW_HDNI void model_d_finish(ModelD &m) {
  PhaseConnParts c;
  finish_fref_phase(m, c);
  finish_f3_terms(m, m.s.f3, c);
  c.a1fit = lambda_elem(m.s, 14);
  model_d_finish_parts(m, c);
}

// ------------------------------------------------------------- IMRPhenomPv2
GW_HD double L2PN(double eta, double MF2third, double PI2third) {  // IMRPhenomP.cpp:1214-1220
  double x = MF2third * PI2third, x2 = x * x, eta2 = eta * eta;
  return (eta * (1.0 + (1.5 + eta / 6.0) * x + (3.375 - (19.0 * eta) / 8. - eta2 / 24.0) * x2)) / sqrt(x);
}
// PhenomPv2_Param_Transform (IMRPhenomP.cpp:1082-1210) / _reduced (:822-938)
GW_HDNI void pv2_transform(Source &s, int reduced) {
  double chi1_l = s.spin1z, chi2_l = s.spin2z;
  double q = s.mass1 / s.mass2;
  double chi_eff = (s.mass1 * chi1_l + s.mass2 * chi2_l) / s.M;
  s.chil = (1.0 + q) / q * chi_eff;
  double m1_2 = s.mass1 * s.mass1, m2_2 = s.mass2 * s.mass2;
  if (!reduced) {
    double S1_perp = m1_2 * sqrt(s.spin1y * s.spin1y + s.spin1x * s.spin1x);
    double S2_perp = m2_2 * sqrt(s.spin2y * s.spin2y + s.spin2x * s.spin2x);
    double A1 = 2 + (3 * s.mass2) / (2 * s.mass1), A2 = 2 + (3 * s.mass1) / (2 * s.mass2);
    double ASp1 = A1 * S1_perp, ASp2 = A2 * S2_perp;
    double num = (ASp2 > ASp1) ? ASp2 : ASp1;
    double denom = (s.mass2 > s.mass1) ? A2 * m2_2 : A1 * m1_2;
    s.chip = num / denom;
  }
  double m1 = q / (1 + q), m2 = 1. / (1 + q);
  s.SP = s.chip * m1 * m1;
  s.SL = chi1_l * m1 * m1 + chi2_l * m2 * m2;
  Pows pw, pp;
  precalc_powers_PI(pp);
  precalc_powers_ins(s.f_ref, s.M, pw);
  double L0 = s.M * s.M * L2PN(s.eta, pw.MF2third, pp.PI2third);
  double J0x, J0y, J0z;
  if (!reduced) {
    J0x = m1_2 * s.spin1x + m2_2 * s.spin2x;
    J0y = m1_2 * s.spin1y + m2_2 * s.spin2y;
  } else {
    double sp, cp;
    sincos(s.phip, &sp, &cp);
    J0x = m1_2 * s.chip * cp;
    J0y = m1_2 * s.chip * sp;
  }
  J0z = L0 + m1_2 * s.spin1z + m2_2 * s.spin2z;
  double J0 = sqrt(J0x * J0x + J0y * J0y + J0z * J0z);
  double thetaJ_sf = acos(J0z / J0);
  double phiJ_sf = atan2(J0y, J0x);
  s.phi_aligned = -phiJ_sf;
  // the reference's rotations (ROTATEZ / ROTATEY), each angle's sine and
  // cosine evaluated once
  double incl = s.incl_angle, phiRef = s.phiRef;
  double si, ci, sq, cq, sr, cr, sA, cA, sB, cB, sK, cK;
  sincos(incl, &si, &ci);
  sincos(kPi / 2. - phiRef, &sq, &cq);
  sincos(phiRef, &sr, &cr);
  sincos(-phiJ_sf, &sA, &cA);
  sincos(-thetaJ_sf, &sB, &cB);
  auto rotz = [](double c, double sn, double &vx, double &vy) {
    const double t1 = vx * c - vy * sn, t2 = vx * sn + vy * c;
    vx = t1;
    vy = t2;
  };
  auto roty = [](double c, double sn, double &vx, double &vz) {
    const double t1 = vx * c + vz * sn, t2 = -vx * sn + vz * c;
    vx = t1;
    vz = t2;
  };
  double Nx_sf = si * cq, Ny_sf = si * sq, Nz_sf = ci;
  double tx = Nx_sf, ty = Ny_sf, tz = Nz_sf;
  rotz(cA, sA, tx, ty);
  roty(cB, sB, tx, tz);
  double kappa = -atan2(ty, tx);
  sincos(kappa, &sK, &cK);
  tx = 0.;
  ty = 0.;
  tz = 1.;
  rotz(cA, sA, tx, ty);
  roty(cB, sB, tx, tz);
  rotz(cK, sK, tx, ty);
  s.alpha0 = atan2(ty, tx);
  tx = Nx_sf;
  ty = Ny_sf;
  tz = Nz_sf;
  rotz(cA, sA, tx, ty);
  roty(cB, sB, tx, tz);
  rotz(cK, sK, tx, ty);
  double Nx_Jf = tx, Nz_Jf = tz;
  s.thetaJN = acos(Nz_Jf);
  tx = -ci * sr;
  ty = -ci * cr;
  tz = si;
  rotz(cA, sA, tx, ty);
  roty(cB, sB, tx, tz);
  rotz(cK, sK, tx, ty);
  double XdotPArun = tx * 0. + ty * -1. + tz * 0.;
  double XdotQArun = tx * Nz_Jf + ty * 0. + tz * -Nx_Jf;
  s.zeta_polariz = atan2(XdotQArun, XdotPArun);
}

GW_HDNI void pv2_euler_coeffs(double *a, double *e, const Source &s) {  // IMRPhenomP.cpp:65-144
  double m2 = s.q / (1. + s.q), m1 = 1. / (1. + s.q), dm = m1 - m2;
  double eta = m1 * m2, eta2 = eta * eta;
  double chil = s.chil, chil2 = chil * chil, chip2 = s.chip * s.chip, chip4 = chip2 * chip2;
  double dm2 = dm * dm, dm3 = dm2 * dm;
  double m2_2 = m2 * m2, m2_3 = m2_2 * m2, m2_4 = m2_3 * m2, m2_5 = m2_4 * m2, m2_6 = m2_5 * m2, m2_7 = m2_6 * m2,
         m2_8 = m2_7 * m2;
  // the reference's quotients as products with these inverses (mtot = 1), and
  // constant denominators folded
  const double im2 = 1. / m2, ieta = 1. / eta;
  const double im2_2 = im2 * im2, im2_3 = im2_2 * im2, ieta2 = ieta * ieta, ieta3 = ieta2 * ieta, ieta4 = ieta3 * ieta;
  a[0] = (-0.18229166666666666 - ((5 * dm) * (1. / 64.) * im2));
  a[1] = (((-15 * dm * m2 * chil) * (1. / 128.) * ieta) - ((35 * m2_2 * chil) * (1. / 128.) * ieta));
  a[2] = (-1.7952473958333333 - ((4555 * dm) * (1. / 7168.) * im2) - ((15 * chip2 * dm * m2_3) * (1. / 128.) * ieta2) -
          ((35 * chip2 * m2_4) * (1. / 128.) * ieta2) - ((515 * eta) * (1. / 384.)) - ((15 * dm2 * eta) * (1. / 256.) * im2_2) -
          ((175 * dm * eta) * (1. / 256.) * im2));
  a[3] = -((35 * kPi) * (1. / 48.)) - ((5 * dm * kPi) * (1. / 16.) * im2) + ((5 * dm2 * chil) * (1. / 16.)) +
         ((5 * dm * m2 * chil) * (1. / 3.)) + ((2545 * m2_2 * chil) * (1. / 1152.)) -
         ((5 * chip2 * dm * m2_5 * chil) * (1. / 128.) * ieta3) - ((35 * chip2 * m2_6 * chil) * (1. / 384.) * ieta3) +
         ((2035 * dm * m2 * chil) * (1. / 21504.) * ieta) + ((2995 * m2_2 * chil) * (1. / 9216.) * ieta);
  a[4] = (4.318908476114694 + ((27895885 * dm) * (1. / 2.1676032e7) * im2) - ((15 * chip4 * dm * m2_7) * (1. / 512.) * ieta4) -
          ((35 * chip4 * m2_8) * (1. / 512.) * ieta4) - ((485 * chip2 * dm * m2_3) * (1. / 14336.) * ieta2) +
          ((475 * chip2 * m2_4) * (1. / 6144.) * ieta2) + ((15 * chip2 * dm2 * m2_2) * (1. / 256.) * ieta) +
          ((145 * chip2 * dm * m2_3) * (1. / 512.) * ieta) + ((575 * chip2 * m2_4) * (1. / 1536.) * ieta) +
          ((39695 * eta) * (1. / 86016.)) + ((1615 * dm2 * eta) * (1. / 28672.) * im2_2) - ((265 * dm * eta) * (1. / 14336.) * im2) +
          ((955 * eta2) * (1. / 576.)) + ((15 * dm3 * eta2) * (1. / 1024.) * im2_3) + ((35 * dm2 * eta2) * (1. / 256.) * im2_2) +
          ((2725 * dm * eta2) * (1. / 3072.) * im2) - ((15 * dm * m2 * kPi * chil) * (1. / 16.) * ieta) -
          ((35 * m2_2 * kPi * chil) * (1. / 16.) * ieta) + ((15 * chip2 * dm * m2_7 * chil2) * (1. / 128.) * ieta4) +
          ((35 * chip2 * m2_8 * chil2) * (1. / 128.) * ieta4) + ((375 * dm2 * m2_2 * chil2) * (1. / 256.) * ieta) +
          ((1815 * dm * m2_3 * chil2) * (1. / 256.) * ieta) + ((1645 * m2_4 * chil2) * (1. / 192.) * ieta));
  e[0] = (-0.18229166666666666 - ((5 * dm) * (1. / 64.) * im2));
  e[1] = (((-15 * dm * m2 * chil) * (1. / 128.) * ieta) - ((35 * m2_2 * chil) * (1. / 128.) * ieta));
  e[2] = (-1.7952473958333333 - ((4555 * dm) * (1. / 7168.) * im2) - ((515 * eta) * (1. / 384.)) - ((15 * dm2 * eta) * (1. / 256.) * im2_2) -
          ((175 * dm * eta) * (1. / 256.) * im2));
  e[3] = -((35 * kPi) * (1. / 48.)) - ((5 * dm * kPi) * (1. / 16.) * im2) + ((5 * dm2 * chil) * (1. / 16.)) +
         ((5 * dm * m2 * chil) * (1. / 3.)) + ((2545 * m2_2 * chil) * (1. / 1152.)) +
         ((2035 * dm * m2 * chil) * (1. / 21504.) * ieta) + ((2995 * m2_2 * chil) * (1. / 9216.) * ieta);
  e[4] = (4.318908476114694 + ((27895885 * dm) * (1. / 2.1676032e7) * im2) + ((39695 * eta) * (1. / 86016.)) +
          ((1615 * dm2 * eta) * (1. / 28672.) * im2_2) - ((265 * dm * eta) * (1. / 14336.) * im2) + ((955 * eta2) * (1. / 576.)) +
          ((15 * dm3 * eta2) * (1. / 1024.) * im2_3) + ((35 * dm2 * eta2) * (1. / 256.) * im2_2) + ((2725 * dm * eta2) * (1. / 3072.) * im2) -
          ((15 * dm * m2 * kPi * chil) * (1. / 16.) * ieta) - ((35 * m2_2 * kPi * chil) * (1. / 16.) * ieta) +
          ((375 * dm2 * m2_2 * chil2) * (1. / 256.) * ieta) + ((1815 * dm * m2_3 * chil2) * (1. / 256.) * ieta) +
          ((1645 * m2_4 * chil2) * (1. / 192.) * ieta));
}
// calculate_euler_angles (IMRPhenomP.cpp:717-735) from MFthird
GW_HD void pv2_euler_angles(double &alpha, double &eps, double MFthird, double PIthird, const double *a,
                            const double *e) {
  double oc = MFthird * PIthird, oc2 = oc * oc;
  double logomega = log(oc2 * oc), omega = oc2 * oc;
  alpha = (a[0] / omega + a[1] / oc2 + a[2] / oc + a[3] * logomega + a[4] * oc);
  eps = (e[0] / omega + e[1] / oc2 + e[2] / oc + e[3] * logomega + e[4] * oc);
}
// calculate_time_shift (IMRPhenomP.cpp:551-606): d/df of a 10-node natural
// spline of -phi(f) over [0.8, 1.2] fRD, at fRD, over 2 pi.
// Node j of the spline: -phi(f_j), f_j = 0.8 fRD + j (0.4 fRD / 9).
constexpr int kPv2ShiftNodes = 10;
GW_HD double pv2_shift_freq(const ModelD &m, int j) {
  double fs = .8 * (m.s.fRD), fe = 1.2 * (m.s.fRD);
  return fs + j * ((fe - fs) / (kPv2ShiftNodes - 1));
}
GW_HD double pv2_shift_node(const ModelD &m, int j) {
  double pn[12];
  for (int i = 0; i < 12; i++) pn[i] = m.pn_phase[i];
  double f = pv2_shift_freq(m, j);
  Pows pw;
  precalc_powers_ins(f, m.s.M, pw);
  return -build_phase(f, m, pn, pw);
}
GW_HD double pv2_shift_solve(const ModelD &m, const double *ph) {
  double ff[kPv2ShiftNodes], cc[kPv2ShiftNodes], work[3 * kPv2ShiftNodes];
  double fs = .8 * (m.s.fRD), fe = 1.2 * (m.s.fRD);
  double dfx = (fe - fs) / (kPv2ShiftNodes - 1);
  if (dfx != dfx || dfx <= 0) return 0;
  for (int j = 0; j < kPv2ShiftNodes; j++) ff[j] = pv2_shift_freq(m, j);
  cspline_coeffs(ff, ph, kPv2ShiftNodes, cc, work);
  return cspline_eval(ff, ph, cc, kPv2ShiftNodes, m.s.fRD, 1) / (2. * kPi);
}
GW_HDNI double pv2_time_shift(const ModelD &m) {
  double fs = .8 * (m.s.fRD), fe = 1.2 * (m.s.fRD);
  double dfx = (fe - fs) / (kPv2ShiftNodes - 1);
  if (dfx != dfx || dfx <= 0) return 0;
  double ph[kPv2ShiftNodes];
  for (int j = 0; j < kPv2ShiftNodes; j++) ph[j] = pv2_shift_node(m, j);
  return pv2_shift_solve(m, ph);
}

// Full Pv2 per-request setup: transform, D model, Euler/harmonic constants,
// time shift (IMRPhenomP.cpp:195-262, 345-351; waveform_generator.cpp:1272-1281).
// Pv2 stages: the J-frame transform and harmonics (before the D model, whose
// final spin uses chi_p), and the constants that need the D model's matching
// frequencies (before the time shift, which needs its full phase).
GW_HD void model_p_setup(ModelD &m, ModelP &pm, const GenParams &in) {
  Source &s = m.s;
  s.pv2 = 1;
  if ((in.chip + 1) > kCompThresh) {
    s.chip = in.chip;
    s.spin1z = in.spin1[2];
    s.spin2z = in.spin2[2];
    s.phip = in.phip;
    pv2_transform(s, 1);
  } else {
    pv2_transform(s, 0);
  }
  // the s = -2, l = 2 spin-weighted harmonics Y_2m(thetaJN, 0), m = -2..2
  // (XLALSpinWeightedSphericalHarmonic, util.cpp:1953-2333), from one sincos
  double st, ct;
  sincos(s.thetaJN, &st, &ct);
  pm.Y[0] = sqrt(5.0 / (64.0 * kPi)) * (1.0 - ct) * (1.0 - ct);
  pm.Y[1] = sqrt(5.0 / (16.0 * kPi)) * st * (1.0 - ct);
  pm.Y[2] = sqrt(15.0 / (32.0 * kPi)) * st * st;
  pm.Y[3] = sqrt(5.0 / (16.0 * kPi)) * st * (1.0 + ct);
  pm.Y[4] = sqrt(5.0 / (64.0 * kPi)) * (1.0 + ct) * (1.0 + ct);
}
GW_HDNI void model_p_finish(ModelD &m, ModelP &pm) {
  Source &s = m.s;
  m.fref = s.f_ref;
  m.phic = 2 * s.phi_aligned;
  m.tcl = 2 * kPi * s.tc;
  m.A0eff = s.A0 * pow_7_6(s.M) / (2. * sqrt(5. / (64. * kPi)));
  s.q = s.mass1 / s.mass2;
  pv2_euler_coeffs(pm.ac, pm.ec, s);
  double MFthird = cbrt(s.M * s.f_ref);
  double aoff, eoff;
  pv2_euler_angles(aoff, eoff, MFthird, m.pi.PIthird, pm.ac, pm.ec);
  pm.alpha_shift = s.alpha0 - aoff;
  pm.eps_off = eoff;
  sincos(2. * s.zeta_polariz, &pm.s2z, &pm.c2z);
  if (!(s.f_ref > 0)) m.status |= kModelBadInput;
}
GW_HDNI int model_p_prologue(ModelD &m, ModelP &pm, const GenParams &in, const double *qnm) {
  model_p_setup(m, pm, in);
  model_d_prologue(m, qnm);
  model_p_finish(m, pm);
  pm.t_corr = m.s.shift_time ? pv2_time_shift(m) : 0.0;
  return m.status;
}

// ------------------------------------------------------------- detectors
// Sky-position trigonometry shared by every detector of a request.
struct SkyTrig {
  double cg, sg, cd, sd, cp, sp;  // cos/sin of the hour angle gmst - RA, of DEC and of psi
};
GW_HD void sky_trig(double ra, double dec, double psi, double gmst, SkyTrig &t) {
  double gha = gmst - ra;
  sincos(gha, &t.sg, &t.cg);
  sincos(dec, &t.sd, &t.cd);
  sincos(psi, &t.sp, &t.cp);
}
GW_HD void antenna_trig(int det, const SkyTrig &t, double &fp, double &fc) {
  // detector_util.cpp:901-1015, geometric factor detector_util.cpp:1158-1160
  const double *D = GWT_T(gwt_det_tensor)[det];
  double X[3], Y[3];
  const double cg = t.cg, sg = t.sg, cd = t.cd, sd = t.sd, cp = t.cp, sp = t.sp;
  X[0] = -cp * sg - sp * cg * sd;
  X[1] = -cp * cg + sp * sg * sd;
  X[2] = sp * cd;
  Y[0] = sp * sg - cp * cg * sd;
  Y[1] = sp * cg + cp * sg * sd;
  Y[2] = cp * cd;
  fp = 0.0;
  fc = 0.0;
  for (int i = 0; i < 3; i++) {
    double DX = D[i * 3 + 0] * X[0] + D[i * 3 + 1] * X[1] + D[i * 3 + 2] * X[2];
    double DY = D[i * 3 + 0] * Y[0] + D[i * 3 + 1] * Y[1] + D[i * 3 + 2] * Y[2];
    fp += X[i] * DX - Y[i] * DY;
    fc += X[i] * DY + Y[i] * DX;
  }
  fp *= GWT_T(gwt_det_geometric)[det];
  fc *= GWT_T(gwt_det_geometric)[det];
}
GW_HD void antenna(int det, double ra, double dec, double psi, double gmst, double &fp, double &fc) {
  SkyTrig t;
  sky_trig(ra, dec, psi, gmst, t);
  antenna_trig(det, t, fp, fc);
}
GW_HD double dtoa_trig(const SkyTrig &t, int d1, int d2) {  // detector_util.cpp:760-780
  const double *l1 = GWT_T(gwt_det_location)[d1], *l2 = GWT_T(gwt_det_location)[d2];
  double e0 = t.cd * t.cg, e1 = t.cd * -t.sg, e2 = t.sd;
  return ((l1[0] - l2[0]) * e0 + (l1[1] - l2[1]) * e1 + (l1[2] - l2[2]) * e2) / kC;
}
GW_HD double dtoa(double RA, double DEC, double gmst, int d1, int d2) {
  SkyTrig t;
  sky_trig(RA, DEC, 0.0, gmst, t);
  return dtoa_trig(t, d1, d2);
}

// Everything one likelihood request needs.
struct Request {
  ModelD m;
  ModelP p;
  DetProj det[kMaxDet];
  int approximant, ndet;
};

// Full prologue of one request.  `in.tc` must already hold the t_c the model
// sees (MCMC_likelihood_extrinsic replaces it by T - t_c, mcmc_gw.cpp:2466-2473).
GW_HDNI int request_prologue(Request &r, const GenParams &in, int approximant, const int *dets, int ndet,
                             const double *qnm) {
  r.approximant = approximant;
  r.ndet = ndet;
  populate(r.m.s, in);
  int st;
  if (approximant == kPhenomPv2) {
    st = model_p_prologue(r.m, r.p, in, qnm);
  } else {
    st = model_d_prologue(r.m, qnm);
    model_d_finish(r.m);
    st = r.m.status;
  }
  SkyTrig tr;
  sky_trig(in.RA, in.DEC, in.psi, in.gmst, tr);
  for (int i = 0; i < ndet && i < kMaxDet; i++) {
    antenna_trig(dets[i], tr, r.det[i].fp, r.det[i].fc);
    double DTOA = dtoa_trig(tr, dets[0], dets[i]);
    double tc = -DTOA;
    tc *= 2 * kPi;
    r.det[i].tau = tc;
  }
  return st;
}

}  // namespace gwt

namespace gwt {

// ------------------------------------------------------- Fisher parameters
// unpack_parameters (fisher.cpp:1841-1961) / repack_parameters (fisher.cpp:2168-2300)
// for "IMRPhenomD" (method 0: [RA, DEC, psi, iota, phiRef, tc, D_L*, M_c*, eta,
// chi1, chi2], * = log factor) and "MCMC_IMRPhenomD" (method 1: [RA, sin DEC,
// psi, cos iota, phiRef, tc, ln D_L, ln M_c, eta, chi1, chi2]).
constexpr int kFisherDim = 11;

GW_HD void fisher_unpack(const GenParams &p, int method, double *v, int *logf) {
  for (int i = 0; i < kFisherDim; i++) logf[i] = 0;
  int mcmc = (method == 1);
  double mc = calc_chirpmass(p.mass1, p.mass2), eta = calc_eta(p.mass1, p.mass2);
  v[0] = p.RA;
  v[1] = mcmc ? sin(p.DEC) : p.DEC;
  if (p.equatorial_orientation) {  // L's equatorial angles stand for psi, iota (fisher.cpp:1916-1919, 1944-1947)
    v[2] = p.theta_l;
    v[3] = p.phi_l;
  } else {
    v[2] = p.psi;
    v[3] = mcmc ? cos(p.incl_angle) : p.incl_angle;
  }
  v[4] = p.phiRef;
  v[5] = p.tc;
  if (mcmc) {
    v[6] = log(p.Luminosity_Distance);
    v[7] = log(mc);
  } else {
    logf[6] = 1;
    logf[7] = 1;
    v[6] = p.Luminosity_Distance;
    v[7] = mc;
  }
  v[8] = eta;
  v[9] = p.spin1[2];
  v[10] = p.spin2[2];
}

// ------------------------------------------------- equatorial orientation
// Polarisation and inclination of a direction (th, ph) in equatorial
// coordinates seen from the sky position (ra, dec): tan(pi/2 - psi) =
// cos(dec) cot(th) / sin(ph - ra) - cot(ph - ra) sin(dec), and the angle to the
// propagation direction -N (terr_pol_iota_from_equat_sph, util.cpp:1362-1378).
GW_HD void pol_incl_of_direction(double ra, double dec, double th, double ph, double &pol, double &incl) {
  const double cd = cos(dec), sd = sin(dec);
  pol = kPi / 2. - atan(cd * 1. / tan(th) * 1. / sin(ph - ra) - 1. / tan(ph - ra) * sd);
  incl = acos(-(cos(th) * sd) - cd * cos(ph - ra) * sin(th));
}

// transform_orientation_coords (waveform_util.cpp:1523-1586) for a ground
// detector.  IMRPhenomD: inclination and polarisation of L itself.
// IMRPhenomPv2: the inclination is the angle between L and the line of sight N;
// the polarisation is that of the total angular momentum J.  J's direction in
// the source frame (L along z) is J0 = (m1^2 chip cos phip, m1^2 chip sin phip,
// L0 + m1^2 chi1z + m2^2 chi2z), L0 = M^2 L2PN at f_ref
// (PhenomPv2_JSF_from_params, IMRPhenomP.cpp:776-816); it is carried to
// equatorial coordinates by the rotation that takes the source frame's (L, N,
// L x N) to their equatorial directions (equatorial_from_SF, util.cpp:1440-1485).
GW_HD void orientation_transform(GenParams &p, int approx) {
  const double ths = kPi / 2. - p.DEC, phs = p.RA;
  const double n0 = -sin(ths) * cos(phs), n1 = -sin(ths) * sin(phs), n2 = -cos(ths);
  const double l0 = sin(p.theta_l) * cos(p.phi_l), l1 = sin(p.theta_l) * sin(p.phi_l), l2 = cos(p.theta_l);
  p.incl_angle = acos(n0 * l0 + n1 * l1 + n2 * l2);
  if (approx != kPhenomPv2) {
    pol_incl_of_direction(p.RA, p.DEC, p.theta_l, p.phi_l, p.psi, p.incl_angle);
    return;
  }
  // J in the source frame
  const double eta = calc_eta(p.mass1, p.mass2);
  const double m1sq = p.mass1 * p.mass1, m2sq = p.mass2 * p.mass2;
  Pows pw;
  precalc_powers_PI(pw);
  precalc_powers_ins(p.f_ref, (p.mass1 + p.mass2) * kMsolSec, pw);
  const double Mt = p.mass1 + p.mass2;
  const double Lz = Mt * Mt * L2PN(eta, pw.MF2third, pw.PI2third);
  double jx = m1sq * p.chip * cos(p.phip), jy = m1sq * p.chip * sin(p.phip), jz = Lz + m1sq * p.spin1[2] +
                                                                                  m2sq * p.spin2[2];
  const double jn = sqrt(jx * jx + jy * jy + jz * jz);
  jx /= jn;
  jy /= jn;
  jz /= jn;
  // rotated to equatorial coordinates
  const double cp = cos(kPi / 2. - p.phiRef), sp = sin(kPi / 2. - p.phiRef);
  const double ci = cos(p.incl_angle), si = sin(p.incl_angle);
  const double ctl = cos(p.theta_l), stl = sin(p.theta_l), cts = cos(ths), sts = sin(ths);
  const double cps = cos(phs), sps = sin(phs), cpl = cos(p.phi_l), spl = sin(p.phi_l);
  const double cp2 = cp * cp;
  const double ex = (cp2 * cpl * jz * si * stl - ci * cpl * (cp * jx + jy * sp) * stl -
                     cp * (cts * jy * spl * stl + cps * jx * sts - ctl * jy * sps * sts) +
                     sp * (cpl * jz * si * sp * stl + cts * jx * spl * stl - (cps * jy + ctl * jx * sps) * sts)) /
                    si;
  const double ey = (cp2 * jz * si * spl * stl +
                     sp * (-(cpl * cts * jx * stl) - ci * jy * spl * stl + jz * si * sp * spl * stl +
                           cps * ctl * jx * sts - jy * sps * sts) +
                     cp * (cpl * cts * jy * stl - ci * jx * spl * stl - (cps * ctl * jy + jx * sps) * sts)) /
                    si;
  const double ez = (ctl * jz * si - jx * (ci * cp * ctl + cp * cts + sp * (cps * spl - cpl * sps) * stl * sts) -
                     jy * (ci * ctl * sp + cts * sp + cp * (-(cps * spl) + cpl * sps) * stl * sts)) /
                    si;
  // its spherical angles (transform_cart_sph, util.cpp:1882-1891)
  const double r = sqrt(ex * ex + ez * ez + ey * ey);
  const double thj = acos(ez / r);
  double phj = atan2(ey, ex);
  if (phj < 0) phj += 2 * kPi;
  double incl_j;
  pol_incl_of_direction(p.RA, p.DEC, thj, phj, p.psi, incl_j);
}

// repack_non_parameter_options (fisher.cpp:2514-2535) + repack_parameters
GW_HD void fisher_repack(const double *v, const GenParams &in, int method, GenParams &o) {
  for (int k = 0; k < 3; k++) o.spin1[k] = o.spin2[k] = 0;
  o.chip = -1;
  o.phip = -1;
  o.sky_average = in.sky_average;
  o.f_ref = in.f_ref;
  o.gmst = in.gmst;
  o.shift_time = 0;
  o.shift_phase = in.shift_phase;
  o.dep_postmerger = in.dep_postmerger;
  o.equatorial_orientation = in.equatorial_orientation;
  o.theta_l = in.theta_l;
  o.phi_l = in.phi_l;
  o.reserved = 0;
  if (method == 1) {
    o.mass1 = calc_mass1(exp(v[7]), v[8]);
    o.mass2 = calc_mass2(exp(v[7]), v[8]);
    o.Luminosity_Distance = exp(v[6]);
    o.DEC = asin(v[1]);
  } else {
    o.mass1 = calc_mass1(v[7], v[8]);
    o.mass2 = calc_mass2(v[7], v[8]);
    o.Luminosity_Distance = v[6];
    o.DEC = v[1];
  }
  o.RA = v[0];
  o.phiRef = v[4];
  o.tc = v[5];
  o.spin1[2] = v[9];
  o.spin2[2] = v[10];
  if (in.equatorial_orientation) {  // the response takes psi and iota from L (fisher.cpp:2242-2245)
    o.theta_l = v[2];
    o.phi_l = v[3];
    orientation_transform(o, kPhenomD);
  } else {
    o.psi = v[2];
    o.incl_angle = method == 1 ? acos(v[3]) : v[3];
  }
}

// The sampler's parameter vector to the generation parameters: MCMC_prep_params
// (mcmc_gw.cpp:2492-2510: f_ref 20, t_c and phase shifts on, the sampler's
// GMST, no orientation transform) + repack_parameters, MCMC_IMRPhenomD 11-dim
// and MCMC_IMRPhenomPv2 15-dim with spherical spins (fisher.cpp:2171-2284).
GW_HD void mcmc_repack(const double *th, int dim, int approximant, double gmst, GenParams &o) {
  o.spin1[0] = o.spin1[1] = o.spin1[2] = 0;
  o.spin2[0] = o.spin2[1] = o.spin2[2] = 0;
  o.chip = -1;
  o.phip = -1;
  o.sky_average = 0;
  o.dep_postmerger = 0;
  o.f_ref = 20;
  o.shift_time = 1;
  o.shift_phase = 1;
  o.gmst = gmst;
  o.theta_l = 0;
  o.phi_l = 0;
  o.equatorial_orientation = 0;
  o.reserved = 0;
  o.mass1 = calc_mass1(exp(th[7]), th[8]);
  o.mass2 = calc_mass2(exp(th[7]), th[8]);
  o.Luminosity_Distance = exp(th[6]);
  o.RA = th[0];
  o.DEC = asin(th[1]);
  o.psi = th[2];
  o.incl_angle = acos(th[3]);
  o.phiRef = th[4];
  o.tc = th[5];
  if (approximant == kPhenomPv2 && dim >= 15) {
    double t1 = th[11] > 1 ? 0 : (th[11] < -1 ? kPi : acos(th[11]));
    double t2 = th[12] > 1 ? 0 : (th[12] < -1 ? kPi : acos(th[12]));
    o.spin1[0] = th[9] * sin(t1) * cos(th[13]);
    o.spin1[1] = th[9] * sin(t1) * sin(th[13]);
    o.spin1[2] = th[9] * cos(t1);
    o.spin2[0] = th[10] * sin(t2) * cos(th[14]);
    o.spin2[1] = th[10] * sin(t2) * sin(th[14]);
    o.spin2[2] = th[10] * cos(t2);
  } else {
    o.spin1[2] = th[9];
    o.spin2[2] = th[10];
  }
}

// The perturbed parameter vector of calculate_derivatives (fisher.cpp:361-375):
// sign +1 / -1, one-sided at the eta = 1/4 boundary.  Returns the divisor of
// the central difference (2 eps, or eps when one-sided).
GW_HD double fisher_perturb(const double *v, int i, int sign, double eps, double *out) {
  for (int j = 0; j < kFisherDim; j++) out[j] = v[j];
  bool onesided = (i == 8 && v[i] > .25 - eps);
  if (sign > 0) out[i] = onesided ? v[i] : v[i] + eps;
  else out[i] = v[i] - eps;
  return onesided ? eps : 2. * eps;
}
GW_HD double fisher_step(const double *v, int i, double epsilon, int step_mode) {
  if (step_mode == 1) return epsilon * (v[i] != 0 ? fabs(v[i]) : 1.0);
  return epsilon;
}

}  // namespace gwt
