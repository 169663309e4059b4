// phenom_model.h -- FP64 IMRPhenomD / IMRPhenomPv2 model, host and device.
//
// One header compiled twice: by nvcc into the kernels (per-request prologue
// and the FP64 per-bin evaluation of the plain form) and by the host compiler
// into the drop-in layer (host-side prologue for the one-request-per-launch
// path) and into a CPU test build.  The arithmetic restates the reference
// model (src/IMRPhenomD.cpp, src/IMRPhenomP.cpp, src/waveform_generator.cpp);
// functions cite the lines they follow.  Per-request work is split from
// per-bin work: ModelD/ModelP hold every constant a bin needs.
#pragma once

#include <cmath>
#include <vector>
#include <cstdint>
#include <cstring>

#include "phenom_tables.h"

#if defined(__CUDACC__)
#define GW_HD __host__ __device__ __forceinline__
#define GW_HDNI inline __host__ __device__ __noinline__
#else
#define GW_HD inline
#define GW_HDNI inline
#endif

namespace gwt {

constexpr double kPi = 3.14159265358979323846;
constexpr double kLnPi = 1.1447298858494002;  // ln(pi)
constexpr double kGammaE = 0.5772156649015328606065120900824024310421;
constexpr double kC = 299792458.;
constexpr double kMsolSec = 4.925491025543575903411922162094833998e-6;
constexpr double kMpcSI = 3.085677581491367278913937957796471611e22;
constexpr double kLog64 = 4.15888308336;  // IMRPhenomD.cpp:25
constexpr double kSqrt6 = 2.44948974278317788;
constexpr double kCompThresh = 1e-10;
constexpr int kQnmLen = GWT_QNM_LEN;
constexpr int kMaxDet = 4;

enum Approximant { kPhenomD = 0, kPhenomPv2 = 1 };

// Status bits set by the prologue.
enum { kModelOK = 0, kModelBadInput = 1, kModelQnmRange = 2 };

// Mirror of gwgpu_gen_params (include/gwgpu.h); same layout.
struct GenParams {
  double mass1, mass2;
  double spin1[3], spin2[3];
  double Luminosity_Distance;
  double incl_angle, phiRef, f_ref, tc;
  double RA, DEC, psi, gmst;
  double chip, phip;
  int32_t shift_time, shift_phase, sky_average, dep_postmerger;
  double theta_l, phi_l;  // equatorial direction of L, read when equatorial_orientation is set
  int32_t equatorial_orientation, reserved;
};

// source_parameters<double> subset (include/gwat/util.h:426-665)
struct Source {
  double mass1, mass2, M, eta, chirpmass, chi_s, chi_a, chi_eff, chi_pn, DL, delta_mass, A0;
  double spin1x, spin1y, spin1z, spin2x, spin2y, spin2z;
  double phiRef, tc, incl_angle, f_ref;
  int shift_time, shift_phase, sky_average, dep_postmerger, pv2;
  double fRD, fdamp, f1, f3, f1_phase, f2_phase;
  double chip, phip, chil, SP, SL, phi_aligned, alpha0, thetaJN, zeta_polariz, q;
  double cos_incl, fac_incl;  // cos(incl_angle), (1 + cos^2) / 2
  double inv_eta, k_tf2;      // 1 / eta and 3 / (128 eta), the divisions of the phase formulas
};

struct Lambda {
  double rho[4], v2, gamma[4], sigma[5], beta[5], alpha[7];
};

struct Pows {
  double MFthird, MFsixth, MF7sixth, MF2third, MF4third, MF5third, MFsquare, MF7third, MF8third, MFcube,
      MFminus_5third;
  double PIsquare, PIcube, PIthird, PI2third, PI4third, PI5third, PI7third, PIminus_5third;
};

// All per-request constants of the D model (and the D part of Pv2).
struct ModelD {
  Source s;
  Lambda l;
  Pows pi;  // only the PI* members are meaningful
  double deltas[5], pn_amp[7], pn_phase[12];
  double A0eff;   // A0 * M^(7/6) (D) or A0 * M^(7/6) / (2 sqrt(5/(64 pi))) (Pv2)
  double tcl;     // D: 2 pi tc + tc_shift; Pv2: 2 pi tc
  double phic;    // D: 2 phiRef + phi(f_ref) or phiRef; Pv2: 2 phi_aligned
  double fref;    // f_ref used in tc*(f - f_ref) (0 when shift_phase is off, D only)
  double fcut;    // 0.2 / M
  int status;
};

// Extra per-request constants of Pv2.
struct ModelP {
  double ac[5], ec[5];  // Euler alpha / epsilon coefficients (IMRPhenomP.cpp:65-144)
  double alpha_shift;   // alpha0 - alpha(f_ref)
  double eps_off;       // epsilon(f_ref)
  double t_corr;        // calculate_time_shift (IMRPhenomP.cpp:551-606)
  double Y[5];          // -2Y2m(thetaJN, 0), m=-2..2, all real
  double c2z, s2z;      // polarisation rotation by 2 zeta (waveform_generator.cpp:257-266)
};

// Per-detector projection constants of one request.
struct DetProj {
  double fp, fc;  // F+, Fx (detector_util.cpp:901-1015, geometric factor :1160)
  double tau;     // -2 pi DTOA relative to detector 0 (waveform_util.cpp:172-179)
};

// ---------------------------------------------------------------- util.cpp
GW_HD double pow_int(double base, int power) {  // util.cpp:1585-1597
  if (power == 0) return 1.;
  double prod = 1;
  int pw = power < 0 ? -power : power;
  for (int i = 0; i < pw; i++) prod = prod * base;
  if (power > 0) return prod;
  return 1. / prod;
}
// FP64 pow costs about as much as a log and an exp together; where the
// exponent allows, products, sqrt and cbrt take its place (a few ulp apart).
GW_HD double calc_chirpmass(double m1, double m2) { return pow(m1 * m2, 3. / 5) / pow(m1 + m2, 1. / 5); }
GW_HD double calc_eta(double m1, double m2) { return (m1 * m2) / ((m1 + m2) * (m1 + m2)); }
GW_HD double pow_m7_6(double x) { return 1.0 / (x * sqrt(cbrt(x))); }  // x^(-7/6)
GW_HD double pow_7_6(double x) { return x * sqrt(cbrt(x)); }           // x^(7/6)
GW_HD double calc_mass1(double mc, double eta) {  // util.cpp:1516
  double etapow = pow(eta, 3. / 5);
  return 1. / 2 * (mc / etapow + sqrt(1. - 4 * eta) * mc / etapow);
}
GW_HD double calc_mass2(double mc, double eta) {  // util.cpp:1531
  double etapow = pow(eta, 3. / 5);
  return 1. / 2 * (mc / etapow - sqrt(1. - 4 * eta) * mc / etapow);
}

// populate_source_parameters (util.cpp:997-1030) + prep_source_parameters
// (waveform_generator.cpp:1255-1271)
// In three independent parts (the cooperative prologue runs them at once on
// different warps): the masses, spins and ratios; the chirp mass and the
// amplitude normalisation (a pow); the inclination factors.
GW_HD void populate_core(Source &s, const GenParams &in) {
  s.mass1 = in.mass1 * kMsolSec;
  s.mass2 = in.mass2 * kMsolSec;
  s.spin1x = in.spin1[0];
  s.spin2x = in.spin2[0];
  s.spin1y = in.spin1[1];
  s.spin2y = in.spin2[1];
  s.spin1z = in.spin1[2];
  s.spin2z = in.spin2[2];
  s.chi_s = (1. / 2) * (s.spin1z + s.spin2z);
  s.chi_a = (1. / 2) * (s.spin1z - s.spin2z);
  s.eta = calc_eta(s.mass1, s.mass2);
  s.inv_eta = 1. / s.eta;
  s.k_tf2 = 3. / (128. * s.eta);
  s.M = s.mass1 + s.mass2;
  s.chi_eff = (s.mass1 * (s.spin1z) + s.mass2 * (s.spin2z)) / (s.M);
  s.chi_pn = s.chi_eff - ((38. / 113) * s.eta) * (2 * s.chi_s);
  s.DL = in.Luminosity_Distance * (kMpcSI / kC);
  s.delta_mass = sqrt(1. - 4 * s.eta);
  s.phiRef = in.phiRef;
  s.tc = in.tc;
  s.sky_average = in.sky_average;
  s.incl_angle = in.incl_angle;
  s.f_ref = in.f_ref;
  s.shift_time = in.shift_time;
  s.shift_phase = in.shift_phase;
  s.dep_postmerger = in.dep_postmerger;
  s.pv2 = 0;
  s.chip = in.chip;
  s.phip = in.phip;
}
GW_HD void populate_amp(Source &s, const GenParams &in) {
  const double m1 = in.mass1 * kMsolSec, m2 = in.mass2 * kMsolSec;
  const double M = m1 + m2, eta = calc_eta(m1, m2), DL = in.Luminosity_Distance * (kMpcSI / kC);
  const double mc = M * pow(eta, 3. / 5);  // (m1 m2)^(3/5) / M^(1/5)
  s.chirpmass = mc;
  // A0_from_DL (util.cpp:1271-1279)
  if (in.sky_average)
    s.A0 = sqrt(kPi / 30) * mc * mc / DL * pow_m7_6(kPi * mc);
  else
    s.A0 = sqrt(kPi * 40. / 192.) * mc * mc / DL * pow_m7_6(kPi * mc);
}
GW_HD void populate_incl(Source &s, const GenParams &in) {
  s.cos_incl = cos(in.incl_angle);
  s.fac_incl = .5 * (1 + s.cos_incl * s.cos_incl);
}
GW_HD void populate(Source &s, const GenParams &in) {
  populate_core(s, in);
  populate_amp(s, in);
  populate_incl(s, in);
}

// ------------------------------------------- natural cubic spline (QNM table)
// Spline layout in one array: x[n], y1[n], y2[n], c1[n], c2[n].
// On [x_i, x_{i+1}], S(x) = y_i + b_i t + c_i t^2 + d_i t^3, t = x - x_i,
// h_i = x_{i+1} - x_i; natural ends c_0 = c_{n-1} = 0 (c is half of S'').
// Continuity of S' at the interior knots gives
//   h_{i-1} c_{i-1} + 2 (h_{i-1} + h_i) c_i + h_i c_{i+1} = 3 (s_i - s_{i-1}),
// s_i = (y_{i+1} - y_i) / h_i (Burden & Faires, Numerical Analysis, sec. 3.5):
// a symmetric tridiagonal system, solved by its L D L^T factorisation -- one
// forward sweep for the pivots, the multipliers and the reduced right-hand
// side, then back substitution.  Solved once on the host (QNM table) or per
// request (the 10-node Pv2 time shift).  work: 3 (n - 2) doubles.
GW_HD void cspline_coeffs(const double *x, const double *y, int n, double *c, double *work) {
  const int m = n - 2;  // unknowns: the interior knots 1..n-2
  c[0] = 0.0;
  c[n - 1] = 0.0;
  if (m < 1) return;
  double *piv = work, *mul = work + m, *rhs = work + 2 * m;
  double h_left = x[1] - x[0];
  double s_left = (y[1] - y[0]) * (h_left != 0.0 ? 1.0 / h_left : 0.0);
  for (int k = 0; k < m; k++) {
    const double h_right = x[k + 2] - x[k + 1];
    const double s_right = (y[k + 2] - y[k + 1]) * (h_right != 0.0 ? 1.0 / h_right : 0.0);
    const double diag = 2.0 * (h_right + h_left), load = 3.0 * (s_right - s_left);
    if (k == 0) {
      piv[0] = diag;
      rhs[0] = load;
    } else {  // the row's sub-diagonal entry is the previous row's h_right = h_left here
      piv[k] = diag - h_left * mul[k - 1];
      rhs[k] = load - mul[k - 1] * rhs[k - 1];
    }
    if (k < m - 1) mul[k] = h_right / piv[k];
    h_left = h_right;
    s_left = s_right;
  }
  c[m] = rhs[m - 1] / piv[m - 1];
  for (int k = m - 2; k >= 0; k--) c[k + 1] = rhs[k] / piv[k] - mul[k] * c[k + 2];
}
// Interval of xv in the knots x[0..n): the last ilo <= n - 2 with x[ilo] <= xv
// (what a bisection finds), or -1 outside [x[0], x[n-1]].
GW_HD int cspline_locate(const double *x, int n, double xv) {
  if (!(xv >= x[0] && xv <= x[n - 1])) return -1;
  int ilo = 0, ihi = n - 1;
  while (ihi > ilo + 1) {
    int i = (ihi + ilo) / 2;
    if (x[i] > xv) ihi = i;
    else ilo = i;
  }
  return ilo;
}
// The same interval on a knot array that is nearly uniform with spacing h:
// a guess from the spacing corrected by a short walk (bounded by n).
GW_HD int cspline_locate_near_uniform(const double *x, int n, double xv, double h) {
  if (!(xv >= x[0] && xv <= x[n - 1])) return -1;
  int g = (int)((xv - x[0]) * (1.0 / h));  // a guess: the walk below corrects it
  if (g < 0) g = 0;
  if (g > n - 2) g = n - 2;
  for (int it = 0; it < n && g > 0 && x[g] > xv; it++) g--;
  for (int it = 0; it < n && g < n - 2 && x[g + 1] <= xv; it++) g++;
  return g;
}
// A knot interval's cubic from per-interval coefficients b, d prepared once
// (the values cspline_eval_at forms on each call): no division per call.
GW_HD double cspline_eval_pre(const double *x, const double *y, const double *b, const double *c, const double *d,
                              int ilo, double xv) {
  if (ilo < 0) return NAN;
  const double delx = xv - x[ilo];
  return y[ilo] + delx * (b[ilo] + delx * (c[ilo] + delx * d[ilo]));
}
// S (deriv 0) or S' (deriv 1) on knot interval i:
// b_i = s_i - h_i (c_{i+1} + 2 c_i) / 3, d_i = (c_{i+1} - c_i) / (3 h_i).
GW_HD double cspline_eval_at(const double *x, const double *y, const double *c, int ilo, double xv, int deriv) {
  if (ilo < 0) return NAN;
  double x_lo = x[ilo], dx = x[ilo + 1] - x_lo, y_lo = y[ilo], dy = y[ilo + 1] - y_lo, delx = xv - x_lo;
  double c_i = c[ilo], c_ip1 = c[ilo + 1];
  double b_i = (dy / dx) - dx * (c_ip1 + 2.0 * c_i) / 3.0, d_i = (c_ip1 - c_i) / (3.0 * dx);
  if (deriv) return b_i + delx * (2.0 * c_i + 3.0 * d_i * delx);
  return y_lo + delx * (b_i + delx * (c_i + delx * d_i));
}
GW_HD double cspline_eval(const double *x, const double *y, const double *c, int n, double xv, int deriv) {
  if (!(xv >= x[0] && xv <= x[n - 1])) return NAN;
  int ilo = cspline_locate(x, n, xv);
  double x_lo = x[ilo], dx = x[ilo + 1] - x_lo, y_lo = y[ilo], dy = y[ilo + 1] - y_lo, delx = xv - x_lo;
  double c_i = c[ilo], c_ip1 = c[ilo + 1];
  double b_i = (dy / dx) - dx * (c_ip1 + 2.0 * c_i) / 3.0, d_i = (c_ip1 - c_i) / (3.0 * dx);
  if (deriv) return b_i + delx * (2.0 * c_i + 3.0 * d_i * delx);
  return y_lo + delx * (b_i + delx * (c_i + delx * d_i));
}

// ------------------------------------------------------------- IMRPhenomD
GW_HD double lambda_elem(const Source &s, int i) {  // IMRPhenomD.cpp:855-870
  const double *pl = GWT_T(gwt_lambda_fit)[i];
  double spin_coeff = s.chi_pn - 1;
  double eta = s.eta;
  const double sc2 = spin_coeff * spin_coeff, sc3 = sc2 * spin_coeff;
  return pl[0] + pl[1] * eta + (spin_coeff) * (pl[2] + pl[3] * eta + pl[4] * eta * eta) +
         sc2 * (pl[5] + pl[6] * eta + pl[7] * eta * eta) + sc3 * (pl[8] + pl[9] * eta + pl[10] * eta * eta);
}
GW_HD void precalc_powers_ins(double f, double M, Pows &p) {  // IMRPhenomD.cpp:877-893
  double Mf = M * f;
  p.MFsquare = Mf * Mf;
  p.MFcube = Mf * Mf * Mf;
  p.MFsixth = sqrt(cbrt(Mf));
  p.MF7sixth = p.MFsixth * M * f;
  p.MFthird = p.MFsixth * p.MFsixth;
  p.MF2third = p.MFthird * p.MFthird;
  p.MF4third = p.MFthird * Mf;
  p.MF5third = p.MF2third * Mf;
  p.MF7third = p.MF4third * Mf;
  p.MF8third = p.MF5third * Mf;
  p.MFminus_5third = 1. / p.MF5third;
}
GW_HD void precalc_powers_PI(Pows &p) {  // IMRPhenomD.cpp:937-950
  p.PIsquare = kPi * kPi;
  p.PIcube = kPi * kPi * kPi;
  p.PIthird = 1.4645918875615231;  // pow(pi, 1/3)
  p.PI2third = p.PIthird * p.PIthird;
  p.PI4third = p.PIthird * kPi;
  p.PI5third = p.PI2third * kPi;
  p.PI7third = p.PI4third * kPi;
  p.PIminus_5third = 1. / p.PI5third;
}
// The PN coefficients with every constant ratio folded (k * eta / n written
// (k / n) * eta): a runtime FP64 division costs tens of instructions.
GW_HD void pn_amp_coeff(const Source &s, double *coeff) {  // IMRPhenomD.cpp:955-986
  double md = s.delta_mass, eta = s.eta, ca = s.chi_a, cs = s.chi_s;
  double eta2 = eta * eta, eta3 = eta2 * eta, cs2 = cs * cs, ca2 = ca * ca;
  constexpr double pi2 = kPi * kPi;
  coeff[0] = 1.;
  coeff[1] = 0.;
  coeff[2] = (-323. / 224 + (451. / 168) * eta);
  coeff[3] = ((27. / 8) * md * ca + (27. / 8 - (11. / 6) * eta) * cs);
  coeff[4] = (-27312085. / 8128512 - (1975055. / 338688) * eta + (105271. / 24192) * eta2 +
              (-81. / 32 + 8 * eta) * ca2 - (81. / 16) * md * ca * cs + (-81. / 32 + (17. / 8) * eta) * cs2);
  coeff[5] = 1. * (-85 * kPi / 64 + (85 * kPi / 16) * eta + md * (285197. / 16128 - (1579. / 4032) * eta) * ca +
                   (285197. / 16128 - (15317. / 672) * eta - (2227. / 1008) * eta2) * cs);
  coeff[6] = 1. * (-177520268561. / 8583708672 + (545384828789. / 5007163392 - 205 * pi2 / 48) * eta -
                   (3248849057. / 178827264) * eta2 + (34473079. / 6386688) * eta3 +
                   (1614569. / 64512 - (1873643. / 16128) * eta + (2167. / 42) * eta2) * ca2 +
                   (31 * kPi / 12 - (7 * kPi / 3) * eta) * cs +
                   (1614569. / 64512 - (61391. / 1344) * eta + (57451. / 4032) * eta2) * cs2 +
                   md * ca * (31 * kPi / 12 + (1614569. / 32256 - (165961. / 2688) * eta) * cs));
}
GW_HD void pn_phase_coeff_static(const Source &s, double *coeff) {  // IMRPhenomD.cpp:992-1032
  double delta = s.delta_mass, eta = s.eta, ca = s.chi_a, cs = s.chi_s;
  double eta2 = eta * eta, eta3 = eta2 * eta, cs2 = cs * cs, ca2 = ca * ca;
  constexpr double pi2 = kPi * kPi;
  coeff[0] = 1.;
  coeff[1] = 0.;
  coeff[2] = 3715. / 756 + (55. / 9) * eta;
  coeff[3] = -16. * kPi + (113. / 3) * delta * ca + (113. / 3 - (76. / 3) * eta) * cs;
  coeff[4] = 15293365. / 508032 + (27145. / 504) * eta + (3085. / 72) * eta2 + (-405. / 8 + 200. * eta) * ca2 -
             (405. / 4) * delta * ca * cs + (-405. / 8 + (5. / 2) * eta) * cs2;
  coeff[5] = 0.;
  coeff[6] = 0.;
  coeff[7] = 77096675. * kPi / 254016 + (378515. * kPi / 1512) * eta - (74045. * kPi / 756) * eta2 +
             delta * (-25150083775. / 3048192 + (26804935. / 6048) * eta - (1985. / 48) * eta2) * ca +
             (-25150083775. / 3048192 + (10566655595. / 762048) * eta - (1042165. / 3024) * eta2 +
              (5345. / 36) * eta3) *
                 cs;
  coeff[8] = (38645. * kPi / 756 - (65. * kPi / 9) * eta + delta * (-732985. / 2268 - (140. / 9) * eta) * ca +
              (-732985. / 2268 + (24260. / 81) * eta + (340. / 9) * eta2) * cs);
  coeff[9] = coeff[8];
  coeff[10] = 11583231236531. / 4694215680 - 6848. * kGammaE / 21 - 640. * pi2 / 3 +
              (-15737765635. / 3048192 + 2255. * pi2 / 12) * eta + (76055. / 1728) * eta2 - (127825. / 1296) * eta3 +
              (2270. * kPi / 3) * delta * ca + (2270. * kPi / 3 - 520. * kPi * eta) * cs - 6848. * (kLog64) / 63;
  coeff[11] = 6848. / 63.;
}
GW_HD void pn_phase_coeff_nonstatic(const Source &s, double *coeff, double f) {  // IMRPhenomD.cpp:1040-1060
  double M = s.mass1 + s.mass2;
  double logF = log(kPi * M * f);
  coeff[5] = coeff[8] + logF * coeff[9];
  coeff[6] = coeff[10] - coeff[11] * (logF);
}
GW_HD double FinalSpin0815(double eta, double chi1, double chi2) {  // IMRPhenomD.cpp:1229-1257
  double Seta = sqrt(1.0 - 4.0 * eta);
  double m1 = 0.5 * (1.0 + Seta), m2 = 0.5 * (1.0 - Seta);
  double s = (m1 * m1 * chi1 + m2 * m2 * chi2);
  double eta2 = eta * eta, eta3 = eta2 * eta, s2 = s * s, s3 = s2 * s;
  return eta * (3.4641016151377544 - 4.399247300629289 * eta + 9.397292189321194 * eta2 - 13.180949901606242 * eta3 +
                s * ((1.0 / eta - 0.0850917821418767 - 5.837029316602263 * eta) +
                     (0.1014665242971878 - 2.0967746996832157 * eta) * s +
                     (-1.3546806617824356 + 4.108962025369336 * eta) * s2 +
                     (-0.8676969352555539 + 2.064046835273906 * eta) * s3));
}
GW_HD double EradRational0815(double eta, double chi1, double chi2) {  // IMRPhenomD.cpp:1264-1286
  double Seta = sqrt(1.0 - 4.0 * eta);
  double m1 = 0.5 * (1.0 + Seta), m2 = 0.5 * (1.0 - Seta);
  double m1s = m1 * m1, m2s = m2 * m2;
  double s = (m1s * chi1 + m2s * chi2) / (m1s + m2s);
  double eta2 = eta * eta, eta3 = eta2 * eta;
  return (eta * (0.055974469826360077 + 0.5809510763115132 * eta - 0.9606726679372312 * eta2 + 3.352411249771192 * eta3) *
          (1. + (-0.0030302335878845507 - 2.0066110851351073 * eta + 7.7050567802399215 * eta2) * s)) /
         (1. + (-0.6714403054720589 - 1.4756929437702908 * eta + 7.304676214885011 * eta2) * s);
}
GW_HD double final_spin(const Source &s) {
  if (!s.pv2) return FinalSpin0815(s.eta, s.spin1z, s.spin2z);  // IMRPhenomD.cpp:1222
  // FinalSpinIMRPhenomD_all_in_plane_spin_on_larger_BH (IMRPhenomP.cpp:1232-1253)
  double m1 = s.mass1, m2 = s.mass2, M = m1 + m2;
  double eta = m1 * m2 / (M * M), af_parallel, q_factor;
  if (m1 >= m2) {
    q_factor = m1 / M;
    af_parallel = FinalSpin0815(eta, s.spin1z, s.spin2z);
  } else {
    q_factor = m2 / M;
    af_parallel = FinalSpin0815(eta, s.spin2z, s.spin1z);
  }
  double Sperp = s.chip * q_factor * q_factor;
  double sgn = sqrt(1.0 * 1.0 / (af_parallel * af_parallel)) * af_parallel;  // copysign_internal (util.cpp:566)
  return sgn * sqrt(Sperp * Sperp + af_parallel * af_parallel);
}
// The QNM part of post_merger, with the final spin and radiated energy given.
GW_HD void post_merger_qnm(Source &s, const double *qnm, double finspin, double Erad) {
  const double *a = qnm, *yr = qnm + kQnmLen, *yd = qnm + 2 * kQnmLen, *cr = qnm + 3 * kQnmLen,
               *cd = qnm + 4 * kQnmLen, *br = qnm + 5 * kQnmLen, *dr = qnm + 6 * kQnmLen,
               *bd = qnm + 7 * kQnmLen, *dd = qnm + 8 * kQnmLen;
  // both splines share the knots (spacing 0.002 inside, 0.001 at the ends)
  const int ilo = cspline_locate_near_uniform(a, kQnmLen, finspin, 0.002);
  const double sc = 1.0 / ((1.0 - Erad) * s.M);
  s.fRD = cspline_eval_pre(a, yr, br, cr, dr, ilo, finspin) * sc;
  s.fdamp = cspline_eval_pre(a, yd, bd, cd, dd, ilo, finspin) * sc;
}
GW_HD void post_merger(Source &s, const double *qnm) {  // IMRPhenomD.cpp:1091-1217
  if (s.dep_postmerger) {  // _calc_fring / _calc_fdamp (IMRPhenomD.cpp:1113-1176)
    double eta = s.eta, eta2 = eta * eta, eta3 = eta2 * eta, eta4 = eta3 * eta, M = s.M;
    double S = (s.spin1z * s.mass1 * s.mass1 + s.spin2z * s.mass2 * s.mass2) / (M * M);
    double S_red = S / (1. - 2. * eta);
    double a = final_spin(s);
    double E_rad_ns = 0.0559745 * eta + 0.580951 * eta2 - 0.960673 * eta3 + 3.35241 * eta4;
    double E_rad = E_rad_ns * (1. + S_red * (-0.00303023 - 2.00661 * eta + 7.70506 * eta2)) /
                   (1 + S_red * (-0.67144 - 1.47569 * eta + 7.30468 * eta2));
    double MWRD = (1.5251 - 1.1568 * pow(1 - a, 0.1292));
    double MWdamp = ((1.5251 - 1.1568 * pow(1. - a, 0.1292)) / (2. * (0.700 + 1.4187 * pow(1. - a, -.4990))));
    s.fRD = (1. / (2 * kPi)) * (MWRD) / (M * (1. - E_rad));
    s.fdamp = (1. / (2 * kPi)) * (MWdamp) / (M * (1. - E_rad));
    return;
  }
  post_merger_qnm(s, qnm, final_spin(s), EradRational0815(s.eta, s.spin1z, s.spin2z));
}
// The QNM table: knots a, fring and fdamp, the natural cubic spline
// coefficients c of both, then their per-interval b and d (kQnmArrays arrays
// of kQnmLen).  Host code.
constexpr int kQnmArrays = 9;
inline void qnm_fill(double *o, const double *a_h, const double *fring_h, const double *fdamp_h) {
  const int n = kQnmLen;
  for (int i = 0; i < n; i++) {
    o[i] = a_h[i];
    o[n + i] = fring_h[i];
    o[2 * n + i] = fdamp_h[i];
  }
  std::vector<double> work(6 * n);
  cspline_coeffs(o, o + n, n, o + 3 * n, work.data());
  cspline_coeffs(o, o + 2 * n, n, o + 4 * n, work.data());
  for (int sp = 0; sp < 2; sp++) {
    const double *x = o, *y = o + (1 + sp) * n, *c = o + (3 + sp) * n;
    double *b = o + (5 + 2 * sp) * n, *d = o + (6 + 2 * sp) * n;
    for (int i = 0; i < n; i++) {
      if (i + 1 >= n) {
        b[i] = d[i] = 0.0;
        continue;
      }
      const double dx = x[i + 1] - x[i], dy = y[i + 1] - y[i];
      b[i] = (dy / dx) - dx * (c[i + 1] + 2.0 * c[i]) / 3.0;
      d[i] = (c[i + 1] - c[i]) / (3.0 * dx);
    }
  }
}
GW_HD double fpeak(const Source &s, const Lambda &l) {  // IMRPhenomD.cpp:1312-1326
  double fRD = s.fRD, fdamp = s.fdamp, g3 = l.gamma[2], g2 = l.gamma[1];
  if (g2 > 1) {
    double out = fRD + (fdamp * (-1.) * g3) / g2;
    return sqrt(out * out);
  }
  double v = (fRD + fdamp * g3 * (sqrt(1 - g2 * g2) - 1) / g2);
  return sqrt(v * v);
}
GW_HD double amp_ins(double f, const ModelD &m, const Pows &p) {  // IMRPhenomD.cpp:1336-1355
  const double *pn = m.pn_amp;
  double M = m.s.M;
  double pn_amp = pn[0] + pn[1] * m.pi.PIthird * p.MFthird + pn[2] * m.pi.PI2third * p.MF2third + pn[3] * kPi * M * f +
                  pn[4] * m.pi.PI4third * p.MF4third + pn[5] * m.pi.PI5third * p.MF5third +
                  pn[6] * m.pi.PIsquare * p.MFsquare;
  double nr_amp = (m.l.rho[0]) * p.MF7third + (m.l.rho[1]) * p.MF8third + (m.l.rho[2]) * p.MFcube;
  return pn_amp + nr_amp;
}
GW_HD double phase_ins(double f, const Source &s, double *pn, const Lambda &l, const Pows &pi, const Pows &p) {
  // IMRPhenomD.cpp:1365-1399
  double M = s.M;
  pn_phase_coeff_nonstatic(s, pn, f);
  double pn_phase = pn[0] + pn[1] * pi.PIthird * p.MFthird + pn[2] * pi.PI2third * p.MF2third + pn[3] * kPi * M * f +
                    pn[4] * pi.PI4third * p.MF4third + pn[5] * pi.PI5third * p.MF5third +
                    pn[6] * pi.PIsquare * p.MFsquare + pn[7] * pi.PI7third * p.MF7third;
  double phase_TF2 = -kPi / 4. + s.k_tf2 * pi.PIminus_5third * p.MFminus_5third * pn_phase;
  return phase_TF2 + s.inv_eta * (0 + l.sigma[1] * M * f + (3. / 4.) * l.sigma[2] * p.MF4third +
                                   (3. / 5) * l.sigma[3] * p.MF5third + (1. / 2.) * l.sigma[4] * p.MFsquare);
}
GW_HD double amp_mr(double f, const Source &s, const Lambda &l) {  // IMRPhenomD.cpp:1468-1478
  double M = s.M, M2 = M * M;
  double numerator = ((l.gamma[0]) * (l.gamma[2]) * (s.fdamp) * (s.M)) *
                     exp(-(l.gamma[1]) * (f - (s.fRD)) / ((l.gamma[2]) * (s.fdamp)));
  double denominator = M2 * (((f - (s.fRD)) * (f - (s.fRD))) + ((l.gamma[2]) * (s.fdamp) * (l.gamma[2]) * (s.fdamp)));
  return numerator / denominator;
}
GW_HD double phase_mr(double f, const Source &s, const Lambda &l) {  // IMRPhenomD.cpp:1485-1503
  double M = s.M, Mf = M * f, Mfcube = Mf * Mf * Mf, Mf3fourths = sqrt(sqrt(Mfcube));
  return s.inv_eta * (l.alpha[0] + l.alpha[1] * (Mf)-l.alpha[2] * (1. / (Mf)) + (4. / 3) * l.alpha[3] * Mf3fourths +
                       l.alpha[4] * atan((f - l.alpha[5] * s.fRD) / s.fdamp));
}
GW_HD double amp_int(double f, const ModelD &m) {  // IMRPhenomD.cpp:1560-1570
  const double *d = m.deltas;
  double Mf = m.s.M * f, Mf2 = Mf * Mf, Mf3 = Mf2 * Mf, Mf4 = Mf3 * Mf;
  return (d[0] + d[1] * Mf + d[2] * Mf2 + d[3] * Mf3 + d[4] * Mf4);
}
GW_HD double phase_int(double f, const Source &s, const Lambda &l) {  // IMRPhenomD.cpp:1577-1589
  double Mf = s.M * f, Mf3 = Mf * Mf * Mf;
  return s.inv_eta * (l.beta[0] + l.beta[1] * (Mf) + l.beta[2] * log(Mf) - l.beta[3] / 3. * 1. / Mf3);
}
GW_HD double Dphase_int(double f, const Source &s, const Lambda &l) {  // IMRPhenomD.cpp:1597-1607
  const double M3 = s.M * s.M * s.M, f2 = f * f;
  return s.inv_eta * (l.beta[1] * (s.M) + l.beta[2] / f + l.beta[3] / M3 / (f2 * f2));
}
GW_HD double Dphase_mr(double f, const Source &s, const Lambda &l) {  // IMRPhenomD.cpp:1539-1554
  double M = s.M, fdamp = s.fdamp, fRD = s.fRD, u = f - l.alpha[5] * fRD;
  return (l.alpha[4] / (fdamp * (1. + (u * u) / (fdamp * fdamp))) + l.alpha[2] / ((f * f) * M) +
          M * (l.alpha[1] + l.alpha[3] / sqrt(sqrt(f * M)))) /
         s.eta;
}
GW_HD double build_amp(double f, const ModelD &m, const Pows &p) {  // IMRPhenomD.cpp:747-796
  if (f < m.s.f1) return 1. / (p.MF7sixth) * amp_ins(f, m, p);
  if (f > m.s.f3) return 1. / p.MF7sixth * amp_mr(f, m.s, m.l);
  return 1. / p.MF7sixth * amp_int(f, m);
}
GW_HD double build_phase(double f, const ModelD &m, double *pn, const Pows &p) {  // IMRPhenomD.cpp:804-821
  if (f < m.s.f1_phase) return phase_ins(f, m.s, pn, m.l, m.pi, p);
  if (f > m.s.f2_phase) return phase_mr(f, m.s, m.l);
  return phase_int(f, m.s, m.l);
}

// Prologue pieces that are not needed per bin
GW_HDNI void d_connections(ModelD &m);
GW_HDNI int model_d_prologue(ModelD &m, const double *qnm);

}  // namespace gwt

#include "phenom_prologue.h"
