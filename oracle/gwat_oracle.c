/*
 * gwat_oracle.c -- FP64 CPU oracle (test infrastructure, see gwat_oracle.h).
 *
 * Plain-C restatement of the reference's likelihood path.  Operation order
 * follows the cited reference lines so that, compiled with the same compiler
 * and flags, the waveform agrees bit for bit with the reference's own
 * IMRPhenomD.cpp / IMRPhenomP.cpp (checked in tests/test_oracle_pins.py
 * against oracle/_ref).  Complex arithmetic uses C99 _Complex, whose
 * multiplication and division lower to the same runtime helpers as
 * std::complex<double> in the reference.
 */
#include "gwat_oracle.h"
#include "gwo_tables.h"

#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Physical constants: include/gwat/util.h:44-58 */
static const double GWO_GAMMA_E = 0.5772156649015328606065120900824024310421;
static const double GWO_C_SI = 299792458.;
static const double GWO_MSOL_SEC = 4.925491025543575903411922162094833998e-6;
static const double GWO_MPC_SI = 3.085677581491367278913937957796471611e22;
static const double GWO_DOUBLE_COMP_THRESH = 1e-10; /* util.h:80 */
static const double GWO_LOG_64 = 4.15888308336;     /* IMRPhenomD.cpp:25 */
static const double GWO_SQRT_6 = 2.44948974278317788; /* IMRPhenomP.h:50 */

#define GWO_PI 3.14159265358979323846

/* source_parameters<double> (util.h:426-665), only the fields on the path */
typedef struct {
  double mass1, mass2, M, eta, chirpmass, chi_s, chi_a, chi_eff, chi_pn, DL, delta_mass, A0;
  double spin1x, spin1y, spin1z, spin2x, spin2y, spin2z;
  double phiRef, tc, incl_angle, f_ref;
  int shift_time, shift_phase, sky_average, dep_postmerger;
  double fRD, fdamp, f1, f3, f1_phase, f2_phase;
  double chip, phip, chil, SP, SL, phi_aligned, alpha0, thetaJN, zeta_polariz, q;
  int pv2;
} src_t;

typedef struct { double rho[4], v2, gamma[4], sigma[5], beta[5], alpha[7]; } lambda_t;

typedef struct {
  double MFthird, MFsixth, MF7sixth, MF2third, MF4third, MF5third, MFsquare, MF7third, MF8third,
      MFcube, MFminus_5third;
  double PIsquare, PIcube, PIthird, PI2third, PI4third, PI5third, PI7third, PIminus_5third;
} pows_t;

void gwo_default_params(gwo_gen_params *p) {
  memset(p, 0, sizeof(*p));
  /* util.h defaults: f_ref=0, shift_time=shift_phase=true, chip=phip=-1 */
  p->shift_time = 1;
  p->shift_phase = 1;
  p->chip = -1;
  p->phip = -1;
}

/* ---------------------------------------------------------------- util.cpp */
static double pow_int(double base, int power) { /* util.cpp:1585-1597 */
  if (power == 0) return 1.;
  double prod = 1;
  int pw = abs(power);
  for (int i = 0; i < pw; i++) prod = prod * base;
  if (power > 0) return prod;
  return 1. / prod;
}
static double calc_chirpmass(double m1, double m2) { return pow(m1 * m2, 3. / 5) / pow(m1 + m2, 1. / 5); } /* util.cpp:1492 */
static double calc_eta(double m1, double m2) { return (m1 * m2) / pow(m1 + m2, 2); }                          /* util.cpp:1503 */
static double calc_mass1(double mc, double eta) {                                                           /* util.cpp:1516 */
  double etapow = pow(eta, 3. / 5);
  return 1. / 2 * (mc / etapow + sqrt(1. - 4 * eta) * mc / etapow);
}
static double calc_mass2(double mc, double eta) { /* util.cpp:1531 */
  double etapow = pow(eta, 3. / 5);
  return 1. / 2 * (mc / etapow - sqrt(1. - 4 * eta) * mc / etapow);
}
static double copysign_internal(double val, double sign) { return sqrt(val * val / (sign * sign)) * sign; } /* util.cpp:566 */
static double A0_from_DL(double chirpmass, double DL, int sky_average) {                                   /* util.cpp:1271 */
  if (sky_average) return sqrt(GWO_PI / 30) * chirpmass * chirpmass / DL * pow(GWO_PI * chirpmass, -7. / 6);
  return sqrt(GWO_PI * 40. / 192.) * chirpmass * chirpmass / DL * pow(GWO_PI * chirpmass, -7. / 6);
}
/* XLALSpinWeightedSphericalHarmonic, s=-2, l=2 (util.cpp:1953-2333), phi=0 as used by Pv2 */
static double complex swsh_m2_2m(double theta, double phi, int m) {
  double fac = 0.0;
  switch (m) {
    case -2: fac = sqrt(5.0 / (64.0 * GWO_PI)) * (1.0 - cos(theta)) * (1.0 - cos(theta)); break;
    case -1: fac = sqrt(5.0 / (16.0 * GWO_PI)) * sin(theta) * (1.0 - cos(theta)); break;
    case 0: fac = sqrt(15.0 / (32.0 * GWO_PI)) * sin(theta) * sin(theta); break;
    case 1: fac = sqrt(5.0 / (16.0 * GWO_PI)) * sin(theta) * (1.0 + cos(theta)); break;
    case 2: fac = sqrt(5.0 / (64.0 * GWO_PI)) * (1.0 + cos(theta)) * (1.0 + cos(theta)); break;
  }
  if (m) {
    /* cpolar(1, m*phi) * fac (util.cpp:1944-1947) */
    double complex e = cexp(CMPLX(0.0 * (m * phi), 1.0 * (m * phi)));
    double complex cp = CMPLX(1.0 * creal(e), 1.0 * cimag(e));
    return CMPLX(creal(cp) * fac, cimag(cp) * fac);
  }
  return CMPLX(fac, 0.0);
}

/* populate_source_parameters (util.cpp:997-1030) + prep_source_parameters
 * (waveform_generator.cpp:1255-1292) */
static void populate(src_t *s, const gwo_gen_params *in) {
  memset(s, 0, sizeof(*s));
  s->mass1 = in->mass1 * GWO_MSOL_SEC;
  s->mass2 = in->mass2 * GWO_MSOL_SEC;
  s->spin1x = in->spin1[0];
  s->spin2x = in->spin2[0];
  s->spin1y = in->spin1[1];
  s->spin2y = in->spin2[1];
  s->spin1z = in->spin1[2];
  s->spin2z = in->spin2[2];
  s->chi_s = (1. / 2) * (s->spin1z + s->spin2z);
  s->chi_a = (1. / 2) * (s->spin1z - s->spin2z);
  s->chirpmass = calc_chirpmass(s->mass1, s->mass2);
  s->eta = calc_eta(s->mass1, s->mass2);
  s->M = s->mass1 + s->mass2;
  s->chi_eff = (s->mass1 * (s->spin1z) + s->mass2 * (s->spin2z)) / (s->M);
  s->chi_pn = s->chi_eff - (38 * s->eta / 113) * (2 * s->chi_s);
  s->DL = in->Luminosity_Distance * (GWO_MPC_SI / GWO_C_SI);
  s->delta_mass = sqrt(1. - 4 * s->eta);
  s->phiRef = in->phiRef;
  s->tc = in->tc;
  s->sky_average = in->sky_average;
  s->A0 = A0_from_DL(s->chirpmass, s->DL, s->sky_average);
  s->incl_angle = in->incl_angle;
  s->f_ref = in->f_ref;
  s->shift_time = in->shift_time;
  s->shift_phase = in->shift_phase;
  s->dep_postmerger = in->dep_postmerger;
}

/* ------------------------------------------------- natural cubic spline */
/* The natural cubic spline the reference takes from GSL's "cspline"
 * (IMRPhenomD.cpp:1190-1217, IMRPhenomP.cpp:595-602); GSL is not part of the
 * reference, so this is the published algorithm (Burden & Faires, Numerical
 * Analysis, sec. 3.5): c[i] = S''(x_i)/2, c[0] = c[n-1] = 0, and for the
 * interior knots h_{i-1} c_{i-1} + 2 (h_{i-1} + h_i) c_i + h_i c_{i+1}
 * = 3 (s_i - s_{i-1}), s_i the interval slopes.  The symmetric tridiagonal
 * system is solved by its L D L^T factorisation: a forward sweep (pivots,
 * multipliers, reduced right-hand side), then back substitution.  The same
 * arithmetic, in the same order, as the test-only spline of oracle/shim that
 * the reference's own model code is compiled against. */
void gwo_cspline_coeffs(const double *x, const double *y, int n, double *c) {
  const int m = n - 2;
  c[0] = 0.0;
  c[n - 1] = 0.0;
  if (m < 1) return;
  double *piv = (double *)malloc(sizeof(double) * (size_t)m * 3);
  double *mul = piv + m, *rhs = mul + m;
  double h_left = x[1] - x[0];
  double s_left = (y[1] - y[0]) * (h_left != 0.0 ? 1.0 / h_left : 0.0);
  for (int k = 0; k < m; k++) {
    const double h_right = x[k + 2] - x[k + 1];
    const double s_right = (y[k + 2] - y[k + 1]) * (h_right != 0.0 ? 1.0 / h_right : 0.0);
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
  for (int k = m - 2; k >= 0; k--) c[k + 1] = rhs[k] / piv[k] - mul[k] * c[k + 2];
  free(piv);
}

/* S (deriv 0) or S' (deriv 1): on [x_i, x_{i+1}], S = y_i + b t + c_i t^2 + d t^3,
 * b = s_i - h_i (c_{i+1} + 2 c_i)/3, d = (c_{i+1} - c_i)/(3 h_i); outside the
 * knots NaN (GSL_EDOM). */
double gwo_cspline_eval(const double *x, const double *y, const double *c, int n, double xv, int deriv) {
  if (!(xv >= x[0] && xv <= x[n - 1])) return NAN; /* GSL_EDOM */
  int ilo = 0, ihi = n - 1;
  while (ihi > ilo + 1) {
    int i = (ihi + ilo) / 2;
    if (x[i] > xv) ihi = i;
    else ilo = i;
  }
  double x_lo = x[ilo], x_hi = x[ilo + 1], dx = x_hi - x_lo;
  double y_lo = y[ilo], y_hi = y[ilo + 1], dy = y_hi - y_lo;
  double delx = xv - x_lo;
  double c_i = c[ilo], c_ip1 = c[ilo + 1];
  double b_i = (dy / dx) - dx * (c_ip1 + 2.0 * c_i) / 3.0;
  double d_i = (c_ip1 - c_i) / (3.0 * dx);
  if (deriv) return b_i + delx * (2.0 * c_i + 3.0 * d_i * delx);
  return y_lo + delx * (b_i + delx * (c_i + delx * d_i));
}

static double qnm_c_fring[GWO_QNM_LEN], qnm_c_fdamp[GWO_QNM_LEN];
static int qnm_ready = 0;
static void qnm_init(void) {
  if (qnm_ready) return;
#ifdef _OPENMP
#pragma omp critical(gwo_qnm)
#endif
  {
    if (!qnm_ready) {
      gwo_cspline_coeffs(gwo_qnm_a, gwo_qnm_fring, GWO_QNM_LEN, qnm_c_fring);
      gwo_cspline_coeffs(gwo_qnm_a, gwo_qnm_fdamp, GWO_QNM_LEN, qnm_c_fdamp);
      qnm_ready = 1;
    }
  }
}

/* ------------------------------------------------------------- IMRPhenomD */
static double lambda_elem(const src_t *s, int i) { /* IMRPhenomD.cpp:855-870 */
  const double *pl = gwo_lambda_fit[i];
  double spin_coeff = s->chi_pn - 1;
  double eta = s->eta;
  return pl[0] + pl[1] * eta + (spin_coeff) * (pl[2] + pl[3] * eta + pl[4] * eta * eta) +
         pow(spin_coeff, 2) * (pl[5] + pl[6] * eta + pl[7] * eta * eta) +
         pow(spin_coeff, 3) * (pl[8] + pl[9] * eta + pl[10] * eta * eta);
}
static void assign_lambda(const src_t *s, lambda_t *l) { /* IMRPhenomD.cpp:833-852 */
  memset(l, 0, sizeof(*l));
  for (int i = 0; i < 3; i++) l->rho[i] = lambda_elem(s, i);
  l->v2 = lambda_elem(s, 3);
  for (int i = 0; i < 3; i++) l->gamma[i] = lambda_elem(s, i + 4);
  for (int i = 0; i < 4; i++) l->sigma[i + 1] = lambda_elem(s, i + 7);
  for (int i = 0; i < 3; i++) l->beta[i + 1] = lambda_elem(s, i + 11);
  for (int i = 0; i < 5; i++) l->alpha[i + 1] = lambda_elem(s, i + 14);
}
static void precalc_powers_ins(double f, double M, pows_t *p) { /* IMRPhenomD.cpp:877-893 */
  double Mf = M * f;
  p->MFsquare = Mf * Mf;
  p->MFcube = Mf * Mf * Mf;
  p->MFsixth = pow(M * f, 1. / 6.);
  p->MF7sixth = p->MFsixth * M * f;
  p->MFthird = p->MFsixth * p->MFsixth;
  p->MF2third = p->MFthird * p->MFthird;
  p->MF4third = p->MFthird * Mf;
  p->MF5third = p->MF2third * Mf;
  p->MF7third = p->MF4third * Mf;
  p->MF8third = p->MF5third * Mf;
  p->MFminus_5third = 1. / p->MF5third;
}
static void precalc_powers_PI(pows_t *p) { /* IMRPhenomD.cpp:937-950 */
  p->PIsquare = GWO_PI * GWO_PI;
  p->PIcube = GWO_PI * GWO_PI * GWO_PI;
  p->PIthird = pow(GWO_PI, 1. / 3.);
  p->PI2third = p->PIthird * p->PIthird;
  p->PI4third = p->PIthird * GWO_PI;
  p->PI5third = p->PI2third * GWO_PI;
  p->PI7third = p->PI4third * GWO_PI;
  p->PIminus_5third = 1. / p->PI5third;
}
static void pn_amp_coeff(const src_t *s, double *coeff) { /* IMRPhenomD.cpp:955-986 */
  double massdelta = s->delta_mass, eta = s->eta, chi_a = s->chi_a, chi_s = s->chi_s;
  double eta2 = eta * eta, eta3 = eta2 * eta, chi_s2 = chi_s * chi_s, chi_a2 = chi_a * chi_a;
  double pi2 = GWO_PI * GWO_PI;
  coeff[0] = 1.;
  coeff[1] = 0.;
  coeff[2] = (-323. / 224 + 451 * eta / 168);
  coeff[3] = (27. * massdelta * chi_a / 8 + (27. / 8 - 11. * eta / 6) * chi_s);
  coeff[4] = (-27312085. / 8128512 - 1975055 * eta / 338688 + 105271 * eta2 / 24192 +
              (-81. / 32 + 8 * eta) * chi_a2 - 81 * massdelta * chi_a * chi_s / 16 +
              (-81. / 32 + 17 * eta / 8) * chi_s2);
  coeff[5] = 1. * (-85 * GWO_PI / 64 + 85 * GWO_PI * eta / 16 +
                   massdelta * (285197. / 16128 - 1579 * eta / 4032) * chi_a +
                   (285197. / 16128 - 15317 * eta / 672 - 2227 * eta2 / 1008) * chi_s);
  coeff[6] = 1. * (-177520268561. / 8583708672 + (545384828789. / 5007163392 - 205 * pi2 / 48) * eta -
                   3248849057 * eta2 / 178827264 + 34473079 * eta3 / 6386688 +
                   (1614569. / 64512 - 1873643. * eta / 16128 + 2167 * eta2 / 42) * chi_a2 +
                   (31 * GWO_PI / 12 - 7 * GWO_PI * eta / 3) * chi_s +
                   (1614569. / 64512 - 61391 * eta / 1344 + 57451 * eta2 / 4032) * chi_s2 +
                   massdelta * chi_a * (31 * GWO_PI / 12 + (1614569. / 32256 - 165961 * eta / 2688) * chi_s));
}
static void pn_phase_coeff_static(const src_t *s, double *coeff) { /* IMRPhenomD.cpp:992-1032 */
  double delta = s->delta_mass, eta = s->eta, chi_a = s->chi_a, chi_s = s->chi_s;
  double eta2 = eta * eta, eta3 = eta2 * eta, chi_s2 = chi_s * chi_s, chi_a2 = chi_a * chi_a;
  double pi2 = GWO_PI * GWO_PI;
  coeff[0] = 1.;
  coeff[1] = 0.;
  coeff[2] = 3715. / 756 + 55. * eta / 9;
  coeff[3] = -16. * GWO_PI + 113. * delta * chi_a / 3 + (113. / 3 - 76. * eta / 3) * chi_s;
  coeff[4] = 15293365. / 508032 + 27145. * eta / 504 + 3085. * eta2 / 72 + (-405. / 8 + 200. * eta) * chi_a2 -
             (405. / 4) * delta * chi_a * chi_s + (-405. / 8 + 5. * eta / 2) * chi_s2;
  coeff[7] = 77096675. * GWO_PI / 254016 + 378515. * GWO_PI * eta / 1512 - 74045. * GWO_PI * eta2 / 756 +
             delta * (-25150083775. / 3048192 + 26804935. * eta / 6048 - 1985. * eta2 / 48) * chi_a +
             (-25150083775. / 3048192 + 10566655595. * eta / 762048 - 1042165. * eta2 / 3024 + 5345. * eta3 / 36) * chi_s;
  coeff[8] = (38645. * GWO_PI / 756 - 65. * GWO_PI * eta / 9 + delta * (-732985. / 2268 - 140. * eta / 9) * chi_a +
              (-732985. / 2268 + 24260. * eta / 81 + 340. * eta2 / 9) * chi_s);
  coeff[9] = coeff[8];
  coeff[10] = 11583231236531. / 4694215680 - 6848. * GWO_GAMMA_E / 21 - 640. * pi2 / 3 +
              (-15737765635. / 3048192 + 2255. * pi2 / 12) * eta + 76055. * eta2 / 1728 - 127825. * eta3 / 1296 +
              2270. * delta * chi_a * GWO_PI / 3 + (2270. * GWO_PI / 3 - 520. * GWO_PI * eta) * chi_s -
              6848. * (GWO_LOG_64) / 63;
  coeff[11] = 6848. / 63.;
}
static void pn_phase_coeff_nonstatic(const src_t *s, double *coeff, double f) { /* IMRPhenomD.cpp:1040-1060 */
  double M = s->mass1 + s->mass2;
  double logF = log(GWO_PI * M * f);
  coeff[5] = coeff[8] + logF * coeff[9];
  coeff[6] = coeff[10] - coeff[11] * (logF);
}
static void pn_phase_coeff_nonstatic_deriv(const src_t *s, double *Dc, double f) { /* IMRPhenomD.cpp:1067-1081 */
  double delta = s->delta_mass, eta = s->eta, chi_a = s->chi_a, chi_s = s->chi_s;
  double eta2 = eta * eta;
  Dc[0] = (1. / f) * (38645. * GWO_PI / 756 - 65 * GWO_PI * eta / 9 + delta * (-732985. / 2268 - 140 * eta / 9) * chi_a +
                      (-732985. / 2268 + 24260 * eta / 81 + 340 * eta2 / 9) * chi_s);
  Dc[1] = (-6848. * (1. / f) / 63);
}

static double FinalSpin0815_s(double eta, double s) { /* IMRPhenomD.cpp:1229-1242 */
  double eta2 = eta * eta, eta3 = eta2 * eta, s2 = s * s, s3 = s2 * s;
  return eta * (3.4641016151377544 - 4.399247300629289 * eta + 9.397292189321194 * eta2 - 13.180949901606242 * eta3 +
                s * ((1.0 / eta - 0.0850917821418767 - 5.837029316602263 * eta) +
                     (0.1014665242971878 - 2.0967746996832157 * eta) * s +
                     (-1.3546806617824356 + 4.108962025369336 * eta) * s2 +
                     (-0.8676969352555539 + 2.064046835273906 * eta) * s3));
}
static double FinalSpin0815(double eta, double chi1, double chi2) { /* IMRPhenomD.cpp:1247-1257 */
  double Seta = sqrt(1.0 - 4.0 * eta);
  double m1 = 0.5 * (1.0 + Seta), m2 = 0.5 * (1.0 - Seta);
  double m1s = m1 * m1, m2s = m2 * m2;
  double s = (m1s * chi1 + m2s * chi2);
  return FinalSpin0815_s(eta, s);
}
static double EradRational0815_s(double eta, double s) { /* IMRPhenomD.cpp:1264-1270 */
  double eta2 = eta * eta, eta3 = eta2 * eta;
  return (eta * (0.055974469826360077 + 0.5809510763115132 * eta - 0.9606726679372312 * eta2 + 3.352411249771192 * eta3) *
          (1. + (-0.0030302335878845507 - 2.0066110851351073 * eta + 7.7050567802399215 * eta2) * s)) /
         (1. + (-0.6714403054720589 - 1.4756929437702908 * eta + 7.304676214885011 * eta2) * s);
}
static double EradRational0815(double eta, double chi1, double chi2) { /* IMRPhenomD.cpp:1275-1286 */
  double Seta = sqrt(1.0 - 4.0 * eta);
  double m1 = 0.5 * (1.0 + Seta), m2 = 0.5 * (1.0 - Seta);
  double m1s = m1 * m1, m2s = m2 * m2;
  double s = (m1s * chi1 + m2s * chi2) / (m1s + m2s);
  return EradRational0815_s(eta, s);
}
/* FinalSpinIMRPhenomD_all_in_plane_spin_on_larger_BH (IMRPhenomP.cpp:1232-1253) */
static double final_spin_pv2(double m1, double m2, double chi1_l, double chi2_l, double chip) {
  double M = m1 + m2;
  double eta = m1 * m2 / (M * M);
  double af_parallel, q_factor;
  if (m1 >= m2) {
    q_factor = m1 / M;
    af_parallel = FinalSpin0815(eta, chi1_l, chi2_l);
  } else {
    q_factor = m2 / M;
    af_parallel = FinalSpin0815(eta, chi2_l, chi1_l);
  }
  double Sperp = chip * q_factor * q_factor;
  return copysign_internal((double)1.0, af_parallel) * sqrt(Sperp * Sperp + af_parallel * af_parallel);
}
static double final_spin(const src_t *s) {
  if (s->pv2) return final_spin_pv2(s->mass1, s->mass2, s->spin1z, s->spin2z, s->chip);
  return FinalSpin0815(s->eta, s->spin1z, s->spin2z); /* IMRPhenomD.cpp:1222 */
}
/* _calc_fring/_calc_fdamp: deprecated analytic fits (IMRPhenomD.cpp:1113-1176) */
static void calc_fring_fdamp_dep(src_t *s) {
  double chi1 = s->spin1z, chi2 = s->spin2z, eta = s->eta, M = s->M, m1 = s->mass1, m2 = s->mass2;
  double eta2 = eta * eta, eta3 = eta2 * eta, eta4 = eta3 * eta;
  double m12 = m1 * m1, m22 = m2 * m2, M2 = M * M;
  double S = (chi1 * m12 + chi2 * m22) / M2;
  double S_red = S / (1. - 2. * eta);
  double a = final_spin(s);
  double E_rad_ns = 0.0559745 * eta + 0.580951 * eta2 - 0.960673 * eta3 + 3.35241 * eta4;
  double E_rad = E_rad_ns * (1. + S_red * (-0.00303023 - 2.00661 * eta + 7.70506 * eta2)) /
                 (1 + S_red * (-0.67144 - 1.47569 * eta + 7.30468 * eta2));
  double MWRD = (1.5251 - 1.1568 * pow(1 - a, 0.1292));
  double MWdamp = ((1.5251 - 1.1568 * pow(1. - a, 0.1292)) / (2. * (0.700 + 1.4187 * pow(1. - a, -.4990))));
  s->fRD = (1. / (2 * GWO_PI)) * (MWRD) / (M * (1. - E_rad));
  s->fdamp = (1. / (2 * GWO_PI)) * (MWdamp) / (M * (1. - E_rad));
}
static void post_merger_variables(src_t *s) { /* IMRPhenomD.cpp:1091-1101, 1183-1217 */
  if (s->dep_postmerger) {
    calc_fring_fdamp_dep(s);
    return;
  }
  qnm_init();
  double finspin = final_spin(s);
  double Erad = EradRational0815(s->eta, s->spin1z, s->spin2z);
  double rv = gwo_cspline_eval(gwo_qnm_a, gwo_qnm_fring, qnm_c_fring, GWO_QNM_LEN, finspin, 0) / (1.0 - Erad);
  s->fRD = rv / s->M;
  finspin = final_spin(s);
  Erad = EradRational0815(s->eta, s->spin1z, s->spin2z);
  rv = gwo_cspline_eval(gwo_qnm_a, gwo_qnm_fdamp, qnm_c_fdamp, GWO_QNM_LEN, finspin, 0) / (1.0 - Erad);
  s->fdamp = rv / s->M;
}
static double fpeak(const src_t *s, const lambda_t *l) { /* IMRPhenomD.cpp:1312-1326 */
  double fRD = s->fRD, fdamp = s->fdamp, gamma3 = l->gamma[2], gamma2 = l->gamma[1], out;
  if (gamma2 > 1) {
    out = fRD + (fdamp * (-1.) * gamma3) / gamma2;
    return sqrt(out * out);
  }
  return sqrt((fRD + fdamp * gamma3 * (sqrt(1 - gamma2 * gamma2) - 1) / gamma2) *
              (fRD + fdamp * gamma3 * (sqrt(1 - gamma2 * gamma2) - 1) / gamma2));
}
static double amp_ins(double f, const src_t *s, const double *pn, const lambda_t *l, const pows_t *p) { /* :1336-1355 */
  double M = s->M;
  double pn_amp = pn[0] + pn[1] * p->PIthird * p->MFthird + pn[2] * p->PI2third * p->MF2third + pn[3] * GWO_PI * M * f +
                  pn[4] * p->PI4third * p->MF4third + pn[5] * p->PI5third * p->MF5third + pn[6] * p->PIsquare * p->MFsquare;
  double nr_amp = (l->rho[0]) * p->MF7third + (l->rho[1]) * p->MF8third + (l->rho[2]) * p->MFcube;
  return pn_amp + nr_amp;
}
static double phase_ins(double f, const src_t *s, double *pn, const lambda_t *l, const pows_t *p) { /* :1365-1399 */
  double M = s->M, eta = s->eta;
  pn_phase_coeff_nonstatic(s, pn, f);
  double pn_phase = pn[0] + pn[1] * p->PIthird * p->MFthird + pn[2] * p->PI2third * p->MF2third + pn[3] * GWO_PI * M * f +
                    pn[4] * p->PI4third * p->MF4third + pn[5] * p->PI5third * p->MF5third +
                    pn[6] * p->PIsquare * p->MFsquare + pn[7] * p->PI7third * p->MF7third;
  double phase_TF2 = -GWO_PI / 4. + 3. / (128. * eta) * p->PIminus_5third * p->MFminus_5third * pn_phase;
  double sigma0 = 0, sigma1 = l->sigma[1], sigma2 = l->sigma[2], sigma3 = l->sigma[3], sigma4 = l->sigma[4];
  return phase_TF2 + (1. / eta) * (sigma0 + sigma1 * M * f + (3. / 4.) * sigma2 * p->MF4third +
                                   (3. / 5) * sigma3 * p->MF5third + (1. / 2.) * sigma4 * p->MFsquare);
}
static double Damp_ins(double f, const src_t *s, const double *pn, const lambda_t *l) { /* :1407-1419 */
  double pn_amp = 0, M = s->M;
  for (int i = 0; i < 7; i++) pn_amp += pn[i] * pow(GWO_PI * (M), i / 3.) * pow(f, i / 3. - 1.) * (i / 3.);
  double nr_amp = 0;
  for (int i = 0; i < 3; i++) nr_amp += (l->rho[i]) * pow(M, (7. + i) / 3.) * pow(f, (7. + i) / 3. - 1.) * (7. + i) / 3.;
  return pn_amp + nr_amp;
}
static double Dphase_ins(double f, const src_t *s, double *pn, const lambda_t *l) { /* :1427-1460 */
  double M = s->M, eta = s->eta;
  pn_phase_coeff_nonstatic(s, pn, f);
  double pnderiv[3];
  pn_phase_coeff_nonstatic_deriv(s, pnderiv, f);
  double pn_phase = 0;
  for (int i = 0; i < 8; i++) pn_phase += pn[i] * pow(GWO_PI * M * f, i / 3.);
  double phase_TF2 = +3. / (128 * eta) * pow(GWO_PI * M, -5. / 3.) * (-5. / 3.) * pow(f, -5. / 3 - 1.) * pn_phase;
  double pn_phase_deriv = 0;
  for (int i = 0; i < 8; i++) pn_phase_deriv += pn[i] * pow(GWO_PI * M, i / 3.) * (i / 3.) * pow(f, i / 3. - 1.);
  pn_phase_deriv += pnderiv[0] * pow(GWO_PI * M * f, 5. / 3) + pnderiv[1] * pow(GWO_PI * M * f, 6. / 3);
  phase_TF2 += pn_phase_deriv * (3. / (128 * eta) * pow(GWO_PI * M * f, -5. / 3));
  double sigma1 = l->sigma[1], sigma2 = l->sigma[2], sigma3 = l->sigma[3], sigma4 = l->sigma[4];
  return phase_TF2 + (1. / eta) * (sigma1 * M + sigma2 * pow(M, 4. / 3.) * pow(f, 1. / 3) +
                                   sigma3 * pow(M, 5. / 3.) * pow(f, 2. / 3) + sigma4 * pow(M, 2.) * f);
}
static double amp_mr(double f, const src_t *s, const lambda_t *l) { /* :1468-1478 */
  double M = s->M, M2 = M * M;
  double numerator = ((l->gamma[0]) * (l->gamma[2]) * (s->fdamp) * (s->M)) *
                     exp(-(l->gamma[1]) * (f - (s->fRD)) / ((l->gamma[2]) * (s->fdamp)));
  double denominator =
      M2 * (((f - (s->fRD)) * (f - (s->fRD))) + ((l->gamma[2]) * (s->fdamp) * (l->gamma[2]) * (s->fdamp)));
  return numerator / denominator;
}
static double phase_mr(double f, const src_t *s, const lambda_t *l) { /* :1485-1503 */
  double M = s->M, eta = s->eta, fdamp = s->fdamp, fRD = s->fRD;
  double alpha0 = l->alpha[0], alpha1 = l->alpha[1], alpha2 = l->alpha[2], alpha3 = l->alpha[3], alpha4 = l->alpha[4],
         alpha5 = l->alpha[5];
  double Mf = M * f, Mfcube = Mf * Mf * Mf, Mf3fourths = sqrt(sqrt(Mfcube));
  return (1. / eta) * (alpha0 + alpha1 * (Mf)-alpha2 * (1. / (Mf)) + (4. / 3) * alpha3 * Mf3fourths +
                       alpha4 * atan((f - alpha5 * fRD) / fdamp));
}
static double Damp_mr(double f, const src_t *s, const lambda_t *l) { /* :1514-1532 */
  double gamma1 = l->gamma[0], gamma2 = l->gamma[1], gamma3 = l->gamma[2], fdamp = s->fdamp, fRD = s->fRD, M = s->M;
  return -((exp(((-f + fRD) * gamma2) / (fdamp * gamma3)) * gamma1 *
            (pow_int(f - fRD, 2) * gamma2 + 2 * fdamp * (f - fRD) * gamma3 + pow_int(fdamp, 2) * gamma2 * pow(gamma3, 2))) /
           (pow(pow_int(f - fRD, 2) + pow_int(fdamp, 2) * pow_int(gamma3, 2), 2) * M));
}
static double Dphase_mr(double f, const src_t *s, const lambda_t *l) { /* :1539-1554 */
  double M = s->M, eta = s->eta, fdamp = s->fdamp, fRD = s->fRD;
  double alpha1 = l->alpha[1], alpha2 = l->alpha[2], alpha3 = l->alpha[3], alpha4 = l->alpha[4], alpha5 = l->alpha[5];
  return (alpha4 / (fdamp * (1. + pow(f - alpha5 * fRD, 2.) / pow(fdamp, 2.))) + alpha2 / (pow(f, 2.) * M) +
          M * (alpha1 + alpha3 / pow(f * M, 0.25))) /
         eta;
}
static double amp_int(double f, const src_t *s, const double *d) { /* :1560-1570 */
  double M = s->M, Mf = M * f, Mf2 = Mf * Mf, Mf3 = Mf2 * Mf, Mf4 = Mf3 * Mf;
  return (d[0] + d[1] * Mf + d[2] * Mf2 + d[3] * Mf3 + d[4] * Mf4);
}
static double phase_int(double f, const src_t *s, const lambda_t *l) { /* :1577-1589 */
  double beta0 = l->beta[0], beta1 = l->beta[1], beta2 = l->beta[2], beta3 = l->beta[3];
  double M = s->M, Mf = M * f, Mf3 = Mf * Mf * Mf, eta = s->eta;
  return (1. / eta) * (beta0 + beta1 * (Mf) + beta2 * log(Mf) - beta3 / 3. * 1. / Mf3);
}
static double Dphase_int(double f, const src_t *s, const lambda_t *l) { /* :1597-1607 */
  double beta1 = l->beta[1], beta2 = l->beta[2], beta3 = l->beta[3], M = s->M, eta = s->eta;
  return (1. / eta) * (beta1 * (M) + beta2 / f + beta3 * pow(M, -3.) * pow(f, -4.));
}
static void phase_connection(const src_t *s, lambda_t *l, double *pn) { /* :1614-1674 */
  l->beta[0] = 0;
  l->beta[1] = 0;
  l->alpha[0] = 0;
  l->alpha[1] = 0;
  double M = s->M, eta = s->eta;
  {
    double f1 = s->f1_phase;
    double Dins = Dphase_ins(f1, s, pn, l);
    double Dint = Dphase_int(f1, s, l);
    l->beta[1] = (eta / M) * Dins - (eta / M) * Dint;
  }
  {
    double f1 = s->f1_phase;
    pows_t pw;
    precalc_powers_ins(f1, M, &pw);
    precalc_powers_PI(&pw);
    double ins = phase_ins(f1, s, pn, l, &pw);
    double intval = phase_int(f1, s, l);
    l->beta[0] = (eta)*ins - eta * intval;
  }
  {
    double f2 = s->f2_phase;
    double Dint = Dphase_int(f2, s, l);
    double Dmr = Dphase_mr(f2, s, l);
    l->alpha[1] = (eta / M) * Dint - eta / M * Dmr;
  }
  {
    double f2 = s->f2_phase;
    double intval = phase_int(f2, s, l);
    double mr = phase_mr(f2, s, l);
    l->alpha[0] = (eta)*intval - eta * mr;
  }
}
/* calculate_delta_parameter_0..4 (IMRPhenomD.cpp:1709-1785) */
static double delta0(double f1, double f2, double f3, double v1, double v2, double v3, double dd1, double dd3, double M) {
  (void)M;
  return (-(dd3 * pow(f1, 2) * pow(f1 - f2, 2) * f2 * (f1 - f3) * (f2 - f3) * f3) +
          dd1 * f1 * (f1 - f2) * f2 * (f1 - f3) * pow(f2 - f3, 2) * pow(f3, 2) - 4 * pow(f1, 2) * pow(f2, 3) * pow(f3, 2) * v1 +
          3 * f1 * pow(f2, 4) * pow(f3, 2) * v1 + 8 * pow(f1, 2) * pow(f2, 2) * pow(f3, 3) * v1 -
          4 * f1 * pow(f2, 3) * pow(f3, 3) * v1 - pow(f2, 4) * pow(f3, 3) * v1 - 4 * pow(f1, 2) * f2 * pow(f3, 4) * v1 -
          f1 * pow(f2, 2) * pow(f3, 4) * v1 + 2 * pow(f2, 3) * pow(f3, 4) * v1 + 2 * f1 * f2 * pow(f3, 5) * v1 -
          pow(f2, 2) * pow(f3, 5) * v1 + pow(f1, 5) * pow(f3, 2) * v2 - 3 * pow(f1, 4) * pow(f3, 3) * v2 +
          3 * pow(f1, 3) * pow(f3, 4) * v2 - pow(f1, 2) * pow(f3, 5) * v2 + pow(f1, 5) * pow(f2, 2) * v3 -
          2 * pow(f1, 4) * pow(f2, 3) * v3 + pow(f1, 3) * pow(f2, 4) * v3 - 2 * pow(f1, 5) * f2 * f3 * v3 +
          pow(f1, 4) * pow(f2, 2) * f3 * v3 + 4 * pow(f1, 3) * pow(f2, 3) * f3 * v3 - 3 * pow(f1, 2) * pow(f2, 4) * f3 * v3 +
          4 * pow(f1, 4) * f2 * pow(f3, 2) * v3 - 8 * pow(f1, 3) * pow(f2, 2) * pow(f3, 2) * v3 +
          4 * pow(f1, 2) * pow(f2, 3) * pow(f3, 2) * v3) /
         (pow(f1 - f2, 2) * pow(f1 - f3, 3) * pow(f2 - f3, 2));
}
static double delta1(double f1, double f2, double f3, double v1, double v2, double v3, double dd1, double dd3, double M) {
  return (dd3 * f1 * pow(f1 - f2, 2) * (f1 - f3) * (f2 - f3) * (2 * f2 * f3 + f1 * (f2 + f3)) +
          f3 * (-(dd1 * (f1 - f2) * (f1 - f3) * pow(f2 - f3, 2) * (f2 * f3 + f1 * (2 * f2 + f3))) -
                2 * f1 *
                    (pow(f3, 4) * (v1 - v2) +
                     f1 * (2 * pow(f3, 3) * (-v1 + v2) - 4 * pow(f2, 3) * (v1 - v3) + 6 * pow(f2, 2) * f3 * (v1 - v3)) +
                     3 * pow(f2, 4) * (v1 - v3) + pow(f1, 4) * (v2 - v3) + 4 * pow(f2, 3) * f3 * (-v1 + v3) +
                     2 * pow(f1, 3) * f3 * (-v2 + v3)))) /
         (pow(f1 - f2, 2) * pow(f1 - f3, 3) * pow(f2 - f3, 2) * M);
}
static double delta2(double f1, double f2, double f3, double v1, double v2, double v3, double dd1, double dd3, double M) {
  return (-(dd3 * pow(f1 - f2, 2) * (f1 - f3) * (f2 - f3) * (pow(f1, 2) + f2 * f3 + 2. * f1 * (f2 + f3))) +
          dd1 * (f1 - f3) * pow(f2 - f3, 2) * (-(f2 * f3 * (2 * f2 + f3)) + pow(f1, 2) * (f2 + 2 * f3) + f1 * (-pow(f2, 2) + pow(f3, 2))) -
          4 * pow(f1, 2) * pow(f2, 3) * v1 + 3 * f1 * pow(f2, 4) * v1 - 4 * f1 * pow(f2, 3) * f3 * v1 + 3 * pow(f2, 4) * f3 * v1 +
          12 * pow(f1, 2) * f2 * pow(f3, 2) * v1 - 4 * pow(f2, 3) * pow(f3, 2) * v1 - 8 * pow(f1, 2) * pow(f3, 3) * v1 +
          f1 * pow(f3, 4) * v1 + pow(f3, 5) * v1 + pow(f1, 5) * v2 + pow(f1, 4) * f3 * v2 - 8 * pow(f1, 3) * pow(f3, 2) * v2 +
          8 * pow(f1, 2) * pow(f3, 3) * v2 - f1 * pow(f3, 4) * v2 - pow(f3, 5) * v2 - pow(f1, 5) * v3 +
          4 * pow(f1, 2) * pow(f2, 3) * v3 - 3 * f1 * pow(f2, 4) * v3 - pow(f1, 4) * f3 * v3 + 4 * f1 * pow(f2, 3) * f3 * v3 -
          3 * pow(f2, 4) * f3 * v3 + 8 * pow(f1, 3) * pow(f3, 2) * v3 - 12 * pow(f1, 2) * f2 * pow(f3, 2) * v3 +
          4 * pow(f2, 3) * pow(f3, 2) * v3) /
         (pow(f1 - f2, 2) * pow(f1 - f3, 3) * pow(f2 - f3, 2) * pow(M, 2));
}
static double delta3(double f1, double f2, double f3, double v1, double v2, double v3, double dd1, double dd3, double M) {
  return (dd3 * pow(f1 - f2, 2) * (f1 - f3) * (f2 - f3) * (2 * f1 + f2 + f3) -
          dd1 * (f1 - f2) * (f1 - f3) * pow(f2 - f3, 2) * (f1 + f2 + 2 * f3) +
          2 * (pow(f3, 4) * (-v1 + v2) + 2 * pow(f1, 2) * pow(f2 - f3, 2) * (v1 - v3) + 2 * pow(f2, 2) * pow(f3, 2) * (v1 - v3) +
               2 * pow(f1, 3) * f3 * (v2 - v3) + pow(f2, 4) * (-v1 + v3) + pow(f1, 4) * (-v2 + v3) +
               2 * f1 * f3 * (pow(f3, 2) * (v1 - v2) + pow(f2, 2) * (v1 - v3) + 2 * f2 * f3 * (-v1 + v3)))) /
         (pow(f1 - f2, 2) * pow(f1 - f3, 3) * pow(f2 - f3, 2) * pow(M, 3));
}
static double delta4(double f1, double f2, double f3, double v1, double v2, double v3, double dd1, double dd3, double M) {
  return (-(dd3 * pow(f1 - f2, 2) * (f1 - f3) * (f2 - f3)) + dd1 * (f1 - f2) * (f1 - f3) * pow(f2 - f3, 2) -
          3 * f1 * pow(f2, 2) * v1 + 2 * pow(f2, 3) * v1 + 6 * f1 * f2 * f3 * v1 - 3 * pow(f2, 2) * f3 * v1 -
          3 * f1 * pow(f3, 2) * v1 + pow(f3, 3) * v1 + pow(f1, 3) * v2 - 3 * pow(f1, 2) * f3 * v2 + 3 * f1 * pow(f3, 2) * v2 -
          pow(f3, 3) * v2 - pow(f1, 3) * v3 + 3 * f1 * pow(f2, 2) * v3 - 2 * pow(f2, 3) * v3 + 3 * pow(f1, 2) * f3 * v3 -
          6 * f1 * f2 * f3 * v3 + 3 * pow(f2, 2) * f3 * v3) /
         (pow(f1 - f2, 2) * pow(f1 - f3, 3) * pow(f2 - f3, 2) * pow(M, 4));
}
static void amp_connection(const src_t *s, const lambda_t *l, const double *pn, double *coeffs) { /* :1679-1702 */
  double M = s->M, f1 = s->f1, f3 = s->f3;
  pows_t pw;
  precalc_powers_ins(f1, M, &pw);
  precalc_powers_PI(&pw);
  double f2 = (f1 + f3) / 2.;
  double v1 = amp_ins(f1, s, pn, l, &pw);
  double v2 = l->v2;
  double v3 = amp_mr(f3, s, l);
  double dd1 = Damp_ins(f1, s, pn, l);
  double dd3 = Damp_mr(f3, s, l);
  coeffs[0] = delta0(f1, f2, f3, v1, v2, v3, dd1, dd3, M);
  coeffs[1] = delta1(f1, f2, f3, v1, v2, v3, dd1, dd3, M);
  coeffs[2] = delta2(f1, f2, f3, v1, v2, v3, dd1, dd3, M);
  coeffs[3] = delta3(f1, f2, f3, v1, v2, v3, dd1, dd3, M);
  coeffs[4] = delta4(f1, f2, f3, v1, v2, v3, dd1, dd3, M);
}
static double build_amp(double f, const lambda_t *l, const src_t *s, const pows_t *p, const double *ac, const double *d) {
  /* IMRPhenomD.cpp:747-796 */
  if (f < s->f1) return 1. / (p->MF7sixth) * amp_ins(f, s, ac, l, p);
  else if (f > s->f3) return 1. / p->MF7sixth * amp_mr(f, s, l);
  return 1. / p->MF7sixth * amp_int(f, s, d);
}
static double build_phase(double f, const lambda_t *l, const src_t *s, const pows_t *p, double *pc) {
  /* IMRPhenomD.cpp:804-821 */
  if (f < s->f1_phase) return phase_ins(f, s, pc, l, p);
  else if (f > s->f2_phase) return phase_mr(f, s, l);
  return phase_int(f, s, l);
}

/* Shared prologue of construct_waveform (IMRPhenomD.cpp:410-432) */
typedef struct {
  lambda_t lambda;
  pows_t pows;
  double deltas[6], pn_amp[7], pn_phase[12];
} dmodel_t;
static void d_prologue(src_t *s, dmodel_t *m) {
  assign_lambda(s, &m->lambda);
  post_merger_variables(s);
  s->f1_phase = 0.018 / (s->M);
  s->f2_phase = s->fRD / 2.;
  s->f1 = 0.014 / (s->M);
  s->f3 = fpeak(s, &m->lambda);
  memset(&m->pows, 0, sizeof(m->pows));
  precalc_powers_PI(&m->pows);
  memset(m->deltas, 0, sizeof(m->deltas));
  memset(m->pn_phase, 0, sizeof(m->pn_phase));
  pn_amp_coeff(s, m->pn_amp);
  pn_phase_coeff_static(s, m->pn_phase);
  amp_connection(s, &m->lambda, m->pn_amp, m->deltas);
  phase_connection(s, &m->lambda, m->pn_phase);
}

/* IMRPhenomD::construct_waveform, array overload (IMRPhenomD.cpp:404-504) */
static int d_construct(const double *freqs, int length, double complex *wf, src_t *s) {
  dmodel_t m;
  d_prologue(s, &m);
  double M = s->M;
  double phic, f_ref, tc, phi_shift, tc_shift;
  if (s->shift_phase) {
    f_ref = s->f_ref;
    precalc_powers_ins(f_ref, M, &m.pows);
    phi_shift = build_phase(f_ref, &m.lambda, s, &m.pows, m.pn_phase);
    phic = 2 * s->phiRef + phi_shift;
  } else {
    f_ref = 0;
    phic = s->phiRef;
  }
  if (s->shift_time) {
    double alpha1_offset = lambda_elem(s, 14);
    tc_shift = Dphase_mr(s->f3, s, &m.lambda) + (-m.lambda.alpha[1] + alpha1_offset) * s->M / s->eta;
  } else {
    tc_shift = 0;
  }
  tc = 2 * GWO_PI * s->tc + tc_shift;
  double A0 = s->A0 * pow(M, 7. / 6.);
  double fcut = .2 / M;
  for (int j = 0; j < length; j++) {
    double f = freqs[j];
    if (f > fcut) {
      wf[j] = 0.0;
    } else {
      if (f < s->f1_phase) {
        precalc_powers_ins(f, M, &m.pows);
      } else {
        m.pows.MFsixth = pow(M * f, 1. / 6.);
        m.pows.MF7sixth = pow_int(m.pows.MFsixth, 7);
      }
      double amp = (A0 * build_amp(f, &m.lambda, s, &m.pows, m.pn_amp, m.deltas));
      double phase = (build_phase(f, &m.lambda, s, &m.pows, m.pn_phase));
      phase -= (double)(tc * (f - f_ref) + phic);
      /* amp * exp(-i*phase) with amp and phase real */
      double complex e = cexp(CMPLX(0.0, -phase));
      wf[j] = CMPLX(amp * creal(e), amp * cimag(e));
    }
  }
  return 1;
}

/* ------------------------------------------------------------- IMRPhenomPv2 */
#define ROTATEZ(angle, vx, vy, vz)                \
  tmp1 = vx * cos(angle) - vy * sin(angle);      \
  tmp2 = vx * sin(angle) + vy * cos(angle);      \
  vx = tmp1;                                     \
  vy = tmp2
#define ROTATEY(angle, vx, vy, vz)                \
  tmp1 = vx * cos(angle) + vz * sin(angle);      \
  tmp2 = -vx * sin(angle) + vz * cos(angle);     \
  vx = tmp1;                                     \
  vz = tmp2

static double L2PN(double eta, const pows_t *p) { /* IMRPhenomP.cpp:1214-1220 */
  double x = p->MF2third * p->PI2third, x2 = x * x, eta2 = eta * eta;
  return (eta * (1.0 + (1.5 + eta / 6.0) * x + (3.375 - (19.0 * eta) / 8. - eta2 / 24.0) * x2)) / sqrt(x);
}
/* PhenomPv2_Param_Transform (IMRPhenomP.cpp:1082-1210) and _reduced (:822-938) */
static void pv2_transform(src_t *s, int reduced) {
  double chi1_l = s->spin1z, chi2_l = s->spin2z;
  double q = s->mass1 / s->mass2;
  double chi_eff = (s->mass1 * chi1_l + s->mass2 * chi2_l) / s->M;
  double chil = (1.0 + q) / q * chi_eff;
  s->chil = chil;
  double m1_2 = s->mass1 * s->mass1, m2_2 = s->mass2 * s->mass2;
  double m1, m2;
  if (!reduced) {
    double S1_perp = m1_2 * sqrt(s->spin1y * s->spin1y + s->spin1x * s->spin1x);
    double S2_perp = m2_2 * sqrt(s->spin2y * s->spin2y + s->spin2x * s->spin2x);
    double A1 = 2 + (3 * s->mass2) / (2 * s->mass1);
    double A2 = 2 + (3 * s->mass1) / (2 * s->mass2);
    double ASp1 = A1 * S1_perp, ASp2 = A2 * S2_perp;
    double num = (ASp2 > ASp1) ? ASp2 : ASp1;
    double denom = (s->mass2 > s->mass1) ? A2 * m2_2 : A1 * m1_2;
    s->chip = num / denom;
  }
  m1 = q / (1 + q);
  m2 = 1. / (1 + q);
  s->SP = s->chip * m1 * m1;
  s->SL = chi1_l * m1 * m1 + chi2_l * m2 * m2;
  pows_t pw;
  memset(&pw, 0, sizeof(pw));
  precalc_powers_PI(&pw);
  precalc_powers_ins(s->f_ref, s->M, &pw);
  double L0 = s->M * s->M * L2PN(s->eta, &pw);
  double J0x_sf, J0y_sf, J0z_sf;
  if (!reduced) {
    J0x_sf = m1_2 * s->spin1x + m2_2 * s->spin2x;
    J0y_sf = m1_2 * s->spin1y + m2_2 * s->spin2y;
    J0z_sf = L0 + m1_2 * s->spin1z + m2_2 * s->spin2z;
  } else {
    J0x_sf = m1_2 * s->chip * cos(s->phip);
    J0y_sf = m1_2 * s->chip * sin(s->phip);
    J0z_sf = L0 + m1_2 * s->spin1z + m2_2 * s->spin2z;
  }
  double J0 = sqrt(J0x_sf * J0x_sf + J0y_sf * J0y_sf + J0z_sf * J0z_sf);
  double thetaJ_sf = acos(J0z_sf / J0);
  double phiJ_sf = atan2(J0y_sf, J0x_sf);
  s->phi_aligned = -phiJ_sf;
  double tmp1, tmp2;
  double incl = s->incl_angle, phiRef = s->phiRef;
  double Nx_sf = sin(incl) * cos(GWO_PI / 2. - phiRef);
  double Ny_sf = sin(incl) * sin(GWO_PI / 2. - phiRef);
  double Nz_sf = cos(incl);
  double tmp_x = Nx_sf, tmp_y = Ny_sf, tmp_z = Nz_sf;
  ROTATEZ(-phiJ_sf, tmp_x, tmp_y, tmp_z);
  ROTATEY(-thetaJ_sf, tmp_x, tmp_y, tmp_z);
  double kappa = -atan2(tmp_y, tmp_x);
  tmp_x = 0.;
  tmp_y = 0.;
  tmp_z = 1.;
  ROTATEZ(-phiJ_sf, tmp_x, tmp_y, tmp_z);
  ROTATEY(-thetaJ_sf, tmp_x, tmp_y, tmp_z);
  ROTATEZ(kappa, tmp_x, tmp_y, tmp_z);
  s->alpha0 = atan2(tmp_y, tmp_x);
  tmp_x = Nx_sf;
  tmp_y = Ny_sf;
  tmp_z = Nz_sf;
  ROTATEZ(-phiJ_sf, tmp_x, tmp_y, tmp_z);
  ROTATEY(-thetaJ_sf, tmp_x, tmp_y, tmp_z);
  ROTATEZ(kappa, tmp_x, tmp_y, tmp_z);
  double Nx_Jf = tmp_x, Nz_Jf = tmp_z;
  s->thetaJN = acos(Nz_Jf);
  double Xx_sf = -cos(incl) * sin(phiRef), Xy_sf = -cos(incl) * cos(phiRef), Xz_sf = sin(incl);
  tmp_x = Xx_sf;
  tmp_y = Xy_sf;
  tmp_z = Xz_sf;
  ROTATEZ(-phiJ_sf, tmp_x, tmp_y, tmp_z);
  ROTATEY(-thetaJ_sf, tmp_x, tmp_y, tmp_z);
  ROTATEZ(kappa, tmp_x, tmp_y, tmp_z);
  double PArunx_Jf = 0., PAruny_Jf = -1., PArunz_Jf = 0.;
  double QArunx_Jf = Nz_Jf, QAruny_Jf = 0., QArunz_Jf = -Nx_Jf;
  double XdotPArun = tmp_x * PArunx_Jf + tmp_y * PAruny_Jf + tmp_z * PArunz_Jf;
  double XdotQArun = tmp_x * QArunx_Jf + tmp_y * QAruny_Jf + tmp_z * QArunz_Jf;
  s->zeta_polariz = atan2(XdotQArun, XdotPArun);
}

typedef struct { double c1, c2, c3, c4, c5; } euler_c;
static void euler_coeffs(euler_c *a, euler_c *e, const src_t *s) { /* IMRPhenomP.cpp:65-144 */
  double m2 = s->q / (1. + s->q), m1 = 1. / (1. + s->q), dm = m1 - m2, mtot = 1.;
  double eta = m1 * m2, eta2 = eta * eta, eta3 = eta2 * eta, eta4 = eta3 * eta;
  double mtot2 = mtot * mtot, mtot4 = mtot2 * mtot2, mtot6 = mtot4 * mtot2, mtot8 = mtot6 * mtot2;
  double chil2 = s->chil * s->chil, chip2 = s->chip * s->chip, chip4 = chip2 * chip2;
  double dm2 = dm * dm, dm3 = dm2 * dm;
  double m2_2 = m2 * m2, m2_3 = m2_2 * m2, m2_4 = m2_3 * m2, m2_5 = m2_4 * m2, m2_6 = m2_5 * m2, m2_7 = m2_6 * m2,
         m2_8 = m2_7 * m2;
  double chil = s->chil;
  a->c1 = (-0.18229166666666666 - (5 * dm) / (64. * m2));
  a->c2 = ((-15 * dm * m2 * chil) / (128. * mtot2 * eta) - (35 * m2_2 * chil) / (128. * mtot2 * eta));
  a->c3 = (-1.7952473958333333 - (4555 * dm) / (7168. * m2) - (15 * chip2 * dm * m2_3) / (128. * mtot4 * eta2) -
           (35 * chip2 * m2_4) / (128. * mtot4 * eta2) - (515 * eta) / 384. - (15 * dm2 * eta) / (256. * m2_2) -
           (175 * dm * eta) / (256. * m2));
  a->c4 = -(35 * GWO_PI) / 48. - (5 * dm * GWO_PI) / (16. * m2) + (5 * dm2 * chil) / (16. * mtot2) +
          (5 * dm * m2 * chil) / (3. * mtot2) + (2545 * m2_2 * chil) / (1152. * mtot2) -
          (5 * chip2 * dm * m2_5 * chil) / (128. * mtot6 * eta3) - (35 * chip2 * m2_6 * chil) / (384. * mtot6 * eta3) +
          (2035 * dm * m2 * chil) / (21504. * mtot2 * eta) + (2995 * m2_2 * chil) / (9216. * mtot2 * eta);
  a->c5 = (4.318908476114694 + (27895885 * dm) / (2.1676032e7 * m2) - (15 * chip4 * dm * m2_7) / (512. * mtot8 * eta4) -
           (35 * chip4 * m2_8) / (512. * mtot8 * eta4) - (485 * chip2 * dm * m2_3) / (14336. * mtot4 * eta2) +
           (475 * chip2 * m2_4) / (6144. * mtot4 * eta2) + (15 * chip2 * dm2 * m2_2) / (256. * mtot4 * eta) +
           (145 * chip2 * dm * m2_3) / (512. * mtot4 * eta) + (575 * chip2 * m2_4) / (1536. * mtot4 * eta) +
           (39695 * eta) / 86016. + (1615 * dm2 * eta) / (28672. * m2_2) - (265 * dm * eta) / (14336. * m2) +
           (955 * eta2) / 576. + (15 * dm3 * eta2) / (1024. * m2_3) + (35 * dm2 * eta2) / (256. * m2_2) +
           (2725 * dm * eta2) / (3072. * m2) - (15 * dm * m2 * GWO_PI * chil) / (16. * mtot2 * eta) -
           (35 * m2_2 * GWO_PI * chil) / (16. * mtot2 * eta) + (15 * chip2 * dm * m2_7 * chil2) / (128. * mtot8 * eta4) +
           (35 * chip2 * m2_8 * chil2) / (128. * mtot8 * eta4) + (375 * dm2 * m2_2 * chil2) / (256. * mtot4 * eta) +
           (1815 * dm * m2_3 * chil2) / (256. * mtot4 * eta) + (1645 * m2_4 * chil2) / (192. * mtot4 * eta));
  e->c1 = (-0.18229166666666666 - (5 * dm) / (64. * m2));
  e->c2 = ((-15 * dm * m2 * chil) / (128. * mtot2 * eta) - (35 * m2_2 * chil) / (128. * mtot2 * eta));
  e->c3 = (-1.7952473958333333 - (4555 * dm) / (7168. * m2) - (515 * eta) / 384. - (15 * dm2 * eta) / (256. * m2_2) -
           (175 * dm * eta) / (256. * m2));
  e->c4 = -(35 * GWO_PI) / 48. - (5 * dm * GWO_PI) / (16. * m2) + (5 * dm2 * chil) / (16. * mtot2) +
          (5 * dm * m2 * chil) / (3. * mtot2) + (2545 * m2_2 * chil) / (1152. * mtot2) +
          (2035 * dm * m2 * chil) / (21504. * mtot2 * eta) + (2995 * m2_2 * chil) / (9216. * mtot2 * eta);
  e->c5 = (4.318908476114694 + (27895885 * dm) / (2.1676032e7 * m2) + (39695 * eta) / 86016. +
           (1615 * dm2 * eta) / (28672. * m2_2) - (265 * dm * eta) / (14336. * m2) + (955 * eta2) / 576. +
           (15 * dm3 * eta2) / (1024. * m2_3) + (35 * dm2 * eta2) / (256. * m2_2) + (2725 * dm * eta2) / (3072. * m2) -
           (15 * dm * m2 * GWO_PI * chil) / (16. * mtot2 * eta) - (35 * m2_2 * GWO_PI * chil) / (16. * mtot2 * eta) +
           (375 * dm2 * m2_2 * chil2) / (256. * mtot4 * eta) + (1815 * dm * m2_3 * chil2) / (256. * mtot4 * eta) +
           (1645 * m2_4 * chil2) / (192. * mtot4 * eta));
}
static void euler_angles(double *alpha, double *epsilon, const pows_t *p, const euler_c *a, const euler_c *e) {
  /* IMRPhenomP.cpp:717-735 */
  double omega_cbrt = p->MFthird * p->PIthird;
  double omega_cbrt2 = omega_cbrt * omega_cbrt;
  double logomega = log(omega_cbrt2 * omega_cbrt);
  double omega = omega_cbrt2 * omega_cbrt;
  *alpha = (a->c1 / omega + a->c2 / omega_cbrt2 + a->c3 / omega_cbrt + a->c4 * logomega + a->c5 * omega_cbrt);
  *epsilon = (e->c1 / omega + e->c2 / omega_cbrt2 + e->c3 / omega_cbrt + e->c4 * logomega + e->c5 * omega_cbrt);
}
static void wignerd(double d2[5], double dm2[5], const pows_t *p, const src_t *s) { /* IMRPhenomP.cpp:665-693 */
  double L = L2PN(s->eta, p);
  double sv = s->SP / (L + s->SL);
  double s_2 = sv * sv;
  double cos_beta = 1. / sqrt(1.0 + s_2);
  double cbh = sqrt((1.0 + cos_beta) / 2.0), sbh = sqrt((1.0 - cos_beta) / 2.0);
  double c2 = cbh * cbh, s2 = sbh * sbh, c3 = c2 * cbh, s3 = s2 * sbh, c4 = c3 * cbh, s4 = s3 * sbh;
  d2[0] = s4;
  d2[1] = 2 * cbh * s3;
  d2[2] = GWO_SQRT_6 * s2 * c2;
  d2[3] = 2 * c3 * sbh;
  d2[4] = c4;
  dm2[0] = d2[4];
  dm2[1] = -d2[3];
  dm2[2] = d2[2];
  dm2[3] = -d2[1];
  dm2[4] = d2[0];
}
static double complex cscale(double complex z, double a) { return CMPLX(creal(z) * a, cimag(z) * a); }
static void twistup(double alpha, double complex *hp, double complex *hc, const double d2[5], const double dm2[5],
                    const double complex Y[5]) { /* IMRPhenomP.cpp:696-715; Y = {Y2m2,Y2m1,Y20,Y21,Y22} */
  double complex exp_a = cexp(CMPLX(0.0 * alpha, 1. * alpha));
  double complex exp_ma = CMPLX(1., 0.0) / exp_a;
  double complex exp_2a = exp_a * exp_a;
  double complex exp_m2a = exp_ma * exp_ma;
  double complex ev[5] = {exp_m2a, exp_ma, CMPLX(1.0, 0.0), exp_a, exp_2a};
  for (int m = -2; m <= 2; m++) {
    double complex T2m = cscale(ev[-m + 2], dm2[m + 2]) * Y[m + 2];
    double complex Tm2m = cscale(ev[m + 2], d2[m + 2]) * conj(Y[m + 2]);
    *hp += T2m + Tm2m;
    *hc += CMPLX(0, 1.) * (T2m - Tm2m);
  }
}
/* calculate_time_shift (IMRPhenomP.cpp:551-606) */
static double pv2_time_shift(src_t *s, pows_t *p, double *pc, const lambda_t *l) {
  double M = s->M;
  int n_fixed = 10;
  double f_final = s->fRD;
  double ff[10], ph[10], cc[10];
  double fs = .8 * (f_final), fe = 1.2 * (f_final);
  double dfx = (fe - fs) / (n_fixed - 1);
  if (isnan(dfx) || dfx <= 0) return 0;
  for (int j = 0; j < n_fixed; j++) ff[j] = fs + j * dfx;
  for (int j = 0; j < n_fixed; j++) {
    double f = ff[j];
    if (f < s->f1_phase) {
      precalc_powers_ins(f, M, p);
    } else {
      p->MFsixth = pow(M * f, 1. / 6);
      p->MF7sixth = p->MFsixth * p->MFsixth * p->MFsixth * p->MFsixth * p->MFsixth * p->MFsixth * p->MFsixth;
      p->MFthird = p->MFsixth * p->MFsixth;
      p->MF2third = p->MFthird * p->MFthird;
    }
    ph[j] = -build_phase(f, l, s, p, pc);
  }
  gwo_cspline_coeffs(ff, ph, n_fixed, cc);
  return gwo_cspline_eval(ff, ph, cc, n_fixed, f_final, 1) / (2. * GWO_PI);
}
/* IMRPhenomPv2::construct_waveform (IMRPhenomP.cpp:195-369) */
static int pv2_construct(const double *freqs, int length, double complex *wp, double complex *wc, src_t *s) {
  double complex Y[5];
  double phiHarm = 0.;
  Y[4] = swsh_m2_2m(s->thetaJN, phiHarm, 2);
  Y[3] = swsh_m2_2m(s->thetaJN, phiHarm, 1);
  Y[2] = swsh_m2_2m(s->thetaJN, phiHarm, 0);
  Y[1] = swsh_m2_2m(s->thetaJN, phiHarm, -1);
  Y[0] = swsh_m2_2m(s->thetaJN, phiHarm, -2);
  double M = s->M;
  dmodel_t m;
  d_prologue(s, &m);
  double f_ref = s->f_ref;
  double phic = 2 * s->phi_aligned;
  double tc = 2 * GWO_PI * s->tc;
  double A0 = s->A0 * pow(M, 7. / 6.) / (2. * sqrt(5. / (64. * GWO_PI)));
  double q = s->mass1 / s->mass2;
  s->q = q;
  double d2[5], dm2[5];
  double complex hpf = 0.0, hcf = 0.0;
  double eps, eps_off, alpha, alpha_off;
  euler_c ac, ec;
  euler_coeffs(&ac, &ec, s);
  double *ampv = (double *)malloc(sizeof(double) * (size_t)(length > 0 ? length : 1) * 2);
  double *phasev = ampv + length;
  double complex *hpv = (double complex *)malloc(sizeof(double complex) * (size_t)(length > 0 ? length : 1) * 2);
  double complex *hcv = hpv + length;
  m.pows.MFthird = pow(s->M * s->f_ref, 1. / 3.);
  m.pows.MF2third = m.pows.MFthird * m.pows.MFthird;
  euler_angles(&alpha_off, &eps_off, &m.pows, &ac, &ec);
  double fcut = .2 / M;
  for (int j = 0; j < length; j++) {
    double f = freqs[j];
    if (f > fcut) {
      wp[j] = 0.0;
      wc[j] = 0.0;
      ampv[j] = 0;
      phasev[j] = 0;
      hpv[j] = 0;
      hcv[j] = 0;
    } else {
      precalc_powers_ins(f, M, &m.pows);
      double amp = (A0 * build_amp(f, &m.lambda, s, &m.pows, m.pn_amp, m.deltas));
      double phase = (build_phase(f, &m.lambda, s, &m.pows, m.pn_phase));
      wignerd(d2, dm2, &m.pows, s);
      euler_angles(&alpha, &eps, &m.pows, &ac, &ec);
      alpha = alpha + s->alpha0 - alpha_off;
      eps = eps - eps_off;
      twistup(alpha, &hpf, &hcf, d2, dm2, Y);
      phase = phase + (2. * eps);
      ampv[j] = amp / 2.; /* amp/std::complex(2,0): exact halving */
      phasev[j] = phase;
      hpv[j] = hpf;
      hcv[j] = hcf;
      hpf = 0.;
      hcf = 0.;
    }
  }
  double t_corr = 0;
  if (s->shift_time) t_corr = pv2_time_shift(s, &m.pows, m.pn_phase, &m.lambda);
  for (int j = 0; j < length; j++) {
    double f = freqs[j];
    double x = ((phasev[j] - tc * (f - f_ref)) - phic) + (2 * GWO_PI * t_corr * f);
    double complex e = cexp(CMPLX(0.0, -x));
    double complex ah = cscale(hpv[j], ampv[j]);
    double complex ax = cscale(hcv[j], ampv[j]);
    wp[j] = ah * e;
    x = ((phasev[j] - tc * (f - f_ref)) - phic) + ((2 * GWO_PI * t_corr) * f);
    e = cexp(CMPLX(0.0, -x));
    wc[j] = ax * e;
  }
  free(ampv);
  free(hpv);
  return 1;
}

/* ---------------------------------------------------------- fourier_waveform */
int gwo_fourier_waveform(const double *freqs, int length, double *hplus, double *hcross, int approximant,
                         const gwo_gen_params *p) {
  src_t s;
  populate(&s, p);
  double complex *hp = (double complex *)hplus, *hc = (double complex *)hcross;
  if (approximant == GWO_IMRPHENOMD) {
    d_construct(freqs, length, hp, &s); /* waveform_generator.cpp:176-200 */
    double ci = cos(s.incl_angle);
    for (int i = 0; i < length; i++) {
      hc[i] = CMPLX(0, -1) * hp[i];
    }
    double fac = .5 * (1 + ci * ci);
    for (int i = 0; i < length; i++) {
      hc[i] = cscale(hc[i], ci);
      hp[i] = cscale(hp[i], fac);
    }
    return 1;
  }
  if (approximant == GWO_IMRPHENOMPV2) {
    s.pv2 = 1;
    if ((p->chip + 1) > GWO_DOUBLE_COMP_THRESH) { /* waveform_generator.cpp:1272-1281 */
      s.chip = p->chip;
      s.spin1z = p->spin1[2];
      s.spin2z = p->spin2[2];
      s.phip = p->phip;
      pv2_transform(&s, 1);
    } else {
      pv2_transform(&s, 0);
    }
    pv2_construct(freqs, length, hp, hc, &s);
    double c2z = cos(2. * s.zeta_polariz), s2z = sin(2. * s.zeta_polariz); /* :257-266 */
    for (int i = 0; i < length; i++) {
      double complex tp = hp[i], tx = hc[i];
      hp[i] = cscale(tp, c2z) + cscale(tx, s2z);
      hc[i] = cscale(tx, c2z) - cscale(tp, s2z);
    }
    return 1;
  }
  return 0;
}

/* ------------------------------------------------------------------ detectors */
int gwo_detector_index(const char *n) {
  static const char *names[9][3] = {{"Hanford", "hanford", ""},         {"Livingston", "livingston", ""},
                                    {"Virgo", "virgo", ""},             {"Kagra", "kagra", ""},
                                    {"Indigo", "indigo", ""},           {"Cosmic Explorer", "cosmic explorer", "CE"},
                                    {"Einstein Telescope 1", "einstein telescope 1", "ET1"},
                                    {"Einstein Telescope 2", "einstein telescope 2", "ET2"},
                                    {"Einstein Telescope 3", "einstein telescope 3", "ET3"}};
  if (!n) return -1;
  for (int i = 0; i < 9; i++)
    for (int j = 0; j < 3; j++)
      if (names[i][j][0] && strcmp(n, names[i][j]) == 0) return i;
  return -1;
}
void gwo_antenna(int det, double ra, double dec, double psi, double gmst, double *fplus, double *fcross) {
  /* detector_util.cpp:901-1015 */
  const double *D = gwo_det_tensor[det];
  double X[3], Y[3];
  double gha = gmst - ra;
  double cosgha = cos(gha), singha = sin(gha), cosdec = cos(dec), sindec = sin(dec), cospsi = cos(psi),
         sinpsi = sin(psi);
  X[0] = -cospsi * singha - sinpsi * cosgha * sindec;
  X[1] = -cospsi * cosgha + sinpsi * singha * sindec;
  X[2] = sinpsi * cosdec;
  Y[0] = sinpsi * singha - cospsi * cosgha * sindec;
  Y[1] = sinpsi * cosgha + cospsi * singha * sindec;
  Y[2] = cospsi * cosdec;
  double fp = 0.0, fc = 0.0;
  for (int i = 0; i < 3; i++) {
    double DX = D[i * 3 + 0] * X[0] + D[i * 3 + 1] * X[1] + D[i * 3 + 2] * X[2];
    double DY = D[i * 3 + 0] * Y[0] + D[i * 3 + 1] * Y[1] + D[i * 3 + 2] * Y[2];
    fp += X[i] * DX - Y[i] * DY;
    fc += X[i] * DY + Y[i] * DX;
  }
  fp *= gwo_det_geometric[det]; /* detector_util.cpp:1158-1160 */
  fc *= gwo_det_geometric[det];
  *fplus = fp;
  *fcross = fc;
}
double gwo_dtoa(double RA, double DEC, double GMST_rad, int d1, int d2) { /* detector_util.cpp:760-780 */
  const double *l1 = gwo_det_location[d1], *l2 = gwo_det_location[d2];
  double dx[3] = {l1[0] - l2[0], l1[1] - l2[1], l1[2] - l2[2]};
  double hour_angle = GMST_rad - RA;
  double ehat[3];
  ehat[0] = cos(DEC) * cos(hour_angle);
  ehat[1] = cos(DEC) * -sin(hour_angle);
  ehat[2] = sin(DEC);
  return (dx[0] * ehat[0] + dx[1] * ehat[1] + dx[2] * ehat[2]) / GWO_C_SI;
}

static void project(const double complex *hp, const double complex *hc, int length, double fp, double fc,
                    double complex *r) { /* waveform_util.cpp:865-873 */
  for (int i = 0; i < length; i++) r[i] = cscale(hp[i], fp) + cscale(hc[i], fc);
}

/* terr_pol_iota_from_equat_sph (util.cpp:1362-1378): polarisation and
 * inclination of a direction (thetaj, phij) seen from the sky position. */
static void terr_pol_iota(double RA, double DEC, double thetaj, double phij, double *pol, double *iota) {
  double t = atan(cos(DEC) * 1. / tan(thetaj) * 1. / sin(phij - RA) - 1. / tan(phij - RA) * sin(DEC));
  *pol = GWO_PI / 2. - t;
  *iota = acos(-(cos(thetaj) * sin(DEC)) - cos(DEC) * cos(phij - RA) * sin(thetaj));
}

/* equatorial_from_SF (util.cpp:1440-1485): a source-frame vector (L along z)
 * rotated to equatorial Cartesian coordinates. */
static void equatorial_from_sf(const double *v, double thetal, double phil, double thetas, double phis, double iota,
                               double phi_ref, double *out) {
  double cp = cos(GWO_PI / 2. - phi_ref), sp = sin(GWO_PI / 2. - phi_ref);
  double ci = cos(iota), si = sin(iota);
  double ctl = cos(thetal), stl = sin(thetal), cts = cos(thetas), sts = sin(thetas);
  double cps = cos(phis), sps = sin(phis), cpl = cos(phil), spl = sin(phil);
  double jx = v[0], jy = v[1], jz = v[2];
  out[0] = (pow_int(cp, 2) * cpl * jz * si * stl - ci * cpl * (cp * jx + jy * sp) * stl -
            cp * (cts * jy * spl * stl + cps * jx * sts - ctl * jy * sps * sts) +
            sp * (cpl * jz * si * sp * stl + cts * jx * spl * stl - (cps * jy + ctl * jx * sps) * sts)) / si;
  out[1] = (pow_int(cp, 2) * jz * si * spl * stl +
            sp * (-(cpl * cts * jx * stl) - ci * jy * spl * stl + jz * si * sp * spl * stl + cps * ctl * jx * sts -
                  jy * sps * sts) +
            cp * (cpl * cts * jy * stl - ci * jx * spl * stl - (cps * ctl * jy + jx * sps) * sts)) / si;
  out[2] = (ctl * jz * si - jx * (ci * cp * ctl + cp * cts + sp * (cps * spl - cpl * sps) * stl * sts) -
            jy * (ci * ctl * sp + cts * sp + cp * (-(cps * spl) + cpl * sps) * stl * sts)) / si;
}

/* transform_orientation_coords (waveform_util.cpp:1523-1586), ground-detector
 * branch: the inclination and polarisation from the equatorial direction
 * (theta_l, phi_l) of the orbital angular momentum.  IMRPhenomD: both from
 * terr_pol_iota_from_equat_sph of L.  IMRPhenomPv2: the inclination is the
 * angle between N and L; the polarisation is that of the total angular
 * momentum J, its source-frame direction from PhenomPv2_JSF_from_params
 * (IMRPhenomP.cpp:776-816) rotated to equatorial coordinates. */
void gwo_transform_orientation_coords(gwo_gen_params *p, int approximant) {
  double theta_s = GWO_PI / 2. - p->DEC, phi_s = p->RA;
  double N[3] = {-sin(theta_s) * cos(phi_s), -sin(theta_s) * sin(phi_s), -cos(theta_s)};
  double L[3] = {sin(p->theta_l) * cos(p->phi_l), sin(p->theta_l) * sin(p->phi_l), cos(p->theta_l)};
  p->incl_angle = acos(N[0] * L[0] + N[1] * L[1] + N[2] * L[2]);
  if (approximant != GWO_IMRPHENOMPV2) {
    terr_pol_iota(p->RA, p->DEC, p->theta_l, p->phi_l, &p->psi, &p->incl_angle);
    return;
  }
  double chi1_l = p->spin1[2], chi2_l = p->spin2[2];
  double eta = calc_eta(p->mass1, p->mass2);
  double m1_2 = p->mass1 * p->mass1, m2_2 = p->mass2 * p->mass2;
  pows_t pw;
  memset(&pw, 0, sizeof(pw));
  precalc_powers_PI(&pw);
  precalc_powers_ins(p->f_ref, (p->mass1 + p->mass2) * GWO_MSOL_SEC, &pw);
  double L0 = pow_int(p->mass1 + p->mass2, 2) * L2PN(eta, &pw);
  double jx = m1_2 * p->chip * cos(p->phip), jy = m1_2 * p->chip * sin(p->phip);
  double jz = L0 + m1_2 * chi1_l + m2_2 * chi2_l;
  double j0 = sqrt(jx * jx + jy * jy + jz * jz);
  double jsf[3] = {jx / j0, jy / j0, jz / j0}, jeq[3];
  equatorial_from_sf(jsf, p->theta_l, p->phi_l, theta_s, phi_s, p->incl_angle, p->phiRef, jeq);
  double r = sqrt(jeq[0] * jeq[0] + jeq[2] * jeq[2] + jeq[1] * jeq[1]); /* transform_cart_sph, util.cpp:1882-1891 */
  double theta_j = acos(jeq[2] / r), phi_j = atan2(jeq[1], jeq[0]);
  if (phi_j < 0) phi_j += 2 * GWO_PI;
  double iota_j;
  terr_pol_iota(p->RA, p->DEC, theta_j, phi_j, &p->psi, &iota_j);
}

int gwo_fourier_detector_response(const double *freqs, int length, double *response, int det, int approximant,
                                  const gwo_gen_params *p_in) {
  gwo_gen_params pc = *p_in;
  const gwo_gen_params *p = &pc;
  if (pc.equatorial_orientation) gwo_transform_orientation_coords(&pc, approximant); /* waveform_util.cpp:946-948 */
  double complex *hp = (double complex *)malloc(sizeof(double complex) * (size_t)(length > 0 ? length : 1) * 2);
  double complex *hc = hp + length;
  int st = gwo_fourier_waveform(freqs, length, (double *)hp, (double *)hc, approximant, p);
  double fp, fc;
  gwo_antenna(det, p->RA, p->DEC, p->psi, p->gmst, &fp, &fc);
  project(hp, hc, length, fp, fc, (double complex *)response);
  free(hp);
  return st;
}

static double simpsons_sum(double delta_x, int length, const double *x) { /* util.h:844-856 */
  double sum = 0;
  for (int i = 1; i < length - 1; i++) {
    if (i % 2 == 0) sum += 2 * x[i];
    else sum += 4 * x[i];
  }
  sum += x[0] + x[length - 1];
  return sum * delta_x / 3;
}

double gwo_log_likelihood_internal(const double *data, const double *psd, const double *freqs, const double *response,
                                   int length) { /* mcmc_gw.cpp:801-873, SIMPSONS */
  if (length < 2) return 0.0;
  const double complex *d = (const double complex *)data, *r = (const double complex *)response;
  double delta_f = freqs[length / 2] - freqs[length / 2 - 1];
  double *integrand = (double *)malloc(sizeof(double) * (size_t)length);
  for (int i = 0; i < length; i++) integrand[i] = creal(r[i] * conj(r[i])) / psd[i];
  double HH = 4. * simpsons_sum(delta_f, length, integrand);
  for (int i = 0; i < length; i++) integrand[i] = creal(d[i] * conj(r[i])) / psd[i];
  double DH = 4. * simpsons_sum(delta_f, length, integrand);
  free(integrand);
  return -0.5 * (HH - 2 * DH);
}

/* GAUSSLEG branch of Log_Likelihood_internal (mcmc_gw.cpp:820-833, 843-862):
 * integral = 4 sum_i w_i integrand_i, times f_i ln 10 when log10F. */
static double gauss_sum(const double *w, const double *freqs, int log10F, int length, const double *x) {
  double integral = 0;
  if (log10F) {
    for (int i = 0; i < length; i++) integral += w[i] * x[i] * freqs[i] * log(10.); /* LOG10, util.h:75 */
  } else {
    for (int i = 0; i < length; i++) integral += w[i] * x[i];
  }
  return integral * 4;
}
double gwo_log_likelihood_internal_gl(const double *data, const double *psd, const double *freqs,
                                      const double *weights, const double *response, int length, int log10F) {
  if (length < 1) return 0.0;
  const double complex *d = (const double complex *)data, *r = (const double complex *)response;
  double *integrand = (double *)malloc(sizeof(double) * (size_t)length);
  for (int i = 0; i < length; i++) integrand[i] = creal(r[i] * conj(r[i])) / psd[i];
  double HH = gauss_sum(weights, freqs, log10F, length, integrand);
  for (int i = 0; i < length; i++) integrand[i] = creal(d[i] * conj(r[i])) / psd[i];
  double DH = gauss_sum(weights, freqs, log10F, length, integrand);
  free(integrand);
  return -0.5 * (HH - 2 * DH);
}

double gwo_loglik_extrinsic_gl(const gwo_gen_params *pin, int approximant, double T_segment, const double *freqs,
                               int length, int ndet, const int *dets, const double *const *data,
                               const double *const *psd, const double *const *weights, int log10F) {
  gwo_gen_params p = *pin;
  p.tc = T_segment - p.tc; /* mcmc_gw.cpp:2466-2473 */
  size_t n = (size_t)(length > 0 ? length : 1);
  double complex *hp = (double complex *)malloc(sizeof(double complex) * n * 3);
  double complex *hc = hp + n, *r = hc + n;
  gwo_fourier_waveform(freqs, length, (double *)hp, (double *)hc, approximant, &p);
  double ll = 0;
  for (int i = 0; i < ndet; i++) {
    double tc = -gwo_dtoa(p.RA, p.DEC, p.gmst, dets[0], dets[i]);
    tc *= 2 * GWO_PI;
    double fp, fc;
    gwo_antenna(dets[i], p.RA, p.DEC, p.psi, p.gmst, &fp, &fc);
    project(hp, hc, length, fp, fc, r);
    for (int j = 0; j < length; j++) r[j] *= cexp(CMPLX(0, tc * freqs[j]));
    ll += gwo_log_likelihood_internal_gl(data[i], psd[i], freqs, weights[i], (const double *)r, length, log10F);
  }
  free(hp);
  return ll;
}

double gwo_loglik_extrinsic(const gwo_gen_params *pin, int approximant, double T_segment, const double *freqs,
                            int length, int ndet, const int *dets, const double *const *data,
                            const double *const *psd) {
  gwo_gen_params p = *pin;
  double tc_ref = T_segment - p.tc; /* mcmc_gw.cpp:2466-2473 */
  p.tc = tc_ref;
  size_t n = (size_t)(length > 0 ? length : 1);
  double complex *hp = (double complex *)malloc(sizeof(double complex) * n * 3);
  double complex *hc = hp + n, *r = hc + n;
  gwo_fourier_waveform(freqs, length, (double *)hp, (double *)hc, approximant, &p); /* waveform_util.cpp:153-184 */
  double ll = 0;
  for (int i = 0; i < ndet; i++) {
    double DTOA = gwo_dtoa(p.RA, p.DEC, p.gmst, dets[0], dets[i]);
    double tc = -DTOA;
    tc *= 2 * GWO_PI;
    double fp, fc;
    gwo_antenna(dets[i], p.RA, p.DEC, p.psi, p.gmst, &fp, &fc);
    project(hp, hc, length, fp, fc, r);
    for (int j = 0; j < length; j++) r[j] *= cexp(CMPLX(0, tc * freqs[j]));
    ll += gwo_log_likelihood_internal(data[i], psd[i], freqs, (const double *)r, length);
  }
  free(hp);
  return ll;
}

void gwo_mcmc_repack(const double *th, int dim, int approximant, double gmst, gwo_gen_params *o) {
  gwo_default_params(o);
  o->sky_average = 0; /* MCMC_prep_params, mcmc_gw.cpp:2494-2507 */
  o->f_ref = 20;
  o->shift_time = 1;
  o->shift_phase = 1;
  o->gmst = gmst;
  o->mass1 = calc_mass1(exp(th[7]), th[8]);
  o->mass2 = calc_mass2(exp(th[7]), th[8]);
  o->Luminosity_Distance = exp(th[6]);
  o->RA = th[0];
  o->DEC = asin(th[1]);
  o->psi = th[2];
  o->incl_angle = acos(th[3]);
  o->phiRef = th[4];
  o->tc = th[5];
  if (approximant == GWO_IMRPHENOMD || dim < 15) { /* fisher.cpp:2263-2284 */
    o->spin1[2] = th[9];
    o->spin2[2] = th[10];
  } else { /* fisher.cpp:2171-2227 */
    double t1, t2;
    if (th[11] > 1) t1 = 0;
    else if (th[11] < -1) t1 = GWO_PI;
    else t1 = acos(th[11]);
    if (th[12] > 1) t2 = 0;
    else if (th[12] < -1) t2 = GWO_PI;
    else t2 = acos(th[12]);
    double s1[3] = {th[9], t1, th[13]}, s2[3] = {th[10], t2, th[14]};
    o->spin1[0] = s1[0] * sin(s1[1]) * cos(s1[2]); /* transform_sph_cart, util.cpp:1909 */
    o->spin1[1] = s1[0] * sin(s1[1]) * sin(s1[2]);
    o->spin1[2] = s1[0] * cos(s1[1]);
    o->spin2[0] = s2[0] * sin(s2[1]) * cos(s2[2]);
    o->spin2[1] = s2[0] * sin(s2[1]) * sin(s2[2]);
    o->spin2[2] = s2[0] * cos(s2[1]);
  }
}

void gwo_loglik_batch(const gwo_gen_params *p, int n, const int *approximant, double T_segment, const double *freqs,
                      int length, int ndet, const int *dets, const double *const *data, const double *const *psd,
                      double *out, int nthreads) {
  qnm_init();
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
  for (int i = 0; i < n; i++)
    out[i] = gwo_loglik_extrinsic(&p[i], approximant[i], T_segment, freqs, length, ndet, dets, data, psd);
  (void)nthreads;
}

/* ------------------------------------------------------------------- Fisher */
/* unpack_parameters (fisher.cpp:1841-1961), non-sky-averaged branches */
static int fisher_unpack(double *v, int *logf, const gwo_gen_params *p, int method) {
  int dim = (method == 0 || method == 1) ? 11 : (method == 2 ? 13 : 15);
  for (int i = 0; i < dim; i++) logf[i] = 0;
  int mcmc = (method == 1 || method == 3);
  double mc = calc_chirpmass(p->mass1, p->mass2), eta = calc_eta(p->mass1, p->mass2);
  v[0] = p->RA;
  v[1] = mcmc ? sin(p->DEC) : p->DEC;
  if (p->equatorial_orientation) { /* L's equatorial angles in place of psi, iota (fisher.cpp:1916-1919, 1944-1947) */
    v[2] = p->theta_l;
    v[3] = p->phi_l;
  } else {
    v[2] = p->psi;
    v[3] = mcmc ? cos(p->incl_angle) : p->incl_angle;
  }
  v[4] = p->phiRef;
  v[5] = p->tc;
  if (mcmc) {
    v[6] = log(p->Luminosity_Distance);
    v[7] = log(mc);
  } else {
    logf[6] = 1;
    logf[7] = 1;
    v[6] = p->Luminosity_Distance;
    v[7] = mc;
  }
  v[8] = eta;
  if (method == 3) { /* transform_cart_sph (util.cpp:1895-1906) */
    const double *sp[2] = {p->spin1, p->spin2};
    double sph[2][3];
    for (int k = 0; k < 2; k++) {
      sph[k][0] = sqrt(sp[k][0] * sp[k][0] + sp[k][1] * sp[k][1] + sp[k][2] * sp[k][2]);
      if (sph[k][0] == 0) {
        sph[k][1] = 0;
        sph[k][2] = 0;
      } else {
        sph[k][1] = acos(sp[k][2] / sph[k][0]);
        sph[k][2] = atan2(sp[k][1], sp[k][0]);
      }
    }
    v[9] = sph[0][0];
    v[10] = sph[1][0];
    v[11] = cos(sph[0][1]);
    v[12] = cos(sph[1][1]);
    v[13] = sph[0][2];
    v[14] = sph[1][2];
  } else {
    v[9] = p->spin1[2];
    v[10] = p->spin2[2];
    if (method == 2) {
      v[11] = p->chip;
      v[12] = p->phip;
    }
  }
  return dim;
}
/* repack_parameters (fisher.cpp:2168-2300), non-sky-averaged branches, on top
 * of repack_non_parameter_options (fisher.cpp:2514-2535) */
static void fisher_repack(const double *v, gwo_gen_params *o, const gwo_gen_params *in, int method) {
  gwo_default_params(o);
  o->sky_average = in->sky_average;
  o->f_ref = in->f_ref;
  o->gmst = in->gmst;
  o->shift_time = 0;
  o->shift_phase = in->shift_phase;
  o->dep_postmerger = in->dep_postmerger;
  o->equatorial_orientation = in->equatorial_orientation;
  int mcmc = (method == 1 || method == 3);
  if (mcmc) {
    o->mass1 = calc_mass1(exp(v[7]), v[8]);
    o->mass2 = calc_mass2(exp(v[7]), v[8]);
    o->Luminosity_Distance = exp(v[6]);
    o->DEC = asin(v[1]);
  } else {
    o->mass1 = calc_mass1(v[7], v[8]);
    o->mass2 = calc_mass2(v[7], v[8]);
    o->Luminosity_Distance = v[6];
    o->DEC = v[1];
  }
  if (in->equatorial_orientation) { /* psi and iota follow from the transform at the response (fisher.cpp:2242-2245) */
    o->theta_l = v[2];
    o->phi_l = v[3];
  } else {
    o->psi = v[2];
    o->incl_angle = mcmc ? acos(v[3]) : v[3];
  }
  o->RA = v[0];
  o->phiRef = v[4];
  o->tc = v[5];
  if (method == 3) {
    double t1, t2;
    if (v[11] > 1) t1 = 0;
    else if (v[11] < -1) t1 = GWO_PI;
    else t1 = acos(v[11]);
    if (v[12] > 1) t2 = 0;
    else if (v[12] < -1) t2 = GWO_PI;
    else t2 = acos(v[12]);
    o->spin1[0] = v[9] * sin(t1) * cos(v[13]);
    o->spin1[1] = v[9] * sin(t1) * sin(v[13]);
    o->spin1[2] = v[9] * cos(t1);
    o->spin2[0] = v[10] * sin(t2) * cos(v[14]);
    o->spin2[1] = v[10] * sin(t2) * sin(v[14]);
    o->spin2[2] = v[10] * cos(t2);
  } else {
    o->spin1[2] = v[9];
    o->spin2[2] = v[10];
    if (method == 2) {
      o->chip = v[11];
      o->phip = v[12];
    }
  }
}

int gwo_fisher_numerical(const double *freqs, int length, int method, int det, int ref_det, double *out,
                         const gwo_gen_params *p, int order, const double *psd, double epsilon, int step_mode) {
  int approx = (method >= 2) ? GWO_IMRPHENOMPV2 : GWO_IMRPHENOMD;
  double v[15], pp[15], pm[15], ppp[15], pmm[15];
  int logf[15];
  int dim = fisher_unpack(v, logf, p, method);
  size_t n = (size_t)(length > 0 ? length : 1);
  double complex *deriv = (double complex *)malloc(sizeof(double complex) * n * (size_t)dim);
  double complex *rp = (double complex *)malloc(sizeof(double complex) * n * 4);
  double complex *rm = rp + n, *rpp = rm + n, *rmm = rpp + n;
  gwo_gen_params wp;
  for (int i = 0; i < dim; i++) { /* fisher.cpp:361-470 */
    double eps = epsilon;
    if (step_mode == 1) eps = epsilon * (v[i] != 0 ? fabs(v[i]) : 1.0);
    for (int j = 0; j < dim; j++) {
      pp[j] = v[j];
      pm[j] = v[j];
      ppp[j] = v[j];
      pmm[j] = v[j];
    }
    pp[i] = v[i] + eps;
    pm[i] = v[i] - eps;
    int onesided = (i == 8 && v[i] > .25 - eps);
    if (onesided) pp[i] = v[i];
    if (order >= 4) {
      ppp[i] = v[i] + 2 * eps;
      pmm[i] = v[i] - 2 * eps;
      if (onesided) ppp[i] = v[i];
    }
    fisher_repack(pp, &wp, p, method);
    gwo_fourier_detector_response(freqs, length, (double *)rp, det, approx, &wp);
    if (ref_det != det) {
      double DTOA = -2 * GWO_PI * gwo_dtoa(wp.RA, wp.DEC, wp.gmst, ref_det, det);
      for (int l = 0; l < length; l++) rp[l] *= cexp(CMPLX(0, DTOA * freqs[l]));
    }
    fisher_repack(pm, &wp, p, method);
    gwo_fourier_detector_response(freqs, length, (double *)rm, det, approx, &wp);
    if (ref_det != det) {
      double DTOA = -2 * GWO_PI * gwo_dtoa(wp.RA, wp.DEC, wp.gmst, ref_det, det);
      for (int l = 0; l < length; l++) rm[l] *= cexp(CMPLX(0, DTOA * freqs[l]));
    }
    if (order >= 4) { /* fisher.cpp:426-458: time shift, not a phase factor */
      fisher_repack(ppp, &wp, p, method);
      if (ref_det != det) wp.tc -= gwo_dtoa(wp.RA, wp.DEC, wp.gmst, ref_det, det);
      gwo_fourier_detector_response(freqs, length, (double *)rpp, det, approx, &wp);
      fisher_repack(pmm, &wp, p, method);
      if (ref_det != det) wp.tc -= gwo_dtoa(wp.RA, wp.DEC, wp.gmst, ref_det, det);
      gwo_fourier_detector_response(freqs, length, (double *)rmm, det, approx, &wp);
    }
    double complex *d = deriv + (size_t)i * n;
    if (order == 2) {
      for (int l = 0; l < length; l++) {
        d[l] = (rp[l] - rm[l]) / (2. * eps);
        if (onesided) d[l] = (rp[l] - rm[l]) / eps;
      }
    } else {
      for (int l = 0; l < length; l++) {
        d[l] = (-rpp[l] + 8. * rp[l] - 8. * rm[l] + rmm[l]) / (12. * eps);
        if (onesided) d[l] = (-rpp[l] + 8. * rp[l] - 8. * rm[l] + rmm[l]) / (6. * eps);
      }
    }
  }
  for (int l = 0; l < dim; l++) /* fisher.cpp:548-553 */
    if (logf[l])
      for (int j = 0; j < length; j++) deriv[(size_t)l * n + j] *= v[l];
  /* calculate_fisher_elements (fisher.cpp:2704-2781) */
  double *integ = (double *)malloc(sizeof(double) * n);
  double dfs = freqs[1] - freqs[0];
  for (int j = 0; j < dim; j++) {
    for (int k = 0; k < j; k++) {
      const double complex *a = deriv + (size_t)j * n, *b = deriv + (size_t)k * n;
      for (int i = 0; i < length; i++) {
        double complex pr = a[i] * conj(b[i]);
        integ[i] = creal(pr) / psd[i];
      }
      out[j * dim + k] = 4 * simpsons_sum(dfs, length, integ);
      out[k * dim + j] = out[j * dim + k];
    }
  }
  for (int j = 0; j < dim; j++) {
    const double complex *a = deriv + (size_t)j * n;
    for (int i = 0; i < length; i++) {
      double complex pr = a[i] * conj(a[i]);
      integ[i] = creal(pr) / psd[i];
    }
    out[j * dim + j] = 4 * simpsons_sum(dfs, length, integ);
  }
  free(integ);
  free(deriv);
  free(rp);
  return dim;
}

int gwo_fisher_network(const double *freqs, int length, int method, int ndet, const int *dets, double *out,
                       const gwo_gen_params *p, int order, const double *const *psd, double epsilon, int step_mode) {
  int dim = (method == 0 || method == 1) ? 11 : (method == 2 ? 13 : 15);
  double tmp[15 * 15];
  for (int j = 0; j < dim * dim; j++) out[j] = 0;
  for (int i = 0; i < ndet; i++) {
    gwo_fisher_numerical(freqs, length, method, dets[i], dets[0], tmp, p, order, psd[i], epsilon, step_mode);
    for (int j = 0; j < dim * dim; j++) out[j] += tmp[j];
  }
  return dim;
}

void gwo_fisher_batch(const gwo_gen_params *p, int n, const double *freqs, int length, int method, int ndet,
                      const int *dets, const double *const *psd, double epsilon, int step_mode, double *out,
                      int nthreads) {
  qnm_init();
  int dim = (method == 0 || method == 1) ? 11 : (method == 2 ? 13 : 15);
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
  for (int i = 0; i < n; i++)
    gwo_fisher_network(freqs, length, method, ndet, dets, out + (size_t)i * dim * dim, &p[i], 2, psd, epsilon,
                       step_mode);
  (void)nthreads;
}

/* gsl_cholesky_matrix_invert (util.cpp:857-900): pivoted Cholesky
 * (gsl_linalg_pcholesky_decomp / _invert).  Restated as: symmetric diagonal
 * pivoting on the largest remaining diagonal, LDL^T factorisation, inverse of
 * P^T L D L^T P.  Returns 0 on success, 1 on failure (non-positive pivot or
 * NaN), as the reference does. */
int gwo_cholesky_invert(const double *a, double *inv, int dim) {
  double A[15 * 15], Linv[15 * 15], Dv[15];
  int perm[15];
  if (dim > 15 || dim <= 0) return 1;
  for (int i = 0; i < dim * dim; i++) A[i] = a[i];
  for (int i = 0; i < dim; i++) perm[i] = i;
  for (int j = 0; j < dim; j++) {
    /* pivot: largest diagonal among remaining */
    int piv = j;
    for (int i = j + 1; i < dim; i++)
      if (A[i * dim + i] > A[piv * dim + piv]) piv = i;
    if (piv != j) {
      for (int k = 0; k < dim; k++) { /* swap rows */
        double t = A[j * dim + k];
        A[j * dim + k] = A[piv * dim + k];
        A[piv * dim + k] = t;
      }
      for (int k = 0; k < dim; k++) { /* swap cols */
        double t = A[k * dim + j];
        A[k * dim + j] = A[k * dim + piv];
        A[k * dim + piv] = t;
      }
      int t = perm[j];
      perm[j] = perm[piv];
      perm[piv] = t;
    }
    double d = A[j * dim + j];
    if (!(d > 0)) return 1;
    Dv[j] = d;
    for (int i = j + 1; i < dim; i++) A[i * dim + j] /= d;
    for (int i = j + 1; i < dim; i++)
      for (int k = j + 1; k <= i; k++) {
        A[i * dim + k] -= A[i * dim + j] * A[k * dim + j] * d;
        A[k * dim + i] = A[i * dim + k];
      }
  }
  /* L unit lower (strict part in A), invert L */
  for (int i = 0; i < dim * dim; i++) Linv[i] = 0;
  for (int i = 0; i < dim; i++) {
    Linv[i * dim + i] = 1;
    for (int j = 0; j < i; j++) {
      double s = 0;
      for (int k = j; k < i; k++) s += A[i * dim + k] * Linv[k * dim + j];
      Linv[i * dim + j] = -s;
    }
  }
  /* (L D L^T)^-1 = L^-T D^-1 L^-1 ; then undo the permutation */
  for (int i = 0; i < dim; i++)
    for (int j = 0; j < dim; j++) {
      double s = 0;
      for (int k = (i > j ? i : j); k < dim; k++) s += Linv[k * dim + i] * Linv[k * dim + j] / Dv[k];
      inv[perm[i] * dim + perm[j]] = s;
    }
  for (int i = 0; i < dim * dim; i++)
    if (isnan(inv[i])) return 1;
  return 0;
}

double gwo_analytic_psd(double f) {
  double x = f / 215.;
  return 1e-49 * (pow(x, -4.14) - 5. * pow(x, -2.) + 111. * (1. - x * x + 0.5 * x * x * x * x) / (1. + 0.5 * x * x));
}

/* Model internals, same layout as ref_d_internals in oracle/ref_driver.cpp. */
int gwo_d_internals(const gwo_gen_params *p, double *out) {
  src_t s;
  populate(&s, p);
  dmodel_t m;
  d_prologue(&s, &m);
  int k = 0;
  out[k++] = s.fRD;
  out[k++] = s.fdamp;
  out[k++] = s.f1;
  out[k++] = s.f3;
  out[k++] = s.f1_phase;
  out[k++] = s.f2_phase;
  for (int i = 0; i < 5; i++) out[k++] = m.deltas[i];
  for (int i = 0; i < 4; i++) out[k++] = m.lambda.beta[i];
  for (int i = 0; i < 6; i++) out[k++] = m.lambda.alpha[i];
  return k;
}
