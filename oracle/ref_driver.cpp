// ref_driver.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Links the reference's own, unmodified src/IMRPhenomD.cpp and
// src/IMRPhenomP.cpp (compiled where they lie, against the test-only shim
// headers in oracle/shim/) into oracle/_ref/libgwatref.so, so the C oracle can
// be pinned against the reference's model code.  What those two translation
// units need from util.cpp is restated here (cited per function), and the
// D/Pv2 branches of fourier_waveform (waveform_generator.cpp:104-273) and
// prep_source_parameters (waveform_generator.cpp:1255-1292) are restated
// around the reference classes.
//
// Built by oracle/ref_build.sh only where the reference sources exist.
#include "IMRPhenomD.h"
#include "IMRPhenomP.h"
#include "util.h"

#include <complex>
#include <cstring>
#include <string>

#include "gwat_oracle.h"

// ---- util.cpp restatements (only what the two model TUs reference) ----
double pow_int(double base, int power) {  // util.cpp:1585-1597
  if (power == 0) return 1.;
  double prod = 1;
  int pw = std::abs(power);
  for (int i = 0; i < pw; i++) prod = prod * base;
  if (power > 0) return prod;
  return 1. / prod;
}
adouble pow_int(adouble base, int power) {
  if (power == 0) return 1.;
  adouble prod = 1;
  int pw = std::abs(power);
  for (int i = 0; i < pw; i++) prod = prod * base;
  if (power > 0) return prod;
  return 1. / prod;
}
long factorial(long num) {  // util.cpp:1569-1580
  int prod = 1;
  int step = num;
  while (step > 0) {
    prod *= step;
    step -= 1;
  }
  return prod;
}
double calculate_chirpmass(double m1, double m2) { return pow(m1 * m2, 3. / 5) / pow(m1 + m2, 1. / 5); }
adouble calculate_chirpmass(adouble m1, adouble m2) { return pow(m1 * m2, 3. / 5) / pow(m1 + m2, 1. / 5); }
double calculate_eta(double m1, double m2) { return (m1 * m2) / pow(m1 + m2, 2); }
adouble calculate_eta(adouble m1, adouble m2) { return (m1 * m2) / pow(m1 + m2, 2); }
double calculate_mass1(double mc, double eta) {
  double etapow = pow(eta, 3. / 5);
  return 1. / 2 * (mc / etapow + sqrt(1. - 4 * eta) * mc / etapow);
}
adouble calculate_mass1(adouble mc, adouble eta) {
  adouble etapow = pow(eta, 3. / 5);
  return 1. / 2 * (mc / etapow + sqrt(1. - 4 * eta) * mc / etapow);
}
double calculate_mass2(double mc, double eta) {
  double etapow = pow(eta, 3. / 5);
  return 1. / 2 * (mc / etapow - sqrt(1. - 4 * eta) * mc / etapow);
}
adouble calculate_mass2(adouble mc, adouble eta) {
  adouble etapow = pow(eta, 3. / 5);
  return 1. / 2 * (mc / etapow - sqrt(1. - 4 * eta) * mc / etapow);
}
template <class T>
T copysign_internal(T val, T sign) {  // util.cpp:566-569
  return sqrt(val * val / (sign * sign)) * sign;
}
template double copysign_internal<double>(double, double);
template adouble copysign_internal<adouble>(adouble, adouble);
template <class T>
T A0_from_DL(T chirpmass, T DL, bool sky_average) {  // util.cpp:1271-1279
  if (sky_average) return sqrt(M_PI / 30) * chirpmass * chirpmass / DL * pow(M_PI * chirpmass, -7. / 6);
  return sqrt(M_PI * 40. / 192.) * chirpmass * chirpmass / DL * pow(M_PI * chirpmass, -7. / 6);
}
template <class T>
std::complex<T> cpolar(T mag, T phase) {  // util.cpp:1944-1947
  return mag * std::exp(std::complex<T>(0, 1) * phase);
}
template <class T>
std::complex<T> XLALSpinWeightedSphericalHarmonic(T theta, T phi, int s, int l, int m) {  // util.cpp:1953-2333 (s=-2,l=2)
  T fac = 0.0;
  std::complex<T> ans = std::complex<T>(0.0, 0.0);
  if (s == -2 && l == 2) {
    switch (m) {
      case -2: fac = sqrt(5.0 / (64.0 * M_PI)) * (1.0 - cos(theta)) * (1.0 - cos(theta)); break;
      case -1: fac = sqrt(5.0 / (16.0 * M_PI)) * sin(theta) * (1.0 - cos(theta)); break;
      case 0: fac = sqrt(15.0 / (32.0 * M_PI)) * sin(theta) * sin(theta); break;
      case 1: fac = sqrt(5.0 / (16.0 * M_PI)) * sin(theta) * (1.0 + cos(theta)); break;
      case 2: fac = sqrt(5.0 / (64.0 * M_PI)) * (1.0 + cos(theta)) * (1.0 + cos(theta)); break;
    }
  }
  if (m) ans = cpolar((T)(1.0), (T)(m * phi)) * fac;
  else ans = fac;
  return ans;
}
template std::complex<double> XLALSpinWeightedSphericalHarmonic<double>(double, double, int, int, int);
template std::complex<adouble> XLALSpinWeightedSphericalHarmonic<adouble>(adouble, adouble, int, int, int);

template <class T>
void source_parameters<T>::populate_source_parameters(gen_params_base<T> *param_in) {  // util.cpp:997-1030
  this->mass1 = param_in->mass1 * MSOL_SEC;
  this->mass2 = param_in->mass2 * MSOL_SEC;
  this->spin1x = param_in->spin1[0];
  this->spin2x = param_in->spin2[0];
  this->spin1y = param_in->spin1[1];
  this->spin2y = param_in->spin2[1];
  this->spin1z = param_in->spin1[2];
  this->spin2z = param_in->spin2[2];
  this->chi_s = (1. / 2) * (this->spin1z + this->spin2z);
  this->chi_a = (1. / 2) * (this->spin1z - this->spin2z);
  this->chirpmass = calculate_chirpmass(this->mass1, this->mass2);
  this->eta = calculate_eta(this->mass1, this->mass2);
  this->M = this->mass1 + this->mass2;
  this->chi_eff = (this->mass1 * (this->spin1z) + this->mass2 * (this->spin2z)) / (this->M);
  this->chi_pn = this->chi_eff - (38 * this->eta / 113) * (2 * this->chi_s);
  this->DL = param_in->Luminosity_Distance * MPC_SEC;
  this->delta_mass = sqrt(1. - 4 * this->eta);
  this->phiRef = param_in->phiRef;
  this->tc = param_in->tc;
  this->sky_average = param_in->sky_average;
  this->A0 = A0_from_DL(this->chirpmass, this->DL, this->sky_average);
}
template <class T>
source_parameters<T> source_parameters<T>::populate_source_parameters_old(T, T, T, T *, T *, T, T, bool) {
  return source_parameters<T>();
}
template struct source_parameters<double>;
template struct source_parameters<adouble>;
template <class T>
void debugger_print(const char *file, const int line, T message) {
  (void)file;
  (void)line;
  (void)message;
}
template void debugger_print<const char *>(const char *, int, const char *);
template void debugger_print<std::string>(const char *, int, std::string);

// ---- restated glue around the reference classes ----
static void to_gen_params(const gwo_gen_params *p, gen_params_base<double> *g) {
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

extern "C" int ref_fourier_waveform(const double *freqs, int length, double *hplus, double *hcross, int approximant,
                                    const gwo_gen_params *p) {
  gen_params_base<double> in;
  to_gen_params(p, &in);
  source_parameters<double> params;
  params.populate_source_parameters(&in);  // waveform_generator.cpp:1258-1271
  params.phi = in.phi;
  params.theta = in.theta;
  params.incl_angle = in.incl_angle;
  params.f_ref = in.f_ref;
  params.phiRef = in.phiRef;
  params.shift_time = in.shift_time;
  params.sky_average = in.sky_average;
  params.shift_phase = in.shift_phase;
  params.dep_postmerger = in.dep_postmerger;
  std::complex<double> *hp = reinterpret_cast<std::complex<double> *>(hplus);
  std::complex<double> *hc = reinterpret_cast<std::complex<double> *>(hcross);
  double *f = const_cast<double *>(freqs);
  if (approximant == GWO_IMRPHENOMD) {
    std::complex<double> ci = std::complex<double>(cos(params.incl_angle), 0);
    IMRPhenomD<double> modeld;
    modeld.construct_waveform(f, length, hp, &params);
    for (int i = 0; i < length; i++) {  // waveform_generator.cpp:191-200
      hc[i] = std::complex<double>(0, -1) * hp[i];
    }
    for (int i = 0; i < length; i++) {
      hc[i] *= ci;
      hp[i] *= std::complex<double>(.5, 0) * (std::complex<double>(1, 0) + ci * ci);
    }
    return 1;
  }
  if (approximant == GWO_IMRPHENOMPV2) {
    IMRPhenomPv2<double> model;
    if ((in.chip + 1) > DOUBLE_COMP_THRESH) {  // waveform_generator.cpp:1272-1281
      params.chip = in.chip;
      params.spin1z = in.spin1[2];
      params.spin2z = in.spin2[2];
      params.phip = in.phip;
      model.PhenomPv2_Param_Transform_reduced(&params);
    } else {
      model.PhenomPv2_Param_Transform(&params);
    }
    model.construct_waveform(f, length, hp, hc, &params);
    std::complex<double> c2z = std::complex<double>(cos(2. * params.zeta_polariz));
    std::complex<double> s2z = std::complex<double>(sin(2. * params.zeta_polariz));
    for (int i = 0; i < length; i++) {  // waveform_generator.cpp:257-266
      std::complex<double> tp = hp[i], tx = hc[i];
      hp[i] = c2z * tp + s2z * tx;
      hc[i] = c2z * tx - s2z * tp;
    }
    return 1;
  }
  return 0;
}

// Model internals for the pin tests: fRD, fdamp, f1, f3, f1_phase, f2_phase,
// deltas[0..4], beta[0..3], alpha[0..5] (19 + 6 = 25 values).
extern "C" int ref_d_internals(const gwo_gen_params *p, double *out) {
  gen_params_base<double> in;
  to_gen_params(p, &in);
  source_parameters<double> params;
  params.populate_source_parameters(&in);
  params.f_ref = in.f_ref;
  params.phiRef = in.phiRef;
  params.shift_time = in.shift_time;
  params.shift_phase = in.shift_phase;
  params.dep_postmerger = in.dep_postmerger;
  IMRPhenomD<double> m;
  lambda_parameters<double> lambda;
  m.assign_lambda_param(&params, &lambda);
  m.post_merger_variables(&params);
  params.f1_phase = 0.018 / (params.M);
  params.f2_phase = params.fRD / 2.;
  params.f1 = 0.014 / (params.M);
  params.f3 = m.fpeak(&params, &lambda);
  double deltas[6], pn_amp[7], pn_phase[12];
  m.assign_pn_amplitude_coeff(&params, pn_amp);
  m.assign_static_pn_phase_coeff(&params, pn_phase);
  m.amp_connection_coeffs(&params, &lambda, pn_amp, deltas);
  m.phase_connection_coefficients(&params, &lambda, pn_phase);
  int k = 0;
  out[k++] = params.fRD;
  out[k++] = params.fdamp;
  out[k++] = params.f1;
  out[k++] = params.f3;
  out[k++] = params.f1_phase;
  out[k++] = params.f2_phase;
  for (int i = 0; i < 5; i++) out[k++] = deltas[i];
  for (int i = 0; i < 4; i++) out[k++] = lambda.beta[i];
  for (int i = 0; i < 6; i++) out[k++] = lambda.alpha[i];
  return k;
}
