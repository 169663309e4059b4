// ref_glue.cpp -- TEST INFRASTRUCTURE ONLY.
//
// C entry points into the reference's own, unmodified translation units
// (detector_util.cpp, waveform_util.cpp, waveform_generator.cpp, util.cpp,
// mcmc_gw.cpp, fisher.cpp, IMRPhenomD.cpp, IMRPhenomP.cpp, ...), compiled
// where they lie against the test-only shim headers of oracle/shim/ into
// oracle/_ref/libgwatref_full.so (oracle/Makefile, target "full").  The pin
// tests call these to check the C oracle (oracle/gwat_oracle.c) against the
// reference's own code for the glue of the path: antenna patterns, arrival
// times, detector responses, Log_Likelihood_internal,
// MCMC_likelihood_extrinsic, MCMC_likelihood_wrapper (with MCMC_prep_params
// and repack_parameters), fisher_numerical, MCMC_fisher_wrapper and the
// maximised likelihoods.
//
// The sampler callback is reached the way the reference reaches it:
// PTMCMC_MH_dynamic_PT_alloc_uncorrelated_GW (mcmc_gw.cpp:1422) sets the
// process state of mcmc_gw.cpp and hands MCMC_likelihood_wrapper and
// MCMC_fisher_wrapper to the sampler PTMCMC_MH_dynamic_PT_alloc_uncorrelated.
// This file defines that sampler symbol: instead of sampling, it evaluates the
// two callbacks at the positions the test asks for.
#include <omp.h>

#include <chrono>
#include <complex>
#include <cstring>
#include <string>
#include <vector>

#include "detector_util.h"
#include "fisher.h"
#include "mcmc_gw.h"
#include "mcmc_io_util.h"
#include "mcmc_sampler.h"
#include "util.h"
#include "waveform_generator.h"
#include "waveform_util.h"

#include "gwat_oracle.h"

static void to_ref(const gwo_gen_params *p, gen_params_base<double> *g) {
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
  g->theta_l = p->theta_l;
  g->phi_l = p->phi_l;
  g->equatorial_orientation = p->equatorial_orientation != 0;
}

static void from_ref(const gen_params_base<double> *g, gwo_gen_params *p) {
  p->mass1 = g->mass1;
  p->mass2 = g->mass2;
  for (int i = 0; i < 3; i++) {
    p->spin1[i] = g->spin1[i];
    p->spin2[i] = g->spin2[i];
  }
  p->Luminosity_Distance = g->Luminosity_Distance;
  p->incl_angle = g->incl_angle;
  p->phiRef = g->phiRef;
  p->f_ref = g->f_ref;
  p->tc = g->tc;
  p->RA = g->RA;
  p->DEC = g->DEC;
  p->psi = g->psi;
  p->gmst = g->gmst;
  p->chip = g->chip;
  p->phip = g->phip;
  p->shift_time = g->shift_time;
  p->shift_phase = g->shift_phase;
  p->sky_average = g->sky_average;
  p->dep_postmerger = g->dep_postmerger;
  p->theta_l = g->theta_l;
  p->phi_l = g->phi_l;
  p->equatorial_orientation = g->equatorial_orientation;
}

extern "C" {

// fourier_waveform (waveform_generator.h:70-74) through the template form.
int gwr_fourier_waveform(double *freqs, int n, double *hp, double *hc, const char *method, const gwo_gen_params *p) {
  gen_params_base<double> g;
  to_ref(p, &g);
  waveform_polarizations<double> wp;
  wp.hplus = (std::complex<double> *)hp;
  wp.hcross = (std::complex<double> *)hc;
  int st = fourier_waveform(freqs, n, &wp, std::string(method), &g);
  wp.hplus = wp.hcross = nullptr;
  return st;
}

// fourier_detector_response (waveform_util.cpp:1070-1088); p_after gets the
// parameters as the call left them (equatorial_orientation rewrites psi and
// the inclination).
int gwr_fourier_detector_response(double *freqs, int n, double *out, const char *det, const char *method,
                                  const gwo_gen_params *p, gwo_gen_params *p_after) {
  gen_params_base<double> g;
  to_ref(p, &g);
  int st = fourier_detector_response(freqs, n, (std::complex<double> *)out, std::string(det), std::string(method), &g,
                                     (double *)nullptr);
  if (p_after) from_ref(&g, p_after);
  return st;
}

// transform_orientation_coords (waveform_util.cpp:1523-1586).
void gwr_transform_orientation_coords(const gwo_gen_params *p, const char *method, const char *det,
                                      gwo_gen_params *out) {
  gen_params_base<double> g;
  to_ref(p, &g);
  transform_orientation_coords(&g, std::string(method), std::string(det));
  from_ref(&g, out);
}

// detector_response_functions_equatorial, string form (detector_util.cpp:1037-).
void gwr_antenna(const char *det, double ra, double dec, double psi, double gmst, double *fp, double *fc) {
  det_res_pat<double> r;
  r.Fplus = fp;
  r.Fcross = fc;
  bool active[6] = {true, true, false, false, false, false};
  r.active_polarizations = active;
  detector_response_functions_equatorial(std::string(det), ra, dec, psi, gmst, &r);
}

// DTOA_DETECTOR (detector_util.cpp:677-790).
double gwr_dtoa(double ra, double dec, double gmst, const char *d1, const char *d2) {
  return DTOA_DETECTOR(ra, dec, gmst, std::string(d1), std::string(d2));
}

// Log_Likelihood_internal (mcmc_gw.cpp:801-873).
double gwr_log_likelihood_internal(double *data, double *psd, double *freqs, double *weights, double *resp, int n,
                                   int log10F, const char *integration) {
  return Log_Likelihood_internal((std::complex<double> *)data, psd, freqs, weights, (std::complex<double> *)resp, n,
                                 log10F != 0, std::string(integration));
}

// MCMC_likelihood_extrinsic (mcmc_gw.cpp:2374-2487).  freqs[d] are the
// caller's arrays: the reference forms T from freqs[1] - freqs[0] as pointers
// (mcmc_gw.cpp:2466), so their placement in memory matters; the T it used and
// the t_c it left are returned.
double gwr_mcmc_likelihood_extrinsic(const gwo_gen_params *p, const char *method, int *lengths, double **freqs,
                                     double **data, double **psd, double **weights, const char *integration,
                                     int log10F, const char **dets, int ndet, double *T_used, double *tc_after) {
  gen_params_base<double> g;
  to_ref(p, &g);
  std::vector<std::string> dn(dets, dets + ndet);
  std::vector<std::complex<double> *> dd(ndet);
  for (int i = 0; i < ndet; i++) dd[i] = (std::complex<double> *)data[i];
  double ll = MCMC_likelihood_extrinsic(true, &g, std::string(method), lengths, freqs, dd.data(), psd, weights,
                                        std::string(integration), log10F != 0, dn.data(), ndet);
  if (T_used) *T_used = ndet > 1 ? 1. / (double)(freqs[1] - freqs[0]) : 0.0;
  if (tc_after) *tc_after = g.tc;
  return ll;
}

// fisher_numerical (fisher.cpp:81-146), output dim x dim row major.
void gwr_fisher_numerical(double *freqs, int n, const char *method, const char *det, const char *refdet, double *out,
                          int dim, const gwo_gen_params *p, int order, double *noise) {
  gen_params_base<double> g;
  to_ref(p, &g);
  std::vector<double *> rows(dim);
  for (int i = 0; i < dim; i++) rows[i] = out + (size_t)i * dim;
  fisher_numerical(freqs, n, std::string(method), std::string(det), std::string(refdet), rows.data(), dim, &g, order,
                   nullptr, nullptr, noise);
}

// maximized_Log_Likelihood_aligned_spin_internal (mcmc_gw.cpp:595-658).
double gwr_maximized_aligned(double *data, double *psd, double *freqs, double *resp, int n) {
  fftw_outline plan;
  allocate_FFTW_mem_forward(&plan, n);
  double ll = maximized_Log_Likelihood_aligned_spin_internal((std::complex<double> *)data, psd, freqs,
                                                            (std::complex<double> *)resp, (size_t)n, &plan);
  deallocate_FFTW_mem(&plan);
  return ll;
}

// maximized_Log_Likelihood_unaligned_spin_internal (mcmc_gw.cpp:660-800).
double gwr_maximized_unaligned(double *data, double *psd, double *freqs, double *hp, double *hc, int n) {
  fftw_outline plan;
  allocate_FFTW_mem_forward(&plan, n);
  double ll = maximized_Log_Likelihood_unaligned_spin_internal((std::complex<double> *)data, psd, freqs,
                                                              (std::complex<double> *)hp, (std::complex<double> *)hc,
                                                              (size_t)n, &plan);
  deallocate_FFTW_mem(&plan);
  return ll;
}

// gps_to_GMST_radian (util.cpp:1840-1845).
double gwr_gps_to_gmst_radian(double gps) { return gps_to_GMST_radian(gps); }

}  // extern "C"

// ---- the sampler callbacks, reached through the reference's own set-up ----
namespace {
struct EvalRequest {
  int npos = 0, dim = 0, nthreads = 1;
  const double *positions = nullptr;
  double *loglik = nullptr;
  double *fisher = nullptr;
  double seconds = 0;
};
EvalRequest g_req;
}  // namespace

// The sampler symbol that PTMCMC_MH_dynamic_PT_alloc_uncorrelated_GW calls
// (mcmc_sampler.h:417).  Evaluates log_likelihood (and fisher, when asked) at
// each requested position; one chain per OpenMP thread with its own
// user_parameters entry, as the reference's sampler runs its chains.
void PTMCMC_MH_dynamic_PT_alloc_uncorrelated(
    mcmc_sampler_output *, double **, int dimension, int, int chain_N, int, double *, double *, double **, double *,
    int, int, int, int, std::string, double (*)(double *, mcmc_data_interface *, void *),
    double (*log_likelihood)(double *, mcmc_data_interface *, void *),
    void (*fisher)(double *, double **, mcmc_data_interface *, void *), void **user_parameters, int, bool, bool,
    std::string, std::string, std::string, std::string) {
  EvalRequest &r = g_req;
  const int nthr = r.nthreads < 1 ? 1 : (r.nthreads > chain_N ? chain_N : r.nthreads);
  auto t0 = std::chrono::steady_clock::now();
#pragma omp parallel num_threads(nthr)
  {
    const int tid = omp_get_thread_num();
    mcmc_data_interface iface;
    iface.min_dim = dimension;
    iface.max_dim = dimension;
    iface.chain_id = tid;
    iface.chain_number = chain_N;
    iface.nested_model_number = 0;
    std::vector<double> pos(dimension);
    std::vector<double> fout((size_t)dimension * dimension);
    std::vector<double *> frows(dimension);
    for (int i = 0; i < dimension; i++) frows[i] = fout.data() + (size_t)i * dimension;
#pragma omp for schedule(dynamic, 1)
    for (int k = 0; k < r.npos; k++) {
      std::memcpy(pos.data(), r.positions + (size_t)k * dimension, sizeof(double) * dimension);
      if (r.loglik) r.loglik[k] = log_likelihood(pos.data(), &iface, user_parameters[tid]);
      if (r.fisher && fisher) {
        std::memcpy(pos.data(), r.positions + (size_t)k * dimension, sizeof(double) * dimension);
        fisher(pos.data(), frows.data(), &iface, user_parameters[tid]);
        std::memcpy(r.fisher + (size_t)k * dimension * dimension, fout.data(),
                    sizeof(double) * dimension * dimension);
      }
    }
  }
  r.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

extern "C" {

// Runs MCMC_likelihood_wrapper (mcmc_gw.cpp:2569) and, if fisher != NULL,
// MCMC_fisher_wrapper (mcmc_gw.cpp:2230) at npos positions of dimension dim,
// after PTMCMC_MH_dynamic_PT_alloc_uncorrelated_GW (mcmc_gw.cpp:1422) has set
// up its data, detectors, GMST from gps_time and the parameterisation.
// freqs[d], data[d] (complex interleaved), psd[d] have lengths[d] entries;
// the reference forms T from freqs[1] - freqs[0] as pointers, which the
// caller controls through where it places the arrays.  Returns the wall time
// of the evaluations in seconds.
double gwr_sampler_eval(const char *method, int dim, int ndet, const char **dets, double **freqs, double **data,
                        double **psd, int *lengths, double gps_time, int npos, const double *positions,
                        double *loglik, double *fisher, int nthreads) {
  g_req.npos = npos;
  g_req.dim = dim;
  g_req.positions = positions;
  g_req.loglik = loglik;
  g_req.fisher = fisher;
  g_req.nthreads = nthreads;
  std::vector<std::string> dn(dets, dets + ndet);
  std::vector<std::complex<double> *> dd(ndet);
  for (int i = 0; i < ndet; i++) dd[i] = (std::complex<double> *)data[i];
  MCMC_modification_struct mod;
  std::vector<double> init(positions, positions + dim);
  const int chains = nthreads < 1 ? 1 : nthreads;
  std::vector<double> temps(chains, 1.0);
  PTMCMC_MH_dynamic_PT_alloc_uncorrelated_GW(nullptr, nullptr, dim, 0, chains, chains, init.data(), nullptr, nullptr,
                                             temps.data(), 1, 1, 1, 1, "cold", nullptr, chains, false, false, ndet,
                                             dd.data(), psd, freqs, lengths, gps_time, dn.data(), &mod,
                                             std::string(method), "", "", "", "");
  return g_req.seconds;
}

}  // extern "C"
