// gwat_dropin.cpp -- definitions of the reference-signature entry points
// (include/gwat_dropin.h) on top of the C ABI (include/gwgpu.h).
//
// One process-wide engine context.  The process-global data arrays of the
// sampler (mcmc_data / mcmc_noise / mcmc_frequencies, mcmc_gw.cpp:1464-1476)
// are registered on the device the first time a (pointer, length, content
// fingerprint) triple is seen and reused afterwards, as the reference treats
// them as read-only during sampling.  The fingerprint reads 64 samples of each
// of the frequency, data and PSD arrays (and the weights) on every likelihood
// call: about 1 us of host time.  At most kMaxHandles registrations are kept;
// the least recently used one is released when a new one would exceed that,
// so a caller that refills or reallocates its arrays does not grow device
// memory without bound.  Callers on several threads are safe: the engine
// serialises them, or, in "served" mode, coalesces them into batched launches
// (one server per segment length T, kept until the process exits).
#include "../../include/gwat_dropin.h"

#include <algorithm>
#include <chrono>
#include <climits>
#include <list>
#include <thread>
#include <cmath>
#include <cstdio>
#include <stdexcept>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "../../include/gwgpu.h"

namespace gwat_dropin {

constexpr size_t kMaxHandles = 64;

using HandleKey = std::tuple<const void *, const void *, const void *, const void *, int, int, uint64_t>;

struct Engine {
  gwgpu_context *ctx = nullptr;
  bool served = false;
  std::mutex mu;
  // registered streams, most recently used first
  std::list<std::pair<HandleKey, int>> lru;
  std::map<HandleKey, std::list<std::pair<HandleKey, int>>::iterator> handles;
  // served mode: the first segment length T is served by the device-resident
  // request loop (2 blocks per SM, leaving room for other kernels of the
  // context); other values of T, and requests the loop does not take (another
  // detector count, a longer grid), by one host-scheduled server per T.
  // GWGPU_DROPIN_SERVER=host: host-scheduled servers only.  No server is
  // destroyed while the process runs, so no caller can be inside one being freed.
  std::map<double, gwgpu_server *> servers;
  gwgpu_server *loop = nullptr;
  double loop_T = 0;
  bool use_loop = true, loop_failed = false;
};

static Engine &engine() {
  static Engine e;
  static std::once_flag once;
  std::call_once(once, [] {
    const char *dev = std::getenv("GWGPU_DROPIN_DEVICE");
    gwgpu_context_create(dev ? std::atoi(dev) : 0, 0, &e.ctx);
    const char *mode = std::getenv("GWGPU_DROPIN_MODE");
    e.served = mode && std::strcmp(mode, "served") == 0;
    const char *sv = std::getenv("GWGPU_DROPIN_SERVER");
    e.use_loop = !(sv && std::strcmp(sv, "host") == 0);
  });
  return e;
}

void set_mode(const char *mode) { engine().served = mode && std::strcmp(mode, "served") == 0; }
void set_server(const char *server) { engine().use_loop = !(server && std::strcmp(server, "host") == 0); }

static uint64_t fingerprint(const double *a, int n) {
  uint64_t h = 1469598103934665603ull;
  int step = n > 64 ? n / 64 : 1;
  for (int i = 0; i < n; i += step) {
    uint64_t v;
    std::memcpy(&v, a + i, 8);
    h = (h ^ v) * 1099511628211ull;
  }
  return h;
}

static void to_abi(const gen_params_base<double> *p, gwgpu_gen_params *o) {
  gwgpu_default_params(o);
  o->mass1 = p->mass1;
  o->mass2 = p->mass2;
  for (int i = 0; i < 3; i++) {
    o->spin1[i] = p->spin1[i];
    o->spin2[i] = p->spin2[i];
  }
  o->Luminosity_Distance = p->Luminosity_Distance;
  o->incl_angle = p->incl_angle;
  o->phiRef = p->phiRef;
  o->f_ref = p->f_ref;
  o->tc = p->tc;
  o->RA = p->RA;
  o->DEC = p->DEC;
  o->psi = p->psi;
  o->gmst = p->gmst;
  o->chip = p->chip;
  o->phip = p->phip;
  o->shift_time = p->shift_time;
  o->shift_phase = p->shift_phase;
  o->sky_average = p->sky_average;
  o->dep_postmerger = p->dep_postmerger;
  o->equatorial_orientation = p->equatorial_orientation;
  o->theta_l = p->theta_l;
  o->phi_l = p->phi_l;
}

// weights: the GAUSSLEG integration (null: Simpson's rule); log10F as the reference's flag
static int handle_for(Engine &e, const std::string &det, const double *f, const std::complex<double> *d,
                      const double *psd, const double *weights, bool log10F, int n) {
  uint64_t fp = fingerprint(f, n) ^ (fingerprint((const double *)d, 2 * n) * 31) ^ (fingerprint(psd, n) * 131);
  if (weights) fp ^= fingerprint(weights, n) * 1031 + (log10F ? 7 : 3);
  auto key = std::make_tuple((const void *)f, (const void *)d, (const void *)psd, (const void *)weights, n,
                             (int)det.size() * 131 + det[0], fp);
  auto it = e.handles.find(key);
  if (it != e.handles.end()) {
    e.lru.splice(e.lru.begin(), e.lru, it->second);
    return it->second->second;
  }
  int h = -1;
  int st = weights ? gwgpu_data_register_weighted(e.ctx, det.c_str(), f, n, (const double *)d, psd, weights,
                                                  log10F ? 1 : 0, &h)
                   : gwgpu_data_register(e.ctx, det.c_str(), f, n, (const double *)d, psd, &h);
  if (st != GWGPU_OK) return -1;
  e.lru.emplace_front(key, h);
  e.handles[key] = e.lru.begin();
  return h;
}

// Release the least recently used registrations beyond kMaxHandles, keeping
// the `keep` handles of the call in progress.  Called with e.mu held, before
// any launch of that call: a released stream is never read by work in flight
// on the context stream, which the engine serialises.  In served mode the
// server may still hold requests on older streams, so nothing is released
// there while any server exists.
static void evict(Engine &e, const int *keep, int nkeep) {
  if (!e.servers.empty() || e.loop) return;
  while (e.lru.size() > kMaxHandles) {
    auto last = std::prev(e.lru.end());
    bool kept = false;
    for (int i = 0; i < nkeep; i++) kept |= keep[i] == last->second;
    if (kept) break;
    gwgpu_data_release(e.ctx, last->second);
    e.handles.erase(last->first);
    e.lru.erase(last);
  }
}

}  // namespace gwat_dropin

using namespace gwat_dropin;

template <class T>
int fourier_waveform(T *frequencies, int length, waveform_polarizations<T> *wp, std::string generation_method,
                     gen_params_base<T> *parameters) {
  gwgpu_gen_params p;
  to_abi(parameters, &p);
  return gwgpu_fourier_waveform(engine().ctx, frequencies, length, (double *)wp->hplus, (double *)wp->hcross,
                                generation_method.c_str(), &p);
}
template int fourier_waveform<double>(double *, int, waveform_polarizations<double> *, std::string,
                                      gen_params_base<double> *);

int fourier_waveform(double *frequencies, int length, std::complex<double> *waveform_plus,
                     std::complex<double> *waveform_cross, std::string generation_method, gen_params *parameters) {
  gwgpu_gen_params p;
  to_abi(parameters, &p);
  return gwgpu_fourier_waveform(engine().ctx, frequencies, length, (double *)waveform_plus, (double *)waveform_cross,
                                generation_method.c_str(), &p);
}

template <class T>
int fourier_detector_response(T *frequencies, int length, std::complex<T> *response, std::string detector,
                              std::string generation_method, gen_params_base<T> *parameters, T *times) {
  (void)times;
  gwgpu_gen_params p;
  to_abi(parameters, &p);
  if (parameters->equatorial_orientation &&
      gwgpu_transform_orientation_coords(&p, generation_method.c_str()) == GWGPU_OK) {
    parameters->psi = p.psi;  // the reference rewrites the caller's psi and inclination (waveform_util.cpp:946-948)
    parameters->incl_angle = p.incl_angle;
  }
  return gwgpu_fourier_detector_response(engine().ctx, frequencies, length, (double *)response, detector.c_str(),
                                         generation_method.c_str(), &p);
}
template int fourier_detector_response<double>(double *, int, std::complex<double> *, std::string, std::string,
                                               gen_params_base<double> *, double *);

double Log_Likelihood_internal(std::complex<double> *data, double *psd, double *frequencies, double *weights,
                               std::complex<double> *detector_response, int length, bool log10F,
                               std::string integration_method) {
  double out = NAN;
  if (integration_method == "SIMPSONS")
    gwgpu_log_likelihood_internal(engine().ctx, (const double *)data, psd, frequencies,
                                  (const double *)detector_response, length, &out);
  else if (integration_method == "GAUSSLEG" && weights)
    gwgpu_log_likelihood_internal_weighted(engine().ctx, (const double *)data, psd, frequencies, weights,
                                           (const double *)detector_response, length, log10F ? 1 : 0, &out);
  return out;
}

double MCMC_likelihood_extrinsic(bool save_waveform, gen_params_base<double> *parameters,
                                 std::string generation_method, int *data_length, double **frequencies,
                                 std::complex<double> **data, double **psd, double **weights,
                                 std::string integration_method, bool log10F, std::string *detectors,
                                 int num_detectors) {
  const bool gauss = integration_method == "GAUSSLEG";
  if (!save_waveform || !(gauss || integration_method == "SIMPSONS") || num_detectors < 1 || num_detectors > 4)
    return NAN;
  if (gauss && !weights) return NAN;
  Engine &e = engine();
  // mcmc_gw.cpp:2466 forms T from frequencies[1] - frequencies[0] of the
  // double** array, i.e. the distance between the first two detectors'
  // frequency arrays; the same expression is used here so that a caller with
  // the same arrays gets the same log L.  With one detector that expression
  // reads past the array in the reference; 1/df of the grid is used instead.
  double T = num_detectors > 1 ? 1. / (double)(frequencies[1] - frequencies[0])
                               : 1. / (frequencies[0][1] - frequencies[0][0]);
  double tc_ref = T - parameters->tc;  // mcmc_gw.cpp:2467-2473: the caller's params are mutated
  int hs[4];
  {
    std::lock_guard<std::mutex> lk(e.mu);
    for (int i = 0; i < num_detectors; i++) {
      hs[i] = handle_for(e, detectors[i], frequencies[i], data[i], psd[i], gauss ? weights[i] : nullptr, log10F,
                         data_length[i]);
      if (hs[i] < 0) return NAN;
    }
    evict(e, hs, num_detectors);
  }
  gwgpu_gen_params p;
  to_abi(parameters, &p);
  parameters->tc = tc_ref;
  double ll = NAN;
  const char *m = generation_method.c_str();
  int approx = generation_method.find("Pv2") != std::string::npos ? GWGPU_IMRPHENOMPV2 : GWGPU_IMRPHENOMD;
  if (e.served && !gauss) {  // the served (mixed) form wants uniform grids; Gauss-Legendre grids run plain
    gwgpu_server *srv = nullptr;
    // the host-scheduled server of this T (e.mu held)
    auto host_server = [&]() -> gwgpu_server * {
      auto it = e.servers.find(T);
      if (it != e.servers.end()) return it->second;
      gwgpu_server_config cfg = {16384, 1024, 4, GWGPU_PREC_MIXED, T, 0, 0, 0, 0, 0};
      gwgpu_server *h = nullptr;
      if (gwgpu_server_create(e.ctx, &cfg, &h) != GWGPU_OK || !h) return nullptr;
      e.servers[T] = h;
      return h;
    };
    {
      std::lock_guard<std::mutex> lk(e.mu);
      if (e.use_loop && !e.loop && !e.loop_failed) {
        gwgpu_server_config cfg = {16384, 1024, 4, GWGPU_PREC_MIXED, T, 0, 1, 0, 0, 2};
        if (gwgpu_server_create(e.ctx, &cfg, &e.loop) == GWGPU_OK && e.loop) {
          e.loop_T = T;
        } else {
          e.loop = nullptr;
          e.loop_failed = true;
        }
      }
      srv = e.use_loop && e.loop && e.loop_T == T ? e.loop : host_server();
      if (!srv) return NAN;
    }
    // every slot taken: back off and retry, for at most a minute
    uint64_t t;
    int st;
    const auto deadline = std::chrono::steady_clock::now() + std::chrono::seconds(60);
    auto pause = std::chrono::microseconds(20);
    for (;;) {
      st = gwgpu_server_submit(srv, &p, approx, hs, num_detectors, &t);
      if (st == GWGPU_EBUSY) {
        if (std::chrono::steady_clock::now() > deadline) return NAN;
        std::this_thread::sleep_for(pause);
        pause = std::min(pause * 2, std::chrono::microseconds(2000));
        continue;
      }
      if ((st == GWGPU_EINVAL || st == GWGPU_ETOOLARGE) && srv == e.loop) {
        // another detector count or a longer grid than the loop was sized for
        std::lock_guard<std::mutex> lk(e.mu);
        srv = host_server();
        if (!srv) return NAN;
        continue;
      }
      break;
    }
    if (st != GWGPU_OK) return NAN;
    int rst = GWGPU_OK;
    if (gwgpu_server_wait(srv, t, 600000, &ll, &rst) != GWGPU_OK || rst != GWGPU_OK) return NAN;
    return ll;
  }
  gwgpu_mcmc_likelihood_extrinsic(e.ctx, &p, m, hs, num_detectors, T, &ll);
  return ll;
}

void fisher_numerical(double *frequency, int length, std::string generation_method, std::string detector,
                      std::string reference_detector, double **output, int dimension,
                      gen_params_base<double> *parameters, int order, int *amp_tapes, int *phase_tapes,
                      double *noise) {
  (void)amp_tapes;
  (void)phase_tapes;
  gwgpu_gen_params p;
  to_abi(parameters, &p);
  std::vector<double> out((size_t)dimension * dimension, NAN);
  if (noise)
    gwgpu_fisher_numerical(engine().ctx, frequency, length, generation_method.c_str(), detector.c_str(),
                           reference_detector.c_str(), out.data(), dimension, &p, order, noise);
  for (int i = 0; i < dimension; i++)
    for (int j = 0; j < dimension; j++) output[i][j] = out[(size_t)i * dimension + j];
}

double maximized_Log_Likelihood_aligned_spin_internal(std::complex<double> *data, double *psd, double *frequencies,
                                                      std::complex<double> *detector_response, size_t length,
                                                      fftw_outline *plan) {
  (void)plan;
  double out = NAN;
  gwgpu_maximized_log_likelihood_internal(engine().ctx, (const double *)data, psd, frequencies,
                                          (const double *)detector_response, (int)length, &out);
  return out;
}

double maximized_Log_Likelihood_unaligned_spin_internal(std::complex<double> *data, double *psd, double *frequencies,
                                                        std::complex<double> *hplus, std::complex<double> *hcross,
                                                        size_t length, fftw_outline *plan) {
  (void)plan;
  double out = NAN;
  gwgpu_maximized_log_likelihood_unaligned_internal(engine().ctx, (const double *)data, psd, frequencies,
                                                    (const double *)hplus, (const double *)hcross, (int)length,
                                                    &out);
  return out;
}

// ---- data and noise ingestion
static void io_fail(int st, const std::string &file) {
  if (st == GWGPU_ENOTFOUND) {
    std::printf("ERROR -- File %s not found\n", file.c_str());
    std::exit(1);
  }
  if (st == GWGPU_EINVAL) throw std::invalid_argument("stod: " + file);
}

void read_LOSC_data_file(std::string filename, double *output, double *data_start_time, double *duration,
                         double *fs) {
  long long n = 0;
  int st = gwgpu_read_losc_data_file(filename.c_str(), output, LLONG_MAX, &n, data_start_time, duration, fs);
  if (st) io_fail(st, filename);
}

void read_LOSC_PSD_file(std::string filename, double **output, int rows, int cols) {
  std::vector<double> flat((size_t)rows * cols);
  int st = gwgpu_read_losc_psd_file(filename.c_str(), flat.data(), rows, cols);
  if (st) io_fail(st, filename);
  for (int i = 0; i < rows; i++)
    for (int j = 0; j < cols; j++) output[i][j] = flat[(size_t)i * cols + j];
}

void allocate_LOSC_data(std::string *data_files, std::string psd_file, int num_detectors, int psd_length,
                        int data_file_length, double trigger_time, double post_merger_duration,
                        std::complex<double> **data, double **psds, double **freqs) {
  std::vector<const char *> names(num_detectors);
  for (int i = 0; i < num_detectors; i++) names[i] = data_files[i].c_str();
  const size_t n = (size_t)num_detectors * psd_length;
  std::vector<double> d(2 * n), p(n), f(n);
  int st = gwgpu_allocate_losc_data(engine().ctx, names.data(), psd_file.c_str(), num_detectors, psd_length,
                                    data_file_length, trigger_time, post_merger_duration, d.data(), p.data(),
                                    f.data());
  if (st == GWGPU_ENOTFOUND || st == GWGPU_EINVAL) io_fail(st, psd_file);
  if (st != GWGPU_OK && st != GWGPU_EDOMAIN) return;
  for (int i = 0; i < num_detectors; i++)
    for (int j = 0; j < psd_length; j++) {
      psds[i][j] = p[(size_t)i * psd_length + j];
      freqs[i][j] = f[(size_t)i * psd_length + j];
    }
  if (st == GWGPU_EDOMAIN) return;  // the trigger window is outside the file: data untouched
  for (int i = 0; i < num_detectors; i++)
    for (int j = 0; j < psd_length; j++) {
      const size_t k = 2 * ((size_t)i * psd_length + j);
      data[i][j] = std::complex<double>(d[k], d[k + 1]);
    }
}

int count_lines_data_file(std::string file, int *count) {
  if (gwgpu_count_lines_data_file(file.c_str(), count) != GWGPU_OK) {
    *count = 0;
    std::printf("ERROR -- could not open file\n");
    return 1;
  }
  return 0;
}

int count_lines_LOSC_PSD_file(std::string file, int *count) {
  count_lines_data_file(file, count);
  *count -= 1;
  return 0;
}

int count_lines_LOSC_data_file(std::string file, int *count) {
  count_lines_data_file(file, count);
  *count -= 3;
  return 0;
}

void populate_noise(double *frequencies, std::string detector, double *noise_root, int length,
                    double integration_time) {
  std::string dir;
  if (const char *e = std::getenv("GWGPU_NOISE_DIR")) dir = e;
#ifdef GWAT_SHARE_DIR
  else dir = std::string(GWAT_SHARE_DIR) + "noise_data/";
#endif
  int st = gwgpu_populate_noise(frequencies, detector.c_str(), noise_root, length, integration_time,
                                dir.empty() ? nullptr : dir.c_str());
  if (st == GWGPU_ENOTFOUND) std::printf("Detector %s not supported\n", detector.c_str());
}

// ---- C entry points for the test suite (ctypes cannot call the C++ symbols)
// allocate_LOSC_data through the reference signature: outputs flat like the C ABI.
extern "C" void gwat_dropin_test_losc(const char *const *files, int nd, const char *psd_file, int psd_length,
                                      int data_file_length, double trigger, double post, double *data, double *psds,
                                      double *freqs) {
  std::vector<std::string> names(files, files + nd);
  std::vector<std::complex<double> *> dr(nd);
  std::vector<double *> pr(nd), fr(nd);
  for (int i = 0; i < nd; i++) {
    dr[i] = (std::complex<double> *)(data + 2 * (size_t)i * psd_length);
    pr[i] = psds + (size_t)i * psd_length;
    fr[i] = freqs + (size_t)i * psd_length;
  }
  allocate_LOSC_data(names.data(), psd_file, nd, psd_length, data_file_length, trigger, post, dr.data(), pr.data(),
                     fr.data());
}

// The maximised likelihood through the reference signatures (hc null: aligned).
extern "C" double gwat_dropin_test_maxll(const double *data, const double *psd, const double *f, const double *hp,
                                         const double *hc, int N) {
  auto *d = (std::complex<double> *)data;
  auto *p = (std::complex<double> *)hp;
  if (!hc)
    return maximized_Log_Likelihood_aligned_spin_internal(d, const_cast<double *>(psd), const_cast<double *>(f), p,
                                                          (size_t)N, nullptr);
  return maximized_Log_Likelihood_unaligned_spin_internal(d, const_cast<double *>(psd), const_cast<double *>(f), p,
                                                          (std::complex<double> *)hc, (size_t)N, nullptr);
}

extern "C" double gwat_dropin_test_loglik_gl(const double *f, int N, const double *const *data,
                                             const double *const *psd, const double *const *weights, int log10F,
                                             const char *const *dets, int ndet, const gwgpu_gen_params *pp,
                                             double *tc_after);
extern "C" double gwat_dropin_test_loglik(const double *f, int N, const double *const *data,
                                          const double *const *psd, const char *const *dets, int ndet,
                                          const gwgpu_gen_params *pp, int served, double *tc_after) {
  gen_params_base<double> g;
  g.mass1 = pp->mass1;
  g.mass2 = pp->mass2;
  for (int i = 0; i < 3; i++) {
    g.spin1[i] = pp->spin1[i];
    g.spin2[i] = pp->spin2[i];
  }
  g.Luminosity_Distance = pp->Luminosity_Distance;
  g.incl_angle = pp->incl_angle;
  g.phiRef = pp->phiRef;
  g.f_ref = pp->f_ref;
  g.tc = pp->tc;
  g.RA = pp->RA;
  g.DEC = pp->DEC;
  g.psi = pp->psi;
  g.gmst = pp->gmst;
  set_mode(served ? "served" : "plain");  // served: 1 the device loop, 2 the host scheduler
  set_server(served == 2 ? "host" : "loop");
  std::vector<int> len(ndet, N);
  std::vector<double *> fs(ndet), ps(ndet), ws(ndet, nullptr);
  std::vector<std::complex<double> *> ds(ndet);
  std::vector<std::string> dn(ndet);
  // one copy of the grid per detector, laid out back to back in one block,
  // so that frequencies[1] - frequencies[0] is N elements
  std::vector<double> fblock((size_t)ndet * N);
  for (int i = 0; i < ndet; i++) {
    std::copy(f, f + N, fblock.begin() + (size_t)i * N);
    fs[i] = fblock.data() + (size_t)i * N;
    ps[i] = const_cast<double *>(psd[i]);
    ds[i] = (std::complex<double> *)data[i];
    dn[i] = dets[i];
  }
  double ll = MCMC_likelihood_extrinsic(true, &g, "IMRPhenomD", len.data(), fs.data(), ds.data(), ps.data(),
                                        ws.data(), "SIMPSONS", false, dn.data(), ndet);
  if (tc_after) tc_after[0] = g.tc;
  if (tc_after) tc_after[1] = ndet > 1 ? 1. / (double)(fs[1] - fs[0]) : 1. / (f[1] - f[0]);
  return ll;
}

// The same with the GAUSSLEG integration (weights per detector), plain mode.
extern "C" double gwat_dropin_test_loglik_gl(const double *f, int N, const double *const *data,
                                             const double *const *psd, const double *const *weights, int log10F,
                                             const char *const *dets, int ndet, const gwgpu_gen_params *pp,
                                             double *tc_after) {
  gen_params_base<double> g;
  g.mass1 = pp->mass1;
  g.mass2 = pp->mass2;
  for (int i = 0; i < 3; i++) {
    g.spin1[i] = pp->spin1[i];
    g.spin2[i] = pp->spin2[i];
  }
  g.Luminosity_Distance = pp->Luminosity_Distance;
  g.incl_angle = pp->incl_angle;
  g.phiRef = pp->phiRef;
  g.f_ref = pp->f_ref;
  g.tc = pp->tc;
  g.RA = pp->RA;
  g.DEC = pp->DEC;
  g.psi = pp->psi;
  g.gmst = pp->gmst;
  set_mode("plain");
  std::vector<int> len(ndet, N);
  std::vector<double *> fs(ndet), ps(ndet), ws(ndet);
  std::vector<std::complex<double> *> ds(ndet);
  std::vector<std::string> dn(ndet);
  std::vector<double> fblock((size_t)ndet * N);
  for (int i = 0; i < ndet; i++) {
    std::copy(f, f + N, fblock.begin() + (size_t)i * N);
    fs[i] = fblock.data() + (size_t)i * N;
    ps[i] = const_cast<double *>(psd[i]);
    ws[i] = const_cast<double *>(weights[i]);
    ds[i] = (std::complex<double> *)data[i];
    dn[i] = dets[i];
  }
  double ll = MCMC_likelihood_extrinsic(true, &g, "IMRPhenomD", len.data(), fs.data(), ds.data(), ps.data(),
                                        ws.data(), "GAUSSLEG", log10F != 0, dn.data(), ndet);
  if (tc_after) tc_after[0] = g.tc;
  if (tc_after) tc_after[1] = ndet > 1 ? 1. / (double)(fs[1] - fs[0]) : 1. / (f[1] - f[0]);
  return ll;
}
