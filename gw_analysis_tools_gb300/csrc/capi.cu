// capi.cu -- the C ABI (include/gwgpu.h): context, device-resident data
// registry, per-bin tables, and the plain / batched / waveform entry points.
//
// Thread safety: every entry point takes the context mutex, so callers on
// several host threads (the reference sampler evaluates one chain per thread,
// mcmc_sampler.cpp:4585-4590) are serialised onto the context stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/gwgpu.h"
#include "capi_internal.h"
#include "cufft_rt.h"
#include "kernels.h"

using gwk::StreamDev;

static_assert(sizeof(gwgpu_gen_params) == sizeof(gwt::GenParams), "gen params layout");

namespace {

int det_index(const char *n) {  // detector names of detector_util.cpp:1037-1160
  static const char *names[9][3] = {{"Hanford", "hanford", ""},
                                    {"Livingston", "livingston", ""},
                                    {"Virgo", "virgo", ""},
                                    {"Kagra", "kagra", ""},
                                    {"Indigo", "indigo", ""},
                                    {"Cosmic Explorer", "cosmic explorer", "CE"},
                                    {"Einstein Telescope 1", "einstein telescope 1", "ET1"},
                                    {"Einstein Telescope 2", "einstein telescope 2", "ET2"},
                                    {"Einstein Telescope 3", "einstein telescope 3", "ET3"}};
  if (!n) return -1;
  for (int i = 0; i < 9; i++)
    for (int j = 0; j < 3; j++)
      if (names[i][j][0] && std::strcmp(n, names[i][j]) == 0) return i;
  return -1;
}

int method_approx(const char *m) {  // fourier_waveform dispatch (waveform_generator.cpp:129-273)
  if (!m) return -1;
  std::string s(m);
  if (s == "IMRPhenomD" || s == "MCMC_IMRPhenomD") return gwt::kPhenomD;
  if (s == "IMRPhenomPv2" || s == "MCMC_IMRPhenomPv2") return gwt::kPhenomPv2;
  return -1;
}

}  // namespace

// ------------------------------------------------------------------ context
gwgpu_context::~gwgpu_context() {}

int gwgpu_context::fail(cudaError_t e, const char *where) {
  last_error = std::string(where) + ": " + cudaGetErrorString(e);
  return GWGPU_ECUDA;
}

int gwgpu_context::dalloc(void **p, size_t bytes, const char *what) {
  if (budget && in_use + bytes > budget) {
    last_error = std::string("HBM budget exceeded allocating ") + what;
    return GWGPU_ENOMEM;
  }
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) return fail(e, what);
  sizes[*p] = bytes;
  in_use += bytes;
  return GWGPU_OK;
}
void gwgpu_context::dfree(void *p) {
  if (!p) return;
  auto it = sizes.find(p);
  if (it != sizes.end()) {
    in_use -= it->second;
    sizes.erase(it);
  }
  cudaFree(p);
}
int gwgpu_context::workspace(int slot, size_t bytes, void **out) {
  Workspace &w = ws[slot];
  if (w.bytes < bytes) {
    dfree(w.ptr);
    w.ptr = nullptr;
    w.bytes = 0;
    size_t nb = std::max(bytes, (size_t)4096);
    int st = dalloc(&w.ptr, nb, "workspace");
    if (st) return st;
    w.bytes = nb;
  }
  *out = w.ptr;
  return GWGPU_OK;
}
int gwgpu_context::pinned(int slot, size_t bytes, void **out) {
  Workspace &w = hws[slot];
  if (w.bytes < bytes) {
    if (w.ptr) cudaFreeHost(w.ptr);
    w.ptr = nullptr;
    w.bytes = 0;
    size_t nb = std::max(bytes, (size_t)4096);
    cudaError_t e = cudaMallocHost(&w.ptr, nb);
    if (e != cudaSuccess) return fail(e, "cudaMallocHost");
    w.bytes = nb;
  }
  *out = w.ptr;
  return GWGPU_OK;
}

// Per-bin tables n^(1/3), n^(-5/3), ln n, n^(3/4) (FP64) and n^(1/3), n^(-7/6) (FP32).
int gwgpu_context::ensure_tables(int nmax) {
  if (nmax <= tables.nmax) return GWGPU_OK;
  int nm = std::max(nmax, 1 << 16);
  size_t n1 = (size_t)nm + 1;
  std::vector<double> t13(n1), tm53(n1), tln(n1), t34(n1);
  std::vector<float> t13f(n1), tm76f(n1);
  for (size_t n = 1; n < n1; n++) {
    double x = (double)n;
    t13[n] = std::cbrt(x);
    tm53[n] = std::pow(x, -5. / 3.);
    tln[n] = std::log(x);
    t34[n] = std::pow(x, 0.75);
    t13f[n] = (float)std::cbrt(x);
    tm76f[n] = (float)std::pow(x, -7. / 6.);
  }
  t13[0] = tm53[0] = tln[0] = t34[0] = 0.0;
  t13f[0] = tm76f[0] = 0.f;
  for (void *p : table_mem) dfree(p);
  table_mem.clear();
  void *p[6];
  size_t sz[6] = {8, 8, 8, 8, 4, 4};
  const void *src[6] = {t13.data(), tm53.data(), tln.data(), t34.data(), t13f.data(), tm76f.data()};
  for (int i = 0; i < 6; i++) {
    int st = dalloc(&p[i], sz[i] * n1, "tables");
    if (st) return st;
    table_mem.push_back(p[i]);
    cudaError_t e = cudaMemcpyAsync(p[i], src[i], sz[i] * n1, cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) return fail(e, "tables upload");
  }
  cudaError_t e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return fail(e, "tables upload");
  tables.t13 = (const double *)p[0];
  tables.tm53 = (const double *)p[1];
  tables.tln = (const double *)p[2];
  tables.t34 = (const double *)p[3];
  tables.t13f = (const float *)p[4];
  tables.tm76f = (const float *)p[5];
  tables.nmax = nm;
  tm76d_n = 0;
  return GWGPU_OK;
}

int gwgpu_context::ensure_tm76d(int nmax) {
  int st = ensure_tables(nmax);
  if (st) return st;
  if (tm76d && tm76d_n >= tables.nmax) return GWGPU_OK;
  dfree(tm76d);
  tm76d = nullptr;
  size_t n1 = (size_t)tables.nmax + 1;
  std::vector<double> v(n1, 0.0);
  for (size_t n = 1; n < n1; n++) v[n] = std::pow((double)n, -7. / 6.);
  st = dalloc((void **)&tm76d, 8 * n1, "tm76d");
  if (st) return st;
  cudaError_t e = cudaMemcpy(tm76d, v.data(), 8 * n1, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return fail(e, "tm76d upload");
  tm76d_n = tables.nmax;
  return GWGPU_OK;
}

int gwgpu_context::sync_streams_table() {
  size_t bytes = sizeof(StreamDev) * std::max<size_t>(streams.size(), 1);
  if (streams_dev_cap < streams.size() || !streams_dev) {
    dfree(streams_dev);
    streams_dev = nullptr;
    size_t cap = std::max<size_t>(64, streams.size() * 2);
    int st = dalloc((void **)&streams_dev, sizeof(StreamDev) * cap, "stream table");
    if (st) return st;
    streams_dev_cap = cap;
  }
  std::vector<StreamDev> v(streams.size());
  for (size_t i = 0; i < streams.size(); i++) v[i] = streams[i].dev;
  streams_epoch++;
  cudaError_t e = cudaMemcpyAsync(streams_dev, v.data(), bytes, cudaMemcpyHostToDevice, stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return fail(e, "stream table upload");
  return GWGPU_OK;
}

const gwgpu_context::Stream *gwgpu_context::get_stream(int handle) const {
  if (handle < 0 || handle >= (int)streams.size() || !streams[handle].live) return nullptr;
  return &streams[handle];
}

extern "C" {

void gwgpu_default_params(gwgpu_gen_params *p) {
  std::memset(p, 0, sizeof(*p));
  p->shift_time = 1;
  p->shift_phase = 1;
  p->chip = -1;
  p->phip = -1;
}

const char *gwgpu_status_string(int s) {
  switch (s) {
    case GWGPU_OK: return "ok";
    case GWGPU_EINVAL: return "invalid argument";
    case GWGPU_ECUDA: return "CUDA error";
    case GWGPU_ENOMEM: return "HBM budget exceeded";
    case GWGPU_EDOMAIN: return "request outside the model domain";
    case GWGPU_ETIMEDOUT: return "timed out";
    case GWGPU_EBUSY: return "busy";
    case GWGPU_ENOTFOUND: return "not found";
    case GWGPU_ETOOLARGE: return "size beyond the fixed maximum";
    case GWGPU_ESINGULAR: return "Fisher matrix not positive definite";
  }
  return "unknown status";
}

int gwgpu_context_create(int device, size_t budget, gwgpu_context **out) {
  if (!out) return GWGPU_EINVAL;
  *out = nullptr;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return GWGPU_ECUDA;
  gwgpu_context *c = new gwgpu_context();
  c->device = device;
  c->budget = budget;
  // GWGPU_PROLOGUE=serial: one thread per request for the batched prologue
  // (the reference's order of operations) instead of the cooperative kernel
  const char *pro = std::getenv("GWGPU_PROLOGUE");
  c->prologue_serial = pro && std::strcmp(pro, "serial") == 0;
  // GWGPU_ITEM_ORDER=listed: the mixed batch's items in plan order instead of
  // most live bins first
  const char *io = std::getenv("GWGPU_ITEM_ORDER");
  c->order_items = !(io && std::strcmp(io, "listed") == 0);
  // GWGPU_PDL=0: the batch kernels launched as plain stream successors
  const char *pd = std::getenv("GWGPU_PDL");
  c->pdl = !(pd && std::strcmp(pd, "0") == 0);
  // GWGPU_MAXLL=fp64: the maximised likelihood with FP64 transforms only
  const char *mx = std::getenv("GWGPU_MAXLL");
  c->maxll_fp64 = mx && std::strcmp(mx, "fp64") == 0;
  e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete c;
    return GWGPU_ECUDA;
  }
  cudaEventCreateWithFlags(&c->ev_in, cudaEventDisableTiming);
  cudaEventCreateWithFlags(&c->ev_out, cudaEventDisableTiming);
  std::vector<double> q(gwt::kQnmArrays * gwt::kQnmLen);
  gwk::qnm_host_table(q.data());
  c->qnm_host = q;
  int st = c->dalloc((void **)&c->qnm_dev, q.size() * sizeof(double), "qnm table");
  if (st) {
    gwgpu_context_destroy(c);
    return st;
  }
  e = cudaMemcpy(c->qnm_dev, q.data(), q.size() * sizeof(double), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    gwgpu_context_destroy(c);
    return GWGPU_ECUDA;
  }
  *out = c;
  return GWGPU_OK;
}

int gwgpu_context_destroy(gwgpu_context *c) {
  if (!c) return GWGPU_EINVAL;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  gwfft::release(c);
  for (auto &kv : c->sizes) cudaFree(kv.first);
  for (auto &w : c->hws)
    if (w.second.ptr) cudaFreeHost(w.second.ptr);
  c->lane.stream = c->stream;
  for (auto &g : c->lane.graphs) cudaGraphExecDestroy(g.second.exec);
  if (c->lane.hio) cudaFreeHost(c->lane.hio);
  if (c->ev_in) cudaEventDestroy(c->ev_in);
  for (int i = 0; i < 3; i++)
    if (c->t_ev[i]) cudaEventDestroy(c->t_ev[i]);
  if (c->ev_out) cudaEventDestroy(c->ev_out);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return GWGPU_OK;
}

const char *gwgpu_last_error_string(gwgpu_context *c) { return c ? c->last_error.c_str() : "no context"; }
void *gwgpu_context_stream(gwgpu_context *c) { return c ? (void *)c->stream : nullptr; }
size_t gwgpu_context_bytes_in_use(gwgpu_context *c) { return c ? c->in_use : 0; }

// ------------------------------------------------------------ data registry
// One detector stream; weights (GAUSSLEG) or null (Simpson's rule).
static int register_stream(gwgpu_context *c, const char *detector, const double *freqs, int N, const double *data,
                           const double *psd, const double *weights, int log10F, int *handle) {
  if (!c || !freqs || !data || !psd || !handle || N < 2) return GWGPU_EINVAL;
  int det = det_index(detector);
  if (det < 0) {
    c->last_error = "unknown detector";
    return GWGPU_EINVAL;
  }
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  gwgpu_context::Stream s;
  StreamDev &d = s.dev;
  std::memset(&d, 0, sizeof(d));
  d.det = det;
  d.N = N;
  d.df = freqs[1] - freqs[0];
  d.simpson_df = freqs[N / 2] - freqs[N / 2 - 1];
  // uniform grid with f0 an integer multiple of df -> table-driven mixed form
  bool uniform = d.df > 0;
  for (int k = 0; k < N && uniform; k++)
    if (std::fabs(freqs[k] - (freqs[0] + k * d.df)) > 1e-9 * d.df * (1 + k)) uniform = false;
  double n0f = freqs[0] / d.df;
  d.n0 = (int)std::llround(n0f);
  d.uniform_int = uniform && d.n0 >= 1 && std::fabs(n0f - d.n0) < 1e-6 && (d.n0 + (double)N) < 1.5e9;
  // integration weights: Simpson's rule, (4 df/3) s_k (util.h:844-856), or the
  // GAUSSLEG branch, 4 w_k (times f_k ln 10 for log10F) (mcmc_gw.cpp:820-862);
  // whitening for the mixed form W_k = weight_k / S_k
  std::vector<double> iw(N), W(N);
  double c3 = 4. * d.simpson_df / 3.;
  for (int k = 0; k < N; k++) {
    double sw = (k == 0 || k == N - 1) ? 1.0 : ((k & 1) ? 4.0 : 2.0);
    iw[k] = weights ? 4.0 * weights[k] * (log10F ? freqs[k] * std::log(10.) : 1.0) : c3 * sw;
  }
  double wmax = 0, dmax = 0;
  for (int k = 0; k < N; k++) {
    W[k] = iw[k] / psd[k];
    if (std::isfinite(W[k])) wmax = std::max(wmax, std::fabs(W[k]));
    double m = std::fabs(W[k] * data[2 * k]) + std::fabs(W[k] * data[2 * k + 1]);
    if (std::isfinite(m)) dmax = std::max(dmax, m);
  }
  d.wscale = wmax > 0 ? wmax : 1.0;
  d.dscale = dmax > 0 ? dmax : 1.0;
  std::vector<float> dh(2 * (size_t)N), wh(N);
  for (int k = 0; k < N; k++) {
    dh[2 * k] = (float)(W[k] * data[2 * k] / d.dscale);
    dh[2 * k + 1] = (float)(W[k] * data[2 * k + 1] / d.dscale);
    wh[k] = (float)(W[k] / d.wscale);
  }
  int st;
  void *pf, *pd, *pp, *pip, *pdh, *pwh, *piw = nullptr;
  std::vector<double> ip(N);  // the reciprocal PSD: the FP64 kernels multiply instead of dividing
  for (int k = 0; k < N; k++) ip[k] = 1.0 / psd[k];
  if ((st = c->dalloc(&pf, 8 * (size_t)N, "freqs")) || (st = c->dalloc(&pd, 16 * (size_t)N, "data")) ||
      (st = c->dalloc(&pp, 8 * (size_t)N, "psd")) || (st = c->dalloc(&pip, 8 * (size_t)N, "inverse psd")) ||
      (st = c->dalloc(&pdh, 8 * (size_t)N, "dhat")) || (st = c->dalloc(&pwh, 4 * (size_t)N, "what")) ||
      (weights && (st = c->dalloc(&piw, 8 * (size_t)N, "integration weights"))))
    return st;
  cudaMemcpyAsync(pip, ip.data(), 8 * (size_t)N, cudaMemcpyHostToDevice, c->stream);
  if (piw) cudaMemcpyAsync(piw, iw.data(), 8 * (size_t)N, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(pf, freqs, 8 * (size_t)N, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(pd, data, 16 * (size_t)N, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(pp, psd, 8 * (size_t)N, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(pdh, dh.data(), 8 * (size_t)N, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(pwh, wh.data(), 4 * (size_t)N, cudaMemcpyHostToDevice, c->stream);
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return c->fail(e, "data upload");
  d.freqs = (const double *)pf;
  d.data = (const double *)pd;
  d.psd = (const double *)pp;
  d.ipsd = (const double *)pip;
  d.dhat = (const float *)pdh;
  d.what = (const float *)pwh;
  d.iw = (const double *)piw;
  s.live = true;
  s.mem = {pf, pd, pp, pip, pdh, pwh};
  if (piw) s.mem.push_back(piw);
  s.host_freqs.assign(freqs, freqs + N);
  uint64_t hsh = 1469598103934665603ull;
  const unsigned char *pb = (const unsigned char *)psd;
  for (size_t i = 0; i < 8 * (size_t)N; i++) hsh = (hsh ^ pb[i]) * 1099511628211ull;
  if (weights) {
    const unsigned char *wb = (const unsigned char *)iw.data();
    for (size_t i = 0; i < 8 * (size_t)N; i++) hsh = (hsh ^ wb[i]) * 1099511628211ull;
  }
  s.psd_hash = hsh ^ (uint64_t)N;
  {  // the weights follow from the PSD, the integration rule and the grid
    uint64_t gk = s.psd_hash;
    const double gv[3] = {d.simpson_df, d.df, (double)d.n0};
    const unsigned char *gb = (const unsigned char *)gv;
    for (size_t i = 0; i < sizeof(gv); i++) gk = (gk ^ gb[i]) * 1099511628211ull;
    s.dev.wkey = gk;
  }
  if (d.uniform_int) {
    st = c->ensure_tables(d.n0 + N);
    if (st) return st;
  }
  c->streams.push_back(s);
  *handle = (int)c->streams.size() - 1;
  return c->sync_streams_table();
}

int gwgpu_data_register(gwgpu_context *c, const char *detector, const double *freqs, int N, const double *data,
                        const double *psd, int *handle) {
  return register_stream(c, detector, freqs, N, data, psd, nullptr, 0, handle);
}

int gwgpu_data_register_weighted(gwgpu_context *c, const char *detector, const double *freqs, int N,
                                 const double *data, const double *psd, const double *weights, int log10F,
                                 int *handle) {
  if (!weights) return GWGPU_EINVAL;
  return register_stream(c, detector, freqs, N, data, psd, weights, log10F, handle);
}

int gwgpu_data_release(gwgpu_context *c, int handle) {
  if (!c) return GWGPU_EINVAL;
  std::lock_guard<std::mutex> lk(c->mu);
  if (handle < 0 || handle >= (int)c->streams.size() || !c->streams[handle].live) return GWGPU_ENOTFOUND;
  cudaStreamSynchronize(c->stream);
  for (void *p : c->streams[handle].mem) c->dfree(p);
  c->streams[handle].live = false;
  c->streams[handle].dev.N = 0;
  return c->sync_streams_table();
}

// ------------------------------------------------------------------ waveform
static int waveform_common(gwgpu_context *c, const double *freqs, int N, double *out_a, double *out_b,
                           const char *method, const gwgpu_gen_params *p, int det, int apply_shift) {
  int ap = method_approx(method);
  if (!c || !freqs || N < 1 || !out_a || !p || ap < 0) return 0;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  gwt::Request r;
  gwt::GenParams gp;
  std::memcpy(&gp, p, sizeof(gp));
  if (det >= 0 && gp.equatorial_orientation) gwt::orientation_transform(gp, ap);  // waveform_util.cpp:946-948
  int dets[1] = {det < 0 ? 0 : det};
  gwt::request_prologue(r, gp, ap, dets, 1, c->qnm_host.data());
  void *dev;
  size_t nb = 8 * (size_t)N + 32 * (size_t)N;
  if (c->workspace(gwgpu_context::kWsWave, nb, &dev)) return 0;
  double *df = (double *)dev, *da = df + N, *db = da + 2 * (size_t)N;
  cudaMemcpyAsync(df, freqs, 8 * (size_t)N, cudaMemcpyHostToDevice, c->stream);
  cudaError_t e;
  if (det < 0) e = gwk::launch_waveform(r, df, N, da, db, c->stream);
  else e = gwk::launch_response(r, 0, apply_shift, df, N, da, c->stream);
  if (e != cudaSuccess) return c->fail(e, "waveform launch"), 0;
  cudaMemcpyAsync(out_a, da, 16 * (size_t)N, cudaMemcpyDeviceToHost, c->stream);
  if (det < 0 && out_b) cudaMemcpyAsync(out_b, db, 16 * (size_t)N, cudaMemcpyDeviceToHost, c->stream);
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return c->fail(e, "waveform"), 0;
  return 1;
}

int gwgpu_fourier_waveform(gwgpu_context *c, const double *freqs, int N, double *hp, double *hc, const char *method,
                           const gwgpu_gen_params *p) {
  if (!hc) return 0;
  return waveform_common(c, freqs, N, hp, hc, method, p, -1, 0);
}

int gwgpu_transform_orientation_coords(gwgpu_gen_params *p, const char *method) {
  int ap = method_approx(method);
  if (!p || ap < 0) return GWGPU_EINVAL;
  gwt::GenParams gp;
  std::memcpy(&gp, p, sizeof(gp));
  gwt::orientation_transform(gp, ap);
  p->psi = gp.psi;
  p->incl_angle = gp.incl_angle;
  return GWGPU_OK;
}

int gwgpu_fourier_detector_response(gwgpu_context *c, const double *freqs, int N, double *resp, const char *detector,
                                    const char *method, const gwgpu_gen_params *p) {
  int det = det_index(detector);
  if (det < 0) return 0;
  return waveform_common(c, freqs, N, resp, nullptr, method, p, det, 0);
}

// ---------------------------------------------------------------- plain form
int gwgpu_log_likelihood_internal(gwgpu_context *c, const double *data, const double *psd, const double *freqs,
                                  const double *resp, int N, double *out) {
  if (!c || !data || !psd || !freqs || !resp || !out || N < 2) return GWGPU_EINVAL;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  void *dev;
  size_t nb = 16 * (size_t)N * 2 + 8 * (size_t)N + 8 * 2048 + 64;
  int st = c->workspace(gwgpu_context::kWsInner, nb, &dev);
  if (st) return st;
  double *dd = (double *)dev, *dr = dd + 2 * (size_t)N, *dp = dr + 2 * (size_t)N, *part = dp + N,
         *res = part + 2048;
  unsigned *cnt = c->counter(0);
  if (!cnt) return GWGPU_ECUDA;
  cudaMemcpyAsync(dd, data, 16 * (size_t)N, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(dr, resp, 16 * (size_t)N, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(dp, psd, 8 * (size_t)N, cudaMemcpyHostToDevice, c->stream);
  double sdf = freqs[N / 2] - freqs[N / 2 - 1];
  cudaError_t e = gwk::launch_inner_product(dd, dp, dr, N, sdf, part, cnt, res, c->stream);
  if (e != cudaSuccess) return c->fail(e, "inner product launch");
  cudaMemcpyAsync(out, res, 8, cudaMemcpyDeviceToHost, c->stream);
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return c->fail(e, "inner product");
  return GWGPU_OK;
}

int gwgpu_log_likelihood_internal_weighted(gwgpu_context *c, const double *data, const double *psd,
                                           const double *freqs, const double *weights, const double *resp, int N,
                                           int log10F, double *out) {
  if (!c || !data || !psd || !freqs || !weights || !resp || !out || N < 1) return GWGPU_EINVAL;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  // integration weights of the GAUSSLEG branch (mcmc_gw.cpp:820-833, 843-862)
  double *iwh;
  int st = c->pinned(gwgpu_context::kHwsInner, 8 * (size_t)N, (void **)&iwh);
  if (st) return st;
  for (int k = 0; k < N; k++) iwh[k] = 4.0 * weights[k] * (log10F ? freqs[k] * std::log(10.) : 1.0);
  void *dev;
  size_t nb = 16 * (size_t)N * 2 + 8 * (size_t)N * 2 + 8 * 2048 + 64;
  st = c->workspace(gwgpu_context::kWsInner, nb, &dev);
  if (st) return st;
  double *dd = (double *)dev, *dr = dd + 2 * (size_t)N, *dp = dr + 2 * (size_t)N, *diw = dp + N, *part = diw + N,
         *res = part + 2048;
  unsigned *cnt = c->counter(0);
  if (!cnt) return GWGPU_ECUDA;
  cudaMemcpyAsync(dd, data, 16 * (size_t)N, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(dr, resp, 16 * (size_t)N, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(dp, psd, 8 * (size_t)N, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(diw, iwh, 8 * (size_t)N, cudaMemcpyHostToDevice, c->stream);
  cudaError_t e = gwk::launch_inner_product_weighted(dd, dp, dr, diw, N, part, cnt, res, c->stream);
  if (e != cudaSuccess) return c->fail(e, "inner product launch");
  cudaMemcpyAsync(out, res, 8, cudaMemcpyDeviceToHost, c->stream);
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return c->fail(e, "inner product");
  return GWGPU_OK;
}

int gwgpu_mcmc_likelihood_extrinsic(gwgpu_context *c, const gwgpu_gen_params *p, const char *method,
                                    const int *handles, int ndet, double T_segment, double *loglik) {
  int ap = method_approx(method);
  if (!c || !p || !handles || ndet < 1 || ndet > gwt::kMaxDet || !loglik || ap < 0) return GWGPU_EINVAL;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  StreamDev sd[gwt::kMaxDet];
  int dets[gwt::kMaxDet];
  for (int d = 0; d < ndet; d++) {
    const gwgpu_context::Stream *s = c->get_stream(handles[d]);
    if (!s) return GWGPU_ENOTFOUND;
    sd[d] = s->dev;
    dets[d] = s->dev.det;
    if (sd[d].N != sd[0].N) return GWGPU_EINVAL;
  }
  gwt::GenParams gp;
  std::memcpy(&gp, p, sizeof(gp));
  gp.tc = T_segment - gp.tc;  // mcmc_gw.cpp:2466-2473
  gwt::Request r;
  gwt::request_prologue(r, gp, ap, dets, ndet, c->qnm_host.data());
  void *dev;
  int nblk = gwk::plain_blocks(sd[0].N);
  int st = c->workspace(gwgpu_context::kWsPlain, sizeof(double) * ((size_t)nblk * 2 * gwt::kMaxDet + 8), &dev);
  if (st) return st;
  double *part = (double *)dev;
  unsigned *cnt = c->counter(1);
  if (!cnt) return GWGPU_ECUDA;
  // the last block writes log L straight into pinned host memory (mapped:
  // no copy after the kernel)
  double *h, *hd;
  st = c->pinned(gwgpu_context::kHwsPlain, 64, (void **)&h);
  if (st) return st;
  cudaError_t e = cudaHostGetDevicePointer((void **)&hd, h, 0);
  if (e != cudaSuccess) return c->fail(e, "plain result mapping");
  // IMRPhenomD on uniform grids: the waveform from the request's coefficients
  // on the grid and the power tables
  gwk::PlainTab pt;
  bool uni = ap == gwt::kPhenomD && !r.m.status && sd[0].n0 >= 1;
  for (int d = 0; d < ndet; d++) uni = uni && sd[d].uniform_int;
  if (uni && sd[0].n0 + sd[0].N - 1 <= c->tables.nmax && c->ensure_tm76d(sd[0].n0 + sd[0].N - 1) == GWGPU_OK &&
      sd[0].n0 + sd[0].N - 1 <= c->tm76d_n) {
    gwt::wave64_prologue(r, sd[0].df, pt.w);
    pt.t = c->tables;
    pt.tm76d = c->tm76d;
    pt.use = 1;
  }
  e = gwk::launch_plain(r, sd, ndet, part, cnt, hd, nullptr, c->stream, &pt);
  if (e != cudaSuccess) return c->fail(e, "plain launch");
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return c->fail(e, "plain");
  *loglik = r.m.status ? NAN : h[0];
  return r.m.status ? GWGPU_EDOMAIN : GWGPU_OK;
}

}  // extern "C"

unsigned *gwgpu_context::counter(int i) {
  if (!counters) {
    if (dalloc((void **)&counters, sizeof(unsigned) * 64, "counters")) return nullptr;
    if (cudaMemset(counters, 0, sizeof(unsigned) * 64) != cudaSuccess) return nullptr;
  }
  return counters + i;
}
