// maxll.cu -- the likelihood maximised over arrival time and phase,
// maximized_Log_Likelihood_aligned_spin_internal (mcmc_gw.cpp:595-658), and
// the sampler's intrinsic mode that sums it over detectors
// (MCMC_likelihood_wrapper, mcmc_gw.cpp:2611-2631).
//
// Per (request, detector): HH = 4 S(|r|^2 / S_n) by Simpson's rule,
// g_k = 4 conj(d_k) r_k / S_n,k, G = DFT(g), and
// log L = 1/2 max_j |G_j|^2 df^2 / HH.  The products and sums are fused in
// hand-written kernels (FP64); the length-N transforms of all pairs run as one
// batched cuFFT double-complex plan (a library transform, loaded at run time
// so that the engine builds and runs without it: the entry points then return
// GWGPU_ECUDA with a message).
#include <cuda_runtime.h>
#include <dlfcn.h>

#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <utility>
#include <vector>

#include "../../include/gwgpu.h"
#include "capi_internal.h"
#include "kernels.h"

namespace {

using gwk::StreamDev;
using gwt::Request;

// ------------------------------------------------------------- cuFFT loader
struct CuFft {
  typedef int (*PlanMany)(int *, int, int *, int *, int, int, int *, int, int, int, int);
  typedef int (*ExecZ2Z)(int, void *, void *, int);
  typedef int (*SetStream)(int, cudaStream_t);
  typedef int (*Destroy)(int);
  void *lib = nullptr;
  PlanMany plan_many = nullptr;
  ExecZ2Z exec_z2z = nullptr;
  SetStream set_stream = nullptr;
  Destroy destroy = nullptr;
  bool ok = false;
};
constexpr int kCufftZ2Z = 0x69, kCufftForward = -1;  // cufftType CUFFT_Z2Z, CUFFT_FORWARD

CuFft &cufft() {
  static CuFft f;
  static std::once_flag once;
  std::call_once(once, [] {
    const char *names[] = {"libcufft.so.12", "libcufft.so.13", "libcufft.so", "/usr/local/cuda/lib64/libcufft.so.12",
                           "/usr/local/cuda/lib64/libcufft.so"};
    for (const char *nm : names)
      if ((f.lib = dlopen(nm, RTLD_NOW | RTLD_LOCAL))) break;
    if (!f.lib) return;
    f.plan_many = (CuFft::PlanMany)dlsym(f.lib, "cufftPlanMany");
    f.exec_z2z = (CuFft::ExecZ2Z)dlsym(f.lib, "cufftExecZ2Z");
    f.set_stream = (CuFft::SetStream)dlsym(f.lib, "cufftSetStream");
    f.destroy = (CuFft::Destroy)dlsym(f.lib, "cufftDestroy");
    f.ok = f.plan_many && f.exec_z2z && f.set_stream && f.destroy;
  });
  return f;
}

// One plan per (length, batch) and context, kept for reuse.
struct Plans {
  std::map<std::pair<int, int>, int> plans;
};
std::mutex g_plans_mu;
std::map<gwgpu_context *, Plans> g_plans;

int plan_for(gwgpu_context *c, int N, int batch, int *plan) {
  CuFft &f = cufft();
  if (!f.ok) {
    c->last_error = "cuFFT library not found";
    return GWGPU_ECUDA;
  }
  std::lock_guard<std::mutex> lk(g_plans_mu);
  auto &m = g_plans[c].plans;
  auto it = m.find({N, batch});
  if (it != m.end()) {
    *plan = it->second;
    return GWGPU_OK;
  }
  int p = 0, n = N;
  if (f.plan_many(&p, 1, &n, nullptr, 1, N, nullptr, 1, N, kCufftZ2Z, batch) != 0) {
    c->last_error = "cuFFT plan";
    return GWGPU_ECUDA;
  }
  m[{N, batch}] = p;
  *plan = p;
  return GWGPU_OK;
}

constexpr int kBlock = 256;

// ------------------------------------------------------------------ kernels
// g_k = 4 conj(d_k) r_k / S_k and the block partial sums of w_k |r_k|^2 / S_k
// (Simpson weights w) for pair q = blockIdx.y; the response r is the model's
// h+ (the horizon frame at theta = phi = psi = 0 and inclination 0 that the
// sampler's intrinsic mode uses: F+ = 1, Fx = 0), or given.
__global__ void k_maxll_prep(const Request *__restrict__ req, const double2 *__restrict__ resp, int ndet,
                             const StreamDev *__restrict__ streams, const int *__restrict__ handles, int N,
                             double2 *__restrict__ g, double *__restrict__ hh_part) {
  __shared__ double s_red[kBlock / 32];
  const int q = blockIdx.y, r = q / ndet;
  const StreamDev &st = streams[handles[q]];
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  double hh = 0.0;
  if (k < N && !(req && req[r].m.status)) {
    double2 h;
    if (req) {
      gwt::cd hp, hc;
      gwt::wave_bin(req[r], st.freqs[k], hp, hc);
      h = make_double2(hp.re, hp.im);
    } else {
      h = resp[(size_t)q * N + k];
    }
    const double2 d = ((const double2 *)st.data)[k];
    const double S = st.psd[k];
    // 4 conj(d) h / S
    g[(size_t)q * N + k] = make_double2(4.0 * (d.x * h.x + d.y * h.y) / S, 4.0 * (d.x * h.y - d.y * h.x) / S);
    hh = gwt::simpson_weight(k, N) * ((h.x * h.x + h.y * h.y) / S);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) hh += __shfl_xor_sync(0xffffffffu, hh, o);
  if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = hh;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < kBlock / 32; w++) s += s_red[w];
    hh_part[(size_t)q * gridDim.x + blockIdx.x] = s;
  }
}

// log L of pair q = 1/2 max |G|^2 df^2 / HH, then summed over each request's
// detectors in order by the last block of the request.
__global__ void k_maxll_reduce(const double2 *__restrict__ G, const double *__restrict__ hh_part, int nblk, int N,
                               int ndet, const StreamDev *__restrict__ streams, const int *__restrict__ handles,
                               const int *__restrict__ req_status, double *__restrict__ ll_pair,
                               unsigned *__restrict__ done, double *__restrict__ out, int *__restrict__ status) {
  __shared__ double s_max[kBlock / 32];
  __shared__ bool s_last;
  const int q = blockIdx.x, r = q / ndet;
  double m = 0.0;
  for (int k = threadIdx.x; k < N; k += blockDim.x) {
    const double2 v = G[(size_t)q * N + k];
    m = fmax(m, v.x * v.x + v.y * v.y);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) s_max[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double mx = 0.0, hh = 0.0;
    for (int w = 0; w < kBlock / 32; w++) mx = fmax(mx, s_max[w]);
    for (int b = 0; b < nblk; b++) hh += hh_part[(size_t)q * nblk + b];
    const StreamDev &st = streams[handles[q]];
    const double df = st.freqs[1] - st.freqs[0];  // mcmc_gw.cpp:604, also the Simpson step
    hh *= 4.0 * df / 3.0;
    ll_pair[q] = 0.5 * (mx * df * df) / hh;
    __threadfence();
    s_last = atomicAdd(done + r, 1u) == (unsigned)ndet - 1;
  }
  __syncthreads();
  if (s_last && threadIdx.x == 0) {
    __threadfence();
    double ll = 0.0;
    for (int d = 0; d < ndet; d++) ll += __ldcg(ll_pair + (size_t)r * ndet + d);
    const int st = req_status ? req_status[r] : 0;
    out[r] = st ? __longlong_as_double(0x7ff8000000000000ll) : ll;
    if (status) status[r] = st;
  }
}

size_t up256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

extern "C" {

int gwgpu_maximized_log_likelihood_internal(gwgpu_context *c, const double *data, const double *psd,
                                            const double *freqs, const double *response, int N, double *out) {
  if (!c || !data || !psd || !freqs || !response || !out || N < 2) return GWGPU_EINVAL;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  int plan;
  int st = plan_for(c, N, 1, &plan);
  if (st) return st;
  const int nblk = (N + kBlock - 1) / kBlock;
  const size_t o_f = 0, o_d = up256(8 * (size_t)N), o_s = o_d + up256(16 * (size_t)N),
               o_r = o_s + up256(8 * (size_t)N), o_g = o_r + up256(16 * (size_t)N), o_h = o_g + up256(16 * (size_t)N),
               o_sd = o_h + up256(8 * (size_t)nblk), o_misc = o_sd + up256(sizeof(StreamDev)), total = o_misc + 256;
  void *dev;
  if ((st = c->workspace(gwgpu_context::kWsMaxll, total, &dev))) return st;
  char *b = (char *)dev;
  cudaMemcpyAsync(b + o_f, freqs, 8 * (size_t)N, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(b + o_d, data, 16 * (size_t)N, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(b + o_s, psd, 8 * (size_t)N, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(b + o_r, response, 16 * (size_t)N, cudaMemcpyHostToDevice, c->stream);
  StreamDev sd;
  std::memset(&sd, 0, sizeof(sd));
  sd.N = N;
  sd.freqs = (const double *)(b + o_f);
  sd.data = (const double *)(b + o_d);
  sd.psd = (const double *)(b + o_s);
  int zero = 0;
  cudaMemcpyAsync(b + o_sd, &sd, sizeof(sd), cudaMemcpyHostToDevice, c->stream);
  int *dh = (int *)(b + o_misc);
  unsigned *done = (unsigned *)(b + o_misc + 16);
  double *ll_pair = (double *)(b + o_misc + 64), *res = ll_pair + 1;
  cudaMemcpyAsync(dh, &zero, sizeof(int), cudaMemcpyHostToDevice, c->stream);
  cudaMemsetAsync(done, 0, sizeof(unsigned), c->stream);
  double2 *g = (double2 *)(b + o_g);
  k_maxll_prep<<<dim3(nblk, 1), kBlock, 0, c->stream>>>(nullptr, (const double2 *)(b + o_r), 1,
                                                       (const StreamDev *)(b + o_sd), dh, N, g, (double *)(b + o_h));
  CuFft &f = cufft();
  if (f.set_stream(plan, c->stream) != 0 || f.exec_z2z(plan, g, g, kCufftForward) != 0) {
    c->last_error = "cuFFT exec";
    return GWGPU_ECUDA;
  }
  k_maxll_reduce<<<1, kBlock, 0, c->stream>>>(g, (const double *)(b + o_h), nblk, N, 1, (const StreamDev *)(b + o_sd),
                                              dh, nullptr, ll_pair, done, res, nullptr);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return c->fail(e, "maximised likelihood launch");
  cudaMemcpyAsync(out, res, 8, cudaMemcpyDeviceToHost, c->stream);
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return c->fail(e, "maximised likelihood");
  return GWGPU_OK;
}

int gwgpu_maximized_loglik_batch(gwgpu_context *c, const gwgpu_gen_params *params, int n, const int *handles,
                                 int ndet, double *loglik, int *status) {
  if (!c || !params || n < 1 || !handles || ndet < 1 || ndet > gwt::kMaxDet || !loglik) return GWGPU_EINVAL;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  const gwgpu_context::Stream *s0 = c->get_stream(handles[0]);
  if (!s0) return GWGPU_ENOTFOUND;
  const int N = s0->dev.N;
  for (int i = 0; i < n * ndet; i++) {
    const gwgpu_context::Stream *s = c->get_stream(handles[i]);
    if (!s) return GWGPU_ENOTFOUND;
    if (s->dev.N != N || s->dev.iw) {
      c->last_error = "maximised likelihood: one Simpson grid length for the whole batch";
      return GWGPU_EINVAL;
    }
  }
  const int pairs = n * ndet;
  int plan;
  int st = plan_for(c, N, pairs, &plan);
  if (st) return st;
  const int nblk = (N + kBlock - 1) / kBlock;
  const size_t o_p = 0, o_a = up256(sizeof(gwgpu_gen_params) * n), o_h = o_a + up256(4 * (size_t)n),
               o_req = o_h + up256(4 * (size_t)pairs), o_g = o_req + up256(sizeof(Request) * n),
               o_hh = o_g + up256(16 * (size_t)pairs * N), o_ll = o_hh + up256(8 * (size_t)pairs * nblk),
               o_out = o_ll + up256(8 * (size_t)pairs), o_st = o_out + up256(8 * (size_t)n),
               o_done = o_st + up256(4 * (size_t)n), total = o_done + up256(4 * (size_t)n);
  void *dev;
  if ((st = c->workspace(gwgpu_context::kWsMaxll, total, &dev))) return st;
  char *b = (char *)dev;
  // the sampler's intrinsic mode fixes the extrinsic parameters (mcmc_gw.cpp:2614-2620)
  std::vector<gwgpu_gen_params> hp(params, params + n);
  for (auto &p : hp) {
    p.RA = p.DEC = p.psi = 0;
    p.phiRef = 1;
    p.f_ref = 10;
    p.incl_angle = 0;
    p.tc = 1;
  }
  std::vector<int> ap(n, gwt::kPhenomD);
  cudaMemcpyAsync(b + o_p, hp.data(), sizeof(gwgpu_gen_params) * n, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(b + o_a, ap.data(), 4 * (size_t)n, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(b + o_h, handles, 4 * (size_t)pairs, cudaMemcpyHostToDevice, c->stream);
  cudaMemsetAsync(b + o_done, 0, 4 * (size_t)n, c->stream);
  cudaError_t e = gwk::launch_prologue((const gwt::GenParams *)(b + o_p), (const int *)(b + o_a), n,
                                       (const int *)(b + o_h), ndet, 0.0, 0, c->streams_dev, c->qnm_dev,
                                       (Request *)(b + o_req), nullptr, 0, (int *)(b + o_st), c->stream);
  if (e != cudaSuccess) return c->fail(e, "maximised likelihood prologue");
  double2 *g = (double2 *)(b + o_g);
  k_maxll_prep<<<dim3(nblk, pairs), kBlock, 0, c->stream>>>((const Request *)(b + o_req), nullptr, ndet,
                                                           c->streams_dev, (const int *)(b + o_h), N, g,
                                                           (double *)(b + o_hh));
  CuFft &f = cufft();
  if (f.set_stream(plan, c->stream) != 0 || f.exec_z2z(plan, g, g, kCufftForward) != 0) {
    c->last_error = "cuFFT exec";
    return GWGPU_ECUDA;
  }
  k_maxll_reduce<<<pairs, kBlock, 0, c->stream>>>(g, (const double *)(b + o_hh), nblk, N, ndet, c->streams_dev,
                                                  (const int *)(b + o_h), (const int *)(b + o_st),
                                                  (double *)(b + o_ll), (unsigned *)(b + o_done),
                                                  (double *)(b + o_out), (int *)(b + o_st));
  e = cudaGetLastError();
  if (e != cudaSuccess) return c->fail(e, "maximised likelihood launch");
  std::vector<int> hs(n);
  cudaMemcpyAsync(loglik, b + o_out, 8 * (size_t)n, cudaMemcpyDeviceToHost, c->stream);
  cudaMemcpyAsync(hs.data(), b + o_st, 4 * (size_t)n, cudaMemcpyDeviceToHost, c->stream);
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return c->fail(e, "maximised likelihood");
  if (status)
    for (int i = 0; i < n; i++) status[i] = gwk::status_code(hs[i]);
  return GWGPU_OK;
}

}  // extern "C"
