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
constexpr int kWarps = kBlock / 32;

// ------------------------------------------------------------------ kernels
// Pair q = blockIdx.y is (request q / ndet, detector q % ndet).
//
// Aligned (UN = false): g = 4 conj(d) h / S into g[q], and the block partial
// sums of w_k |h|^2 / S (Simpson weights w).  h is the model's h+ (the
// horizon frame at theta = phi = psi = 0 and inclination 0 that the sampler's
// intrinsic mode uses gives F+ = 1, Fx = 0), or a given response.
// Unaligned (UN = true): the same for h+ and hx into g[2q] and g[2q+1], and
// partial sums of |h+|^2/S, |hx|^2/S and Re(h+ conj(hx))/S.  The
// normalisation by sqrt(<h+|h+>) and sqrt(<hx|hx>) is applied after the
// transform (it is linear).
// The waveform of request r is evaluated on the grid of its first detector
// (the reference evaluates it once on local_freqs[0], mcmc_gw.cpp:2651-2653,
// 2697-2701).
template <bool UN>
__global__ void k_maxll_prep(const Request *__restrict__ req, const double2 *__restrict__ resp_p,
                             const double2 *__restrict__ resp_c, int ndet, const StreamDev *__restrict__ streams,
                             const int *__restrict__ handles, int N, double2 *__restrict__ g,
                             double *__restrict__ part) {
  constexpr int NS = UN ? 3 : 1, NP = UN ? 2 : 1;
  __shared__ double s_red[NS][kWarps];
  const int q = blockIdx.y, r = q / ndet;
  const StreamDev &st = streams[handles[q]];
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  double acc[NS];
#pragma unroll
  for (int j = 0; j < NS; j++) acc[j] = 0.0;
  if (k < N) {
    // a request outside the model domain contributes zeros (its result is NaN)
    double2 hp = make_double2(0.0, 0.0), hc = make_double2(0.0, 0.0);
    if (req) {
      if (!req[r].m.status) {
        gwt::cd p, c;
        gwt::wave_bin(req[r], streams[handles[(size_t)r * ndet]].freqs[k], p, c);
        hp = make_double2(p.re, p.im);
        hc = make_double2(c.re, c.im);
      }
    } else {
      hp = resp_p[(size_t)q * N + k];
      if (UN) hc = resp_c[(size_t)q * N + k];
    }
    const double2 d = ((const double2 *)st.data)[k];
    const double S = st.psd[k], w = gwt::simpson_weight(k, N);
    // 4 conj(d) h / S
    g[((size_t)q * NP) * N + k] =
        make_double2(4.0 * (d.x * hp.x + d.y * hp.y) / S, 4.0 * (d.x * hp.y - d.y * hp.x) / S);
    acc[0] = w * ((hp.x * hp.x + hp.y * hp.y) / S);
    if (UN) {
      g[((size_t)q * NP + 1) * N + k] =
          make_double2(4.0 * (d.x * hc.x + d.y * hc.y) / S, 4.0 * (d.x * hc.y - d.y * hc.x) / S);
      acc[1] = w * ((hc.x * hc.x + hc.y * hc.y) / S);
      acc[2] = w * ((hp.x * hc.x + hp.y * hc.y) / S);
    }
  }
#pragma unroll
  for (int j = 0; j < NS; j++) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc[j] += __shfl_xor_sync(0xffffffffu, acc[j], o);
  }
  if ((threadIdx.x & 31) == 0)
#pragma unroll
    for (int j = 0; j < NS; j++) s_red[j][threadIdx.x >> 5] = acc[j];
  __syncthreads();
  if (threadIdx.x < NS) {
    double t = 0.0;
    for (int w = 0; w < kWarps; w++) t += s_red[threadIdx.x][w];
    part[((size_t)q * NS + threadIdx.x) * gridDim.x + blockIdx.x] = t;
  }
}

// Sum of v over the block (every thread gets it).
__device__ double block_sum(double v, double *s_tmp) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) s_tmp[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  for (int w = 0; w < kWarps; w++) t += s_tmp[w];
  return t;
}

// One block per pair: the Simpson sums from the partials, then the maximum
// over the transform and log L of the pair; the last block of each request
// sums its detectors in order.
//   aligned   (mcmc_gw.cpp:595-658): 1/2 max|G|^2 df^2 / <h|h>
//   unaligned (mcmc_gw.cpp:660-800): 1/4 max lambda, with
//     rho+ = df G+ / sqrt(<h+|h+>), rhox = df Gx / sqrt(<hx|hx>),
//     gamma = Re(rho+ conj(rhox)), I = <h+|hx> / sqrt(<h+|h+><hx|hx>),
//     lambda = (|rho+|^2 + |rhox|^2 - 2 gamma I + sqrt((|rho+|^2 - |rhox|^2)^2
//              + 4 (I |rho+|^2 - gamma)(I |rhox|^2 - gamma))) / (1 - I^2).
template <bool UN>
__global__ void k_maxll_reduce(const double2 *__restrict__ G, const double *__restrict__ part, int nblk, int N,
                               int ndet, const StreamDev *__restrict__ streams, const int *__restrict__ handles,
                               const int *__restrict__ req_status, double *__restrict__ ll_pair,
                               unsigned *__restrict__ done, double *__restrict__ out, int *__restrict__ status) {
  constexpr int NS = UN ? 3 : 1, NP = UN ? 2 : 1;
  __shared__ double s_tmp[kWarps];
  __shared__ bool s_last;
  const int q = blockIdx.x, r = q / ndet;
  const StreamDev &st = streams[handles[q]];
  const double df = st.freqs[1] - st.freqs[0];  // mcmc_gw.cpp:604, also the Simpson step
  double sums[NS];
#pragma unroll
  for (int j = 0; j < NS; j++) {
    double t = 0.0;
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) t += part[((size_t)q * NS + j) * nblk + b];
    sums[j] = 4.0 * block_sum(t, s_tmp) * df / 3.0;
  }
  double m = 0.0;
  if (!UN) {
    for (int k = threadIdx.x; k < N; k += blockDim.x) {
      const double2 v = G[(size_t)q * N + k];
      m = fmax(m, v.x * v.x + v.y * v.y);
    }
  } else {
    const double ap = df / sqrt(sums[0]), ac = df / sqrt(sums[1]);
    const double I = sums[2] / (sqrt(sums[0]) * sqrt(sums[1]));
    m = -HUGE_VAL;
    for (int k = threadIdx.x; k < N; k += blockDim.x) {
      const double2 a = G[((size_t)q * NP) * N + k], c = G[((size_t)q * NP + 1) * N + k];
      const double rpx = ap * a.x, rpy = ap * a.y, rcx = ac * c.x, rcy = ac * c.y;
      const double p2 = rpx * rpx + rpy * rpy, c2 = rcx * rcx + rcy * rcy;
      const double gam = rpx * rcx + rpy * rcy;
      const double lam =
          (p2 + c2 - 2 * gam * I + sqrt((p2 - c2) * (p2 - c2) + 4. * (I * p2 - gam) * (I * c2 - gam))) / (1. - I * I);
      m = fmax(m, lam);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) s_tmp[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double mx = s_tmp[0];
    for (int w = 1; w < kWarps; w++) mx = fmax(mx, s_tmp[w]);
    ll_pair[q] = UN ? 0.25 * mx : 0.5 * (mx * df * df) / sums[0];
    __threadfence();
    s_last = atomicAdd(done + r, 1u) == (unsigned)ndet - 1;
  }
  __syncthreads();
  if (s_last && threadIdx.x == 0) {
    __threadfence();
    double ll = 0.0;
    for (int d = 0; d < ndet; d++) ll += __ldcg(ll_pair + (size_t)r * ndet + d);
    const int rs = req_status ? req_status[r] : 0;
    out[r] = rs ? __longlong_as_double(0x7ff8000000000000ll) : ll;
    if (status) status[r] = rs;
  }
}

size_t up256(size_t x) { return (x + 255) & ~(size_t)255; }

// One pair from host arrays: hp (and hc when unaligned) given.
int maximized_single(gwgpu_context *c, const double *data, const double *psd, const double *freqs, const double *hp,
                     const double *hc, int N, double *out) {
  const bool un = hc != nullptr;
  const int np = un ? 2 : 1, ns = un ? 3 : 1;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  int plan;
  int st = plan_for(c, N, np, &plan);
  if (st) return st;
  const int nblk = (N + kBlock - 1) / kBlock;
  const size_t o_f = 0, o_d = up256(8 * (size_t)N), o_s = o_d + up256(16 * (size_t)N),
               o_rp = o_s + up256(8 * (size_t)N), o_rc = o_rp + up256(16 * (size_t)N),
               o_g = o_rc + up256(16 * (size_t)N), o_h = o_g + up256(16 * (size_t)N * np),
               o_sd = o_h + up256(8 * (size_t)nblk * ns), o_misc = o_sd + up256(sizeof(StreamDev)),
               total = o_misc + 256;
  void *dev;
  if ((st = c->workspace(gwgpu_context::kWsMaxll, total, &dev))) return st;
  char *b = (char *)dev;
  cudaMemcpyAsync(b + o_f, freqs, 8 * (size_t)N, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(b + o_d, data, 16 * (size_t)N, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(b + o_s, psd, 8 * (size_t)N, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(b + o_rp, hp, 16 * (size_t)N, cudaMemcpyHostToDevice, c->stream);
  if (un) cudaMemcpyAsync(b + o_rc, hc, 16 * (size_t)N, cudaMemcpyHostToDevice, c->stream);
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
  const StreamDev *sdd = (const StreamDev *)(b + o_sd);
  const double2 *rp = (const double2 *)(b + o_rp), *rc = (const double2 *)(b + o_rc);
  if (un)
    k_maxll_prep<true><<<dim3(nblk, 1), kBlock, 0, c->stream>>>(nullptr, rp, rc, 1, sdd, dh, N, g, (double *)(b + o_h));
  else
    k_maxll_prep<false><<<dim3(nblk, 1), kBlock, 0, c->stream>>>(nullptr, rp, nullptr, 1, sdd, dh, N, g,
                                                                (double *)(b + o_h));
  CuFft &f = cufft();
  if (f.set_stream(plan, c->stream) != 0 || f.exec_z2z(plan, g, g, kCufftForward) != 0) {
    c->last_error = "cuFFT exec";
    return GWGPU_ECUDA;
  }
  if (un)
    k_maxll_reduce<true><<<1, kBlock, 0, c->stream>>>(g, (const double *)(b + o_h), nblk, N, 1, sdd, dh, nullptr,
                                                      ll_pair, done, res, nullptr);
  else
    k_maxll_reduce<false><<<1, kBlock, 0, c->stream>>>(g, (const double *)(b + o_h), nblk, N, 1, sdd, dh, nullptr,
                                                       ll_pair, done, res, nullptr);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return c->fail(e, "maximised likelihood launch");
  cudaMemcpyAsync(out, res, 8, cudaMemcpyDeviceToHost, c->stream);
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return c->fail(e, "maximised likelihood");
  return GWGPU_OK;
}

}  // namespace

extern "C" {

int gwgpu_maximized_log_likelihood_internal(gwgpu_context *c, const double *data, const double *psd,
                                            const double *freqs, const double *response, int N, double *out) {
  if (!c || !data || !psd || !freqs || !response || !out || N < 2) return GWGPU_EINVAL;
  return maximized_single(c, data, psd, freqs, response, nullptr, N, out);
}

int gwgpu_maximized_log_likelihood_unaligned_internal(gwgpu_context *c, const double *data, const double *psd,
                                                      const double *freqs, const double *hplus, const double *hcross,
                                                      int N, double *out) {
  if (!c || !data || !psd || !freqs || !hplus || !hcross || !out || N < 2) return GWGPU_EINVAL;
  return maximized_single(c, data, psd, freqs, hplus, hcross, N, out);
}

int gwgpu_maximized_loglik_batch(gwgpu_context *c, const gwgpu_gen_params *params, int n, int approximant,
                                 const int *handles, int ndet, double *loglik, int *status) {
  if (!c || !params || n < 1 || !handles || ndet < 1 || ndet > gwt::kMaxDet || !loglik) return GWGPU_EINVAL;
  if (approximant != GWGPU_IMRPHENOMD && approximant != GWGPU_IMRPHENOMPV2) return GWGPU_EINVAL;
  const bool un = approximant == GWGPU_IMRPHENOMPV2;
  const int np = un ? 2 : 1, ns = un ? 3 : 1;
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
  int st = plan_for(c, N, pairs * np, &plan);
  if (st) return st;
  const int nblk = (N + kBlock - 1) / kBlock;
  const size_t o_p = 0, o_a = up256(sizeof(gwgpu_gen_params) * n), o_h = o_a + up256(4 * (size_t)n),
               o_req = o_h + up256(4 * (size_t)pairs), o_g = o_req + up256(sizeof(Request) * n),
               o_hh = o_g + up256(16 * (size_t)pairs * np * N), o_ll = o_hh + up256(8 * (size_t)pairs * ns * nblk),
               o_out = o_ll + up256(8 * (size_t)pairs), o_st = o_out + up256(8 * (size_t)n),
               o_done = o_st + up256(4 * (size_t)n), total = o_done + up256(4 * (size_t)n);
  void *dev;
  if ((st = c->workspace(gwgpu_context::kWsMaxll, total, &dev))) return st;
  char *b = (char *)dev;
  // the sampler's intrinsic mode fixes the extrinsic parameters
  // (IMRPhenomD: mcmc_gw.cpp:2614-2620, 2645-2651; IMRPhenomPv2: 2693-2699)
  std::vector<gwgpu_gen_params> hp(params, params + n);
  for (auto &p : hp) {
    p.RA = p.DEC = p.psi = 0;
    p.phiRef = 1;
    p.f_ref = un ? 20 : 10;
    p.incl_angle = 0;
    p.tc = 1;
  }
  std::vector<int> ap(n, un ? gwt::kPhenomPv2 : gwt::kPhenomD);
  cudaMemcpyAsync(b + o_p, hp.data(), sizeof(gwgpu_gen_params) * n, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(b + o_a, ap.data(), 4 * (size_t)n, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(b + o_h, handles, 4 * (size_t)pairs, cudaMemcpyHostToDevice, c->stream);
  cudaMemsetAsync(b + o_done, 0, 4 * (size_t)n, c->stream);
  cudaError_t e = gwk::launch_prologue((const gwt::GenParams *)(b + o_p), (const int *)(b + o_a), n,
                                       (const int *)(b + o_h), ndet, 0.0, 0, c->streams_dev, c->qnm_dev,
                                       (Request *)(b + o_req), nullptr, 0, (int *)(b + o_st), c->stream);
  if (e != cudaSuccess) return c->fail(e, "maximised likelihood prologue");
  double2 *g = (double2 *)(b + o_g);
  const Request *rq = (const Request *)(b + o_req);
  const int *hd = (const int *)(b + o_h);
  double *hh = (double *)(b + o_hh);
  if (un)
    k_maxll_prep<true><<<dim3(nblk, pairs), kBlock, 0, c->stream>>>(rq, nullptr, nullptr, ndet, c->streams_dev, hd,
                                                                   N, g, hh);
  else
    k_maxll_prep<false><<<dim3(nblk, pairs), kBlock, 0, c->stream>>>(rq, nullptr, nullptr, ndet, c->streams_dev, hd,
                                                                    N, g, hh);
  CuFft &f = cufft();
  if (f.set_stream(plan, c->stream) != 0 || f.exec_z2z(plan, g, g, kCufftForward) != 0) {
    c->last_error = "cuFFT exec";
    return GWGPU_ECUDA;
  }
  int *dst = (int *)(b + o_st);
  if (un)
    k_maxll_reduce<true><<<pairs, kBlock, 0, c->stream>>>(g, hh, nblk, N, ndet, c->streams_dev, hd, dst,
                                                          (double *)(b + o_ll), (unsigned *)(b + o_done),
                                                          (double *)(b + o_out), dst);
  else
    k_maxll_reduce<false><<<pairs, kBlock, 0, c->stream>>>(g, hh, nblk, N, ndet, c->streams_dev, hd, dst,
                                                           (double *)(b + o_ll), (unsigned *)(b + o_done),
                                                           (double *)(b + o_out), dst);
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
