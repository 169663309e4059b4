// maxll.cu -- the likelihood maximised over arrival time and phase,
// maximized_Log_Likelihood_aligned_spin_internal (mcmc_gw.cpp:595-658) and
// maximized_Log_Likelihood_unaligned_spin_internal (:660-800), and the
// sampler's intrinsic mode that sums them over detectors
// (MCMC_likelihood_wrapper, mcmc_gw.cpp:2611-2720).
//
// Per (request, detector): HH = 4 S(|r|^2 / S_n) by Simpson's rule,
// g_k = 4 conj(d_k) r_k / S_n,k, G = DFT_N(g), and
// log L = 1/2 max_j |G_j|^2 df^2 / HH.  The products and sums are fused in
// hand-written FP64 kernels; the transforms of all pairs run as batched cuFFT
// double-complex plans (cufft_rt.h).
//
// Grid lengths N with a prime factor above 7 (32128 = 2^7 * 251 is typical)
// use Bluestein's identity nk = (n^2 + k^2 - (k - n)^2) / 2 with power-of-two
// transforms of length M >= 2N - 1:
//   G_k = e^{-i pi k^2/N} sum_n [g_n e^{-i pi n^2/N}] e^{i pi (k-n)^2/N},
// a cyclic convolution of a_n = g_n e^{-i pi n^2/N} with b_m = e^{i pi m^2/N}
// (FFT_M, a pointwise product with the transform of b, inverse FFT_M).  The
// outer factor e^{-i pi k^2/N} is never applied: every quantity taken from G
// (|G_k|^2, Re(G+_k conj(Gx_k))) is invariant to a phase common to the pair.
// The chirp phases use n^2 mod 2N in integers, so they are exact to FP64.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <utility>
#include <vector>

#include "../../include/gwgpu.h"
#include "capi_internal.h"
#include "cufft_rt.h"
#include "kernels.h"

namespace {

using gwk::StreamDev;
using gwt::Request;

constexpr int kBlock = 256;
constexpr int kWarps = kBlock / 32;

// e^{sign i pi m^2 / N}, the phase reduced exactly (m^2 mod 2N in integers).
__device__ __forceinline__ double2 chirp(long long m, int N, double sign) {
  const long long t = (m * m) % (2LL * N);
  double sn, cs;
  sincospi((double)t / (double)N, &sn, &cs);
  return make_double2(cs, sign * sn);
}

// ------------------------------------------------------------------ kernels
// Block (x, r): bins x*256.. of request r, for each of its detectors d (pair
// q = r*ndet + d); rows of g have stride ld (N, or M for Bluestein, the bins
// N..M-1 zero).  The waveform is evaluated once per bin and request, on the
// grid of the request's first detector (the reference evaluates it once on
// local_freqs[0], mcmc_gw.cpp:2651-2653, 2697-2701).
//
// Aligned (UN = false): g = 4 conj(d) h / S into row q, and the block partial
// sums of w_k |h|^2 / S (Simpson weights w).  h is the model's h+ (the
// horizon frame at theta = phi = psi = 0 and inclination 0 that the sampler's
// intrinsic mode uses gives F+ = 1, Fx = 0), or a given response per pair.
// Unaligned (UN = true): the same for h+ and hx into rows 2q and 2q+1, and
// partial sums of |h+|^2/S, |hx|^2/S and Re(h+ conj(hx))/S.  The
// normalisation by sqrt(<h+|h+>) and sqrt(<hx|hx>) is applied after the
// transform (it is linear).  With Bluestein, g is multiplied by
// e^{-i pi k^2/N}.
template <bool UN>
__global__ void k_maxll_prep(const Request *__restrict__ req, const double2 *__restrict__ resp_p,
                             const double2 *__restrict__ resp_c, int ndet, const StreamDev *__restrict__ streams,
                             const int *__restrict__ handles, int N, int ld, int blue, double2 *__restrict__ g,
                             double *__restrict__ part) {
  constexpr int NS = UN ? 3 : 1, NP = UN ? 2 : 1;
  __shared__ double s_red[NS][kWarps];
  const int r = blockIdx.y;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  // a request outside the model domain contributes zeros (its result is NaN)
  double2 hp = make_double2(0.0, 0.0), hc = make_double2(0.0, 0.0);
  if (req && k < N && !req[r].m.status) {
    gwt::cd p, c;
    gwt::wave_bin(req[r], streams[handles[(size_t)r * ndet]].freqs[k], p, c);
    hp = make_double2(p.re, p.im);
    hc = make_double2(c.re, c.im);
  }
  const double2 ch = (blue && k < N) ? chirp(k, N, -1.0) : make_double2(1.0, 0.0);
  for (int dd = 0; dd < ndet; dd++) {
    const int q = r * ndet + dd;
    const StreamDev &st = streams[handles[q]];
    double acc[NS];
#pragma unroll
    for (int j = 0; j < NS; j++) acc[j] = 0.0;
    if (k < N) {
      if (!req) {
        hp = resp_p[(size_t)q * N + k];
        if (UN) hc = resp_c[(size_t)q * N + k];
      }
      const double2 d = ((const double2 *)st.data)[k];
      const double S = st.psd[k], w = gwt::simpson_weight(k, N);
      // 4 conj(d) h / S, then the Bluestein chirp
      double2 v = make_double2(4.0 * (d.x * hp.x + d.y * hp.y) / S, 4.0 * (d.x * hp.y - d.y * hp.x) / S);
      g[((size_t)q * NP) * ld + k] = make_double2(v.x * ch.x - v.y * ch.y, v.x * ch.y + v.y * ch.x);
      acc[0] = w * ((hp.x * hp.x + hp.y * hp.y) / S);
      if (UN) {
        v = make_double2(4.0 * (d.x * hc.x + d.y * hc.y) / S, 4.0 * (d.x * hc.y - d.y * hc.x) / S);
        g[((size_t)q * NP + 1) * ld + k] = make_double2(v.x * ch.x - v.y * ch.y, v.x * ch.y + v.y * ch.x);
        acc[1] = w * ((hc.x * hc.x + hc.y * hc.y) / S);
        acc[2] = w * ((hp.x * hc.x + hp.y * hc.y) / S);
      }
    } else if (k < ld) {
      g[((size_t)q * NP) * ld + k] = make_double2(0.0, 0.0);
      if (UN) g[((size_t)q * NP + 1) * ld + k] = make_double2(0.0, 0.0);
    }
#pragma unroll
    for (int j = 0; j < NS; j++) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc[j] += __shfl_xor_sync(0xffffffffu, acc[j], o);
    }
    __syncthreads();  // the previous detector's partials have been read
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
}

// The Bluestein kernel: B = FFT_M(b) / M is made from b_m = e^{i pi m^2/N} at
// index m (0 <= m < N) and M - m (0 < m < N), zero elsewhere.
__global__ void k_chirp_fill(double2 *__restrict__ b, int N, int M) {
  const double inv = 1.0 / (double)M;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M; i += gridDim.x * blockDim.x) {
    long long m = -1;
    if (i < N) m = i;
    else if (i > M - N) m = M - i;
    double2 v = make_double2(0.0, 0.0);
    if (m >= 0) {
      v = chirp(m, N, 1.0);
      v.x *= inv;
      v.y *= inv;
    }
    b[i] = v;
  }
}

// g[row][i] *= B[i] over all rows (the convolution's pointwise product).
__global__ void k_chirp_mul(double2 *__restrict__ g, const double2 *__restrict__ B, int M, long long total) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const double2 a = g[i], c = B[i % M];
    g[i] = make_double2(a.x * c.x - a.y * c.y, a.x * c.y + a.y * c.x);
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
// over the transform (rows of stride ld, the first N entries) and log L of the
// pair; the last block of each request sums its detectors in order.
//   aligned   (mcmc_gw.cpp:595-658): 1/2 max|G|^2 df^2 / <h|h>
//   unaligned (mcmc_gw.cpp:660-800): 1/4 max lambda, with
//     rho+ = df G+ / sqrt(<h+|h+>), rhox = df Gx / sqrt(<hx|hx>),
//     gamma = Re(rho+ conj(rhox)), I = <h+|hx> / sqrt(<h+|h+><hx|hx>),
//     lambda = (|rho+|^2 + |rhox|^2 - 2 gamma I + sqrt((|rho+|^2 - |rhox|^2)^2
//              + 4 (I |rho+|^2 - gamma)(I |rhox|^2 - gamma))) / (1 - I^2).
template <bool UN>
__global__ void k_maxll_reduce(const double2 *__restrict__ G, const double *__restrict__ part, int nblk, int N,
                               int ld, int ndet, const StreamDev *__restrict__ streams,
                               const int *__restrict__ handles, const int *__restrict__ req_status,
                               double *__restrict__ ll_pair, unsigned *__restrict__ done, double *__restrict__ out,
                               int *__restrict__ status) {
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
      const double2 v = G[(size_t)q * ld + k];
      m = fmax(m, v.x * v.x + v.y * v.y);
    }
  } else {
    const double ap = df / sqrt(sums[0]), ac = df / sqrt(sums[1]);
    const double I = sums[2] / (sqrt(sums[0]) * sqrt(sums[1]));
    m = -HUGE_VAL;
    for (int k = threadIdx.x; k < N; k += blockDim.x) {
      const double2 a = G[((size_t)q * NP) * ld + k], c = G[((size_t)q * NP + 1) * ld + k];
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

// ------------------------------------------------------------ the transform
// Length-N DFTs of `rows` rows: cuFFT directly when N has no prime factor
// above 7, else Bluestein with a power-of-two M (the kernel B cached in the
// context per N).
struct Xform {
  int N = 0, ld = 0, blue = 0, plan = 0;
  const double2 *B = nullptr;
};

bool smooth7(int n) {
  for (int p : {2, 3, 5, 7})
    while (n % p == 0) n /= p;
  return n == 1;
}

int xform_setup(gwgpu_context *c, int N, int rows, Xform &x) {
  x.N = N;
  x.blue = !smooth7(N);
  x.ld = N;
  if (x.blue) {
    x.ld = 1;
    while (x.ld < 2 * N - 1) x.ld <<= 1;
  }
  int st = gwfft::plan(c, gwfft::kZ2Z, x.ld, rows, &x.plan);
  if (st || !x.blue) return st;
  void *kb;
  if ((st = c->workspace(gwgpu_context::kWsChirp, 16 * (size_t)x.ld, &kb))) return st;
  x.B = (const double2 *)kb;
  if (c->chirp_n != N) {
    int p1;
    if ((st = gwfft::plan(c, gwfft::kZ2Z, x.ld, 1, &p1))) return st;
    const int gb = std::min((x.ld + kBlock - 1) / kBlock, 1024);
    k_chirp_fill<<<gb, kBlock, 0, c->stream>>>((double2 *)kb, N, x.ld);
    if ((st = gwfft::exec_z2z(c, p1, (double2 *)kb, (double2 *)kb, gwfft::kForward, c->stream))) return st;
    c->chirp_n = N;
  }
  return GWGPU_OK;
}

int xform_run(gwgpu_context *c, const Xform &x, double2 *g, int rows) {
  int st = gwfft::exec_z2z(c, x.plan, g, g, gwfft::kForward, c->stream);
  if (st || !x.blue) return st;
  const long long total = (long long)rows * x.ld;
  const int gb = (int)std::min<long long>((total + kBlock - 1) / kBlock, 152 * 16);
  k_chirp_mul<<<gb, kBlock, 0, c->stream>>>(g, x.B, x.ld, total);
  return gwfft::exec_z2z(c, x.plan, g, g, gwfft::kInverse, c->stream);
}

// One pair from host arrays: hp (and hc when unaligned) given.
int maximized_single(gwgpu_context *c, const double *data, const double *psd, const double *freqs, const double *hp,
                     const double *hc, int N, double *out) {
  const bool un = hc != nullptr;
  const int np = un ? 2 : 1, ns = un ? 3 : 1;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  Xform x;
  int st = xform_setup(c, N, np, x);
  if (st) return st;
  const int nblk = (x.ld + kBlock - 1) / kBlock;
  const size_t o_f = 0, o_d = up256(8 * (size_t)N), o_s = o_d + up256(16 * (size_t)N),
               o_rp = o_s + up256(8 * (size_t)N), o_rc = o_rp + up256(16 * (size_t)N),
               o_g = o_rc + up256(16 * (size_t)N), o_h = o_g + up256(16 * (size_t)x.ld * np),
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
  double *hh = (double *)(b + o_h);
  if (un)
    k_maxll_prep<true><<<dim3(nblk, 1), kBlock, 0, c->stream>>>(nullptr, rp, rc, 1, sdd, dh, N, x.ld, x.blue, g, hh);
  else
    k_maxll_prep<false><<<dim3(nblk, 1), kBlock, 0, c->stream>>>(nullptr, rp, nullptr, 1, sdd, dh, N, x.ld, x.blue,
                                                                g, hh);
  if ((st = xform_run(c, x, g, np))) return st;
  if (un)
    k_maxll_reduce<true><<<1, kBlock, 0, c->stream>>>(g, hh, nblk, N, x.ld, 1, sdd, dh, nullptr, ll_pair, done, res,
                                                      nullptr);
  else
    k_maxll_reduce<false><<<1, kBlock, 0, c->stream>>>(g, hh, nblk, N, x.ld, 1, sdd, dh, nullptr, ll_pair, done,
                                                       res, nullptr);
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
  Xform x;
  int st = xform_setup(c, N, pairs * np, x);
  if (st) return st;
  const int nblk = (x.ld + kBlock - 1) / kBlock;
  const size_t o_p = 0, o_a = up256(sizeof(gwgpu_gen_params) * n), o_h = o_a + up256(4 * (size_t)n),
               o_req = o_h + up256(4 * (size_t)pairs), o_g = o_req + up256(sizeof(Request) * n),
               o_hh = o_g + up256(16 * (size_t)pairs * np * x.ld),
               o_ll = o_hh + up256(8 * (size_t)pairs * ns * nblk), o_out = o_ll + up256(8 * (size_t)pairs),
               o_st = o_out + up256(8 * (size_t)n), o_done = o_st + up256(4 * (size_t)n),
               total = o_done + up256(4 * (size_t)n);
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
    k_maxll_prep<true><<<dim3(nblk, n), kBlock, 0, c->stream>>>(rq, nullptr, nullptr, ndet, c->streams_dev, hd, N,
                                                                   x.ld, x.blue, g, hh);
  else
    k_maxll_prep<false><<<dim3(nblk, n), kBlock, 0, c->stream>>>(rq, nullptr, nullptr, ndet, c->streams_dev, hd, N,
                                                                    x.ld, x.blue, g, hh);
  if ((st = xform_run(c, x, g, pairs * np))) return st;
  int *dst = (int *)(b + o_st);
  if (un)
    k_maxll_reduce<true><<<pairs, kBlock, 0, c->stream>>>(g, hh, nblk, N, x.ld, ndet, c->streams_dev, hd, dst,
                                                          (double *)(b + o_ll), (unsigned *)(b + o_done),
                                                          (double *)(b + o_out), dst);
  else
    k_maxll_reduce<false><<<pairs, kBlock, 0, c->stream>>>(g, hh, nblk, N, x.ld, ndet, c->streams_dev, hd, dst,
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
