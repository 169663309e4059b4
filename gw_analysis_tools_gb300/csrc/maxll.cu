// maxll.cu -- the likelihood maximised over arrival time and phase,
// maximized_Log_Likelihood_aligned_spin_internal (mcmc_gw.cpp:595-658) and
// maximized_Log_Likelihood_unaligned_spin_internal (:660-800), and the
// sampler's intrinsic mode that sums them over detectors
// (MCMC_likelihood_wrapper, mcmc_gw.cpp:2611-2720).
//
// Per (request, detector): HH = 4 S(|r|^2 / S_n) by Simpson's rule,
// g_k = 4 conj(d_k) r_k / S_n,k, G = DFT_N(g), and
// log L = 1/2 max_j |G_j|^2 df^2 / HH (the unaligned form: 1/4 max of lambda,
// built from the transforms of the h+ and hx products).
//
// Grid lengths N with a prime factor above 7 (32128 = 2^7 * 251 is typical)
// use Bluestein's identity nk = (n^2 + k^2 - (k - n)^2) / 2 with power-of-two
// transforms of length M >= 2N - 1:
//   G_k = e^{-i pi k^2/N} sum_n [g_n e^{-i pi n^2/N}] e^{i pi (k-n)^2/N},
// a cyclic convolution of a_n = g_n e^{-i pi n^2/N} with b_m = e^{i pi m^2/N}
// (FFT_M, a pointwise product with the transform of b, inverse FFT_M).  The
// outer factor e^{-i pi k^2/N} is never applied: every quantity taken from G
// (|G_k|^2, Re(G+_k conj(Gx_k))) is invariant to a phase common to the pair.
// The chirp phases use n^2 mod 2N in integers.
//
// GB300's FP64 rate makes FP64 transforms the bottleneck, so by default the
// transforms run in FP32 and only locate the maximum: with E a bound on the
// FP32 error of each G_k (tau * ||C||_2, from the transform's norm growth),
// every k whose FP32 value could still be the maximum (|C_k| + E >= max_j
// |C_j| - E, or the same with the lambda bound of the unaligned form) is a
// candidate, and G is evaluated exactly in FP64 at the candidates only (a
// direct sum with exactly reduced twiddles).  The result is the maximum over
// the FP64 values, i.e. the reference's maximum.  A pair with more than
// kCand candidates (a flat spectrum) sends the batch to the FP64 transforms
// (also selected by GWGPU_MAXLL=fp64).
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
      const double iS = st.ipsd ? st.ipsd[k] : 1.0 / st.psd[k], w = gwt::simpson_weight(k, N), s4 = 4.0 * iS;
      // 4 conj(d) h / S, then the Bluestein chirp
      double2 v = make_double2(s4 * (d.x * hp.x + d.y * hp.y), s4 * (d.x * hp.y - d.y * hp.x));
      g[((size_t)q * NP) * ld + k] = make_double2(v.x * ch.x - v.y * ch.y, v.x * ch.y + v.y * ch.x);
      acc[0] = w * ((hp.x * hp.x + hp.y * hp.y) * iS);
      if (UN) {
        v = make_double2(s4 * (d.x * hc.x + d.y * hc.y), s4 * (d.x * hc.y - d.y * hc.x));
        g[((size_t)q * NP + 1) * ld + k] = make_double2(v.x * ch.x - v.y * ch.y, v.x * ch.y + v.y * ch.x);
        acc[1] = w * ((hc.x * hc.x + hc.y * hc.y) * iS);
        acc[2] = w * ((hp.x * hc.x + hp.y * hc.y) * iS);
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

// ======================================================= FP32 search path
constexpr int kCand = 32;              // candidates per pair
constexpr double kTau = 4e-5;          // FP32 transform error / (||a||_2 * kscale), with a 4x margin
constexpr int kMaxTwiddleRows = 12288; // shared twiddle table of the FP64 refinement: N <= 256 * this

// e^{-i pi m^2 / N} in FP32 (phase reduced exactly in integers).
__device__ __forceinline__ float2 chirp32(long long m, int N) {
  const long long t = (m * m) % (2LL * N);
  float sn, cs;
  sincospif((float)t / (float)N, &sn, &cs);
  return make_float2(cs, -sn);
}

// As k_maxll_prep, writing the exact products g (FP64, rows of N) for the
// refinement and their FP32 (chirped) copy a (rows of ld) for the search, with
// the partial sums of |g|^2 per row beside the Simpson sums:
//   aligned:   [<h|h>, |g|^2]
//   unaligned: [<h+|h+>, <hx|hx>, <h+|hx>, |g+|^2, |gx|^2]
template <bool UN>
__global__ void k_mx_prep(const Request *__restrict__ req, const double2 *__restrict__ resp_p,
                          const double2 *__restrict__ resp_c, int ndet, const StreamDev *__restrict__ streams,
                          const int *__restrict__ handles, int N, int ld, int blue, double2 *__restrict__ g64,
                          float2 *__restrict__ a32, double *__restrict__ part) {
  constexpr int NS = UN ? 5 : 2, NP = UN ? 2 : 1;
  __shared__ double s_red[NS][kWarps];
  const int r = blockIdx.y;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  double2 hp = make_double2(0.0, 0.0), hc = make_double2(0.0, 0.0);
  if (req && k < N && !req[r].m.status) {
    gwt::cd p, c;
    gwt::wave_bin(req[r], streams[handles[(size_t)r * ndet]].freqs[k], p, c);
    hp = make_double2(p.re, p.im);
    hc = make_double2(c.re, c.im);
  }
  const float2 ch = (blue && k < N) ? chirp32(k, N) : make_float2(1.f, 0.f);
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
      const double iS = st.ipsd ? st.ipsd[k] : 1.0 / st.psd[k], w = gwt::simpson_weight(k, N), s4 = 4.0 * iS;
      const double2 v = make_double2(s4 * (d.x * hp.x + d.y * hp.y), s4 * (d.x * hp.y - d.y * hp.x));
      g64[((size_t)q * NP) * N + k] = v;
      const float vx = (float)v.x, vy = (float)v.y;
      a32[((size_t)q * NP) * ld + k] = make_float2(vx * ch.x - vy * ch.y, vx * ch.y + vy * ch.x);
      acc[0] = w * ((hp.x * hp.x + hp.y * hp.y) * iS);
      if (UN) {
        const double2 u = make_double2(s4 * (d.x * hc.x + d.y * hc.y), s4 * (d.x * hc.y - d.y * hc.x));
        g64[((size_t)q * NP + 1) * N + k] = u;
        const float ux = (float)u.x, uy = (float)u.y;
        a32[((size_t)q * NP + 1) * ld + k] = make_float2(ux * ch.x - uy * ch.y, ux * ch.y + uy * ch.x);
        acc[1] = w * ((hc.x * hc.x + hc.y * hc.y) * iS);
        acc[2] = w * ((hp.x * hc.x + hp.y * hc.y) * iS);
        acc[3] = v.x * v.x + v.y * v.y;
        acc[4] = u.x * u.x + u.y * u.y;
      } else {
        acc[NS - 1] = v.x * v.x + v.y * v.y;
      }
    } else if (k < ld) {
      a32[((size_t)q * NP) * ld + k] = make_float2(0.f, 0.f);
      if (UN) a32[((size_t)q * NP + 1) * ld + k] = make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int j = 0; j < NS; j++) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc[j] += __shfl_xor_sync(0xffffffffu, acc[j], o);
    }
    __syncthreads();
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

__global__ void k_chirp_mul32(float2 *__restrict__ a, const float2 *__restrict__ B, int M, long long total) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const float2 x = a[i], c = B[i % M];
    a[i] = make_float2(x.x * c.x - x.y * c.y, x.x * c.y + x.y * c.x);
  }
}

// Block max of v (every thread gets it).
__device__ float block_max(float v, float *s_tmp) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) s_tmp[threadIdx.x >> 5] = v;
  __syncthreads();
  float t = s_tmp[0];
  for (int w = 1; w < kWarps; w++) t = fmaxf(t, s_tmp[w]);
  return t;
}

// One block per pair: the sums (Simpson sums scaled, |g|^2 raw, kept for the
// refinement), the FP32 score of every k < N with its error bound, and the
// candidates k whose score plus bound reaches the largest score minus bound.
template <bool UN>
__global__ void k_mx_cand(const float2 *__restrict__ C, const double *__restrict__ part, int nblk, int N, int ld,
                          int ndet, const StreamDev *__restrict__ streams, const int *__restrict__ handles,
                          const int *__restrict__ req_status, double kscale, double *__restrict__ sums,
                          int *__restrict__ cand, int *__restrict__ ncand, int *__restrict__ overflow) {
  constexpr int NS = UN ? 5 : 2, NP = UN ? 2 : 1;
  __shared__ double s_tmp[kWarps];
  __shared__ float s_tmpf[kWarps];
  __shared__ int s_cnt;
  const int q = blockIdx.x, r = q / ndet;
  if (req_status && req_status[r]) {  // outside the model domain: no candidates, the result is NaN
    if (threadIdx.x == 0) ncand[q] = 0;
    return;
  }
  const StreamDev &st = streams[handles[q]];
  const double df = st.freqs[1] - st.freqs[0];
  double sm[NS];
#pragma unroll
  for (int j = 0; j < NS; j++) {
    double t = 0.0;
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) t += part[((size_t)q * NS + j) * nblk + b];
    t = block_sum(t, s_tmp);
    sm[j] = (UN ? j < 3 : j < 1) ? 4.0 * t * df / 3.0 : t;
  }
  if (threadIdx.x < NS) sums[(size_t)q * NS + threadIdx.x] = sm[threadIdx.x];
  if (threadIdx.x == 0) s_cnt = 0;
  // score and bound of bin k
  float ap = 1.f, ac = 1.f, I = 0.f, eps = 0.f, E = 0.f, inv1mI = 1.f;
  if (UN) {
    ap = (float)(df / sqrt(sm[0]));
    ac = (float)(df / sqrt(sm[1]));
    I = (float)(sm[2] / (sqrt(sm[0]) * sqrt(sm[1])));
    eps = (float)fmax(ap * kTau * kscale * sqrt(sm[3]), ac * kTau * kscale * sqrt(sm[4]));
    inv1mI = 1.f / (1.f - fabsf(I));
  } else {
    E = (float)(kTau * kscale * sqrt(sm[1]));
  }
  auto score = [&](int k, float &lo, float &hi) {
    if (!UN) {
      const float2 v = C[(size_t)q * ld + k];
      const float m = sqrtf(v.x * v.x + v.y * v.y);
      lo = m - E;
      hi = m + E;
    } else {
      const float2 a = C[((size_t)q * NP) * ld + k], c = C[((size_t)q * NP + 1) * ld + k];
      const float rpx = ap * a.x, rpy = ap * a.y, rcx = ac * c.x, rcy = ac * c.y;
      const float p2 = rpx * rpx + rpy * rpy, c2 = rcx * rcx + rcy * rcy, gam = rpx * rcx + rpy * rcy;
      const float lam =
          (p2 + c2 - 2.f * gam * I + sqrtf(fmaxf((p2 - c2) * (p2 - c2) + 4.f * (I * p2 - gam) * (I * c2 - gam), 0.f))) /
          (1.f - I * I);
      // |d lambda| <= (4 (|rho+| + |rhox|) eps + 4 eps^2) / (1 - |I|), doubled, plus FP32 rounding of lambda
      const float D = 2.f * (4.f * (sqrtf(p2) + sqrtf(c2) + 2.f * eps) * eps + 4.f * eps * eps) * inv1mI +
                      1e-5f * fabsf(lam);
      lo = lam - D;
      hi = lam + D;
    }
  };
  float L = -INFINITY;
  for (int k = threadIdx.x; k < N; k += blockDim.x) {
    float lo, hi;
    score(k, lo, hi);
    L = fmaxf(L, lo);
  }
  L = block_max(L, s_tmpf);
  for (int k = threadIdx.x; k < N; k += blockDim.x) {
    float lo, hi;
    score(k, lo, hi);
    if (hi >= L || hi != hi) {  // NaN scores are candidates too
      const int i = atomicAdd(&s_cnt, 1);
      if (i < kCand) cand[(size_t)q * kCand + i] = k;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    ncand[q] = min(s_cnt, kCand);
    if (s_cnt > kCand) atomicExch(overflow, 1);
  }
}

// G_k of the candidate rows exactly in FP64: sum_n g_n e^{-2 pi i nk/N}, the
// twiddle of n = 256 j + i as e^{-2 pi i (256 j k mod N)/N} e^{-2 pi i (i k mod N)/N}
// (both phases reduced exactly in integers).  candval = |G_k|^2 (aligned) or
// lambda (unaligned).  Persistent over the (pair, candidate) slots.
template <bool UN>
__global__ void k_mx_refine(const double2 *__restrict__ g64, int N, int pairs, const int *__restrict__ cand,
                            const int *__restrict__ ncand, const double *__restrict__ sums,
                            const StreamDev *__restrict__ streams, const int *__restrict__ handles,
                            double *__restrict__ candval) {
  constexpr int NS = UN ? 5 : 2, NP = UN ? 2 : 1, NV = UN ? 4 : 2;
  extern __shared__ double2 s_wj[];
  __shared__ double s_red[NV][kWarps];
  const int nj = (N + kBlock - 1) / kBlock;
  // slot s = (candidate ci, pair q) with ci major, so that the first
  // candidates of all pairs take consecutive blocks
  for (int sl = blockIdx.x; sl < pairs * kCand; sl += gridDim.x) {
    const int q = sl % pairs, ci = sl / pairs, it = q * kCand + ci;
    if (ci >= ncand[q]) continue;
    const long long k = cand[it];
    __syncthreads();  // the previous slot's table has been read
    for (int j = threadIdx.x; j < nj; j += blockDim.x) {
      const long long t = ((long long)j * kBlock % N) * k % N;
      double sn, cs;
      sincospi(2.0 * (double)t / (double)N, &sn, &cs);
      s_wj[j] = make_double2(cs, -sn);
    }
    double2 wi;
    {
      const long long t = (long long)threadIdx.x * k % N;
      double sn, cs;
      sincospi(2.0 * (double)t / (double)N, &sn, &cs);
      wi = make_double2(cs, -sn);
    }
    __syncthreads();
    double v[NV];
#pragma unroll
    for (int u = 0; u < NV; u++) v[u] = 0.0;
    // this thread's bins n = 256 j + i: sum_j g_n e^{-2 pi i 256 j k/N}, then
    // one product with e^{-2 pi i i k/N}
    const double2 *row = g64 + ((size_t)q * NP) * N;
    for (int j = 0; j < nj; j++) {
      const int n = j * kBlock + threadIdx.x;
      if (n >= N) break;
      const double2 w = s_wj[j];
      const double2 x = row[n];
      v[0] += x.x * w.x - x.y * w.y;
      v[1] += x.x * w.y + x.y * w.x;
      if (UN) {
        const double2 y = row[N + n];
        v[2] += y.x * w.x - y.y * w.y;
        v[3] += y.x * w.y + y.y * w.x;
      }
    }
#pragma unroll
    for (int u = 0; u < NV; u += 2) {
      const double re = v[u] * wi.x - v[u + 1] * wi.y, im = v[u] * wi.y + v[u + 1] * wi.x;
      v[u] = re;
      v[u + 1] = im;
    }
#pragma unroll
    for (int u = 0; u < NV; u++) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v[u] += __shfl_xor_sync(0xffffffffu, v[u], o);
    }
    if ((threadIdx.x & 31) == 0)
#pragma unroll
      for (int u = 0; u < NV; u++) s_red[u][threadIdx.x >> 5] = v[u];
    __syncthreads();
    if (threadIdx.x == 0) {
      double G[NV];
#pragma unroll
      for (int u = 0; u < NV; u++) {
        G[u] = 0.0;
        for (int w = 0; w < kWarps; w++) G[u] += s_red[u][w];
      }
      if (!UN) {
        candval[it] = G[0] * G[0] + G[1] * G[1];
      } else {
        const double *sm = sums + (size_t)q * NS;
        const StreamDev &st = streams[handles[q]];
        const double df = st.freqs[1] - st.freqs[0];
        const double ap = df / sqrt(sm[0]), ac = df / sqrt(sm[1]);
        const double I = sm[2] / (sqrt(sm[0]) * sqrt(sm[1]));
        const double rpx = ap * G[0], rpy = ap * G[1], rcx = ac * G[2], rcy = ac * G[3];
        const double p2 = rpx * rpx + rpy * rpy, c2 = rcx * rcx + rcy * rcy, gam = rpx * rcx + rpy * rcy;
        candval[it] =
            (p2 + c2 - 2 * gam * I + sqrt((p2 - c2) * (p2 - c2) + 4. * (I * p2 - gam) * (I * c2 - gam))) / (1. - I * I);
      }
    }
  }
}

// One thread per request: log L of each pair from its best candidate, summed
// over the detectors in order.
template <bool UN>
__global__ void k_mx_final(const double *__restrict__ candval, const int *__restrict__ ncand,
                           const double *__restrict__ sums, int n, int ndet, const StreamDev *__restrict__ streams,
                           const int *__restrict__ handles, const int *__restrict__ req_status,
                           double *__restrict__ out, int *__restrict__ status) {
  constexpr int NS = UN ? 5 : 2;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int rs = req_status ? req_status[r] : 0;
  double ll = 0.0;
  for (int d = 0; d < ndet; d++) {
    const int q = r * ndet + d;
    double mx = -HUGE_VAL;
    for (int c = 0; c < ncand[q]; c++) mx = fmax(mx, candval[(size_t)q * kCand + c]);
    if (UN) {
      ll += 0.25 * mx;
    } else {
      const StreamDev &st = streams[handles[q]];
      const double df = st.freqs[1] - st.freqs[0];
      ll += 0.5 * (mx * df * df) / sums[(size_t)q * NS];
    }
  }
  out[r] = rs ? __longlong_as_double(0x7ff8000000000000ll) : ll;
  if (status) status[r] = rs;
}

// max |B_j| over the Bluestein kernel (one block).
__global__ void k_absmax(const double2 *__restrict__ B, int M, double *__restrict__ out) {
  __shared__ double s[kWarps];
  double m = 0.0;
  for (int i = threadIdx.x; i < M; i += blockDim.x) m = fmax(m, hypot(B[i].x, B[i].y));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = s[0];
    for (int w = 1; w < kWarps; w++) t = fmax(t, s[w]);
    *out = t;
  }
}

__global__ void k_to_f32(const double2 *__restrict__ x, float2 *__restrict__ y, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    y[i] = make_float2((float)x[i].x, (float)x[i].y);
}

size_t up256(size_t x) { return (x + 255) & ~(size_t)255; }

bool smooth7(int n) {
  for (int p : {2, 3, 5, 7})
    while (n % p == 0) n /= p;
  return n == 1;
}

// Transform length: N itself when cuFFT handles it directly, else the
// Bluestein power of two M >= 2N - 1.
int xform_len(int N, int *blue) {
  *blue = !smooth7(N);
  if (!*blue) return N;
  int M = 1;
  while (M < 2 * N - 1) M <<= 1;
  return M;
}

// The Bluestein kernel for N, FFT_M(b)/M in FP64 (kWsChirp) and FP32
// (kWsChirp32), and the search's error scale M max|B|, kept until N changes.
int ensure_chirp(gwgpu_context *c, int N, int M, const double2 **B64, const float2 **B32) {
  void *kb, *kb32;
  int st = c->workspace(gwgpu_context::kWsChirp, 16 * (size_t)M + 256, &kb);
  if (st) return st;
  if ((st = c->workspace(gwgpu_context::kWsChirp32, 8 * (size_t)M, &kb32))) return st;
  *B64 = (const double2 *)kb;
  *B32 = (const float2 *)kb32;
  if (c->chirp_n == N) return GWGPU_OK;
  int p1;
  if ((st = gwfft::plan(c, gwfft::kZ2Z, M, 1, &p1))) return st;
  const int gb = std::min((M + kBlock - 1) / kBlock, 1024);
  k_chirp_fill<<<gb, kBlock, 0, c->stream>>>((double2 *)kb, N, M);
  if ((st = gwfft::exec_z2z(c, p1, (double2 *)kb, (double2 *)kb, gwfft::kForward, c->stream))) return st;
  double *dmax = (double *)((char *)kb + 16 * (size_t)M);
  k_absmax<<<1, kBlock, 0, c->stream>>>((const double2 *)kb, M, dmax);
  k_to_f32<<<gb, kBlock, 0, c->stream>>>((const double2 *)kb, (float2 *)kb32, M);
  double bmax = 0;
  cudaMemcpyAsync(&bmax, dmax, 8, cudaMemcpyDeviceToHost, c->stream);
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return c->fail(e, "Bluestein kernel");
  c->chirp_kscale = (double)M * bmax;
  c->chirp_n = N;
  return GWGPU_OK;
}

// What both entry points hand to the pipeline (device pointers).
struct MxIn {
  const Request *req = nullptr;               // requests (intrinsic mode), or null
  const double2 *rp = nullptr, *rc = nullptr;  // responses per pair, rows of N, when req is null
  const StreamDev *streams = nullptr;
  const int *handles = nullptr;                // [n * ndet]
  const int *req_status = nullptr;             // per request, or null
  int n = 0, ndet = 0, N = 0;
  bool un = false;
};

// The FP64 transforms: prep, FFT_M (Bluestein) or FFT_N, reduction.
int run_fp64(gwgpu_context *c, const MxIn &in, double *out, int *status) {
  const int np = in.un ? 2 : 1, ns = in.un ? 3 : 1, pairs = in.n * in.ndet, rows = pairs * np;
  int blue;
  const int ld = xform_len(in.N, &blue);
  const double2 *B64 = nullptr;
  const float2 *B32 = nullptr;
  int st = blue ? ensure_chirp(c, in.N, ld, &B64, &B32) : GWGPU_OK;
  if (st) return st;
  int plan;  // fetched last: a new plan may reset the cache (cufft_rt.cu)
  if ((st = gwfft::plan(c, gwfft::kZ2Z, ld, rows, &plan))) return st;
  const int nblk = (ld + kBlock - 1) / kBlock;
  const size_t o_g = 0, o_h = up256(16 * (size_t)rows * ld), o_ll = o_h + up256(8 * (size_t)pairs * ns * nblk),
               o_done = o_ll + up256(8 * (size_t)pairs), total = o_done + up256(4 * (size_t)in.n);
  void *dev;
  if ((st = c->workspace(gwgpu_context::kWsMaxllRun, total, &dev))) return st;
  char *b = (char *)dev;
  double2 *g = (double2 *)(b + o_g);
  double *hh = (double *)(b + o_h);
  unsigned *done = (unsigned *)(b + o_done);
  cudaMemsetAsync(done, 0, 4 * (size_t)in.n, c->stream);
  const dim3 grid(nblk, in.n);
  if (in.un)
    k_maxll_prep<true><<<grid, kBlock, 0, c->stream>>>(in.req, in.rp, in.rc, in.ndet, in.streams, in.handles, in.N,
                                                        ld, blue, g, hh);
  else
    k_maxll_prep<false><<<grid, kBlock, 0, c->stream>>>(in.req, in.rp, in.rc, in.ndet, in.streams, in.handles, in.N,
                                                         ld, blue, g, hh);
  if ((st = gwfft::exec_z2z(c, plan, g, g, gwfft::kForward, c->stream))) return st;
  if (blue) {
    const long long tot = (long long)rows * ld;
    const int gb = (int)std::min<long long>((tot + kBlock - 1) / kBlock, 152 * 16);
    k_chirp_mul<<<gb, kBlock, 0, c->stream>>>(g, B64, ld, tot);
    if ((st = gwfft::exec_z2z(c, plan, g, g, gwfft::kInverse, c->stream))) return st;
  }
  if (in.un)
    k_maxll_reduce<true><<<pairs, kBlock, 0, c->stream>>>(g, hh, nblk, in.N, ld, in.ndet, in.streams, in.handles,
                                                          in.req_status, (double *)(b + o_ll), done, out, status);
  else
    k_maxll_reduce<false><<<pairs, kBlock, 0, c->stream>>>(g, hh, nblk, in.N, ld, in.ndet, in.streams, in.handles,
                                                           in.req_status, (double *)(b + o_ll), done, out, status);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? GWGPU_OK : c->fail(e, "maximised likelihood launch");
}

// The FP32 search and FP64 refinement; *fallback set when a pair had more
// candidates than kCand (nothing written to out then).
int run_search(gwgpu_context *c, const MxIn &in, double *out, int *status, bool *fallback) {
  const int np = in.un ? 2 : 1, ns = in.un ? 5 : 2, pairs = in.n * in.ndet, rows = pairs * np;
  *fallback = false;
  int blue;
  const int ld = xform_len(in.N, &blue);
  const double2 *B64 = nullptr;
  const float2 *B32 = nullptr;
  double kscale = std::sqrt((double)in.N);
  int st = GWGPU_OK;
  if (blue) {
    if ((st = ensure_chirp(c, in.N, ld, &B64, &B32))) return st;
    kscale = c->chirp_kscale;
  }
  int plan;  // fetched last: a new plan may reset the cache (cufft_rt.cu)
  if ((st = gwfft::plan(c, gwfft::kC2C, ld, rows, &plan))) return st;
  const int nblk = (ld + kBlock - 1) / kBlock;
  const size_t o_g = 0, o_a = up256(16 * (size_t)rows * in.N), o_h = o_a + up256(8 * (size_t)rows * ld),
               o_s = o_h + up256(8 * (size_t)pairs * ns * nblk), o_c = o_s + up256(8 * (size_t)pairs * ns),
               o_nc = o_c + up256(4 * (size_t)pairs * kCand), o_v = o_nc + up256(4 * (size_t)pairs),
               o_o = o_v + up256(8 * (size_t)pairs * kCand), total = o_o + 256;
  void *dev;
  if ((st = c->workspace(gwgpu_context::kWsMaxllRun, total, &dev))) return st;
  char *b = (char *)dev;
  double2 *g64 = (double2 *)(b + o_g);
  float2 *a32 = (float2 *)(b + o_a);
  double *hh = (double *)(b + o_h), *sums = (double *)(b + o_s), *cv = (double *)(b + o_v);
  int *cand = (int *)(b + o_c), *ncand = (int *)(b + o_nc), *ovf = (int *)(b + o_o);
  cudaMemsetAsync(ovf, 0, 4, c->stream);
  const dim3 grid(nblk, in.n);
  if (in.un)
    k_mx_prep<true><<<grid, kBlock, 0, c->stream>>>(in.req, in.rp, in.rc, in.ndet, in.streams, in.handles, in.N, ld,
                                                     blue, g64, a32, hh);
  else
    k_mx_prep<false><<<grid, kBlock, 0, c->stream>>>(in.req, in.rp, in.rc, in.ndet, in.streams, in.handles, in.N, ld,
                                                      blue, g64, a32, hh);
  if ((st = gwfft::exec_c2c(c, plan, a32, a32, gwfft::kForward, c->stream))) return st;
  if (blue) {
    const long long tot = (long long)rows * ld;
    const int gb = (int)std::min<long long>((tot + kBlock - 1) / kBlock, 152 * 16);
    k_chirp_mul32<<<gb, kBlock, 0, c->stream>>>(a32, B32, ld, tot);
    if ((st = gwfft::exec_c2c(c, plan, a32, a32, gwfft::kInverse, c->stream))) return st;
  }
  if (in.un)
    k_mx_cand<true><<<pairs, kBlock, 0, c->stream>>>(a32, hh, nblk, in.N, ld, in.ndet, in.streams, in.handles,
                                                      in.req_status, kscale, sums, cand, ncand, ovf);
  else
    k_mx_cand<false><<<pairs, kBlock, 0, c->stream>>>(a32, hh, nblk, in.N, ld, in.ndet, in.streams, in.handles,
                                                       in.req_status, kscale, sums, cand, ncand, ovf);
  int h_ovf = 0;
  cudaMemcpyAsync(&h_ovf, ovf, 4, cudaMemcpyDeviceToHost, c->stream);
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return c->fail(e, "maximised likelihood search");
  if (h_ovf) {
    *fallback = true;
    return GWGPU_OK;
  }
  const int nj = (in.N + kBlock - 1) / kBlock;
  const size_t smem = 16 * (size_t)nj;
  const int gr = std::min(pairs * kCand, 152 * 8);
  if (in.un) {
    if (smem > 48 * 1024) cudaFuncSetAttribute(k_mx_refine<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_mx_refine<true><<<gr, kBlock, smem, c->stream>>>(g64, in.N, pairs, cand, ncand, sums, in.streams, in.handles,
                                                        cv);
    k_mx_final<true><<<(in.n + 127) / 128, 128, 0, c->stream>>>(cv, ncand, sums, in.n, in.ndet, in.streams,
                                                                 in.handles, in.req_status, out, status);
  } else {
    if (smem > 48 * 1024)
      cudaFuncSetAttribute(k_mx_refine<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_mx_refine<false><<<gr, kBlock, smem, c->stream>>>(g64, in.N, pairs, cand, ncand, sums, in.streams,
                                                         in.handles, cv);
    k_mx_final<false><<<(in.n + 127) / 128, 128, 0, c->stream>>>(cv, ncand, sums, in.n, in.ndet, in.streams,
                                                                  in.handles, in.req_status, out, status);
  }
  e = cudaGetLastError();
  return e == cudaSuccess ? GWGPU_OK : c->fail(e, "maximised likelihood launch");
}

int maxll_run(gwgpu_context *c, const MxIn &in, double *out, int *status) {
  if (!c->maxll_fp64 && (in.N + kBlock - 1) / kBlock <= kMaxTwiddleRows) {
    bool fb = false;
    int st = run_search(c, in, out, status, &fb);
    if (st || !fb) return st;
  }
  return run_fp64(c, in, out, status);
}

// One pair from host arrays: hp (and hc when unaligned) given.
int maximized_single(gwgpu_context *c, const double *data, const double *psd, const double *freqs, const double *hp,
                     const double *hc, int N, double *out) {
  const bool un = hc != nullptr;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  const size_t o_f = 0, o_d = up256(8 * (size_t)N), o_s = o_d + up256(16 * (size_t)N),
               o_rp = o_s + up256(8 * (size_t)N), o_rc = o_rp + up256(16 * (size_t)N),
               o_sd = o_rc + up256(16 * (size_t)N), o_misc = o_sd + up256(sizeof(StreamDev)), total = o_misc + 256;
  void *dev;
  int st = c->workspace(gwgpu_context::kWsMaxll, total, &dev);
  if (st) return st;
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
  cudaMemcpyAsync(b + o_sd, &sd, sizeof(sd), cudaMemcpyHostToDevice, c->stream);
  int *dh = (int *)(b + o_misc);
  double *res = (double *)(b + o_misc + 64);
  cudaMemsetAsync(dh, 0, sizeof(int), c->stream);
  MxIn in;
  in.rp = (const double2 *)(b + o_rp);
  in.rc = un ? (const double2 *)(b + o_rc) : nullptr;
  in.streams = (const StreamDev *)(b + o_sd);
  in.handles = dh;
  in.n = 1;
  in.ndet = 1;
  in.N = N;
  in.un = un;
  if ((st = maxll_run(c, in, res, nullptr))) return st;
  cudaMemcpyAsync(out, res, 8, cudaMemcpyDeviceToHost, c->stream);
  cudaError_t e = cudaStreamSynchronize(c->stream);
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
  const size_t o_p = 0, o_a = up256(sizeof(gwgpu_gen_params) * n), o_h = o_a + up256(4 * (size_t)n),
               o_req = o_h + up256(4 * (size_t)pairs), o_out = o_req + up256(sizeof(Request) * n),
               o_st = o_out + up256(8 * (size_t)n), total = o_st + up256(4 * (size_t)n);
  void *dev;
  int st = c->workspace(gwgpu_context::kWsMaxll, total, &dev);
  if (st) return st;
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
  cudaError_t e = gwk::launch_prologue((const gwt::GenParams *)(b + o_p), (const int *)(b + o_a), n,
                                       (const int *)(b + o_h), ndet, 0.0, 0, c->streams_dev, c->qnm_dev,
                                       (Request *)(b + o_req), nullptr, 0, (int *)(b + o_st), c->stream);
  if (e != cudaSuccess) return c->fail(e, "maximised likelihood prologue");
  int *dst = (int *)(b + o_st);
  MxIn in;
  in.req = (const Request *)(b + o_req);
  in.streams = c->streams_dev;
  in.handles = (const int *)(b + o_h);
  in.req_status = dst;
  in.n = n;
  in.ndet = ndet;
  in.N = N;
  in.un = un;
  if ((st = maxll_run(c, in, (double *)(b + o_out), dst))) return st;
  std::vector<int> hs(n);
  cudaMemcpyAsync(loglik, b + o_out, 8 * (size_t)n, cudaMemcpyDeviceToHost, c->stream);
  cudaMemcpyAsync(hs.data(), dst, 4 * (size_t)n, cudaMemcpyDeviceToHost, c->stream);
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return c->fail(e, "maximised likelihood");
  if (status)
    for (int i = 0; i < n; i++) status[i] = gwk::status_code(hs[i]);
  return GWGPU_OK;
}

}  // extern "C"
