// fisher.cu -- numerical Fisher matrices (fisher.cpp:81-557, 2704-2781).
//
// Plain form (gwgpu_fisher_numerical): the reference algorithm for one source
// and one detector -- complex central differences of the FP64 detector
// response at theta +- eps (one-sided at eta = 1/4), DTOA phase factor for a
// non-reference detector, log-factor chain rule, then the Simpson Gram matrix.
//
// Batched form (gwgpu_fisher_batch): many sources x detectors in one pass.
// The same central differences are taken of the FP64 amplitude A and phase
// Phi separately and combined at the centre,
//   d r_d = e^{-i Psi_d} (dA G_d + A dG_d - i A G_d (dPhi - f dtau_d)),
// so the common phase factor cancels in Re(d_j r d_k r*): the Gram matrix
// needs no per-bin sincos, only the four intrinsic parameters (M_c, eta,
// chi1, chi2) are re-evaluated per bin (FP64), and the seven extrinsic ones
// reduce to per-request constants times three moments of A^2.  The
// per-bin products are FP32 with Kahan sums; assembly and the pivoted
// Cholesky inverse (util.cpp:857-900) are FP64.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/gwgpu.h"
#include "capi_internal.h"
#include "fisher_math.h"
#include "fisher_ref.h"
#include "kernels.h"

namespace gwf {
using namespace gwt;
using gwk::StreamDev;

constexpr int kBlock = 128;
constexpr int kStatusBounds = 0x100;  // set by a tile whose bins fall outside the tables
constexpr int kStatusRedo = 10;       // five-point source left to the reference algorithm (never returned)

// ------------------------------------------------------------- batched form
__global__ void k_fisher_slots(const GenParams *__restrict__ params, int nsrc, int method, const int *__restrict__ dets,
                               int ndet, double df, double epsilon, int step_mode, const double *__restrict__ qnm,
                               SlotOut *out) {
  int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= nsrc * kSlots) return;
  fisher_slot(params[g / kSlots], g % kSlots, method, dets, ndet, df, epsilon, step_mode, qnm, out[g]);
}

__global__ void k_fisher_setup(const GenParams *__restrict__ params, int nsrc, int method, int ndet, double epsilon,
                               int step_mode, int order, const SlotOut *__restrict__ slots, FisherSrc *out,
                               int *status) {
  int src = blockIdx.x * blockDim.x + threadIdx.x;
  if (src >= nsrc) return;
  status[src] =
      fisher_setup(params[src], method, ndet, epsilon, step_mode, order, slots + (size_t)src * kSlots, out[src]);
}

struct FisherArgs {
  const FisherSrc *src;
  int nsrc, ndet, nw;       // nw: distinct weight streams (1 when every detector has the same PSD)
  const int *wslot;         // detector -> weight stream
  const float *what[kMaxDet];
  double wscale[kMaxDet];
  // FP64 sums: the weight of bin k is c3 s_k / (S_k wscale) from the stream's
  // FP64 reciprocal PSD (Simpson pattern s_k, c3 = 4 df_s / 3), or iw_k / (S_k
  // wscale) for a stream registered with its own integration weights iw
  const double *ipsd[kMaxDet];
  const double *iw[kMaxDet];
  double c3[kMaxDet];
  int n0, N, tile, ntiles;
  double df, fisher_df_ratio;  // (f1 - f0) / simpson_df
  float df_f;                  // df in FP32 (the bins' frequency in the moment sums)
  gwt::Tables tab;
  const double *tm76d;
  int tm76d_n;              // tm76d valid for n <= tm76d_n
  unsigned *item_counter, *src_done;
  double *partials;  // items * kMaxDet * kSums
  double *fisher, *cov;
  int *status;
};

// ACC64: the per-bin differences, weights and moment sums in FP64 instead of
// FP32 values with compensated FP32 sums.
template <int NW, bool ACC64>
__global__ void __launch_bounds__(kBlock, 3) k_fisher_main(const FisherArgs a) {
  __shared__ int s_item;
  __shared__ __align__(16) unsigned char s_buf[sizeof(FisherSrc)];
  __shared__ double s_red[32 * 8];
  const int tid = threadIdx.x;
  const int nitems = a.nsrc * a.ntiles;
  for (;;) {
    if (tid == 0) s_item = (int)atomicAdd(a.item_counter, 1u);
    __syncthreads();
    const int it = s_item;
    if (it >= nitems) break;
    const int src = it / a.ntiles, tile = it % a.ntiles;
    {
      const unsigned *p = (const unsigned *)(a.src + src);
      unsigned *q = (unsigned *)s_buf;
      for (int w = tid; w < (int)(sizeof(FisherSrc) / 4); w += blockDim.x) q[w] = p[w];
    }
    __syncthreads();
    const FisherSrc &F = *(const FisherSrc *)s_buf;
    using Acc = typename std::conditional<ACC64, double, KSum>::type;
    Acc acc[NW * kSums];
#pragma unroll
    for (int j = 0; j < NW * kSums; j++) {
      if constexpr (ACC64) acc[j] = 0.0;
      else acc[j] = KSum{0.f, 0.f};
    }
    const int k0 = tile * a.tile, k1 = min(k0 + a.tile, a.N);
    const bool in_tables = a.n0 >= 1 && a.n0 + k1 - 1 <= a.tab.nmax && a.n0 + k1 - 1 <= a.tm76d_n;
    if (!in_tables && tid == 0) atomicOr(a.status + src, kStatusBounds);
    if (F.status == 0 && in_tables) {
      for (int k = k0 + tid; k < k1; k += blockDim.x) {
        const int n = a.n0 + k;
        if constexpr (ACC64) {
          double a0, qr[kIntr], qi[kIntr];
          if (!fisher_bin_q(F, n, a.tab.t13[n], a.tab.tm53[n], a.tab.tln[n], a.tab.t34[n], a.tm76d[n],
                            a.tab.tm76f[n], a0, qr, qi))
            continue;
          const double fk = (double)n * a.df, sw = simpson_weight(k, a.N);
#pragma unroll
          for (int w = 0; w < NW; w++)
            fisher_accumulate64((a.iw[w] ? a.iw[w][k] : a.c3[w] * sw) * a.ipsd[w][k] / a.wscale[w], a0, fk, qr, qi,
                                acc + w * kSums);
        } else {
          float a0, qr[kIntr], qi[kIntr];
          if (!fisher_bin_q(F, n, a.tab.t13[n], a.tab.tm53[n], a.tab.tln[n], a.tab.t34[n], a.tm76d[n],
                            a.tab.tm76f[n], a0, qr, qi))
            continue;
          const float fk = (float)n * a.df_f;
#pragma unroll
          for (int w = 0; w < NW; w++) fisher_accumulate(a.what[w][k], a0, fk, qr, qi, acc + w * kSums);
        }
      }
    }
    // block reduction in FP64, 8 values at a time
    double *part = a.partials + (size_t)it * kMaxDet * kSums;
    for (int base = 0; base < NW * kSums; base += 8) {
      double v[8];
#pragma unroll
      for (int j = 0; j < 8; j++) {
        if (base + j >= NW * kSums) v[j] = 0.0;
        else if constexpr (ACC64) v[j] = acc[base + j];
        else v[j] = (double)acc[base + j].s - (double)acc[base + j].c;
      }
#pragma unroll
      for (int j = 0; j < 8; j++)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[j] += __shfl_xor_sync(0xffffffffu, v[j], o);
      const int lane = tid & 31, warp = tid >> 5;
      if (lane == 0)
#pragma unroll
        for (int j = 0; j < 8; j++) s_red[warp * 8 + j] = v[j];
      __syncthreads();
      if (tid < 8 && base + tid < NW * kSums) {
        double s = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += s_red[w * 8 + tid];
        part[base + tid] = s;
      }
      __syncthreads();
    }
    // last tile of this source: assemble Gamma in FP64 and invert
    __shared__ bool s_last;
    __syncthreads();
    if (tid == 0) {
      __threadfence();
      unsigned prev = atomicAdd(a.src_done + src, 1u);
      s_last = (prev == (unsigned)a.ntiles - 1);
    }
    __syncthreads();
    // the source's sums over its tiles, one sum per thread in tile order
    __shared__ double s_sum[kMaxDet * kSums];
    if (s_last) {
      __threadfence();
      for (int j = tid; j < NW * kSums; j += blockDim.x) {
        double sj = 0;
        for (int tt = 0; tt < a.ntiles; tt++)
          sj += __ldcg(&a.partials[((size_t)(src * a.ntiles + tt)) * kMaxDet * kSums + j]);
        s_sum[j] = sj;
      }
    }
    __syncthreads();
    if (s_last && tid == 0) {
      const double *Ssum = s_sum;
      double Gm[kDim * kDim];
      fisher_assemble(F, Ssum, a.ndet, a.wslot, a.wscale, a.fisher_df_ratio, Gm);
      double *outF = a.fisher + (size_t)src * kDim * kDim;
      int st = F.status;
      if (__ldcg(a.status + src) & kStatusBounds) st = 5;
      for (int j = 0; j < kDim * kDim; j++) outF[j] = st ? __longlong_as_double(0x7ff8000000000000ll) : Gm[j];
      if (a.cov) {
        double inv[kDim * kDim];
        int cs = st ? 1 : chol_invert(Gm, inv, kDim);
        double *outC = a.cov + (size_t)src * kDim * kDim;
        for (int j = 0; j < kDim * kDim; j++) outC[j] = cs ? __longlong_as_double(0x7ff8000000000000ll) : inv[j];
        if (!st && cs) st = 9;  // inversion failed
      }
      if (!st && F.needs_ref) st = kStatusRedo;
      a.status[src] = st;
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------- plain form
// One parameter's central difference of the FP64 response (fisher.cpp:361-470).
struct FDReq {
  Request rp, rm, rpp, rmm;
};
__global__ void k_fisher_fd(const FDReq *__restrict__ fr, int order, int apply_shift, double div, double logscale,
                            const double *__restrict__ freqs, int N, double2 *__restrict__ deriv) {
  const FDReq &R = *fr;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < N; k += gridDim.x * blockDim.x) {
    double f = freqs[k];
    cd a, b, xp, xm;
    wave_bin(R.rp, f, a, b);
    xp = response_bin(R.rp.det[0], a, b, f, false);
    wave_bin(R.rm, f, a, b);
    xm = response_bin(R.rm.det[0], a, b, f, false);
    if (apply_shift) {  // exp(i (-2 pi DTOA) f) with DTOA from the perturbed sky position (:403-409)
      double s, c;
      sincos(R.rp.det[1].tau * f, &s, &c);
      xp = cmul(xp, cd{c, s});
      sincos(R.rm.det[1].tau * f, &s, &c);
      xm = cmul(xm, cd{c, s});
    }
    cd d;
    if (order >= 4) {  // five-point rule; the +-2 eps responses are time shifted, not phase shifted (:426-458)
      cd xpp, xmm;
      wave_bin(R.rpp, f, a, b);
      xpp = response_bin(R.rpp.det[0], a, b, f, false);
      wave_bin(R.rmm, f, a, b);
      xmm = response_bin(R.rmm.det[0], a, b, f, false);
      d.re = (-xpp.re + 8. * xp.re - 8. * xm.re + xmm.re) / div;
      d.im = (-xpp.im + 8. * xp.im - 8. * xm.im + xmm.im) / div;
    } else {
      d.re = (xp.re - xm.re) / div;
      d.im = (xp.im - xm.im) / div;
    }
    deriv[k] = make_double2(d.re * logscale, d.im * logscale);
  }
}

// Gram matrix 4 Simpson(Re(d_j d_k*)/S) (fisher.cpp:2704-2781), one block per (j, k).
__global__ void k_fisher_gram(const double2 *__restrict__ deriv, int dim, int N, const double *__restrict__ psd,
                              double df, double *out) {
  int j = blockIdx.x, k = blockIdx.y;
  if (k > j) return;
  const double2 *a = deriv + (size_t)j * N, *b = deriv + (size_t)k * N;
  double s = 0;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    double w = simpson_weight(i, N);
    double2 x = a[i], y = b[i];
    s += w * ((x.x * y.x + x.y * y.y) / psd[i]);
  }
  __shared__ double sm[32];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sm[w];
    double v = 4 * (t * df / 3);
    out[j * dim + k] = v;
    out[k * dim + j] = v;
  }
}

int det_index(const char *n) {
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

}  // namespace gwf

using namespace gwf;

extern "C" {

int gwgpu_fisher_numerical(gwgpu_context *c, const double *freqs, int N, const char *method, const char *detector,
                           const char *reference_detector, double *output, int dim, const gwgpu_gen_params *params,
                           int order, const double *noise) {
  if (!c || !freqs || N < 2 || !method || !output || !params || !noise) return GWGPU_EINVAL;
  std::string m(method);
  int meth = (m == "IMRPhenomD") ? 0 : (m == "MCMC_IMRPhenomD" ? 1 : -1);
  if (meth < 0 || dim != kDim || (order != 2 && order != 4)) return GWGPU_EINVAL;
  int det = det_index(detector), ref = det_index(reference_detector);
  if (det < 0 || ref < 0) return GWGPU_EINVAL;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  GenParams in;
  std::memcpy(&in, params, sizeof(in));
  double v[kDim];
  int logf[kDim];
  fisher_unpack(in, meth, v, logf);
  const double epsilon = 1e-8;  // fisher.cpp:158
  size_t need = sizeof(double) * (size_t)N * (2 + 2 * (size_t)dim) + sizeof(double) * N + sizeof(FDReq) +
                sizeof(double) * dim * dim + 256;
  void *dev;
  int st = c->workspace(gwgpu_context::kWsFisher, need, &dev);
  if (st) return st;
  char *p = (char *)dev;
  double *df = (double *)p;
  p += sizeof(double) * N;
  double *dpsd = (double *)p;
  p += sizeof(double) * N;
  double2 *deriv = (double2 *)p;
  p += sizeof(double2) * (size_t)N * dim;
  double *dout = (double *)p;
  p += sizeof(double) * dim * dim;
  p = (char *)(((uintptr_t)p + 255) & ~(uintptr_t)255);
  FDReq *dreq = (FDReq *)p;
  cudaMemcpyAsync(df, freqs, sizeof(double) * N, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(dpsd, noise, sizeof(double) * N, cudaMemcpyHostToDevice, c->stream);
  FDReq *h;
  st = c->pinned(gwgpu_context::kHwsFisher, sizeof(FDReq) * dim, (void **)&h);
  if (st) return st;
  for (int i = 0; i < dim; i++) {
    double eps = epsilon, pv[kDim];
    GenParams q;
    double div = fisher_perturb(v, i, 1, eps, pv);
    fisher_repack(pv, in, meth, q);
    // det[0]: this detector's F+/Fx; det[1].tau: -2 pi DTOA(ref -> det) when ref != det
    int dd[2] = {det, ref};
    request_prologue(h[i].rp, q, kPhenomD, dd, 1, c->qnm_host.data());
    h[i].rp.det[1].tau = -2 * kPi * dtoa(q.RA, q.DEC, q.gmst, ref, det);
    fisher_perturb(v, i, -1, eps, pv);
    fisher_repack(pv, in, meth, q);
    request_prologue(h[i].rm, q, kPhenomD, dd, 1, c->qnm_host.data());
    h[i].rm.det[1].tau = -2 * kPi * dtoa(q.RA, q.DEC, q.gmst, ref, det);
    double d4 = div == eps ? 6. * eps : 12. * eps;
    if (order >= 4) {
      double pp[kDim];
      for (int j = 0; j < kDim; j++) pp[j] = v[j];
      bool onesided = (i == 8 && v[i] > .25 - eps);
      pp[i] = onesided ? v[i] : v[i] + 2 * eps;
      fisher_repack(pp, in, meth, q);
      if (ref != det) q.tc -= dtoa(q.RA, q.DEC, q.gmst, ref, det);
      request_prologue(h[i].rpp, q, kPhenomD, dd, 1, c->qnm_host.data());
      pp[i] = v[i] - 2 * eps;
      fisher_repack(pp, in, meth, q);
      if (ref != det) q.tc -= dtoa(q.RA, q.DEC, q.gmst, ref, det);
      request_prologue(h[i].rmm, q, kPhenomD, dd, 1, c->qnm_host.data());
    }
    double divisor = order >= 4 ? d4 : div;
    double logscale = logf[i] ? v[i] : 1.0;
    cudaMemcpyAsync(dreq, &h[i], sizeof(FDReq), cudaMemcpyHostToDevice, c->stream);
    int grid = (N + 127) / 128;
    k_fisher_fd<<<grid, 128, 0, c->stream>>>(dreq, order, ref != det, divisor, logscale, df, N, deriv + (size_t)i * N);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return c->fail(e, "fisher fd launch");
    e = cudaStreamSynchronize(c->stream);  // dreq is reused for the next parameter
    if (e != cudaSuccess) return c->fail(e, "fisher fd");
  }
  k_fisher_gram<<<dim3(dim, dim), 256, 0, c->stream>>>(deriv, dim, N, dpsd, freqs[1] - freqs[0], dout);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return c->fail(e, "fisher gram launch");
  cudaMemcpyAsync(output, dout, sizeof(double) * dim * dim, cudaMemcpyDeviceToHost, c->stream);
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return c->fail(e, "fisher");
  return GWGPU_OK;
}

}  // extern "C"

// The moment form for n sources; acc64 selects FP64 per-bin values and sums.
int gwf_moment_run(gwgpu_context *c, const gwgpu_gen_params *params, int n, int method, int order, const int *handles,
                   int ndet, double epsilon, int step_mode, double *fisher, double *covariance, int *status,
                   bool acc64) {
  if (!c || !params || n < 1 || !handles || ndet < 1 || ndet > kMaxDet || !fisher || (method != 0 && method != 1) ||
      (order != 2 && order != 4))
    return GWGPU_EINVAL;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  const gwgpu_context::Stream *s0 = c->get_stream(handles[0]);
  if (!s0) return GWGPU_ENOTFOUND;
  if (!s0->dev.uniform_int || s0->dev.iw) {
    c->last_error = "fisher_batch needs Simpson streams on a uniform grid with f0 a multiple of df";
    return GWGPU_EINVAL;
  }
  FisherArgs a;
  std::memset(&a, 0, sizeof(a));
  int dets[kMaxDet];
  std::vector<int> wslot(ndet);
  int nw = 0;
  std::vector<const gwgpu_context::Stream *> ws;
  for (int d = 0; d < ndet; d++) {
    const gwgpu_context::Stream *s = c->get_stream(handles[d]);
    if (!s) return GWGPU_ENOTFOUND;
    if (s->dev.N != s0->dev.N || s->dev.n0 != s0->dev.n0 || s->dev.iw) return GWGPU_EINVAL;
    dets[d] = s->dev.det;
    int found = -1;
    for (int w = 0; w < nw; w++) {  // same PSD and grid -> same weight stream
      if (ws[w]->dev.wscale == s->dev.wscale && ws[w]->psd_hash == s->psd_hash) {
        found = w;
        break;
      }
    }
    if (found < 0) {
      found = nw++;
      ws.push_back(s);
    }
    wslot[d] = found;
  }
  // the FP64 n^(-7/6) table
  int st = c->ensure_tm76d(s0->dev.n0 + s0->dev.N);
  if (st) return st;
  const int N = s0->dev.N, tile = 4096, ntiles = (N + tile - 1) / tile;
  const double df = s0->dev.df;
  // chunk sources to bound the scratch
  const int chunk = std::min(n, 2048);
  size_t bytes = sizeof(GenParams) * chunk + sizeof(SlotOut) * (size_t)chunk * kSlots + sizeof(FisherSrc) * chunk +
                 sizeof(double) * (size_t)chunk * ntiles * kMaxDet * kSums + sizeof(double) * (size_t)chunk * 2 * kDim * kDim +
                 sizeof(int) * (chunk + 8) + sizeof(unsigned) * (chunk + 8) + 1024;
  void *dev;
  st = c->workspace(gwgpu_context::kWsFisher + 10, bytes, &dev);
  if (st) return st;
  auto align = [](char *p) { return (char *)(((uintptr_t)p + 255) & ~(uintptr_t)255); };
  char *p = (char *)dev;
  GenParams *dparams = (GenParams *)p;
  p = align(p + sizeof(GenParams) * chunk);
  SlotOut *slots = (SlotOut *)p;
  p = align(p + sizeof(SlotOut) * (size_t)chunk * kSlots);
  FisherSrc *srcs = (FisherSrc *)p;
  p = align(p + sizeof(FisherSrc) * chunk);
  double *partials = (double *)p;
  p = align(p + sizeof(double) * (size_t)chunk * ntiles * kMaxDet * kSums);
  double *dfish = (double *)p;
  p = align(p + sizeof(double) * (size_t)chunk * kDim * kDim);
  double *dcov = (double *)p;
  p = align(p + sizeof(double) * (size_t)chunk * kDim * kDim);
  int *dstat = (int *)p;
  p = align(p + sizeof(int) * (chunk + 8));
  unsigned *cnt = (unsigned *)p;
  int *dwslot, *ddets;
  void *small;
  st = c->workspace(gwgpu_context::kWsFisher + 11, 256, &small);
  if (st) return st;
  dwslot = (int *)small;
  ddets = dwslot + kMaxDet;
  cudaMemcpyAsync(dwslot, wslot.data(), sizeof(int) * ndet, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(ddets, dets, sizeof(int) * ndet, cudaMemcpyHostToDevice, c->stream);
  a.ndet = ndet;
  a.nw = nw;
  a.wslot = dwslot;
  for (int w = 0; w < nw; w++) {
    a.what[w] = ws[w]->dev.what;
    a.wscale[w] = ws[w]->dev.wscale;
    a.ipsd[w] = ws[w]->dev.ipsd;
    a.iw[w] = ws[w]->dev.iw;
    a.c3[w] = 4. * ws[w]->dev.simpson_df / 3.;
  }
  a.n0 = s0->dev.n0;
  a.N = N;
  a.tile = tile;
  a.ntiles = ntiles;
  a.df = df;
  a.df_f = (float)df;
  a.fisher_df_ratio = (s0->host_freqs[1] - s0->host_freqs[0]) / s0->dev.simpson_df;
  a.tab = c->tables;
  a.tm76d = c->tm76d;
  a.tm76d_n = c->tm76d_n;
  static int grid_cache = 0;
  if (!grid_cache) {
    cudaDeviceProp pr;
    cudaGetDeviceProperties(&pr, c->device);
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_fisher_main<1, false>, kBlock, 0);
    grid_cache = pr.multiProcessorCount * std::max(per, 1);
  }
  for (int s0i = 0; s0i < n; s0i += chunk) {
    int m = std::min(chunk, n - s0i);
    cudaMemcpyAsync(dparams, params + s0i, sizeof(GenParams) * m, cudaMemcpyHostToDevice, c->stream);
    cudaMemsetAsync(cnt, 0, sizeof(unsigned) * (m + 8), c->stream);
    int tot = m * kSlots;
    k_fisher_slots<<<(tot + 63) / 64, 64, 0, c->stream>>>(dparams, m, method, ddets, ndet, df, epsilon, step_mode,
                                                          c->qnm_dev, slots);
    k_fisher_setup<<<(m + 63) / 64, 64, 0, c->stream>>>(dparams, m, method, ndet, epsilon, step_mode, order, slots,
                                                        srcs, dstat);
    a.src = srcs;
    a.nsrc = m;
    a.item_counter = cnt + m;
    a.src_done = cnt;
    a.partials = partials;
    a.fisher = dfish;
    a.cov = covariance ? dcov : nullptr;
    a.status = dstat;
    int grid = std::min(m * ntiles, grid_cache);
    switch (nw) {
      case 1:
        if (acc64) k_fisher_main<1, true><<<grid, kBlock, 0, c->stream>>>(a);
        else k_fisher_main<1, false><<<grid, kBlock, 0, c->stream>>>(a);
        break;
      case 2:
        if (acc64) k_fisher_main<2, true><<<grid, kBlock, 0, c->stream>>>(a);
        else k_fisher_main<2, false><<<grid, kBlock, 0, c->stream>>>(a);
        break;
      case 3:
        if (acc64) k_fisher_main<3, true><<<grid, kBlock, 0, c->stream>>>(a);
        else k_fisher_main<3, false><<<grid, kBlock, 0, c->stream>>>(a);
        break;
      default:
        if (acc64) k_fisher_main<4, true><<<grid, kBlock, 0, c->stream>>>(a);
        else k_fisher_main<4, false><<<grid, kBlock, 0, c->stream>>>(a);
        break;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return c->fail(e, "fisher batch launch");
    cudaMemcpyAsync(fisher + (size_t)s0i * kDim * kDim, dfish, sizeof(double) * m * kDim * kDim,
                    cudaMemcpyDeviceToHost, c->stream);
    if (covariance)
      cudaMemcpyAsync(covariance + (size_t)s0i * kDim * kDim, dcov, sizeof(double) * m * kDim * kDim,
                      cudaMemcpyDeviceToHost, c->stream);
    std::vector<int> hs(m);
    cudaMemcpyAsync(hs.data(), dstat, sizeof(int) * m, cudaMemcpyDeviceToHost, c->stream);
    e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return c->fail(e, "fisher batch");
    // Sources whose matrix the sums leave indefinite (a normalised smallest
    // eigenvalue below their precision: ~1e-8 for the FP32-compensated sums,
    // near-equal masses and face-on orientations) are recomputed by the FP64
    // reference algorithm.
    std::vector<int> redo;
    for (int i = 0; i < m; i++)
      if (hs[i] == 9 || hs[i] == kStatusRedo) redo.push_back(i);
    if (!redo.empty()) {
      std::vector<GenParams> rp(redo.size());
      for (size_t j = 0; j < redo.size(); j++) std::memcpy(&rp[j], params + s0i + redo[j], sizeof(GenParams));
      std::vector<double> rf(redo.size() * kDim * kDim), rc(redo.size() * kDim * kDim);
      std::vector<int> rs(redo.size());
      st = gwf_ref_run(c, rp.data(), (int)redo.size(), method, order, handles, ndet, epsilon, step_mode, 0, rf.data(),
                       covariance ? rc.data() : nullptr, rs.data());
      if (st) return st;
      for (size_t j = 0; j < redo.size(); j++) {
        const size_t o = (size_t)(s0i + redo[j]) * kDim * kDim;
        std::memcpy(fisher + o, &rf[j * kDim * kDim], sizeof(double) * kDim * kDim);
        if (covariance) std::memcpy(covariance + o, &rc[j * kDim * kDim], sizeof(double) * kDim * kDim);
        hs[redo[j]] = rs[j];
      }
    }
    if (status)
      for (int i = 0; i < m; i++) status[s0i + i] = hs[i] == 9 ? GWGPU_ESINGULAR : gwk::status_code(hs[i]);
  }
  return GWGPU_OK;
}

extern "C" int gwgpu_fisher_batch(gwgpu_context *c, const gwgpu_gen_params *params, int n, int method,
                                  const int *handles, int ndet, double epsilon, int step_mode, double *fisher,
                                  double *covariance, int *status) {
  return gwf_moment_run(c, params, n, method, 2, handles, ndet, epsilon, step_mode, fisher, covariance, status, true);
}
