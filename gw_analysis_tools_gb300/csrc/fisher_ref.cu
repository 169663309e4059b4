// fisher_ref.cu -- the reference's numerical Fisher algorithm for many sources
// on the device (fisher.cpp:81-146 -> calculate_derivatives :337-557 ->
// calculate_fisher_elements :2704-2781), summed over a detector network as
// MCMC_fisher_wrapper does (mcmc_gw.cpp:2230-2340, reference detector = the
// first detector), and the sampler's Fisher proposal built on it.
//
// Every perturbed detector response is the FP64 waveform of the perturbed
// parameters, as in the reference: for parameter i and step k the response
// r_k = (F+ h+ + Fx hx) times, for a detector other than the reference one,
// e^{-2 pi i DTOA f} at the steps +-eps (fisher.cpp:403-409) and the same
// arrival time taken into t_c at the steps +-2 eps of the five-point rule
// (fisher.cpp:426-458), which leaves an extra constant phase
// 2 pi DTOA f_ref on those two responses -- kept, since the reference's
// order-4 Fisher (the sampler's, mcmc_gw.h:45) carries it.  Derivatives
// (r+ - r-)/(2 eps) or (-r++ + 8 r+ - 8 r- + r--)/(12 eps) (one-sided at
// eta = 1/4), the log-factor chain rule (:548-553), and
// Gamma_ij = 4 Simpson(Re(d_i d_j*) / S_n) per detector (util.h:844-856), all in
// FP64.
//
// Work layout: a set-up kernel builds the model constants of every perturbed
// parameter set (one thread per source, parameter and step); the main kernel
// is persistent over (source, bin tile) items; each thread evaluates one bin's
// 2 or 4 perturbed waveforms per parameter, writes that bin's derivatives to
// shared memory, and then the block's first 66 threads each accumulate one
// Gram pair over the block's bins.  The last tile of a source sums the tiles'
// partials in a fixed order (the same result every run).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/gwgpu.h"
#include "capi_internal.h"
#include "fisher_math.h"
#include "fisher_ref.h"
#include "kernels.h"

namespace gwf {
using namespace gwt;

constexpr int kRefBlock = 128;
constexpr int kPairs = kDim * (kDim + 1) / 2;  // the lower triangle of Gamma

struct RefSrc {
  double scale[kDim];  // (log factor) / divisor of parameter i
  int status;
};

// Five-point / central weights of the step slots (+eps, -eps, +2eps, -2eps).
__constant__ double c_fd_w2[2] = {1.0, -1.0};
__constant__ double c_fd_w4[4] = {8.0, -8.0, -1.0, 1.0};

__global__ void k_fref_setup(const GenParams *__restrict__ params, int nsrc, int method, int order,
                             const int *__restrict__ dets, int ndet, double epsilon, int step_mode,
                             const double *__restrict__ qnm, Request *req, RefSrc *rs) {
  const int nk = order >= 4 ? 4 : 2;
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= nsrc * kDim * nk) return;
  const int src = g / (kDim * nk), rem = g % (kDim * nk), i = rem / nk, k = rem % nk;
  const GenParams in = params[src];
  double v[kDim], pv[kDim];
  int logf[kDim];
  fisher_unpack(in, method, v, logf);
  const double eps = fisher_step(v, i, epsilon, step_mode);
  const bool onesided = (i == 8 && v[i] > .25 - eps);  // fisher.cpp:376-379, 391-394
  for (int j = 0; j < kDim; j++) pv[j] = v[j];
  const double mult = k == 0 ? 1.0 : (k == 1 ? -1.0 : (k == 2 ? 2.0 : -2.0));
  pv[i] = (onesided && mult > 0) ? v[i] : v[i] + mult * eps;
  GenParams q;
  fisher_repack(pv, in, method, q);
  const int st = request_prologue(req[g], q, kPhenomD, dets, ndet, qnm);
  const bool bad = !(q.mass1 > 0) || !(q.mass2 > 0) || !(q.Luminosity_Distance > 0) || st != 0;
  if (bad) atomicOr(&rs[src].status, 4);
  if (k == 0) {
    const double div = order >= 4 ? (onesided ? 6. * eps : 12. * eps) : (onesided ? eps : 2. * eps);
    rs[src].scale[i] = (logf[i] ? v[i] : 1.0) / div;
  }
}

struct RefArgs {
  const Request *req;
  const RefSrc *rs;
  int nsrc, ndet, nk;
  const double *freqs;
  const double *psd[kMaxDet];
  int N, tile, ntiles;
  double df;  // f1 - f0: the Simpson step of calculate_fisher_elements
  unsigned *item_counter, *src_done;
  double *partials;  // items x kPairs
  double *fisher;    // nsrc x kDim x kDim
};

__global__ void __launch_bounds__(kRefBlock) k_fref_main(const RefArgs a) {
  extern __shared__ double smem[];
  double2 *der = (double2 *)smem;                      // [kDim][ndet][kRefBlock]
  double *wsm = smem + 2 * kDim * a.ndet * kRefBlock;  // [ndet][kRefBlock]: Simpson weight / S_n
  __shared__ int s_item, s_last;
  const int tid = threadIdx.x;
  int pi = 0, pj = 0;  // this thread's Gram pair (i >= j) when tid < kPairs
  if (tid < kPairs) {
    int t = tid;
    while (t > pi) {
      pi++;
      t -= pi;
    }
    pj = t;
  }
  const double *fdw = a.nk == 4 ? c_fd_w4 : c_fd_w2;
  const int nitems = a.nsrc * a.ntiles;
  for (;;) {
    if (tid == 0) s_item = (int)atomicAdd(a.item_counter, 1u);
    __syncthreads();
    const int it = s_item;
    if (it >= nitems) break;
    const int src = it / a.ntiles, tile = it % a.ntiles;
    const Request *R = a.req + (size_t)src * kDim * a.nk;
    const bool ok = a.rs[src].status == 0;
    const int k0 = tile * a.tile, k1 = min(k0 + a.tile, a.N);
    double acc = 0.0;
    for (int base = k0; base < k1; base += kRefBlock) {
      const int kb = base + tid;
      const bool live = ok && kb < k1;
      const double f = live ? a.freqs[kb] : 0.0;
      for (int d = 0; d < a.ndet; d++)
        wsm[d * kRefBlock + tid] = live ? simpson_weight(kb, a.N) / a.psd[d][kb] : 0.0;
      for (int i = 0; i < kDim; i++) {
        cd sum[kMaxDet];
        for (int d = 0; d < kMaxDet; d++) sum[d] = cd{0., 0.};
        if (live) {
          for (int s = 0; s < a.nk; s++) {
            const Request &r = R[i * a.nk + s];
            cd hp, hc;
            wave_bin(r, f, hp, hc);
            const double w = fdw[s];
            for (int d = 0; d < a.ndet; d++) {
              cd x = response_bin(r.det[d], hp, hc, f, false);
              const double tau = r.det[d].tau;
              if (tau != 0.0) {  // a detector other than the reference one
                double sn, cs;
                sincos(s < 2 ? tau * f : tau * (f - r.m.fref), &sn, &cs);
                x = cmul(x, cd{cs, sn});
              }
              sum[d].re += w * x.re;
              sum[d].im += w * x.im;
            }
          }
        }
        const double sc = a.rs[src].scale[i];
        for (int d = 0; d < a.ndet; d++)
          der[(i * a.ndet + d) * kRefBlock + tid] = make_double2(sum[d].re * sc, sum[d].im * sc);
      }
      __syncthreads();
      if (tid < kPairs) {
        const int nb = min(kRefBlock, k1 - base);
        for (int d = 0; d < a.ndet; d++) {
          const double2 *x = der + (pi * a.ndet + d) * kRefBlock, *y = der + (pj * a.ndet + d) * kRefBlock;
          const double *w = wsm + d * kRefBlock;
          for (int t = 0; t < nb; t++) acc += w[t] * (x[t].x * y[t].x + x[t].y * y[t].y);
        }
      }
      __syncthreads();
    }
    if (tid < kPairs) a.partials[(size_t)it * kPairs + tid] = acc;
    __threadfence();
    __syncthreads();
    if (tid == 0) s_last = (atomicAdd(a.src_done + src, 1u) == (unsigned)(a.ntiles - 1));
    __syncthreads();
    if (s_last) {
      __threadfence();
      if (tid < kPairs) {
        double s = 0.0;
        const volatile double *p = a.partials + (size_t)src * a.ntiles * kPairs + tid;
        for (int t = 0; t < a.ntiles; t++) s += p[(size_t)t * kPairs];
        const double g = 4 * (s * a.df / 3);
        a.fisher[(size_t)src * kDim * kDim + pi * kDim + pj] = g;
        a.fisher[(size_t)src * kDim * kDim + pj * kDim + pi] = g;
      }
    }
    __syncthreads();
  }
}

// MCMC_fisher_transformations (mcmc_gw.cpp:2136-2160), non-intrinsic
// IMRPhenomD: the prior widths added to the diagonal.
__constant__ double c_prior_diag[kDim] = {1. / (4 * kPi * kPi), 1. / 4, 1. / (4 * kPi * kPi), 1. / 4,
                                          1. / (4 * kPi * kPi), 1. / (.01), 0., 0., 1. / .25, 1. / 4, 1. / 4};

__global__ void k_fref_finish(int nsrc, const RefSrc *__restrict__ rs, int add_prior, double *fisher, double *cov,
                              int *status) {
  const int src = blockIdx.x * blockDim.x + threadIdx.x;
  if (src >= nsrc) return;
  double *F = fisher + (size_t)src * kDim * kDim;
  int st = rs[src].status;
  if (add_prior)
    for (int i = 0; i < kDim; i++) F[i * kDim + i] += c_prior_diag[i];
  if (st) {
    for (int j = 0; j < kDim * kDim; j++) F[j] = NAN;
  }
  if (cov) {
    double *C = cov + (size_t)src * kDim * kDim;
    if (st || chol_invert(F, C, kDim)) {
      for (int j = 0; j < kDim * kDim; j++) C[j] = NAN;
      if (!st) st = 9;
    }
  }
  status[src] = st;
}

}  // namespace gwf

using namespace gwf;

// The reference algorithm for n sources whose parameters are on the host.
// Writes fisher/cov (host, n x 11 x 11) and the kernel status per source
// (0, 4 outside the model domain, 9 not invertible).
int gwf_ref_run(gwgpu_context *c, const GenParams *params, int n, int method, int order, const int *handles,
                int ndet, double epsilon, int step_mode, int add_prior, double *fisher, double *cov, int *kstatus) {
  if (order != 2 && order != 4) {
    c->last_error = "fisher: order must be 2 or 4";
    return GWGPU_EINVAL;
  }
  const gwgpu_context::Stream *s0 = c->get_stream(handles[0]);
  if (!s0) return GWGPU_ENOTFOUND;
  RefArgs a;
  std::memset(&a, 0, sizeof(a));
  int dets[kMaxDet];
  for (int d = 0; d < ndet; d++) {
    const gwgpu_context::Stream *s = c->get_stream(handles[d]);
    if (!s) return GWGPU_ENOTFOUND;
    if (s->dev.N != s0->dev.N || s->dev.iw || s->host_freqs != s0->host_freqs) {
      c->last_error = "fisher: the detectors need Simpson streams on one grid";
      return GWGPU_EINVAL;
    }
    dets[d] = s->dev.det;
    a.psd[d] = s->dev.psd;
  }
  const int nk = order >= 4 ? 4 : 2;
  const int N = s0->dev.N, tile = 2048, ntiles = (N + tile - 1) / tile;
  const int chunk = std::min(n, 1024);
  auto align = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const size_t b_par = align(sizeof(GenParams) * chunk), b_req = align(sizeof(Request) * (size_t)chunk * kDim * nk),
               b_rs = align(sizeof(RefSrc) * chunk), b_part = align(sizeof(double) * (size_t)chunk * ntiles * kPairs),
               b_f = align(sizeof(double) * (size_t)chunk * kDim * kDim), b_st = align(sizeof(int) * chunk),
               b_cnt = align(sizeof(unsigned) * (chunk + 8)), b_dets = align(sizeof(int) * kMaxDet);
  void *dev;
  int st = c->workspace(gwgpu_context::kWsFisherRef, b_par + b_req + b_rs + b_part + 2 * b_f + b_st + b_cnt + b_dets,
                        &dev);
  if (st) return st;
  char *p = (char *)dev;
  GenParams *dparams = (GenParams *)p;
  p += b_par;
  Request *dreq = (Request *)p;
  p += b_req;
  RefSrc *drs = (RefSrc *)p;
  p += b_rs;
  double *dpart = (double *)p;
  p += b_part;
  double *dfish = (double *)p;
  p += b_f;
  double *dcov = (double *)p;
  p += b_f;
  int *dstat = (int *)p;
  p += b_st;
  unsigned *dcnt = (unsigned *)p;
  p += b_cnt;
  int *ddets = (int *)p;
  cudaMemcpyAsync(ddets, dets, sizeof(int) * ndet, cudaMemcpyHostToDevice, c->stream);
  a.req = dreq;
  a.rs = drs;
  a.ndet = ndet;
  a.nk = nk;
  a.freqs = s0->dev.freqs;
  a.N = N;
  a.tile = tile;
  a.ntiles = ntiles;
  a.df = s0->host_freqs[1] - s0->host_freqs[0];
  a.partials = dpart;
  a.fisher = dfish;
  const size_t smem = sizeof(double) * (size_t)(2 * kDim + 1) * ndet * kRefBlock;
  static int attr_set = 0, per_sm = 0, nsm = 0;
  if (!attr_set) {
    cudaFuncSetAttribute(k_fref_main, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(sizeof(double) * (2 * kDim + 1) * kMaxDet * kRefBlock));
    cudaDeviceProp pr;
    cudaGetDeviceProperties(&pr, c->device);
    nsm = pr.multiProcessorCount;
    attr_set = 1;
  }
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fref_main, kRefBlock, smem);
  for (int s0i = 0; s0i < n; s0i += chunk) {
    const int m = std::min(chunk, n - s0i);
    cudaMemcpyAsync(dparams, params + s0i, sizeof(GenParams) * m, cudaMemcpyHostToDevice, c->stream);
    cudaMemsetAsync(drs, 0, sizeof(RefSrc) * m, c->stream);
    cudaMemsetAsync(dcnt, 0, sizeof(unsigned) * (m + 8), c->stream);
    const int tot = m * kDim * nk;
    k_fref_setup<<<(tot + 63) / 64, 64, 0, c->stream>>>(dparams, m, method, order, ddets, ndet, epsilon, step_mode,
                                                        c->qnm_dev, dreq, drs);
    a.nsrc = m;
    a.src_done = dcnt;
    a.item_counter = dcnt + m;
    const int grid = std::min(m * ntiles, nsm * std::max(per_sm, 1));
    k_fref_main<<<grid, kRefBlock, smem, c->stream>>>(a);
    k_fref_finish<<<(m + 63) / 64, 64, 0, c->stream>>>(m, drs, add_prior, dfish, cov ? dcov : nullptr, dstat);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return c->fail(e, "fisher (reference algorithm) launch");
    cudaMemcpyAsync(fisher + (size_t)s0i * kDim * kDim, dfish, sizeof(double) * m * kDim * kDim,
                    cudaMemcpyDeviceToHost, c->stream);
    if (cov)
      cudaMemcpyAsync(cov + (size_t)s0i * kDim * kDim, dcov, sizeof(double) * m * kDim * kDim, cudaMemcpyDeviceToHost,
                      c->stream);
    cudaMemcpyAsync(kstatus + s0i, dstat, sizeof(int) * m, cudaMemcpyDeviceToHost, c->stream);
    e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return c->fail(e, "fisher (reference algorithm)");
  }
  return GWGPU_OK;
}

static int fisher_status_code(int k) {
  if (k == 0) return GWGPU_OK;
  if (k == 9) return GWGPU_ESINGULAR;
  return gwk::status_code(k);
}

extern "C" {

int gwgpu_fisher_batch_ex(gwgpu_context *c, const gwgpu_gen_params *params, int n, const int *handles, int ndet,
                          const gwgpu_fisher_options *opt, double *fisher, double *covariance, int *status) {
  if (!c || !params || n < 1 || !handles || ndet < 1 || ndet > kMaxDet || !fisher || !opt) return GWGPU_EINVAL;
  if (opt->method != GWGPU_FISHER_IMRPHENOMD && opt->method != GWGPU_FISHER_MCMC_IMRPHENOMD) return GWGPU_EINVAL;
  if (opt->order != 2 && opt->order != 4) return GWGPU_EINVAL;
  if (opt->precision != GWGPU_PREC_FP64 && opt->precision != GWGPU_PREC_MIXED) return GWGPU_EINVAL;
  if (opt->algorithm == GWGPU_FISHER_MOMENTS) {
    int st = gwf_moment_run(c, params, n, opt->method, opt->order, handles, ndet, opt->epsilon, opt->step_mode, fisher,
                            covariance, status, opt->precision == GWGPU_PREC_FP64);
    if (st || !opt->add_prior) return st;
    double prior[kDim];
    cudaMemcpyFromSymbol(prior, c_prior_diag, sizeof(prior));
    for (int i = 0; i < n; i++) {  // the prior diagonal, then the inverse again
      double *F = fisher + (size_t)i * kDim * kDim;
      for (int k = 0; k < kDim; k++) F[k * kDim + k] += prior[k];
      if (covariance) {
        double *C = covariance + (size_t)i * kDim * kDim;
        const bool bad = status && status[i] == GWGPU_EDOMAIN;
        if (bad || chol_invert(F, C, kDim)) {
          for (int k = 0; k < kDim * kDim; k++) C[k] = NAN;
          if (status && !bad) status[i] = GWGPU_ESINGULAR;
        } else if (status && status[i] == GWGPU_ESINGULAR) {
          status[i] = GWGPU_OK;
        }
      }
    }
    return GWGPU_OK;
  }
  if (opt->algorithm != GWGPU_FISHER_REFERENCE || opt->precision != GWGPU_PREC_FP64) return GWGPU_EINVAL;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  std::vector<int> ks(n);
  std::vector<GenParams> hp(n);
  std::memcpy(hp.data(), params, sizeof(GenParams) * n);
  int st = gwf_ref_run(c, hp.data(), n, opt->method, opt->order, handles, ndet, opt->epsilon, opt->step_mode,
                       opt->add_prior, fisher, covariance, ks.data());
  if (st) return st;
  if (status)
    for (int i = 0; i < n; i++) status[i] = fisher_status_code(ks[i]);
  return GWGPU_OK;
}

int gwgpu_mcmc_fisher_batch(gwgpu_context *c, const double *theta, int dim, int n, int approximant, double gmst,
                            const int *handles, int ndet, double *fisher, int *status) {
  if (!c || !theta || n < 1 || !handles || ndet < 1 || ndet > kMaxDet || !fisher) return GWGPU_EINVAL;
  if (approximant != GWGPU_IMRPHENOMD || dim != kDim) {
    c->last_error = "mcmc_fisher_batch: the 11-dimensional IMRPhenomD parameterisation";
    return GWGPU_EINVAL;
  }
  std::vector<GenParams> hp(n);
  for (int i = 0; i < n; i++) mcmc_repack(theta + (size_t)i * dim, dim, kPhenomD, gmst, hp[i]);
  // MCMC_fisher_wrapper: fisher_numerical("MCMC_" + method, order mcmc_deriv_order = 4,
  // epsilon 1e-8 absolute) summed over the detectors, plus the prior diagonal.
  // The moment form with FP64 sums at order 4 (the reference algorithm for the
  // sources it leaves to it)
  std::vector<int> ks(n);
  static_assert(sizeof(GenParams) == sizeof(gwgpu_gen_params), "one parameter layout");
  int st = gwf_moment_run(c, (const gwgpu_gen_params *)hp.data(), n, GWGPU_FISHER_MCMC_IMRPHENOMD, 4, handles, ndet,
                          1e-8, GWGPU_FISHER_STEP_ABSOLUTE, fisher, nullptr, ks.data(), true);
  if (st) return st;
  double prior[kDim];
  {
    std::lock_guard<std::mutex> lk(c->mu);
    cudaSetDevice(c->device);
    cudaError_t e = cudaMemcpyFromSymbol(prior, c_prior_diag, sizeof(prior));
    if (e != cudaSuccess) return c->fail(e, "prior diagonal");
  }
  for (int i = 0; i < n; i++)
    for (int k = 0; k < kDim; k++) fisher[(size_t)i * kDim * kDim + k * kDim + k] += prior[k];
  if (status)
    for (int i = 0; i < n; i++) status[i] = ks[i];
  return GWGPU_OK;
}

}  // extern "C"
