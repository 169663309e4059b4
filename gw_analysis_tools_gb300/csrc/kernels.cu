// kernels.cu -- sm_103a kernels of the likelihood path.
//
//   k_waveform / k_response   fourier_waveform / fourier_detector_response arrays (FP64)
//   k_inner                   Log_Likelihood_internal on given arrays (FP64 Simpson)
//   k_plain                   the drop-in: one request per launch, FP64, fused
//                             waveform -> projection -> Simpson inner product
//   k_prologue                batched per-request FP64 prologue, one thread per request
//   k_batch<fp64|mixed>       persistent fused bin kernel over (request, bin tile) items
//
// Reductions are deterministic: per-block partial sums are written to a
// scratch array and the last block to finish (per request) adds them in a
// fixed order in FP64.
#include <cstdint>
#include <cstdio>

#include "kernels.h"

namespace gwk {
using namespace gwt;

struct PlainStreams {
  StreamDev s[kMaxDet];
};

__device__ __forceinline__ double2 to_d2(cd a) { return make_double2(a.re, a.im); }

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide FP64 sums of NV values per thread; result valid in thread 0.
// smem must hold 32 * NV doubles.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double *smem) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int j = 0; j < NV; j++) v[j] = warp_sum(v[j]);
  if (lane == 0)
#pragma unroll
    for (int j = 0; j < NV; j++) smem[warp * NV + j] = v[j];
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int j = 0; j < NV; j++) {
      double x = (lane < nw) ? smem[lane * NV + j] : 0.0;
      v[j] = warp_sum(x);
    }
  }
  __syncthreads();
}

// ------------------------------------------------------------- waveform
__global__ void k_waveform(const __grid_constant__ Request r, const double *__restrict__ freqs, int N,
                           double2 *__restrict__ hp, double2 *__restrict__ hc) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < N; k += gridDim.x * blockDim.x) {
    cd a, b;
    wave_bin(r, freqs[k], a, b);
    hp[k] = to_d2(a);
    hc[k] = to_d2(b);
  }
}
__global__ void k_response(const __grid_constant__ Request r, int slot, int apply_shift,
                           const double *__restrict__ freqs, int N, double2 *__restrict__ out) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < N; k += gridDim.x * blockDim.x) {
    cd a, b;
    double f = freqs[k];
    wave_bin(r, f, a, b);
    out[k] = to_d2(response_bin(r.det[slot], a, b, f, apply_shift != 0));
  }
}

cudaError_t launch_waveform(const Request &r, const double *freqs, int N, double *hp, double *hc, cudaStream_t s) {
  int block = 128, grid = (N + block - 1) / block;
  k_waveform<<<grid, block, 0, s>>>(r, freqs, N, (double2 *)hp, (double2 *)hc);
  return cudaGetLastError();
}
cudaError_t launch_response(const Request &r, int slot, int apply_shift, const double *freqs, int N, double *out,
                            cudaStream_t s) {
  int block = 128, grid = (N + block - 1) / block;
  k_response<<<grid, block, 0, s>>>(r, slot, apply_shift, freqs, N, (double2 *)out);
  return cudaGetLastError();
}

// ------------------------------------------------ last-block finalisation
// Returns true in every thread of the block that finished last.
__device__ __forceinline__ bool arrive_last(unsigned *counter, unsigned expected) {
  __shared__ bool s_last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    unsigned prev = atomicAdd(counter, 1u);
    s_last = (prev == expected - 1);
  }
  __syncthreads();
  if (s_last) __threadfence();
  return s_last;
}

// ------------------------------------------------------ Simpson inner product
// iw: GAUSSLEG integration weights (null: Simpson's rule).
__global__ void k_inner(const double2 *__restrict__ data, const double *__restrict__ psd,
                        const double2 *__restrict__ resp, const double *__restrict__ iw, int N, double simpson_df,
                        double *partials, unsigned *counter, double *out) {
  __shared__ double smem[32 * 2];
  double v[2] = {0.0, 0.0};
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < N; k += gridDim.x * blockDim.x) {
    double w = iw ? iw[k] : simpson_weight(k, N);
    double2 r = resp[k], d = data[k];
    double S = psd[k];
    v[0] += w * ((r.x * r.x + r.y * r.y) / S);
    v[1] += w * ((d.x * r.x + d.y * r.y) / S);
  }
  block_sum<2>(v, smem);
  if (threadIdx.x == 0) {
    partials[blockIdx.x * 2 + 0] = v[0];
    partials[blockIdx.x * 2 + 1] = v[1];
  }
  if (arrive_last(counter, gridDim.x)) {
    double t[2] = {0.0, 0.0};  // the blocks' partials, strided over the block, then reduced
    for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
      t[0] += __ldcg(&partials[b * 2 + 0]);
      t[1] += __ldcg(&partials[b * 2 + 1]);
    }
    block_sum<2>(t, smem);
    if (threadIdx.x == 0) {
      double c = iw ? 1.0 : 4. * simpson_df / 3.;
      out[0] = -0.5 * (c * t[0] - 2 * c * t[1]);
      *counter = 0;
    }
  }
}
cudaError_t launch_inner_product(const double *data, const double *psd, const double *resp, int N, double simpson_df,
                                 double *partials, unsigned *counter, double *out, cudaStream_t s) {
  int block = 256, grid = (N + block - 1) / block;
  if (grid > 1024) grid = 1024;
  k_inner<<<grid, block, 0, s>>>((const double2 *)data, psd, (const double2 *)resp, nullptr, N, simpson_df, partials,
                                 counter, out);
  return cudaGetLastError();
}
cudaError_t launch_inner_product_weighted(const double *data, const double *psd, const double *resp, const double *iw,
                                          int N, double *partials, unsigned *counter, double *out, cudaStream_t s) {
  int block = 256, grid = (N + block - 1) / block;
  if (grid > 1024) grid = 1024;
  k_inner<<<grid, block, 0, s>>>((const double2 *)data, psd, (const double2 *)resp, iw, N, 0.0, partials, counter,
                                 out);
  return cudaGetLastError();
}

// --------------------------------------------------------------- FP64 bins
// Accumulate one bin of the reference arithmetic into v[2*d] (HH) and
// v[2*d+1] (DH), Simpson-weighted (mcmc_gw.cpp:801-873).
template <int NDET>
__device__ __forceinline__ void fp64_bin(const Request &r, const StreamDev *st, int k, int N, double (&v)[2 * NDET]) {
  const double f = st[0].freqs[k];
  cd hp, hc;
  wave_bin(r, f, hp, hc);
  const double ws = simpson_weight(k, N);
#pragma unroll
  for (int d = 0; d < NDET; d++) {
    cd x = response_bin(r.det[d], hp, hc, f, r.det[d].tau != 0.0);
    double2 dd = ((const double2 *)st[d].data)[k];
    const double iS = st[d].ipsd ? st[d].ipsd[k] : 1.0 / st[d].psd[k];
    const double w = st[d].iw ? st[d].iw[k] : ws;
    v[2 * d] += w * ((x.re * x.re + x.im * x.im) * iS);
    v[2 * d + 1] += w * ((dd.x * x.re + dd.y * x.im) * iS);
  }
}
// The same with each detector's arrival-time rotation e^{i tau_d f} given
// (rc, rs): the batched kernel builds it on uniform grids as the product of a
// per-pass and a per-thread factor instead of one sincos per detector-bin.
template <int NDET>
__device__ __forceinline__ void fp64_acc_rot(const Request &r, const StreamDev *st, int k, int N, cd hp, cd hc,
                                             const double *rc, const double *rs, double (&v)[2 * NDET]) {
  const double ws = simpson_weight(k, N);
#pragma unroll
  for (int d = 0; d < NDET; d++) {
    const cd y = response_bin(r.det[d], hp, hc, 0.0, false);  // the frequency enters through (rc, rs)
    const cd x{y.re * rc[d] - y.im * rs[d], y.re * rs[d] + y.im * rc[d]};
    double2 dd = ((const double2 *)st[d].data)[k];
    const double iS = st[d].ipsd ? st[d].ipsd[k] : 1.0 / st[d].psd[k];
    const double w = st[d].iw ? st[d].iw[k] : ws;
    v[2 * d] += w * ((x.re * x.re + x.im * x.im) * iS);
    v[2 * d + 1] += w * ((dd.x * x.re + dd.y * x.im) * iS);
  }
}
template <int NDET>
__device__ __forceinline__ void fp64_bin_rot(const Request &r, const StreamDev *st, int k, int N, const double *rc,
                                             const double *rs, double (&v)[2 * NDET]) {
  cd hp, hc;
  wave_bin(r, st[0].freqs[k], hp, hc);
  fp64_acc_rot<NDET>(r, st, k, N, hp, hc, rc, rs, v);
}
// IMRPhenomD at bin n = n0 + k of a uniform grid from the coefficients and
// tables of PlainTab (d_bin's values to ~1e-12 relative).
__device__ __forceinline__ void d_bin_tab(const Request &r, const gwt::WaveF64 &x, const gwt::Tables &tb,
                                          const double *tm76d, int n, double f, cd &hp, cd &hc) {
  if (n > x.n_cut) {
    hp = cd{0., 0.};
    hc = cd{0., 0.};
    return;
  }
  const double t = __ldg(tb.t13 + n), rr = __ldg(tb.tm53 + n), lnn = __ldg(tb.tln + n), t34 = __ldg(tb.t34 + n),
               m76 = __ldg(tm76d + n);
  const double amp = x.A_scale * wave64_amp(x, n, t, m76);
  const double phase = wave64_phase(x, n, t, rr, lnn, t34) - (x.tcl * (f - x.fref) + x.phic);
  double sn, cs;
  sincos(phase, &sn, &cs);
  const cd h{amp * cs, -(amp * sn)};
  const double ci = r.m.s.cos_incl, fac = r.m.s.fac_incl;
  hc = cd{h.im * ci, -h.re * ci};
  hp = cd{h.re * fac, h.im * fac};
}
template <int NDET>
__device__ __forceinline__ double fp64_finalize(const double *s, const StreamDev *st) {
  double ll = 0;
#pragma unroll
  for (int d = 0; d < NDET; d++) {
    double c = st[d].iw ? 1.0 : 4. * st[d].simpson_df / 3.;
    ll += -0.5 * (c * s[2 * d] - 2 * c * s[2 * d + 1]);
  }
  return ll;
}

// ------------------------------------------------------------------ plain
// On uniform grids each block's arrival-time rotations come from a table:
// thread t = 16 a + b of a block starting at bin k0 takes
// e^{i tau (f_k0 + t df)} = e^{i tau f_k0} e^{i tau 16 a df} e^{i tau b df},
// 25 sincos per detector and block (one per thread for the first 25 NDET
// threads) instead of one per detector-bin.
constexpr int kPlainRot = 1 + 8 + 16;
template <int NDET>
__global__ void __launch_bounds__(128) k_plain(const __grid_constant__ Request r, const __grid_constant__ PlainStreams ps,
                                               const __grid_constant__ PlainTab pt, double *partials,
                                               unsigned *counter, double *out, int *status) {
  __shared__ double smem[32 * 2 * NDET];
  __shared__ double2 s_rot[NDET * kPlainRot];
  const int N = ps.s[0].N;
  double v[2 * NDET];
#pragma unroll
  for (int j = 0; j < 2 * NDET; j++) v[j] = 0.0;
  bool uniform = blockDim.x == 128 && (long long)gridDim.x * 128 >= N;  // one bin per thread
#pragma unroll
  for (int d = 0; d < NDET; d++) uniform = uniform && ps.s[d].uniform_int;
  if (uniform) {
    const int k0 = blockIdx.x * 128;
    for (int e = threadIdx.x; e < NDET * kPlainRot; e += blockDim.x) {
      const int d = e / kPlainRot, j = e - d * kPlainRot;
      const double tau = r.det[d].tau, df = ps.s[0].df;
      const double arg = j == 0 ? tau * ps.s[0].freqs[min(k0, N - 1)]
                                : tau * ((j <= 8 ? 16.0 * (j - 1) : (double)(j - 9)) * df);
      double sn, cs;
      sincos(arg, &sn, &cs);
      s_rot[e] = make_double2(cs, sn);
    }
    __syncthreads();
    const int k = k0 + threadIdx.x;
    if (k < N) {
      const int a = threadIdx.x >> 4, b = threadIdx.x & 15;
      double rc[NDET], rs[NDET];
#pragma unroll
      for (int d = 0; d < NDET; d++) {
        const double2 B = s_rot[d * kPlainRot], A = s_rot[d * kPlainRot + 1 + a], C = s_rot[d * kPlainRot + 9 + b];
        const double xr = B.x * A.x - B.y * A.y, xi = B.x * A.y + B.y * A.x;
        rc[d] = xr * C.x - xi * C.y;
        rs[d] = xr * C.y + xi * C.x;
      }
      cd hp, hc;
      if (pt.use) d_bin_tab(r, pt.w, pt.t, pt.tm76d, ps.s[0].n0 + k, ps.s[0].freqs[k], hp, hc);
      else wave_bin(r, ps.s[0].freqs[k], hp, hc);
      fp64_acc_rot<NDET>(r, ps.s, k, N, hp, hc, rc, rs, v);
    }
  } else {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < N; k += gridDim.x * blockDim.x)
      fp64_bin<NDET>(r, ps.s, k, N, v);
  }
  block_sum<2 * NDET>(v, smem);
  if (threadIdx.x == 0)
#pragma unroll
    for (int j = 0; j < 2 * NDET; j++) partials[blockIdx.x * (2 * NDET) + j] = v[j];
  if (arrive_last(counter, gridDim.x)) {
    // the blocks' partials summed by the whole block (strided, then the
    // block reduction): a fixed order, and no serial chain of L2 loads
    double s[2 * NDET];
#pragma unroll
    for (int j = 0; j < 2 * NDET; j++) s[j] = 0.0;
    for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x)
#pragma unroll
      for (int j = 0; j < 2 * NDET; j++) s[j] += __ldcg(&partials[b * (2 * NDET) + j]);
    block_sum<2 * NDET>(s, smem);
    if (threadIdx.x == 0) {
      out[0] = fp64_finalize<NDET>(s, ps.s);
      if (status) status[0] = r.m.status ? 4 : 0;
      *counter = 0;
    }
  }
}
cudaError_t plain_preload() {
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, k_plain<1>);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, k_plain<2>);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, k_plain<3>);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, k_plain<4>);
  return e;
}
int plain_blocks(int N) {
  int g = (N + 127) / 128;
  return g < 1 ? 1 : g;
}
cudaError_t launch_plain(const Request &r, const StreamDev *streams, int ndet, double *partials, unsigned *counter,
                         double *out, int *status, cudaStream_t s, const PlainTab *tab) {
  PlainStreams ps;
  for (int d = 0; d < ndet; d++) ps.s[d] = streams[d];
  PlainTab pt;
  if (tab) pt = *tab;
  int grid = plain_blocks(streams[0].N);
  switch (ndet) {
    case 1: k_plain<1><<<grid, 128, 0, s>>>(r, ps, pt, partials, counter, out, status); break;
    case 2: k_plain<2><<<grid, 128, 0, s>>>(r, ps, pt, partials, counter, out, status); break;
    case 3: k_plain<3><<<grid, 128, 0, s>>>(r, ps, pt, partials, counter, out, status); break;
    case 4: k_plain<4><<<grid, 128, 0, s>>>(r, ps, pt, partials, counter, out, status); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------- prologue
__global__ void k_prologue(const GenParams *__restrict__ params, const int *__restrict__ approx, int n,
                           const int *__restrict__ handles, int ndet, double T_segment, int tc_from_segment,
                           const StreamDev *__restrict__ streams, const double *__restrict__ qnm, Request *req,
                           MixedReq *mreq, int want_mixed, int *status) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  GenParams p = params[i];
  int ap = approx[i];
  int dets[kMaxDet];
  const StreamDev &s0 = streams[handles[i * ndet]];
  // mcmc_gw.cpp:2466-2473; T_segment <= 0 selects 1/df of this request's grid
  if (tc_from_segment) p.tc = (T_segment > 0 ? T_segment : 1.0 / s0.df) - p.tc;
  int st = 0;
  for (int d = 0; d < ndet; d++) {
    const StreamDev &sd = streams[handles[i * ndet + d]];
    dets[d] = sd.det;
    if (sd.N != s0.N) st = 1;
  }
  bool bad = !(p.mass1 > 0) || !(p.mass2 > 0) || !(p.Luminosity_Distance > 0) || (ap != 0 && ap != 1);
  Request r;
  if (!bad) {
    request_prologue(r, p, ap, dets, ndet, qnm);
    if (r.m.status) st = 4;
    if (req) req[i] = r;
    if (want_mixed) {
      if (!s0.uniform_int) st = st ? st : 1;
      double ds[kMaxDet], ws[kMaxDet];
      unsigned long long wk[kMaxDet];
      for (int d = 0; d < ndet; d++) {
        ds[d] = streams[handles[i * ndet + d]].dscale;
        ws[d] = streams[handles[i * ndet + d]].wscale;
        wk[d] = streams[handles[i * ndet + d]].wkey;
      }
      mixed_prologue(r, s0.df, mreq[i], ds, ws);
      mixed_fold_shared_weights(mreq[i], wk, ndet);
    }
  } else {
    st = 4;
    if (want_mixed) mreq[i] = MixedReq{};
  }
  if (st && want_mixed) mreq[i].status = st;
  if (st && req) req[i].m.status = st;
  status[i] = st;
}
// Cooperative prologue: the same constants as k_prologue, with each request's
// independent parts spread over the four warps of its block.  An FP64
// instruction occupies a sub-partition's FP64 pipe for the same time whatever
// the number of active lanes, so one request per lane leaves the model's
// FP64 chain as the latency; running its independent parts on four
// sub-partitions at once shortens that chain.  Lane j of every warp works on
// request blockIdx.x * kCoopReq + j; shared memory holds the requests between
// stages.  Stage plan (W0..W3 = warps):
//   S0  W0 parameters, source;  W1/W2 detector projections (a detector per half-warp),
//       W2 inclination factors;  W3 chirp mass and amplitude normalisation
//   S1  W0/W3 calibration fits;  W1 D: final spin, radiated energy, ringdown frequencies /
//       Pv2: J-frame transform;  W2 PN coefficients
//   S2  W0 Pv2: ringdown frequencies; matching frequencies;  W1 D: phase at f_ref (inspiral);
//       W2 D: ringdown-phase terms at f3
//   S3  W0/W1 amplitude matching points;  D: phase connection in four pieces after them
//       (W0 f1 terms, W1 inspiral phase, W2 inspiral derivative, W3 f2 terms);
//       Pv2: W2 inspiral part, W1 the other parts, W3 Euler and frame constants
//   S3b Pv2: W2 phase connection constants
//   S4  amplitude deltas (D: W0/W1/W3, Pv2: W0/W1);  W2 D: phase connection constants,
//       phase/time shift / Pv2: time-shift nodes 0-4;  W3 Pv2: nodes 5-9 (two
//       nodes at a time on the half-warps)
//   S5  W0 mixed amplitude;  W1 mixed phase;  W2 regions, D: detector factors / Pv2:
//       angles;  W3 D: detector phases / Pv2: time shift
//   S6  W0 Pv2: detector phases and factors; outputs;  W1-W3 the bin kernel's work order
// (per-warp clock stamps of each stage guided the split: IMRPhenomD, warm,
// before this split S3 20.2k / S5 22.2k / S6 13.0k cycles on the longest warp)
// Programmatic dependent launch: a kernel launched with the programmatic
// stream-serialisation attribute may start while the one before it on the
// stream still runs; grid_dep_wait() returns once that kernel has completed
// and its memory is visible, and grid_dep_trigger() lets the next kernel start
// launching.  Without the attribute both are no-ops.
__device__ __forceinline__ void grid_dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void grid_dep_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Longest-processing-time-first order for the persistent mixed kernel: an
// item's work is its live 256-bin passes (bins below the request's cut
// f <= 0.2/M, where the model is non-zero; beyond it a pass costs nothing), and
// the requests of one batch differ several-fold in it.  Items are bucketed by
// their number of live passes, most first, so that the grid drains on cheap
// items.  The order inside a bucket depends on atomics; results do not
// (partials are indexed by item, and each request's finalize sums them in
// item order).
__device__ __forceinline__ int order_bucket(int kcut, int t, int tile) {
  const int np = (tile + kSegBins - 1) / kSegBins;
  const int live = max(0, min(kcut - t * tile, tile));
  const int lp = min(np, (live + kSegBins - 1) / kSegBins);
  return (int)((long long)(np - lp) * (kOrderBuckets - 1) / np);  // 0: all passes live
}
// Warp-wide: lane l appends the items t = t0, t0 + dt, ... of its request
// (kcut: end of its live bins, nt items from i0) to their buckets.  Lanes that
// draw the same bucket add to it once.  Every lane of the warp calls this
// (nt = 0 for none).
__device__ __forceinline__ void order_append(const OrderArgs &o, int kcut, int nt, int i0, int t0, int dt) {
  const int lane = threadIdx.x & 31;
  const int ntmax = __reduce_max_sync(0xffffffffu, nt);
  for (int t = t0; t < ntmax; t += dt) {
    const int b = t < nt ? order_bucket(kcut, t, o.tile) : -1;
    const unsigned grp = __match_any_sync(0xffffffffu, b);
    const int leader = __ffs(grp) - 1;
    int base = 0;
    if (b >= 0 && lane == leader) base = atomicAdd(o.fill + b, __popc(grp));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (b >= 0) o.items[(size_t)b * o.nitems + base + __popc(grp & ((1u << lane) - 1u))] = i0 + t;
  }
}

constexpr int kCoopWarps = 4, kCoopReq = 16;
// Shared state of one group of kCoopWarps warps serving kCoopReq requests.
struct CoopSmem {
  Request r[kCoopReq];
  GenParams p[kCoopReq];
  AmpConn ac[kCoopReq];
  PhaseConnParts pc[kCoopReq];
  double ds[kCoopReq][kMaxDet], ws[kCoopReq][kMaxDet];  // stream scales of the mixed form
  unsigned long long wk[kCoopReq][kMaxDet];              // and weight keys
  double shift[kCoopReq][kPv2ShiftNodes];
  double df[kCoopReq];
  int st[kCoopReq], bad[kCoopReq], uni[kCoopReq];
};
// The cooperative prologue of requests base .. base + kCoopReq - 1 (those
// below n) on one group of kCoopWarps warps: warp (0..3) and lane are the
// thread's place in the group, sync() the group's barrier.  In S6, while warp
// 0 stores the results, warps 1-3 call tail(warp, lane, act, i, kcut) with
// kcut the end of request i's live bins (0 when it will not be evaluated);
// tail is warp-collective.
template <class Sync, class Tail>
__device__ __forceinline__ void prologue_coop_body(CoopSmem &sm, int base, int warp, int lane,
                                                   const GenParams *__restrict__ params,
                                                   const int *__restrict__ approx, int n,
                                                   const int *__restrict__ handles, int ndet, double T_segment,
                                                   int tc_from_segment, const StreamDev *__restrict__ streams,
                                                   const double *__restrict__ qnm, Request *req, MixedReq *mreq,
                                                   int want_mixed, int *status, Sync sync, Tail tail,
                                                   gwt::WaveF64 *w64 = nullptr) {
  Request *s_r = sm.r;
  GenParams *s_p = sm.p;
  AmpConn *s_ac = sm.ac;
  PhaseConnParts *s_pc = sm.pc;
  double(*s_ds)[kMaxDet] = sm.ds;
  double(*s_ws)[kMaxDet] = sm.ws;
  unsigned long long(*s_wk)[kMaxDet] = sm.wk;
  double(*s_shift)[kPv2ShiftNodes] = sm.shift;
  double *s_df = sm.df;
  int *s_st = sm.st, *s_bad = sm.bad, *s_uni = sm.uni;
  static_assert(2 * kCoopReq == 32, "two half-warps per warp share the group's requests");
  const int i = base + lane;
  const bool act = lane < kCoopReq && i < n;
  // half-warp form: lanes j and j + kCoopReq both serve request j
  const int hl = lane & (kCoopReq - 1);
  const bool hact = base + hl < n;
  Request &r = s_r[lane < kCoopReq ? lane : 0];
  const GenParams &p = s_p[lane < kCoopReq ? lane : 0];
  // S0
  if (act && warp == 0) {
    GenParams q = params[i];
    const int ap = approx[i];
    const StreamDev &s0 = streams[handles[i * ndet]];
    // mcmc_gw.cpp:2466-2473; T_segment <= 0 selects 1/df of this request's grid
    if (tc_from_segment) q.tc = (T_segment > 0 ? T_segment : 1.0 / s0.df) - q.tc;
    int st = 0;
    for (int d = 0; d < ndet; d++)
      if (streams[handles[i * ndet + d]].N != s0.N) st = 1;
    const bool bad = !(q.mass1 > 0) || !(q.mass2 > 0) || !(q.Luminosity_Distance > 0) || (ap != 0 && ap != 1);
    s_p[lane] = q;
    s_st[lane] = st;
    s_bad[lane] = bad;
    s_df[lane] = s0.df;
    s_uni[lane] = s0.uniform_int;
    r.approximant = ap;
    r.ndet = ndet;
    if (!bad) populate_core(r.m.s, q);
  }
  if (act && warp == 3) populate_amp(r.m.s, params[i]);
  if (warp == 1 || warp == 2) {  // projections need only the sky position: detectors over the half-warps of warps 1, 2
    // sky_trig with the hour angle's sincos on lanes j and the declination's
    // on lanes j + kCoopReq at once
    const int ih = base + hl;
    const GenParams &q = params[min(ih, n - 1)];
    double s1, c1, sps, cps;
    sincos(lane < kCoopReq ? q.gmst - q.RA : q.DEC, &s1, &c1);
    sincos(q.psi, &sps, &cps);
    SkyTrig tr;
    tr.sg = __shfl_sync(0xffffffffu, s1, hl);
    tr.cg = __shfl_sync(0xffffffffu, c1, hl);
    tr.sd = __shfl_sync(0xffffffffu, s1, hl + kCoopReq);
    tr.cd = __shfl_sync(0xffffffffu, c1, hl + kCoopReq);
    tr.sp = sps;
    tr.cp = cps;
    if (hact) {  // request hl: warp 1 detectors 0, 2 (+4k), warp 2 detectors 1, 3, half-warp by half-warp
      Request &rh = s_r[hl];
      if (warp == 2 && lane < kCoopReq) populate_incl(rh.m.s, q);
      const int d0 = streams[handles[ih * ndet]].det;
      for (int d = (warp - 1) + (lane >= kCoopReq ? 2 : 0); d < ndet && d < kMaxDet; d += 4) {
        const StreamDev &sd = streams[handles[ih * ndet + d]];
        const int dd = sd.det;
        s_ds[hl][d] = sd.dscale;
        s_ws[hl][d] = sd.wscale;
        s_wk[hl][d] = sd.wkey;
        antenna_trig(dd, tr, rh.det[d].fp, rh.det[d].fc);
        rh.det[d].tau = -dtoa_trig(tr, d0, dd) * (2 * kPi);
      }
    }
  }
  sync();
  const bool run = act && !s_bad[lane < kCoopReq ? lane : 0];
  const bool pv2 = run && r.approximant == kPhenomPv2;
  // S1: the calibration fits in four slots, the half-warps of warps 0 and 3
  if ((warp == 0 || warp == 3) && hact && !s_bad[hl])
    model_d_lambdas_slot(s_r[hl].m, (warp == 3 ? 2 : 0) + (lane >= kCoopReq ? 1 : 0));
  if (run) {
    if (warp == 1) {
      if (pv2) model_p_setup(r.m, r.p, p);
      else if (r.m.s.dep_postmerger) post_merger(r.m.s, qnm);
      else post_merger_qnm(r.m.s, qnm, final_spin(r.m.s), EradRational0815(r.m.s.eta, r.m.s.spin1z, r.m.s.spin2z));
    }
    if (warp == 2) model_d_pn(r.m);
  }
  sync();
  // S2
  if (run && warp == 0) {
    if (pv2) post_merger(r.m.s, qnm);
    model_d_freqs(r.m);
  }
  if (run && warp == 1 && !pv2) finish_fref_phase(r.m, s_pc[lane]);
  if (run && warp == 2 && !pv2) finish_f3_terms(r.m, fpeak(r.m.s, r.m.l), s_pc[lane]);
  sync();
  // S3
  if (run) {
    if (warp == 0) {
      d_amp_conn_low(r.m, s_ac[lane]);
      if (!pv2) phase_conn_imr1(r.m, s_pc[lane]);
    }
    if (warp == 1) {
      d_amp_conn_high(r.m, s_ac[lane]);
      if (pv2) phase_conn_imr(r.m, s_pc[lane]);
      else phase_conn_phins(r.m, s_pc[lane]);
    }
    if (warp == 2) {
      if (pv2) {
        phase_conn_ins(r.m, s_pc[lane]);
      } else {
        phase_conn_dins(r.m, s_pc[lane]);
      }
    }
    if (warp == 3) {
      if (pv2) model_p_finish(r.m, r.p);
      else phase_conn_imr2(r.m, s_pc[lane]);
    }
  }
  sync();
  // S3b  Pv2: the phase connection constants (its time-shift nodes need them)
  if (run && pv2 && warp == 2) phase_conn_combine(r.m, s_pc[lane]);
  sync();
  // S4
  if (run) {
    if (!pv2) {
      if (warp == 0) d_deltas(r.m, s_ac[lane], 0, 2);
      if (warp == 1) d_deltas(r.m, s_ac[lane], 2, 4);
      if (warp == 3) d_deltas(r.m, s_ac[lane], 4, 5);
      if (warp == 2) {
        phase_conn_combine(r.m, s_pc[lane]);
        model_d_finish_parts(r.m, s_pc[lane]);
      }
    } else {
      if (warp == 0) d_deltas(r.m, s_ac[lane], 0, 3);
      if (warp == 1) d_deltas(r.m, s_ac[lane], 3, 5);
    }
  }
  if (warp == 2 || warp == 3) {  // Pv2 time-shift nodes: both half-warps, lanes j and j + kCoopReq on request j
    const Request &rh = s_r[hl];
    if (hact && !s_bad[hl] && rh.approximant == kPhenomPv2 && rh.m.s.shift_time) {
      const int j1 = (warp - 1) * (kPv2ShiftNodes / 2);
      for (int j = (warp - 2) * (kPv2ShiftNodes / 2) + (lane >= kCoopReq ? 1 : 0); j < j1; j += 2)
        s_shift[hl][j] = pv2_shift_node(rh.m, j);
    }
  }
  sync();
  // S5
  if (run) {
    if (warp == 3 && pv2) r.p.t_corr = r.m.s.shift_time ? pv2_shift_solve(r.m, s_shift[lane]) : 0.0;
    if (want_mixed) {
      MixedReq &x = mreq[i];
      const double df = s_df[lane];
      if (warp == 0) mixed_amp_coeffs(r, df, x);
      if (warp == 1) mixed_phase_coeffs(r, df, x);
      if (warp == 2) {
        mixed_regions(r, df, x);  // sets x.A_scale
        if (pv2) mixed_pv2_coeffs(r, df, x);
        else mixed_det_factors_a(r, x, x.A_scale, s_ds[lane], s_ws[lane]);
      }
      if (warp == 3 && !pv2) mixed_det_phase(r, df, x);
    } else if (w64 && warp == 0 && !pv2 && s_uni[lane]) {
      // FP64 batches, IMRPhenomD on a uniform grid: the waveform's
      // coefficients on the grid for the bin kernel's table form
      wave64_prologue(r, s_df[lane], w64[i]);
    }
  }
  sync();
  // S6
  if (act && warp == 0) {
    int st = s_st[lane];
    if (!s_bad[lane]) {
      if (r.m.status) st = 4;
      if (req) req[i] = r;
      if (want_mixed) {
        if (!s_uni[lane]) st = st ? st : 1;
        if (r.approximant == kPhenomPv2) {  // needs the time shift of S5
          mixed_det_phase(r, s_df[lane], mreq[i]);
          mixed_det_factors(r, mreq[i], s_ds[lane], s_ws[lane]);
        }
        mixed_fold_shared_weights(mreq[i], s_wk[lane], ndet);
      }
    } else {
      st = 4;
      if (want_mixed) mreq[i] = MixedReq{};
    }
    if (st && want_mixed) mreq[i].status = st;
    if (st && req) req[i].m.status = st;
    status[i] = st;
  }
  if (warp >= 1 && want_mixed) {
    // a request is live when S6's status will be 0: valid parameters, model
    // status 0, one uniform grid length
    int kcut = 0;
    if (act && !s_bad[lane] && r.m.status == 0 && s_st[lane] == 0 && s_uni[lane]) {
      const StreamDev &s0 = streams[handles[i * ndet]];
      kcut = min(s0.N, mreq[i].n_cut - s0.n0 + 1);  // n_cut: written in S5
    }
    tail(warp, lane, act, i, kcut);
  }
}

__global__ void __launch_bounds__(kCoopWarps * 32) k_prologue_coop(
    const GenParams *__restrict__ params, const int *__restrict__ approx, int n, const int *__restrict__ handles,
    int ndet, double T_segment, int tc_from_segment, const StreamDev *__restrict__ streams,
    const double *__restrict__ qnm, Request *req, MixedReq *mreq, int want_mixed, int *status, const OrderArgs ord,
    gwt::WaveF64 *w64) {
  __shared__ CoopSmem sm;
  grid_dep_trigger();  // the bin kernel may launch and wait for this grid
  // this block's requests into the work order, on the warps idle in S6 (warp
  // w takes the tiles t = w - 1 mod 3)
  auto tail = [&](int warp, int lane, bool act, int i, int kcut) {
    if (!ord.fill) return;
    const int nt = act ? ord.item_count[i] : 0, i0 = act ? ord.item_start[i] : 0;
    order_append(ord, kcut, nt, i0, warp - 1, kCoopWarps - 1);
  };
  prologue_coop_body(sm, blockIdx.x * kCoopReq, threadIdx.x >> 5, threadIdx.x & 31, params, approx, n, handles, ndet,
                     T_segment, tc_from_segment, streams, qnm, req, mreq, want_mixed, status,
                     [] { __syncthreads(); }, tail, w64);
}


cudaError_t launch_prologue(const GenParams *params, const int *approx, int n, const int *handles, int ndet,
                            double T_segment, int tc_from_segment, const StreamDev *streams, const double *qnm,
                            Request *req, MixedReq *mreq, int want_mixed, int *status, cudaStream_t s,
                            const OrderArgs &ord, gwt::WaveF64 *w64) {
  int grid = (n + kCoopReq - 1) / kCoopReq;
  k_prologue_coop<<<grid, kCoopWarps * 32, 0, s>>>(params, approx, n, handles, ndet, T_segment, tc_from_segment,
                                                   streams, qnm, req, mreq, want_mixed, status, ord, w64);
  return cudaGetLastError();
}
cudaError_t launch_prologue_serial(const GenParams *params, const int *approx, int n, const int *handles, int ndet,
                                   double T_segment, int tc_from_segment, const StreamDev *streams, const double *qnm,
                                   Request *req, MixedReq *mreq, int want_mixed, int *status, cudaStream_t s) {
  int block = 32, grid = (n + block - 1) / block;
  k_prologue<<<grid, block, 0, s>>>(params, approx, n, handles, ndet, T_segment, tc_from_segment, streams, qnm, req,
                                    mreq, want_mixed, status);
  return cudaGetLastError();
}

// MCMC_prep_params + repack_parameters (mcmc_gw.cpp:2492-2510; fisher.cpp:2171-2284)
__global__ void k_mcmc_repack(const double *__restrict__ theta, int dim, int n, int approximant, double gmst,
                              GenParams *out, int *approx_out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  GenParams o;
  mcmc_repack(theta + (size_t)i * dim, dim, approximant, gmst, o);
  out[i] = o;
  approx_out[i] = approximant;
}
cudaError_t launch_mcmc_repack(const double *theta, int dim, int n, int approximant, double gmst, GenParams *out,
                               int *approx_out, cudaStream_t s) {
  int block = 128, grid = (n + block - 1) / block;
  k_mcmc_repack<<<grid, block, 0, s>>>(theta, dim, n, approximant, gmst, out, approx_out);
  return cudaGetLastError();
}

// ---------------------------------------------------------- batched kernels
constexpr int kBatchBlock = 256;
static_assert(kBatchBlock == kSegBins, "one block pass covers one phase segment");
constexpr int kMaxSegs = 32;  // segments per chunk of an item (shared buffers)
constexpr int kMaxTile = 16384;  // FP64 form: items up to this many bins use the rotation table
constexpr int kStatusBounds = 0x100;  // set by an item whose bins fall outside the tables; finalize reports 5

// Two-level compensated reduction of NV FP32 values per thread:
// 16-element TwoSum columns, then FP64 across columns.  Result in res[0..NV).
template <int NV>
__device__ __forceinline__ void block_sum_mixed(const float (&v)[NV], float *sm, double *res) {
  const int tid = threadIdx.x, nt = blockDim.x;  // nt == kBatchBlock
#pragma unroll
  for (int j = 0; j < NV; j++) sm[j * kBatchBlock + tid] = v[j];
  __syncthreads();
  constexpr int kCols = kBatchBlock / 16;
  __shared__ float s_hi[kAcc * kCols], s_lo[kAcc * kCols];
  for (int w = tid; w < NV * kCols; w += nt) {
    int j = w / kCols, c = w % kCols;
    const float *p = sm + j * kBatchBlock + c * 16;
    float hi = 0.f, lo = 0.f;
#pragma unroll
    for (int q = 0; q < 16; q++) {
      float a = p[q];
      float s = hi + a;
      float bp = s - hi;
      float e = (hi - (s - bp)) + (a - bp);
      hi = s;
      lo += e;
    }
    s_hi[j * kCols + c] = hi;
    s_lo[j * kCols + c] = lo;
  }
  __syncthreads();
  if (tid < NV) {  // the column pairs with TwoSum in FP32, one conversion to FP64 at the end
    float hi = s_hi[tid * kCols], lo = s_lo[tid * kCols];
    for (int c = 1; c < kCols; c++) {
      float a = s_hi[tid * kCols + c];
      float sum = hi + a, bp = sum - hi;
      lo += ((hi - (sum - bp)) + (a - bp)) + s_lo[tid * kCols + c];
      hi = sum;
    }
    res[tid] = (double)hi + (double)lo;
  }
  __syncthreads();
}

// One item of the mixed form for one approximant class, its sums into
// v[d * kAccPerDet + j]: IMRPhenomD keeps two sums per detector live through
// the item (twelve registers for three detectors instead of thirty), Pv2 five.
template <int NDET, bool PV2>
__device__ __forceinline__ void mixed_item(const BatchArgs &a, const MixedReq &x, const StreamDev *s_st, const Item &I,
                                           int N, int kend, double *s_node, double *s_node_a, SegPoly *s_poly,
                                           SegPoly *s_poly_a, double *s_coef, float2 *s_rot_seg, float2 *s_rot_off,
                                           float (&v)[NDET * kAccPerDet]) {
  const int tid = threadIdx.x;
  constexpr int NA = PV2 ? kAccPerDet : 2;  // sums per detector: Pv2 five, D two
  KSum acc[NDET * NA];
#pragma unroll
  for (int j = 0; j < NDET * NA; j++) acc[j] = KSum{0.f, 0.f};
  if (x.status == 0) {
    const int n0 = s_st[0].n0;
    const float *dh[NDET];
    const float *wh[NDET];
#pragma unroll
    for (int d = 0; d < NDET; d++) {
      dh[d] = s_st[d].dhat;
      wh[d] = s_st[d].what;
    }
    int kcut = min(kend, x.n_cut - n0 + 1);
    if (kcut > I.k0 && (n0 < 1 || n0 + kcut - 1 > a.tables.nmax)) {  // grid beyond the power tables
      if (tid == 0) atomicOr(a.status + I.req, kStatusBounds);
      kcut = I.k0;
    }
    constexpr bool pv2 = PV2;
    const bool wsh = x.wshared != 0;  // one weight stream for every detector
    const gwt::Tables &tb = a.tables;
    // this thread's offset rotations (read back only by this thread)
#pragma unroll
    for (int d = 0; d < NDET; d++) {
      float c, sn;
      det_rot_off(x, d, tid, c, sn);
      s_rot_off[d * kBatchBlock + tid] = make_float2(c, sn);
    }
    // chunks of up to kMaxSegs segments (one segment = one pass of the block over kSegBins bins)
    for (int c0 = I.k0; c0 < kcut; c0 += kMaxSegs * kSegBins) {
      const int nseg = min(kMaxSegs, (kcut - c0 + kSegBins - 1) / kSegBins);
      const int nfn = pv2 ? 2 : 1;  // phase, and alpha for Pv2
      // (A) FP64 phase (and alpha) at the nodes of every usable segment
      for (int e = tid; e < nseg * kSegEval; e += blockDim.x) {
        const int sg = e / kSegEval, j = e - sg * kSegEval, kseg = c0 + sg * kSegBins;
        double vp = 0.0, va = 0.0;
        const int n = seg_node_n(n0, kseg, j);
        if (seg_usable(x, n0, N, kseg) && n <= tb.nmax) {
          const double t = __ldg(tb.t13 + n), r = __ldg(tb.tm53 + n), lnn = __ldg(tb.tln + n);
          vp = mixed_phase_full(x, n, t, r, lnn, __ldg(tb.t34 + n), false);
          if (pv2) va = mixed_pv2_alpha(x, n, t, r, lnn);
        }
        s_node[e] = vp;
        s_node_a[e] = va;
      }
      __syncthreads();
      // (B1) polynomial coefficients and their stored form, one thread per
      // (segment, function, coefficient); a segment the check rejects below
      // keeps unused stored coefficients
      for (int e = tid; e < nseg * nfn * kSegNodes; e += blockDim.x) {
        const int j = e % kSegNodes, q = e / kSegNodes, sg = q / nfn, fn = q - sg * nfn;
        const double *v = (fn ? s_node_a : s_node) + sg * kSegEval;
        double *cf = s_coef + (sg * 2 + fn) * kSegNodes;
        const bool use = seg_usable(x, n0, N, c0 + sg * kSegBins);
        cf[j] = use ? seg_coef(v, j) : 0.0;
        if (use) seg_store(v, cf, j, fn ? s_poly_a[sg] : s_poly[sg]);
      }
      __syncthreads();
      // segment-pass rotations of the detectors
      for (int e = tid; e < nseg * NDET; e += blockDim.x) {
        const int sg = e / NDET, d = e - sg * NDET;
        float c, sn;
        det_rot_seg(x, d, n0 + c0 + sg * kSegBins, c, sn);
        s_rot_seg[sg * NDET + d] = make_float2(c, sn);
      }
      // (B2) acceptance per (segment, function)
      for (int e = tid; e < nseg * 2; e += blockDim.x) {
        const int sg = e >> 1, fn = e & 1, kseg = c0 + sg * kSegBins;
        SegPoly &P = fn ? s_poly_a[sg] : s_poly[sg];
        bool ok = seg_usable(x, n0, N, kseg) && seg_node_n(n0, kseg, 8) <= tb.nmax;
        if (ok && (fn == 0 || pv2))
          ok = seg_check((fn ? s_node_a : s_node) + sg * kSegEval, s_coef + (sg * 2 + fn) * kSegNodes) == 0;
        P.direct = ok ? 0 : 1;
      }
      __syncthreads();
      // (C) bins: the block covers one segment per pass
      for (int sg = 0; sg < nseg; sg++) {
        const int kseg = c0 + sg * kSegBins, k = kseg + tid;
        const bool direct = s_poly[sg].direct | (pv2 ? s_poly_a[sg].direct : 0);
        if (k < kcut) {
          const int n = n0 + k;
          uint64_t ph, al = 0;
          if (!direct) {
            const int m = tid - kSegHalf;
            ph = seg_eval(s_poly[sg], m, n0 + kseg >= x.n_f2p ? seg_atan_extra(x, n) : 0.0f);
            if (pv2) al = seg_eval(s_poly_a[sg], m);
          } else {
            mixed_phase_direct(x, n, __ldg(tb.t13 + n), __ldg(tb.tm53 + n), __ldg(tb.tln + n),
                               __ldg(tb.t34 + n), ph, al);
          }
          float dre[NDET], dim[NDET], w[NDET];
#pragma unroll
          for (int d = 0; d < NDET; d++) {
            float2 v = __ldg(((const float2 *)dh[d]) + k);
            dre[d] = v.x;
            dim[d] = v.y;
            w[d] = (d == 0 || !wsh) ? __ldg(wh[d] + k) : 0.0f;
          }
          float rc[NDET], rs[NDET];
#pragma unroll
          for (int d = 0; d < NDET; d++) {
            const float2 ra = s_rot_seg[sg * NDET + d], rb = s_rot_off[d * kBatchBlock + tid];
            cmulf(ra.x, ra.y, rb.x, rb.y, rc[d], rs[d]);
          }
          if constexpr (PV2)
            mixed_bin_p<NDET>(x, n, ph, al, __ldg(tb.t13f + n), __ldg(tb.tm76f + n), dre, dim, w, rc, rs, acc,
                              wsh);
          else
            mixed_bin_d<NDET, 2>(x, n, ph, __ldg(tb.t13f + n), __ldg(tb.tm76f + n), dre, dim, w, rc, rs, acc,
                                 wsh);
        }
      }
      __syncthreads();  // the node and fit buffers are reused by the next chunk
    }
  }
#pragma unroll
  for (int d = 0; d < NDET; d++)
#pragma unroll
    for (int j = 0; j < kAccPerDet; j++) v[d * kAccPerDet + j] = j < NA ? acc[d * NA + j].s - acc[d * NA + j].c : 0.f;
}

// Shared buffers of one item of the fused bin kernel.
template <int NDET, int MIXED>
struct BinSmem {
  static constexpr int NV = MIXED ? NDET * kAccPerDet : 2 * NDET;
  // mixed form: segment node values and fitted phase / alpha polynomials
  static constexpr int kSegBuf = MIXED ? kMaxSegs : 1;
  // FP64 form on uniform grids: each pass's arrival-time rotations
  static constexpr int kRotPasses = MIXED ? 1 : kMaxTile / kBatchBlock;
  alignas(16) unsigned char req[MIXED ? sizeof(MixedReq) : sizeof(Request)];
  StreamDev st[NDET];
  double res[NV];
  float red[MIXED ? NV * kBatchBlock : 1];
  double dsm[32 * (MIXED ? 1 : NV)];
  double node[kSegBuf * kSegEval], node_a[kSegBuf * kSegEval];
  SegPoly poly[kSegBuf], poly_a[kSegBuf];
  double coef[kSegBuf * 2 * kSegNodes];
  double2 rot64[kRotPasses * NDET];
  // detector rotations: per segment pass (first bin) and per thread offset
  float2 rot_seg[kSegBuf * (MIXED ? NDET : 1)];
  float2 rot_off[(MIXED ? NDET : 1) * (MIXED ? kBatchBlock : 1)];
  alignas(8) unsigned char w64[MIXED ? 8 : sizeof(gwt::WaveF64)];  // FP64 form: the table form's coefficients
};

// One item (iid, I) of a batch on the whole block: its partial sums into
// a.partials[iid]; the block that finishes a request's last item sums them in
// item order and hands log L and the status to fin(request, log L, status)
// (called by thread 0).
template <int NDET, int MIXED, class Fin>
__device__ __forceinline__ void batch_item(const BatchArgs &a, const int iid, const Item I, BinSmem<NDET, MIXED> &sm,
                                           Fin fin) {
  using BS = BinSmem<NDET, MIXED>;
  constexpr int NV = BS::NV;
  constexpr int kRotPasses = BS::kRotPasses;
  unsigned char *s_req = sm.req;
  StreamDev *s_st = sm.st;
  double *s_res = sm.res;
  float *s_red = sm.red;
  double *s_dsm = sm.dsm;
  double *s_node = sm.node, *s_node_a = sm.node_a;
  SegPoly *s_poly = sm.poly, *s_poly_a = sm.poly_a;
  double *s_coef = sm.coef;
  double2 *s_rot64 = sm.rot64;
  float2 *s_rot_seg = sm.rot_seg, *s_rot_off = sm.rot_off;
  const int tid = threadIdx.x;
  // stage the request constants and its streams
  {
    const unsigned *src = MIXED ? (const unsigned *)(a.mreq + I.req) : (const unsigned *)(a.req + I.req);
    unsigned *dst = (unsigned *)s_req;
    constexpr int nw = (MIXED ? sizeof(MixedReq) : sizeof(Request)) / 4;
    for (int w = tid; w < nw; w += blockDim.x) dst[w] = __ldcg(src + w);
    if (tid < NDET) s_st[tid] = a.streams[__ldcg(a.handles + I.req * a.ndet + tid)];
    if constexpr (!MIXED) {
      if (a.w64) {  // the request's FP64 coefficients on the grid (IMRPhenomD, uniform grids)
        static_assert(sizeof(gwt::WaveF64) % 4 == 0, "copied as words");
        const unsigned *ws = (const unsigned *)(a.w64 + I.req);
        unsigned *wd = (unsigned *)sm.w64;
        for (int w = tid; w < (int)(sizeof(gwt::WaveF64) / 4); w += blockDim.x) wd[w] = __ldcg(ws + w);
      }
    }
  }
  __syncthreads();
  const int N = s_st[0].N;
  const int kend = min(I.k0 + a.tile, N);
  if constexpr (MIXED) {
    const MixedReq &x = *(const MixedReq *)s_req;
    float v[NV];
    if (x.approximant == kPhenomPv2)
      mixed_item<NDET, true>(a, x, s_st, I, N, kend, s_node, s_node_a, s_poly, s_poly_a, s_coef, s_rot_seg,
                             s_rot_off, v);
    else
      mixed_item<NDET, false>(a, x, s_st, I, N, kend, s_node, s_node_a, s_poly, s_poly_a, s_coef, s_rot_seg,
                              s_rot_off, v);
    block_sum_mixed<NV>(v, s_red, s_res);
  } else {
    const Request &r = *(const Request *)s_req;
    double v[NV];
#pragma unroll
    for (int j = 0; j < NV; j++) v[j] = 0.0;
    bool uniform = true;
#pragma unroll
    for (int d = 0; d < NDET; d++) uniform = uniform && s_st[d].uniform_int;
    const int npass = (kend - I.k0 + kBatchBlock - 1) / kBatchBlock;
    if (uniform && npass <= kRotPasses) {
      // e^{i tau f_k} = e^{i tau f_(first bin of the pass)} e^{i tau (k - first) df}
      for (int e = tid; e < npass * NDET; e += blockDim.x) {
        const int pass = e / NDET, d = e - pass * NDET;
        double sn, cs;
        sincos(r.det[d].tau * s_st[0].freqs[I.k0 + pass * kBatchBlock], &sn, &cs);
        s_rot64[e] = make_double2(cs, sn);
      }
      double oc[NDET], os[NDET];
#pragma unroll
      for (int d = 0; d < NDET; d++) sincos(r.det[d].tau * (tid * s_st[0].df), &os[d], &oc[d]);
      __syncthreads();
      if (r.m.status == 0) {
        // IMRPhenomD: the waveform from the request's coefficients and the
        // power tables where they cover the item's bins
        const int n0 = s_st[0].n0;
        const bool tab = a.w64 && r.approximant == kPhenomD && n0 >= 1 && n0 + kend - 1 <= a.tables.nmax &&
                         n0 + kend - 1 <= a.tm76d_n;
        const gwt::WaveF64 &W = *(const gwt::WaveF64 *)sm.w64;
        int pass = 0;
        for (int k = I.k0 + tid; k < kend; k += blockDim.x, pass++) {
          double rc[NDET], rs[NDET];
#pragma unroll
          for (int d = 0; d < NDET; d++) {
            const double2 b = s_rot64[pass * NDET + d];
            rc[d] = b.x * oc[d] - b.y * os[d];
            rs[d] = b.y * oc[d] + b.x * os[d];
          }
          cd hp, hc;
          if (tab) d_bin_tab(r, W, a.tables, a.tm76d, n0 + k, s_st[0].freqs[k], hp, hc);
          else wave_bin(r, s_st[0].freqs[k], hp, hc);
          fp64_acc_rot<NDET>(r, s_st, k, N, hp, hc, rc, rs, v);
        }
      }
      __syncthreads();  // s_rot64 is rewritten by the next item
    } else if (r.m.status == 0) {
      for (int k = I.k0 + tid; k < kend; k += blockDim.x) fp64_bin<NDET>(r, s_st, k, N, v);
    }
    block_sum<NV>(v, s_dsm);
    if (tid == 0)
#pragma unroll
      for (int j = 0; j < NV; j++) s_res[j] = v[j];
    __syncthreads();
  }
  if (tid < NV) a.partials[(size_t)iid * kAcc + tid] = s_res[tid];
  // last item of this request: fixed-order FP64 sum and log L
  if (arrive_last(a.req_done + I.req, (unsigned)__ldcg(a.item_count + I.req))) {
    if constexpr (MIXED) {
      // lane j of warp 0: sum j over the request's items, times its factor;
      // then a fixed-order warp sum
      if (tid < 32) {
        const MixedReq &x = *(const MixedReq *)s_req;
        const int i0 = __ldcg(a.item_start + I.req), ic = __ldcg(a.item_count + I.req);
        double v = 0.0;
        if (tid < NV) {
          for (int q = 0; q < ic; q++) v += __ldcg(&a.partials[(size_t)(i0 + q) * kAcc + tid]);
          v *= x.fc[tid];
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (tid == 0) {
          int st = x.status;
          if (__ldcg(a.status + I.req) & kStatusBounds) st = 5;
          fin(I.req, st ? __longlong_as_double(0x7ff8000000000000ll) : v, st);
        }
      }
    } else if (tid == 0) {
      double s[NV];
#pragma unroll
      for (int j = 0; j < NV; j++) s[j] = 0.0;
      const int i0 = __ldcg(a.item_start + I.req), ic = __ldcg(a.item_count + I.req);
      for (int q = 0; q < ic; q++)
#pragma unroll
        for (int j = 0; j < NV; j++) s[j] += __ldcg(&a.partials[(size_t)(i0 + q) * kAcc + j]);
      double ll;
      int st;
      {
        const Request &r = *(const Request *)s_req;
        ll = fp64_finalize<NDET>(s, s_st);
        st = r.m.status;
      }
      if (__ldcg(a.status + I.req) & kStatusBounds) st = 5;
      fin(I.req, st ? __longlong_as_double(0x7ff8000000000000ll) : ll, st);
    }
  }
}

// OCC: the resident blocks per SM the register allocation is bounded for
// (mixed form 3 or 4, a launch-shape choice of the autotuner; FP64 form 2).
template <int NDET, int MIXED, int OCC>
__global__ void __launch_bounds__(kBatchBlock, OCC) k_batch(const BatchArgs a) {
  __shared__ int s_item;
  __shared__ BinSmem<NDET, MIXED> sm;
  __shared__ int s_iid, s_bstart[kOrderBuckets];
  const int tid = threadIdx.x;
  grid_dep_wait();  // the prologue's output
  if (a.bucket_fill && tid < 32) {  // first position of each bucket in the work order
    constexpr int kPerLane = (kOrderBuckets + 31) / 32;
    int v[kPerLane], sum = 0;
#pragma unroll
    for (int q = 0; q < kPerLane; q++) {
      const int b = tid * kPerLane + q;
      v[q] = b < kOrderBuckets ? __ldcg(a.bucket_fill + b) : 0;
      sum += v[q];
    }
    int incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (tid >= o) incl += y;
    }
    int run = incl - sum;
#pragma unroll
    for (int q = 0; q < kPerLane; q++) {
      const int b = tid * kPerLane + q;
      if (b < kOrderBuckets) s_bstart[b] = run;
      run += v[q];
    }
  }
  __syncthreads();
  for (;;) {
    if (tid == 0) {
      const int it = (int)atomicAdd(a.item_counter, 1u);
      int iid = it;
      if (a.bucket_fill && it < a.nitems) {  // the bucket holding position it: the last start <= it
        int lo = 0, hi = kOrderBuckets - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (s_bstart[mid] <= it) lo = mid;
          else hi = mid - 1;
        }
        iid = __ldcg(a.bucket_items + (size_t)lo * a.nitems + (it - s_bstart[lo]));
      }
      s_item = it;
      s_iid = iid;
    }
    __syncthreads();
    const int it = s_item;
    if (it >= a.nitems) break;
    const int iid = s_iid;  // the item's own index: its partials' slot
    batch_item<NDET, MIXED>(a, iid, a.items[iid], sm, [&](int req, double ll, int st) {
      a.out[req] = ll;
      a.status_out[req] = st;
    });
    __syncthreads();
  }
}

// ------------------------------------------------------- serving loop kernel
__device__ __forceinline__ long long global_ns() {
  long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ unsigned long long ld_acquire_sys(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.acquire.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned ld_acquire_sys(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.sys.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned ld_relaxed_gpu(const unsigned *p) {
  unsigned v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long ld_acquire_gpu(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long ld_relaxed_gpu(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_gpu(unsigned long long *p, unsigned long long v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void st_release_sys(unsigned long long *p, unsigned long long v) {
  asm volatile("st.release.sys.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Copies ring entries slot0 .. slot0 + k - 1 (host memory) into the device
// arrays the prologue reads, with their sequence numbers and claim times.
__device__ __forceinline__ void loop_stage(const LoopArgs &L, int slot0, int k, unsigned long long seq0) {
  static_assert(sizeof(GenParams) % 4 == 0, "parameters copied as words");
  constexpr int kW = sizeof(GenParams) / 4;
  const int tid = threadIdx.x, ndet = L.a.ndet;
  for (int w = tid; w < k * kW; w += blockDim.x) {
    const int j = w / kW, q = w - j * kW;
    ((unsigned *)(L.dparams + slot0 + j))[q] = __ldcv((const unsigned *)&L.ring[slot0 + j].p + q);
  }
  const long long now = global_ns();
  for (int j = tid; j < k; j += blockDim.x) {
    const LoopReq *e = L.ring + slot0 + j;
    L.dapprox[slot0 + j] = __ldcv(&e->approx);
    for (int d = 0; d < ndet; d++) L.dhandles[(slot0 + j) * ndet + d] = __ldcv(e->handles + d);
    L.dseq[slot0 + j] = seq0 + j;
    L.dclaim[slot0 + j] = now;
  }
}

// The cooperative prologue of the claimed requests on warps 0-3 (a named
// barrier of their own), then warp 0 publishes each request's live items
// (tiles below its cut, at least one: a request that will not be evaluated
// finishes through its first item with its status) in its claim word.
template <int NDET>
__device__ __forceinline__ void loop_prologue(const LoopArgs &L, CoopSmem &cs, int slot0, int k,
                                              unsigned long long seq0) {
  const BatchArgs &a = L.a;
  loop_stage(L, slot0, k, seq0);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp < kCoopWarps)
    prologue_coop_body(cs, slot0, warp, lane, L.dparams, L.dapprox, slot0 + k, L.dhandles, NDET, L.T_segment, 1,
                       a.streams, L.qnm, nullptr, const_cast<MixedReq *>(a.mreq), 1, a.status,
                       [] { asm volatile("bar.sync 1, 128;" ::: "memory"); }, [](int, int, bool, int, int) {});
  __threadfence();
  __syncthreads();
  if (warp != 0 || lane >= k) return;
  const int slot = slot0 + lane;
  const StreamDev &s0 = a.streams[__ldcg(L.dhandles + slot * NDET)];
  int nlive = 1;
  if (__ldcg(a.status + slot) == 0) {
    const int nt = (s0.N + a.tile - 1) / a.tile;
    const int kcut = min(s0.N, __ldcg(&a.mreq[slot].n_cut) - s0.n0 + 1);
    nlive = max(1, min(nt, (kcut + a.tile - 1) / a.tile));
  }
  L.dcount[slot] = nlive;
  a.req_done[slot] = 0u;
  __threadfence();
  st_release_gpu(L.dwork + slot, loop_word(seq0 + lane, nlive, 0));
}

constexpr unsigned kLoopNapMax = 2048;  // ns between polls of an idle polling block
constexpr int kLoopPairAt = 8;          // candidate requests from which a claim takes two items
template <int NDET>
__global__ void __launch_bounds__(kBatchBlock, 3) k_serve_loop(const __grid_constant__ LoopArgs L) {
  using BS = BinSmem<NDET, 1>;
  constexpr size_t kRaw = sizeof(BS) > sizeof(CoopSmem) ? sizeof(BS) : sizeof(CoopSmem);
  __shared__ __align__(16) unsigned char s_raw[kRaw];
  __shared__ int s_kind, s_a, s_b;
  __shared__ unsigned long long s_seq;
  const int tid = threadIdx.x, lane = tid & 31;
  const unsigned full = 0xffffffffu;
  // pollers read the host's tail and stop flag at every idle poll, the other
  // blocks only once idle for their longest nap
  const bool poller = blockIdx.x % kLoopPollEvery == 0;
  const unsigned nap_max = poller ? kLoopNapMax : kLoopPollEvery * kLoopNapMax;
  const unsigned long long R = (unsigned long long)L.R;
  const long long t0 = global_ns();
  long long t_work = t0;
  unsigned nap = 0;
  for (;;) {
    if (tid < 32) {  // warp 0 finds the block's next work
      int kind = 0, a0 = 0, b0 = 0;  // 0 none, 1 item, 2 prologue, 3 leave
      unsigned long long seq = 0;
      // an item of one of the oldest requests whose prologue is done: lane l
      // reads the claim word of request h + 32 g + l; the block tries the
      // candidates from the (blockIdx mod candidates)-th on, so that blocks
      // spread over them
      unsigned long long h = 0, pend = 0;
      if (lane == 0) {
        h = ld_relaxed_gpu(&L.ctl->scan_head);
        pend = ld_relaxed_gpu(&L.ctl->pro_head);
      }
      h = __shfl_sync(full, h, 0);
      pend = __shfl_sync(full, pend, 0);
      for (int g = 0; g < kLoopWindow / 32 && !kind && h + 32ull * g < pend; g++) {
        const unsigned long long q = h + 32ull * g + lane;
        const int slot = (int)(q % R);
        const unsigned long long w = q < pend ? ld_acquire_gpu(L.dwork + slot) : 0ull;
        const bool ready = q < pend && w >> 24 == ((q + 1) & 0xffffffffffull);
        const int cnt = (int)((w >> 12) & 0xfffu), nxt = (int)(w & 0xfffu);
        if (g == 0) {  // requests at the head with every item claimed: move the head past them
          const unsigned spent = __ballot_sync(full, ready && nxt >= cnt);
          const int lead = spent == full ? 32 : __ffs(~spent) - 1;
          if (lane == 0 && lead > 0) atomicCAS(&L.ctl->scan_head, h, h + (unsigned long long)lead);
        }
        unsigned mask = __ballot_sync(full, ready && nxt < cnt);
        for (int tries = 0; mask && tries < 4; tries++) {
          const int nc = __popc(mask);
          const int pick = (int)__fns(mask, 0, (int)(blockIdx.x % (unsigned)nc) + 1);
          // with many requests waiting, two consecutive items per claim
          const int take = nc >= kLoopPairAt && cnt - nxt >= 2 ? 2 : 1;
          int ok = 0;
          if (lane == pick) ok = atomicCAS(L.dwork + slot, w, w + (unsigned long long)take) == w;
          if (__shfl_sync(full, ok, pick)) {
            kind = 1;
            a0 = __shfl_sync(full, slot, pick);
            b0 = __shfl_sync(full, nxt, pick);
            seq = (unsigned long long)__shfl_sync(full, take, pick);  // items claimed
            break;
          }
          mask &= ~(1u << pick);
        }
      }
      if (lane == 0) {
        const long long now = global_ns();
        const bool old = now - t0 > L.life_ns;
        // new requests: the prologue of up to kLoopClaim of them, in ring order
        if (!kind && !old) {
          const unsigned long long p = ld_relaxed_gpu(&L.ctl->pro_head);
          unsigned long long t = ld_relaxed_gpu(&L.ctl->tail_dev);
          if (p >= t && (poller || nap >= nap_max)) {
            t = ld_acquire_sys(L.tail);
            __threadfence();
            if (t > p) atomicMax(&L.ctl->tail_dev, t);
          }
          if (p < t) {
            const unsigned long long k = min(min(t - p, (unsigned long long)kLoopClaim), R - p % R);
            if (atomicCAS(&L.ctl->pro_head, p, p + k) == p) {
              __threadfence_system();  // the ring entries below the tail seen are read after this
              kind = 2;
              a0 = (int)(p % R);
              b0 = (int)k;
              seq = p;
            }
          }
        }
        if (kind) {
          t_work = now;
        } else {
          int why = -1;
          if (old) why = 2;
          else if (now - t_work > L.idle_ns) why = 0;
          else if (nap >= kLoopNapMax) {
            if ((poller || nap >= nap_max) && ld_acquire_sys(L.stop) == L.launch_id)
              atomicExch(&L.ctl->stop_dev, L.launch_id);
            if (ld_relaxed_gpu(&L.ctl->stop_dev) == L.launch_id) why = 1;
          }
          if (why >= 0) {
            kind = 3;
            atomicAdd(&L.ctl->exits[why], 1u);
          }
        }
        s_kind = kind;
        s_a = a0;
        s_b = b0;
        s_seq = seq;
      }
    }
    __syncthreads();
    const int kind = s_kind, a0 = s_a, b0 = s_b;
    const unsigned long long seq = s_seq;
    __syncthreads();
    if (kind == 3) break;
    if (kind == 0) {
      if (tid == 0) {
        __nanosleep(nap);
        nap = min(2 * nap + 32, nap_max);
      }
      continue;
    }
    nap = 0;
    const long long tw0 = tid == 0 ? global_ns() : 0;
    if (kind == 1) {
      for (int q = 0; q < (int)seq; q++) {  // seq: the number of consecutive items claimed
        if (q) __syncthreads();
        batch_item<NDET, 1>(L.a, a0 * L.max_items + b0 + q, Item{a0, (b0 + q) * L.a.tile}, *(BS *)s_raw,
                            [&](int req, double ll, int st) {
                              const unsigned long long c = atomicAdd(&L.ctl->comp_alloc, 1ull);
                              LoopDone *e = L.comp + c % R;
                              e->seq = __ldcg(L.dseq + req);
                              e->ll = ll;
                              e->status = st;
                              const long long dt = global_ns() - __ldcg(L.dclaim + req);
                              e->service_ns = (int)min(dt, 2000000000ll);
                              st_release_sys(&e->tag, c + 1);
                            });
      }
    } else {
      loop_prologue<NDET>(L, *(CoopSmem *)s_raw, a0, b0, seq);
    }
    if (tid == 0) {
      const unsigned long long dt = (unsigned long long)(global_ns() - tw0);
      if (kind == 1) {
        atomicAdd(&L.ctl->busy_item_ns, dt);
        atomicAdd(&L.ctl->n_item, seq);
      } else {
        atomicAdd(&L.ctl->busy_pro_ns, dt);
        atomicAdd(&L.ctl->n_pro, 1ull);
        atomicAdd(&L.ctl->n_pro_req, (unsigned long long)b0);
      }
    }
    __syncthreads();
  }
}

template <int NDET>
static const void *serve_loop_fn() {
  return (const void *)k_serve_loop<NDET>;
}
static const void *serve_loop_fn(int ndet) {
  switch (ndet) {
    case 1: return serve_loop_fn<1>();
    case 2: return serve_loop_fn<2>();
    case 3: return serve_loop_fn<3>();
    case 4: return serve_loop_fn<4>();
    default: return nullptr;
  }
}

int serve_loop_blocks_per_sm(int ndet) {
  int nb = 0;
  const void *f = serve_loop_fn(ndet);
  if (!f || cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, f, kBatchBlock, 0) != cudaSuccess) return 0;
  return nb;
}

cudaError_t launch_serve_loop(const LoopArgs &L, int grid, cudaStream_t s) {
  const void *f = serve_loop_fn(L.a.ndet);
  if (!f || grid < 1) return cudaErrorInvalidValue;
  void *args[] = {(void *)&L};
  return cudaLaunchKernel(f, dim3(grid), dim3(kBatchBlock), args, 0, s);
}

int batch_block_size(int) { return kBatchBlock; }

template <int NDET>
static const void *batch_fn(int mixed, int occ) {
  if (!mixed) return (const void *)k_batch<NDET, 0, 2>;
  return occ == 3 ? (const void *)k_batch<NDET, 1, 3> : (const void *)k_batch<NDET, 1, 4>;
}
static const void *batch_fn(int mixed, int ndet, int occ) {
  switch (ndet) {
    case 1: return batch_fn<1>(mixed, occ);
    case 2: return batch_fn<2>(mixed, occ);
    case 3: return batch_fn<3>(mixed, occ);
    case 4: return batch_fn<4>(mixed, occ);
    default: return nullptr;
  }
}

int batch_default_occ(int mixed) { return mixed ? 4 : 2; }

int batch_occupancy(int mixed, int ndet, int occ) {
  int nb = 0;
  const void *f = batch_fn(mixed, ndet, occ);
  if (!f) return 1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, f, kBatchBlock, 0) != cudaSuccess) return 1;
  return nb;
}

static cudaError_t launch_dependent(const void *f, dim3 grid, dim3 block, void **args, cudaStream_t s, bool pdl) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelExC(&cfg, f, args);
}

cudaError_t launch_batch(const BatchArgs &a, int mixed, int grid, int occ, cudaStream_t s, bool pdl) {
  const void *f = batch_fn(mixed, a.ndet, occ);
  if (!f) return cudaErrorInvalidValue;
  void *args[] = {(void *)&a};
  return launch_dependent(f, dim3(grid), dim3(kBatchBlock), args, s, pdl);
}

void qnm_host_table(double *o) { qnm_fill(o, gwt_qnm_a_h, gwt_qnm_fring_h, gwt_qnm_fdamp_h); }

}  // namespace gwk
