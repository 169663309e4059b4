// host_check.cpp -- TEST BUILD ONLY: the product's per-request prologue and
// per-bin arithmetic (gw_analysis_tools_gb300/csrc/phenom_*.h) compiled for the
// host, so the CPU test suite can check the kernels' math against the oracle
// without a GPU.  Nothing in the product loads this library.
#include <cmath>
#include <cstring>
#include <vector>

#include "../../gw_analysis_tools_gb300/csrc/phenom_mixed.h"

using namespace gwt;

static std::vector<double> g_qnm;
static const double *qnm() {
  if (g_qnm.empty()) {
    g_qnm.resize(kQnmArrays * kQnmLen);
    qnm_fill(g_qnm.data(), gwt_qnm_a_h, gwt_qnm_fring_h, gwt_qnm_fdamp_h);
  }
  return g_qnm.data();
}

static long g_seg_poly = 0, g_seg_total = 0;

extern "C" {

int gwh_waveform(const double *freqs, int N, double *hp, double *hc, int approx, const GenParams *p) {
  Request r;
  int dets[1] = {0};
  request_prologue(r, *p, approx, dets, 1, qnm());
  for (int k = 0; k < N; k++) {
    cd a, b;
    wave_bin(r, freqs[k], a, b);
    hp[2 * k] = a.re;
    hp[2 * k + 1] = a.im;
    hc[2 * k] = b.re;
    hc[2 * k + 1] = b.im;
  }
  return 1;
}

// Model internals: fRD, fdamp, f1, f3, f1_phase, f2_phase, deltas[5], beta[4], alpha[6]
int gwh_d_internals(const GenParams *p, double *out) {
  Request r;
  int dets[1] = {0};
  request_prologue(r, *p, kPhenomD, dets, 1, qnm());
  const ModelD &m = r.m;
  int k = 0;
  out[k++] = m.s.fRD;
  out[k++] = m.s.fdamp;
  out[k++] = m.s.f1;
  out[k++] = m.s.f3;
  out[k++] = m.s.f1_phase;
  out[k++] = m.s.f2_phase;
  for (int i = 0; i < 5; i++) out[k++] = m.deltas[i];
  for (int i = 0; i < 4; i++) out[k++] = m.l.beta[i];
  for (int i = 0; i < 6; i++) out[k++] = m.l.alpha[i];
  return k;
}

double gwh_loglik_fp64(const GenParams *pin, int approx, double T_segment, const double *freqs, int N, int ndet,
                       const int *dets, const double *const *data, const double *const *psd) {
  GenParams p = *pin;
  p.tc = T_segment - p.tc;
  Request r;
  request_prologue(r, p, approx, dets, ndet, qnm());
  std::vector<double> hh(ndet, 0.0), dh(ndet, 0.0);
  for (int k = 0; k < N; k++) {
    cd a, b;
    double f = freqs[k];
    wave_bin(r, f, a, b);
    double w = simpson_weight(k, N);
    for (int d = 0; d < ndet; d++) {
      cd x = response_bin(r.det[d], a, b, f, r.det[d].tau != 0.0);
      double S = psd[d][k];
      hh[d] += w * ((x.re * x.re + x.im * x.im) / S);
      dh[d] += w * ((data[d][2 * k] * x.re + data[d][2 * k + 1] * x.im) / S);
    }
  }
  double ll = 0, c = 4. * (freqs[N / 2] - freqs[N / 2 - 1]) / 3.;
  for (int d = 0; d < ndet; d++) ll += -0.5 * (c * hh[d] - 2 * c * dh[d]);
  return ll;
}

// Mixed form on the host: same registration whitening, tables, prologue and
// per-bin code as the kernels; FP64 sums of the per-bin FP32 terms.
double gwh_loglik_mixed(const GenParams *pin, int approx, double T_segment, const double *freqs, int N, int ndet,
                        const int *dets, const double *const *data, const double *const *psd) {
  GenParams p = *pin;
  p.tc = T_segment - p.tc;
  Request r;
  request_prologue(r, p, approx, dets, ndet, qnm());
  double df = freqs[1] - freqs[0];
  int n0 = (int)std::llround(freqs[0] / df);
  MixedReq x;
  std::memset(&x, 0, sizeof(x));
  double sdf = freqs[N / 2] - freqs[N / 2 - 1];
  std::vector<std::vector<float>> dh(ndet), wh(ndet);
  std::vector<double> dscale(ndet), wscale(ndet);
  for (int d = 0; d < ndet; d++) {
    std::vector<double> W(N);
    double wmax = 0, dmax = 0;
    for (int k = 0; k < N; k++) {
      double sw = (k == 0 || k == N - 1) ? 1.0 : ((k & 1) ? 4.0 : 2.0);
      W[k] = 4. * sdf / 3. * sw / psd[d][k];
      wmax = std::max(wmax, std::fabs(W[k]));
      dmax = std::max(dmax, std::fabs(W[k] * data[d][2 * k]) + std::fabs(W[k] * data[d][2 * k + 1]));
    }
    wscale[d] = wmax;
    dscale[d] = dmax > 0 ? dmax : 1.0;
    dh[d].resize(2 * N);
    wh[d].resize(N);
    for (int k = 0; k < N; k++) {
      dh[d][2 * k] = (float)(W[k] * data[d][2 * k] / dscale[d]);
      dh[d][2 * k + 1] = (float)(W[k] * data[d][2 * k + 1] / dscale[d]);
      wh[d][k] = (float)(W[k] / wscale[d]);
    }
  }
  mixed_prologue(r, df, x, dscale.data(), wscale.data());
  std::vector<unsigned long long> wk(ndet);  // detectors given the same PSD array share weights
  for (int d = 0; d < ndet; d++) wk[d] = (unsigned long long)(uintptr_t)psd[d];
  mixed_fold_shared_weights(x, wk.data(), ndet);
  if (x.status) return NAN;
  auto tables = [](int n, double &t, double &rr, double &lnn, double &t34) {
    double xn = (double)n;
    t = std::cbrt(xn), rr = std::pow(xn, -5. / 3.), lnn = std::log(xn), t34 = std::pow(xn, 0.75);
  };
  double sums[kMaxDet * kAccPerDet] = {0};
  const bool pv2 = x.approximant == kPhenomPv2;
  for (int kseg = 0; kseg < N; kseg += kSegBins) {
    // the kernel's segment plan: polynomial phase where usable and within tolerance
    SegPoly sp{}, sa{};
    bool poly = seg_usable(x, n0, N, kseg);
    if (poly) {
      double vp[kSegEval], va[kSegEval];
      for (int j = 0; j < kSegEval; j++) {
        int n = seg_node_n(n0, kseg, j);
        double t, rr, lnn, t34;
        tables(n, t, rr, lnn, t34);
        vp[j] = mixed_phase_full(x, n, t, rr, lnn, t34, false);
        va[j] = pv2 ? mixed_pv2_alpha(x, n, t, rr, lnn) : 0.0;
      }
      poly = seg_fit(vp, sp) == 0 && (!pv2 || seg_fit(va, sa) == 0);
    }
    g_seg_poly += poly ? 1 : 0;
    g_seg_total += 1;
    for (int k = kseg; k < std::min(N, kseg + kSegBins); k++) {
      int n = n0 + k;
      double xn = (double)n;
      float tf = (float)std::cbrt(xn), m76 = (float)std::pow(xn, -7. / 6.);
      uint64_t ph, al;
      if (poly) {
        int m = k - kseg - kSegHalf;
        ph = seg_eval(sp, m, n0 + kseg >= x.n_f2p ? seg_atan_extra(x, n) : 0.0f);
        al = pv2 ? seg_eval(sa, m) : 0;
      } else {
        double t, rr, lnn, t34;
        tables(n, t, rr, lnn, t34);
        mixed_phase_direct(x, n, t, rr, lnn, t34, ph, al);
      }
      float dre[kMaxDet], dim[kMaxDet], w[kMaxDet];
      for (int d = 0; d < ndet; d++) {
        dre[d] = dh[d][2 * k];
        dim[d] = dh[d][2 * k + 1];
        w[d] = wh[d][k];
      }
      // the kernel's detector rotations: segment factor times offset factor
      float rc[kMaxDet], rs[kMaxDet];
      for (int d = 0; d < ndet; d++) {
        float ac, as, bc, bs;
        det_rot_seg(x, d, n0 + kseg, ac, as);
        det_rot_off(x, d, k - kseg, bc, bs);
        cmulf(ac, as, bc, bs, rc[d], rs[d]);
      }
      KSum acc[kMaxDet * kAccPerDet];
      for (auto &a : acc) a = KSum{0.f, 0.f};
      switch (ndet) {
        case 1: mixed_bin_q<1>(x, n, ph, al, tf, m76, dre, dim, w, rc, rs, acc, x.wshared != 0); break;
        case 2: mixed_bin_q<2>(x, n, ph, al, tf, m76, dre, dim, w, rc, rs, acc, x.wshared != 0); break;
        case 3: mixed_bin_q<3>(x, n, ph, al, tf, m76, dre, dim, w, rc, rs, acc, x.wshared != 0); break;
        default: mixed_bin_q<4>(x, n, ph, al, tf, m76, dre, dim, w, rc, rs, acc, x.wshared != 0); break;
      }
      for (int j = 0; j < kMaxDet * kAccPerDet; j++) sums[j] += (double)(acc[j].s - acc[j].c);
    }
  }
  return mixed_finalize(x, sums);
}

// Segments that used the polynomial phase / all segments, since the last reset.
void gwh_segment_stats(long *poly, long *total, int reset) {
  *poly = g_seg_poly;
  *total = g_seg_total;
  if (reset) g_seg_poly = g_seg_total = 0;
}

}  // extern "C"

#include "../../gw_analysis_tools_gb300/csrc/fisher_math.h"

// The moment form on the host at order 2 or 4; returns 10 for a five-point
// source the product leaves to the reference algorithm.
extern "C" int gwh_fisher_batch_order(const GenParams *p, int method, int order, const double *freqs, int N, int ndet,
                                      const int *dets, const double *const *psd, double epsilon, int step_mode,
                                      double *out, double *cov) {
  using namespace gwf;
  double df = freqs[1] - freqs[0];
  int n0 = (int)std::llround(freqs[0] / df);
  std::vector<SlotOut> slots(kSlots);
  for (int s = 0; s < kSlots; s++) fisher_slot(*p, s, method, dets, ndet, df, epsilon, step_mode, qnm(), slots[s]);
  FisherSrc F;
  int st = fisher_setup(*p, method, ndet, epsilon, step_mode, order, slots.data(), F);
  if (st) return st;
  if (F.needs_ref) return 10;
  double sdf = freqs[N / 2] - freqs[N / 2 - 1];
  std::vector<double> Ssum(kMaxDet * kSums, 0.0);
  std::vector<int> wslot(ndet);
  std::vector<double> wscale(ndet);
  for (int d = 0; d < ndet; d++) {
    wslot[d] = d;
    double wmax = 0;
    for (int k = 0; k < N; k++) {
      double sw = (k == 0 || k == N - 1) ? 1.0 : ((k & 1) ? 4.0 : 2.0);
      wmax = std::max(wmax, 4. * sdf / 3. * sw / psd[d][k]);
    }
    wscale[d] = wmax;
    std::vector<KSum> acc(kSums, KSum{0.f, 0.f});
    for (int k = 0; k < N; k++) {
      int n = n0 + k;
      double x = n;
      float a0, qr[kIntr], qi[kIntr];
      const double m76 = std::pow(x, -7. / 6.);
      if (!fisher_bin_q(F, n, std::cbrt(x), std::pow(x, -5. / 3.), std::log(x), std::pow(x, 0.75), m76,
                        (float)m76, a0, qr, qi))
        continue;
      double sw = (k == 0 || k == N - 1) ? 1.0 : ((k & 1) ? 4.0 : 2.0);
      float wh = (float)(4. * sdf / 3. * sw / psd[d][k] / wmax);
      fisher_accumulate(wh, a0, (float)(x * df), qr, qi, acc.data());
    }
    for (int j = 0; j < kSums; j++) Ssum[d * kSums + j] = (double)acc[j].s - (double)acc[j].c;
  }
  fisher_assemble(F, Ssum.data(), ndet, wslot.data(), wscale.data(), df / sdf, out);
  if (cov) return chol_invert(out, cov, kDim) ? 9 : 0;
  return 0;
}
extern "C" int gwh_fisher_batch(const GenParams *p, int method, const double *freqs, int N, int ndet, const int *dets,
                                const double *const *psd, double epsilon, int step_mode, double *out, double *cov) {
  return gwh_fisher_batch_order(p, method, 2, freqs, N, ndet, dets, psd, epsilon, step_mode, out, cov);
}

// Each intrinsic pair's per-bin complex difference as fisher_bin_q forms it
// (the polynomial-difference fast path, its series in the half phase step, the
// one-sided and beyond-the-cut cases) against fisher_q_exact, which takes the
// pair's two waveforms bin by bin.  maxerr[q] = max_k |q_fast - q_exact| /
// max_k |q_exact| over every bin of the grid, region boundaries included.
extern "C" int gwh_fisher_pair_check(const GenParams *p, int method, double df, int n0, int N, double epsilon,
                                     int step_mode, double *maxerr) {
  using namespace gwf;
  int dets[1] = {0};
  std::vector<SlotOut> slots(kSlots);
  for (int s = 0; s < kSlots; s++) fisher_slot(*p, s, method, dets, 1, df, epsilon, step_mode, qnm(), slots[s]);
  FisherSrc F;
  int st = fisher_setup(*p, method, 1, epsilon, step_mode, 2, slots.data(), F);
  if (st) return st;
  double emax[kIntr] = {0, 0, 0, 0}, qmax[kIntr] = {0, 0, 0, 0};
  for (int k = 0; k < N; k++) {
    const int n = n0 + k;
    const double x = n, t = std::cbrt(x), r = std::pow(x, -5. / 3.), lnn = std::log(x), t34 = std::pow(x, 0.75);
    const double m76 = std::pow(x, -7. / 6.);
    float a0, qr[kIntr], qi[kIntr];
    if (!fisher_bin_q(F, n, t, r, lnn, t34, m76, (float)m76, a0, qr, qi)) continue;
    for (int q = 0; q < kIntr; q++) {
      float er, ei;
      fisher_q_exact(F, q, n, t, r, lnn, t34, m76, er, ei);
      emax[q] = std::max(emax[q], std::hypot((double)qr[q] - er, (double)qi[q] - ei));
      qmax[q] = std::max(qmax[q], std::hypot((double)er, (double)ei));
    }
  }
  for (int q = 0; q < kIntr; q++) maxerr[q] = qmax[q] > 0 ? emax[q] / qmax[q] : 0.0;
  return 0;
}
