// fisher_math.h -- Fisher matrix arithmetic shared by the kernels
// (fisher.cu) and the CPU test build: per-perturbation prologue, the
// amplitude/phase central differences, the moment-form Gram sums and the FP64
// assembly + pivoted Cholesky inverse.
#pragma once

#include "phenom_mixed.h"

namespace gwf {
using namespace gwt;

constexpr int kDim = kFisherDim;
constexpr int kSlots = 1 + 2 * kDim;  // centre, then (+, -) per parameter
constexpr int kIntr = 4;              // parameters 7..10 change the waveform itself
constexpr int kCheap = 7;             // parameters 0..6: projection, phase offset, tc, D_L
constexpr int kSums = 3 + 10 + 16;    // M0, M1, M2 | Q (4x4 sym) | S_i, T_i (complex)

struct SlotOut {
  WaveF64 w;
  double Gre[kMaxDet], Gim[kMaxDet], tau[kMaxDet];
  int status;
};

// Coefficient differences of the waveforms of one central difference pair
// (+ minus -): the phase polynomials, and the amplitude polynomials times
// their scales relative to the centre (the intermediate one re-centred on the
// centre waveform's n_mid).  Where both waveforms are in the same region at a
// bin, their difference is one polynomial in FP64 instead of two.
struct WaveDiff {
  double qi[12], bi0, bi1, pA, pB, pC, pD, mA, mB, mC, mD, phic;
  double ai[10], ei[5];
};

struct FisherSrc {
  WaveF64 w0, wp[kIntr], wm[kIntr];
  double sp[kIntr], sm[kIntr];  // A_scale(+/-) / A_scale(centre)
  double div[kDim];
  double idiv[kIntr];  // 1 / div[7 + q]
  double amp_lk[kIntr];  // ln(K+ sp / (K- sm)) of the ringdown amplitudes of pair q
  WaveDiff wd[kIntr];
  double v[kDim];
  int logf[kDim];
  double G0re[kMaxDet], G0im[kMaxDet];
  double ar[kMaxDet][kCheap], ai[kMaxDet][kCheap], br[kMaxDet][kCheap], bi[kMaxDet][kCheap];
  int onesided[kIntr];  // pair q is a one-sided difference (eta at 1/4): its + waveform is the centre
  int exact[kIntr];     // pair q is taken as the difference of its two waveforms at every bin
  int n_cut_any;        // the last bin where any of the centre and the perturbed waveforms is non-zero
  int needs_ref;        // five-point rule and a pair taken bin by bin: left to the reference algorithm
  int status;
};
// ----------------------------------------------------- pivoted Cholesky inverse
// Symmetric diagonal pivoting on the largest remaining diagonal, LDL^T, inverse
// (gsl_cholesky_matrix_invert, util.cpp:857-900).  Returns 0 on success.
GW_HD int chol_invert(const double *a, double *inv, int dim) {
  double A[kDim * kDim], Li[kDim * kDim], Dv[kDim];
  int perm[kDim];
  for (int i = 0; i < dim * dim; i++) A[i] = a[i];
  for (int i = 0; i < dim; i++) perm[i] = i;
  for (int j = 0; j < dim; j++) {
    int piv = j;
    for (int i = j + 1; i < dim; i++)
      if (A[i * dim + i] > A[piv * dim + piv]) piv = i;
    if (piv != j) {
      for (int k = 0; k < dim; k++) {
        double t = A[j * dim + k];
        A[j * dim + k] = A[piv * dim + k];
        A[piv * dim + k] = t;
      }
      for (int k = 0; k < dim; k++) {
        double t = A[k * dim + j];
        A[k * dim + j] = A[k * dim + piv];
        A[k * dim + piv] = t;
      }
      int t = perm[j];
      perm[j] = perm[piv];
      perm[piv] = t;
    }
    double d = A[j * dim + j];
    if (!(d > 0)) return 1;
    Dv[j] = d;
    for (int i = j + 1; i < dim; i++) A[i * dim + j] /= d;
    for (int i = j + 1; i < dim; i++)
      for (int k = j + 1; k <= i; k++) {
        A[i * dim + k] -= A[i * dim + j] * A[k * dim + j] * d;
        A[k * dim + i] = A[i * dim + k];
      }
  }
  for (int i = 0; i < dim * dim; i++) Li[i] = 0;
  for (int i = 0; i < dim; i++) {
    Li[i * dim + i] = 1;
    for (int j = 0; j < i; j++) {
      double s = 0;
      for (int k = j; k < i; k++) s += A[i * dim + k] * Li[k * dim + j];
      Li[i * dim + j] = -s;
    }
  }
  for (int i = 0; i < dim; i++)
    for (int j = 0; j < dim; j++) {
      double s = 0;
      for (int k = (i > j ? i : j); k < dim; k++) s += Li[k * dim + i] * Li[k * dim + j] / Dv[k];
      inv[perm[i] * dim + perm[j]] = s;
    }
  for (int i = 0; i < dim * dim; i++)
    if (inv[i] != inv[i]) return 1;
  return 0;
}

// One (source, slot) of the batched Fisher: perturbed parameters, prologue,
// FP64 wave coefficients, projection constants.
GW_HDNI void fisher_slot(const GenParams &in, int slot, int method, const int *dets, int ndet, double df,
                         double epsilon, int step_mode, const double *qnm, SlotOut &o) {
  double v[kDim], pv[kDim];
  int logf[kDim];
  fisher_unpack(in, method, v, logf);
  if (slot == 0) {
    for (int j = 0; j < kDim; j++) pv[j] = v[j];
  } else {
    int i = (slot - 1) / 2, sign = ((slot - 1) % 2 == 0) ? 1 : -1;
    fisher_perturb(v, i, sign, fisher_step(v, i, epsilon, step_mode), pv);
  }
  GenParams p;
  fisher_repack(pv, in, method, p);
  Request r;
  request_prologue(r, p, kPhenomD, dets, ndet, qnm);
  wave64_prologue(r, df, o.w);
  double ci = cos(p.incl_angle);
  for (int d = 0; d < ndet; d++) {
    o.Gre[d] = r.det[d].fp * .5 * (1 + ci * ci);
    o.Gim[d] = -r.det[d].fc * ci;
    o.tau[d] = r.det[d].tau;
  }
  bool bad = !(p.mass1 > 0) || !(p.mass2 > 0) || !(p.Luminosity_Distance > 0) || r.m.status != 0;
  o.status = bad ? 4 : 0;
}

// Combine the slots of one source into the constants of the Gram sums.
// Intermediate amplitude coefficients about n_mid re-centred on H (exact
// binomial shift by the integer H - n_mid).
GW_HD void recentre_ei(const WaveF64 &x, int H, double *e) {
  const double sh = (double)(H - x.n_mid);
  for (int k = 0; k < 5; k++) {
    double acc = 0.0, binom = 1.0, pw = 1.0;  // C(j, k) sh^(j - k) for j = k..4
    for (int j = k; j < 5; j++) {
      acc += binom * x.ei[j] * pw;
      binom = binom * (j + 1) / (j + 1 - k);
      pw *= sh;
    }
    e[k] = acc;
  }
}
// The differences, times inv = 1 / (the difference's divisor).
GW_HD void wave_diff(const WaveF64 &p, const WaveF64 &m, double sp, double sm, int H, double inv, WaveDiff &d) {
  for (int j = 0; j < 12; j++) d.qi[j] = (p.qi[j] - m.qi[j]) * inv;
  d.bi0 = (p.bi0 - m.bi0) * inv;
  d.bi1 = (p.bi1 - m.bi1) * inv;
  d.pA = (p.pA - m.pA) * inv;
  d.pB = (p.pB - m.pB) * inv;
  d.pC = (p.pC - m.pC) * inv;
  d.pD = (p.pD - m.pD) * inv;
  d.mA = (p.mA - m.mA) * inv;
  d.mB = (p.mB - m.mB) * inv;
  d.mC = (p.mC - m.mC) * inv;
  d.mD = (p.mD - m.mD) * inv;
  d.phic = (p.phic - m.phic) * inv;
  for (int j = 0; j < 10; j++) d.ai[j] = (p.ai[j] * sp - m.ai[j] * sm) * inv;
  double ep[5], em[5];
  recentre_ei(p, H, ep);
  recentre_ei(m, H, em);
  for (int j = 0; j < 5; j++) d.ei[j] = (ep[j] * sp - em[j] * sm) * inv;
}

GW_HDNI int fisher_setup(const GenParams &in, int method, int ndet, double epsilon, int step_mode, int order,
                         const SlotOut *S, FisherSrc &F) {
  fisher_unpack(in, method, F.v, F.logf);
  int st = 0;
  for (int s = 0; s < kSlots; s++) st |= S[s].status;
  for (int i = 0; i < kDim; i++) {
    double eps = fisher_step(F.v, i, epsilon, step_mode);
    double tmp[kDim];
    F.div[i] = fisher_perturb(F.v, i, 1, eps, tmp);
  }
  for (int q = 0; q < kIntr; q++) {
    F.idiv[q] = 1.0 / F.div[7 + q];
    F.onesided[q] = F.div[7 + q] == fisher_step(F.v, 7 + q, epsilon, step_mode);
    // The waveform depends on eta through sqrt(1 - 4 eta) (the component
    // masses): within a few thousand steps of eta = 1/4 the pair's mean phase
    // and amplitude offsets are no longer second order in the step, and the
    // difference is taken waveform by waveform.
    F.exact[q] = q == 1 && (0.25 - F.v[8]) < 1000.0 * F.div[8];
  }
  F.w0 = S[0].w;
  F.n_cut_any = F.w0.n_cut;
  for (int s = 1; s < kSlots; s++) F.n_cut_any = F.n_cut_any > S[s].w.n_cut ? F.n_cut_any : S[s].w.n_cut;
  const double A0 = S[0].w.A_scale;
  for (int k = 0; k < kIntr; k++) {
    int i = 7 + k;
    F.wp[k] = S[1 + 2 * i].w;
    F.wm[k] = S[2 + 2 * i].w;
    F.sp[k] = F.wp[k].A_scale / A0;
    F.sm[k] = F.wm[k].A_scale / A0;
    F.amp_lk[k] = log((F.wp[k].mrK * F.sp[k]) / (F.wm[k].mrK * F.sm[k]));
    wave_diff(F.wp[k], F.wm[k], F.sp[k], F.sm[k], F.w0.n_mid, F.idiv[k], F.wd[k]);
  }
  for (int d = 0; d < ndet; d++) {
    double g0r = S[0].Gre[d], g0i = S[0].Gim[d];
    F.G0re[d] = g0r;
    F.G0im[d] = g0i;
    for (int i = 0; i < kCheap; i++) {
      const SlotOut &P = S[1 + 2 * i], &Mn = S[2 + 2 * i];
      double dv = F.div[i];
      double ar = 0, ai = 0, br = 0, bi = 0;
      if (i <= 3) {  // RA, DEC, psi, iota: dG + i G f dtau
        ar = (P.Gre[d] - Mn.Gre[d]) / dv;
        ai = (P.Gim[d] - Mn.Gim[d]) / dv;
        double dt = (P.tau[d] - Mn.tau[d]) / dv;
        br = -g0i * dt;  // i G dtau
        bi = g0r * dt;
      } else if (i == 4) {  // phiRef: i G dphic
        double dph = (P.w.phic - Mn.w.phic) / dv;
        ar = -g0i * dph;
        ai = g0r * dph;
      } else if (i == 5) {  // tc: i G dtcl (f - fref)
        double dt = (P.w.tcl - Mn.w.tcl) / dv;
        double fr = S[0].w.fref;
        br = -g0i * dt;
        bi = g0r * dt;
        ar = g0i * dt * fr;
        ai = -g0r * dt * fr;
      } else {  // D_L: G dA/A
        double rel = (P.w.A_scale - Mn.w.A_scale) / (dv * A0);
        ar = g0r * rel;
        ai = g0i * rel;
      }
      if (F.logf[i]) {
        ar *= F.v[i];
        ai *= F.v[i];
        br *= F.v[i];
        bi *= F.v[i];
      }
      if (order == 4) {
        // Five-point rule (fisher.cpp:426-458): the reference shifts t_c by
        // the detector's arrival time at the +-2 eps steps instead of
        // rotating by e^{-2 pi i DTOA f}, so those two responses carry the
        // extra constant phase phq = -tau f_ref.  To second order in the step
        // the five-point difference is then kappa r' + c r with
        // kappa = (4 - e^{i phq}) / 3 and c = -(i/3) e^{i phq} d(phq)/d(theta)
        // = (i/3) e^{i phq} f_ref dtau (the sky position only); kappa = 1 and
        // c = 0 at the reference detector (tau = 0).  Here a' = kappa a + c G0
        // and b' = kappa b; the intrinsic rows take kappa G0 below.
        const double phq = -S[0].tau[d] * S[0].w.fref;
        double sq, cq;
        sincos(phq, &sq, &cq);
        const double kr = (4.0 - cq) / 3.0, ki = -sq / 3.0;
        double dt = i <= 3 ? (P.tau[d] - Mn.tau[d]) / dv : 0.0;
        if (F.logf[i]) dt *= F.v[i];
        const double cr = -sq * S[0].w.fref * dt / 3.0, ci = cq * S[0].w.fref * dt / 3.0;
        const double ar2 = kr * ar - ki * ai + (cr * g0r - ci * g0i), ai2 = kr * ai + ki * ar + (cr * g0i + ci * g0r);
        const double br2 = kr * br - ki * bi, bi2 = kr * bi + ki * br;
        ar = ar2;
        ai = ai2;
        br = br2;
        bi = bi2;
      }
      F.ar[d][i] = ar;
      F.ai[d][i] = ai;
      F.br[d][i] = br;
      F.bi[d][i] = bi;
    }
    if (order == 4) {  // the intrinsic derivatives: kappa G0 q
      const double phq = -S[0].tau[d] * S[0].w.fref;
      double sq, cq;
      sincos(phq, &sq, &cq);
      const double kr = (4.0 - cq) / 3.0, ki = -sq / 3.0;
      F.G0re[d] = kr * g0r - ki * g0i;
      F.G0im[d] = kr * g0i + ki * g0r;
    }
  }
  // The five-point rule's +-2 eps waveforms are not among the slots: a pair
  // that the moment form takes bin by bin (eta at 1/4, a waveform's cut inside
  // the pair) is left to the reference algorithm.
  F.needs_ref = 0;
  if (order == 4) {
    for (int q = 0; q < kIntr; q++)
      if (F.onesided[q] || F.exact[q] || F.wp[q].n_cut != F.w0.n_cut || F.wm[q].n_cut != F.w0.n_cut) F.needs_ref = 1;
  }
  F.status = st;
  return st;
}


// (A+ s+ - A- s-) / divisor of pair q at bin n (T = float: the amplitude power
// m76 applied in FP32; T = double: all FP64): one polynomial of coefficient
// differences where both waveforms are in the same inspiral or intermediate
// region, the ringdown form of wave64_amp_diff, each waveform on its own at
// the bins between their region boundaries.
template <typename T>
GW_HD T fisher_amp_deriv(const FisherSrc &F, int q, int n, double t, double m76, float m76f) {
  const WaveF64 &p = F.wp[q], &m = F.wm[q];
  const WaveDiff &d = F.wd[q];
  if (n <= p.n_cut && n <= m.n_cut) {
    if (n < p.n_f1 && n < m.n_f1) {
      double a = d.ai[9];
      for (int j = 8; j >= 0; j--) a = a * t + d.ai[j];
      if constexpr (sizeof(T) == sizeof(float)) return (float)a * m76f;
      else return a * m76;
    }
    if (n >= p.n_f1 && n >= m.n_f1 && n < p.n_f3 && n < m.n_f3) {
      const double h = (double)(n - F.w0.n_mid);
      const double a = (((d.ei[4] * h + d.ei[3]) * h + d.ei[2]) * h + d.ei[1]) * h + d.ei[0];
      if constexpr (sizeof(T) == sizeof(float)) return (float)a * m76f;
      else return a * m76;
    }
  }
  return (T)(wave64_amp_diff(p, m, n, t, m76, F.sp[q], F.sm[q], F.amp_lk[q]) * F.idiv[q]);
}
// ((phase+ - phic+) - (phase- - phic-)) / divisor of pair q at bin n, the same way.
GW_HD double fisher_phase_deriv(const FisherSrc &F, int q, int n, double t, double r, double lnn, double t34) {
  const WaveF64 &p = F.wp[q], &m = F.wm[q];
  const WaveDiff &d = F.wd[q];
  if (n <= p.n_cut && n <= m.n_cut) {
    if (n < p.n_f1p && n < m.n_f1p) {
      double s = d.qi[11];
      for (int j = 10; j >= 0; j--) s = s * t + d.qi[j];
      return (r * s + lnn * (d.bi0 + d.bi1 * t)) - d.phic;
    }
    if (n >= p.n_f1p && n >= m.n_f1p && n < p.n_f2p && n < m.n_f2p) {
      const double nd = (double)n;
      return (d.pA + d.pB * nd + d.pC * lnn - d.pD * (r * r * t)) - d.phic;
    }
    if (n >= p.n_f2p && n >= m.n_f2p) {  // ringdown: the atan pair as in wave64_phase_diff
      const double nd = (double)n;
      const double yp = (nd - p.nc) * p.inv_nw, ym = (nd - m.nc) * m.inv_nw;
      const double z = (yp - ym) / (1.0 + yp * ym);
      if (fabs(z) < 1e-3) {
        const double z2 = z * z;
        const double datan = z * (1.0 - z2 * ((1.0 / 3.0) - z2 * 0.2));  // atan z to z^5
        return (d.mA + d.mB * nd - d.mC * (r * t * t) + d.mD * t34 - d.phic) +
               (p.mE * datan + (p.mE - m.mE) * atan(ym)) * F.idiv[q];
      }
    }
  }
  return wave64_phase_diff(p, m, n, t, r, lnn, t34) * F.idiv[q];
}

// The exact difference of pair q relative to the centre's phase, per unit
// step: the sum over the non-zero waveforms of +-A s e^{-i delta},
// delta = (Phi - phic) - (Phi0 - phic0).  Used at a bin where a waveform is
// beyond its cut (f > 0.2/M, where the model is exactly zero: a finite
// difference across the cut is a jump, which the series form below does not
// describe) and for pairs flagged exact.
template <typename T>
GW_HD void fisher_q_exact(const FisherSrc &F, int q, int n, double t, double r, double lnn, double t34, double m76,
                          T &qr, T &qi) {
  const double phi0 = wave64_phase(F.w0, n, t, r, lnn, t34) - F.w0.phic;
  double re = 0.0, im = 0.0;
  for (int side = 0; side < 2; side++) {
    const WaveF64 &w = side == 0 ? F.wp[q] : F.wm[q];
    if (n > w.n_cut) continue;
    const double a = wave64_amp(w, n, t, m76) * (side == 0 ? F.sp[q] : F.sm[q]) * (side == 0 ? 1.0 : -1.0);
    double s, c;
    sincos((wave64_phase(w, n, t, r, lnn, t34) - w.phic) - phi0, &s, &c);
    re += a * c;
    im -= a * s;
  }
  qr = (T)(re * F.idiv[q]);
  qi = (T)(im * F.idiv[q]);
}

// One bin: the intrinsic differences q = (r+ - r-) e^{i Phi0} / (G divisor) of
// the four waveform pairs, for the moment sums.  With h half the phase step
// (Phi+ - Phi-) / 2 and the mean phase offset of the pair second order in the
// step, a central pair is exactly (A+ - A-) cos h - i (A+ + A-) sin h; cos h and
// sin h / h by their series (h stays below 1e-2 for the steps used).  A
// one-sided pair (eta at 1/4, + the centre) is A0 - A- e^{2ih}.
template <typename T>
GW_HD bool fisher_bin_q(const FisherSrc &F, int n, double t, double r, double lnn, double t34, double m76,
                        float m76f, T &a0, T *qr, T *qi) {
  if (n > F.n_cut_any) return false;
  const double amp0 = wave64_amp(F.w0, n, t, m76);
  a0 = (T)amp0;
  for (int q = 0; q < kIntr; q++) {
    if (F.exact[q] || amp0 == 0.0 || n > F.wp[q].n_cut || n > F.wm[q].n_cut) {
      fisher_q_exact(F, q, n, t, r, lnn, t34, m76, qr[q], qi[q]);
      continue;
    }
    const T damp = fisher_amp_deriv<T>(F, q, n, t, m76, m76f);      // (A+ - A-) / divisor
    const double dph = fisher_phase_deriv(F, q, n, t, r, lnn, t34);  // (Phi+ - Phi-) / divisor
    const double h = 0.5 * dph * F.div[7 + q];
    const double h2 = h * h;
    if (!F.onesided[q]) {
      qr[q] = damp * (T)(1.0 - h2 * (0.5 - h2 * (1.0 / 24.0)));
      qi[q] = (T)(-amp0 * dph * (1.0 - h2 * ((1.0 / 6.0) - h2 * (1.0 / 120.0))));
    } else {
      const double am = amp0 - (double)damp * F.div[7 + q];
      double s2, c2;
      sincos(2.0 * h, &s2, &c2);
      qr[q] = (T)((amp0 - am * c2) * F.idiv[q]);
      qi[q] = (T)(-am * s2 * F.idiv[q]);
    }
  }
  return true;
}
GW_HD void fisher_accumulate(float wh, float a0, float fk, const float *qr, const float *qi, KSum *A) {
  float wa2 = wh * a0 * a0;
  kadd(A[0], wa2);
  kadd(A[1], wa2 * fk);
  kadd(A[2], wa2 * fk * fk);
  int o = 3;
  for (int i = 0; i < kIntr; i++)
    for (int j = i; j < kIntr; j++) kadd(A[o++], wh * (qr[i] * qr[j] + qi[i] * qi[j]));
  float wa = wh * a0;
  for (int i = 0; i < kIntr; i++) {
    kadd(A[13 + 4 * i + 0], wa * qr[i]);
    kadd(A[13 + 4 * i + 1], wa * qi[i]);
    kadd(A[13 + 4 * i + 2], wa * qr[i] * fk);
    kadd(A[13 + 4 * i + 3], wa * qi[i] * fk);
  }
}
// The same moment sums in FP64 (weights, differences and sums all FP64).
GW_HD void fisher_accumulate64(double wh, double a0, double fk, const double *qr, const double *qi, double *A) {
  const double wa2 = wh * a0 * a0;
  A[0] += wa2;
  A[1] += wa2 * fk;
  A[2] += wa2 * fk * fk;
  int o = 3;
  for (int i = 0; i < kIntr; i++)
    for (int j = i; j < kIntr; j++) A[o++] += wh * (qr[i] * qr[j] + qi[i] * qi[j]);
  const double wa = wh * a0;
  for (int i = 0; i < kIntr; i++) {
    A[13 + 4 * i + 0] += wa * qr[i];
    A[13 + 4 * i + 1] += wa * qi[i];
    A[13 + 4 * i + 2] += wa * qr[i] * fk;
    A[13 + 4 * i + 3] += wa * qi[i] * fk;
  }
}
// FP64 assembly of Gamma from the moment sums Ssum[w * kSums + j] of each
// weight stream; wscale[w] * ratio restores the whitening scale and the
// Simpson step of calculate_fisher_elements (fisher.cpp:2704-2781).
GW_HDNI void fisher_assemble(const FisherSrc &F, const double *Ssum, int ndet, const int *wslot, const double *wscale,
                         double ratio, double *Gm) {
  for (int j = 0; j < kDim * kDim; j++) Gm[j] = 0;
  const double A0 = F.w0.A_scale;
  for (int d = 0; d < ndet; d++) {
    const int w = wslot[d];
    const double *Sv = Ssum + w * kSums;
    const double c = A0 * A0 * wscale[w] * ratio;
    const double M0 = Sv[0], M1 = Sv[1], M2 = Sv[2];
    const double gr = F.G0re[d], gi = F.G0im[d], g2 = gr * gr + gi * gi;
    // cheap x cheap
    for (int i = 0; i < kCheap; i++)
      for (int j = 0; j <= i; j++) {
        double aiR = F.ar[d][i], aiI = F.ai[d][i], biR = F.br[d][i], biI = F.bi[d][i];
        double ajR = F.ar[d][j], ajI = F.ai[d][j], bjR = F.br[d][j], bjI = F.bi[d][j];
        double t0 = aiR * ajR + aiI * ajI;                            // Re(a_i a_j*)
        double t1 = (aiR * bjR + aiI * bjI) + (biR * ajR + biI * ajI);  // Re(a_i b_j* + b_i a_j*)
        double t2 = biR * bjR + biI * bjI;
        Gm[i * kDim + j] += c * (t0 * M0 + t1 * M1 + t2 * M2);
      }
    // intrinsic x intrinsic
    int o = 3;
    for (int ii = 0; ii < kIntr; ii++)
      for (int jj = ii; jj < kIntr; jj++) {
        double val = c * g2 * Sv[o++];
        int I = 7 + jj, J = 7 + ii;  // I >= J
        Gm[I * kDim + J] += val;
      }
    // intrinsic x cheap: Re[G conj(a_j) S_i + G conj(b_j) T_i]
    for (int ii = 0; ii < kIntr; ii++) {
      double Sr = Sv[13 + 4 * ii], Si = Sv[14 + 4 * ii], Tr = Sv[15 + 4 * ii], Ti = Sv[16 + 4 * ii];
      for (int j = 0; j < kCheap; j++) {
        double ajR = F.ar[d][j], ajI = F.ai[d][j], bjR = F.br[d][j], bjI = F.bi[d][j];
        // G conj(a_j) = (gr + i gi)(ajR - i ajI)
        double car = gr * ajR + gi * ajI, cai = gi * ajR - gr * ajI;
        double cbr = gr * bjR + gi * bjI, cbi = gi * bjR - gr * bjI;
        double val = (car * Sr - cai * Si) + (cbr * Tr - cbi * Ti);
        Gm[(7 + ii) * kDim + j] += c * val;
      }
    }
  }
  // log factor of M_c (parameter 7) on the intrinsic block
  if (F.logf[7]) {
    for (int j = 0; j < kDim; j++) {
      if (j == 7) Gm[7 * kDim + 7] *= F.v[7] * F.v[7];
      else if (j < 7) Gm[7 * kDim + j] *= F.v[7];
      else Gm[j * kDim + 7] *= F.v[7];
    }
  }
  for (int i = 0; i < kDim; i++)
    for (int j = 0; j < i; j++) Gm[j * kDim + i] = Gm[i * kDim + j];
}

}  // namespace gwf
