// phenom_mixed.h -- mixed-precision per-bin evaluation of the extrinsic
// log-likelihood (host and device).
//
// Same quantity as MCMC_likelihood_extrinsic (mcmc_gw.cpp:2374-2487) on a
// uniform grid f_n = n * df (n = n0 + k, integer), regrouped so that:
//  * the smooth PN/intermediate/ringdown phase stays FP64, evaluated as
//    polynomials in per-bin table values n^(1/3), n^(-5/3), ln n, n^(3/4)
//    that are shared by every request (no FP64 transcendental per bin);
//  * every phase term linear in f (2 pi f t_c, phi_c, detector delays, the
//    Pv2 time shift) is an exact 64-bit fixed-point count of turns;
//  * amplitude, antenna projection and the data products are FP32, with
//    per-request constants (A0, |G_d|^2, data scales) factored out and applied
//    in FP64 at the end, and Kahan-compensated FP32 sums.
#pragma once

#include "phenom_bins.h"
#include "segment_basis.h"

#if !defined(__CUDA_ARCH__)
#include <cmath>
#endif

namespace gwt {

// Per-bin tables indexed by n (shared by all requests on grids with integer n0).
struct Tables {
  const double *t13;   // n^(1/3)
  const double *tm53;  // n^(-5/3)
  const double *tln;   // ln n
  const double *t34;   // n^(3/4)
  const float *t13f;   // n^(1/3)
  const float *tm76f;  // n^(-7/6)
  int nmax;            // tables valid for 1 <= n <= nmax
};

// One detector stream of a registered grid, prepared for the mixed form:
// dhat = W d / dscale (complex64), what = W / wscale with the Simpson-weighted
// whitening W_k = (4 df/3) s_k / S_k (mcmc_gw.cpp:811-868, util.h:844-856).
struct MixedStream {
  const float *dhat;  // interleaved (re, im)
  const float *what;
  double dscale, wscale;
};

struct MixedDet {
  uint64_t L0, L1;   // linear phase, turns * 2^64: L0 + L1 * n
  double Gre, Gim;   // D: F+ (1+c^2)/2, -Fx c ; Pv2: P_d, Q_d (real); applied in FP64 at the end
};

constexpr int kAccPerDet = 5;  // D uses 2 (hh, Re z); Pv2 uses 5 (spp, scc, spc, zp, zc)
constexpr float kSegFScale = 268435456.0f;  // FP32 part of a segment phase polynomial: turns * 2^28

struct MixedReq {
  int approximant, status, ndet;
  int wshared;  // every detector has the same whitening weights: the weighted |h|^2 sums are kept for detector 0 only
  int n_f1, n_f3, n_f1p, n_f2p, n_cut;  // region starts (first n in region) and last non-zero n
  int n_mid, n_rd, n_c, pad2;
  double A_scale;                       // amplitude scale applied in FP64
  // phase, FP64
  double qi[12];                        // inspiral: tm53 * sum qi_j t^j + tln * (bi0 + bi1 t)
  double bi0, bi1;
  double pA, pB, pC, pD;                // intermediate: pA + pB n + pC tln - pD n^-3
  double mA, mB, mC, mD, mE;            // ringdown: mA + mB n - mC/n + mD n^(3/4) + mE atan(y)
  // amplitude, FP32
  // Per-request FP32 coefficients are stored as hi + lo pairs so that their
  // rounding does not bias every bin the same way.
  float ai[10], ai_lo[10];              // inspiral: sum ai_j t^j
  float ei[5], ei_lo[5];                // intermediate: sum ei_j (n - n_mid)^j
  float mrK, mrK_lo, mrExp, mrExp_lo;   // ringdown: mrK exp(-mrExp x) / (x^2 + mrG2), x = n - n_rd - frac
  float mrG2, mrG2_lo, mrRDfrac;
  float mEq;                            // mE in the segment polynomials' FP32 units (turns * 2^28)
  float ncfrac, inv_nw;                 // atan argument y = (n - n_c - ncfrac) * inv_nw
  // Pv2
  double ea[6], ee[6];                  // alpha/epsilon: r*(a0 t^2 + a1 n + a2 n t) + a3 + a4 t + a5 tln
  float Y[5], Y_lo[5];
  // 1/s = (w0 + w1 x + w2 x^2)/sqrt(x) + w3 with x = x2c t^2 (L2PN, WignerD)
  float w[4], w_lo[4];
  float x2c, x2c_lo;
  MixedDet det[kMaxDet];
  // log L = sum_j fc[j] * S[j] over the accumulated sums S[d * kAccPerDet + j]
  // (the FP64 amplitude scale, projection and whitening factors of each detector)
  double fc[kMaxDet * kAccPerDet];
};

// FP64 coefficients of the amplitude and phase of one request on a grid
// f_n = n df, as polynomials in the per-bin tables (shared by the mixed form,
// which rounds them to FP32 hi/lo pairs, and by the Fisher, which keeps FP64).
struct WaveF64 {
  int n_f1, n_f3, n_f1p, n_f2p, n_cut, n_mid;
  double A_scale;                 // A0eff (M df)^(-7/6), times 1/2 for Pv2
  double qi[12], bi0, bi1;        // inspiral phase
  double pA, pB, pC, pD;          // intermediate phase
  double mA, mB, mC, mD, mE;      // ringdown phase (atan term: mE atan((n - nc) inv_nw))
  double nc, inv_nw;
  double ai[10];                  // inspiral amplitude, polynomial in t = n^(1/3)
  double ei[5];                   // intermediate amplitude, polynomial in n - n_mid
  double mrK, mrExp, mrG2, nrd;   // ringdown amplitude: mrK exp(-mrExp x)/(x^2 + mrG2), x = n - nrd
  double tcl, fref, phic;         // linear phase: - tcl (f - fref) - phic
};

// First grid index n >= 0 with n df >= fb (strict: n df > fb), clamped to
// 2e9 for NaN or out-of-range boundaries.  ceil(fb / df) is within a step of
// the answer, so each correction loop runs at most a few times.
GW_HD int grid_first(double fb, double df, bool strict) {
  double q = ceil(fb / df);
  if (!(q < 2.0e9)) return 2000000000;
  int n = q > 0 ? (int)q : 0;
  auto ok = [&](int m) { return strict ? (double)m * df > fb : (double)m * df >= fb; };
  for (int it = 0; it < 4 && n > 0 && ok(n - 1); it++) n--;
  for (int it = 0; it < 4 && !ok(n) && n < 2000000000; it++) n++;
  return n;
}

GW_HDNI void wave64_prologue(const Request &r, double df, WaveF64 &x) {
  const ModelD &m = r.m;
  const Source &s = m.s;
  const double M = s.M, Mdf = M * df;
  x.n_f1 = grid_first(s.f1, df, false);          // amp: f < f1 inspiral
  x.n_f1p = grid_first(s.f1_phase, df, false);   // phase: f < f1_phase inspiral
  x.n_f3 = grid_first(s.f3, df, true);           // amp: f > f3 ringdown
  x.n_f2p = grid_first(s.f2_phase, df, true);
  x.n_cut = grid_first(m.fcut, df, true) - 1;    // last n with n df <= fcut
  const bool pv2 = (r.approximant == kPhenomPv2);
  x.A_scale = m.A0eff * pow_m7_6(Mdf) * (pv2 ? 0.5 : 1.0);
  const double cu = cbrt(Mdf), iMdf = 1. / Mdf;
  const double K = s.k_tf2 * m.pi.PIminus_5third;
  const double *pn = m.pn_phase;
  const double Lc = log(kPi * Mdf);
  double q[12];
  q[0] = K * pn[0];
  q[1] = K * pn[1] * m.pi.PIthird;
  q[2] = K * pn[2] * m.pi.PI2third;
  q[3] = K * pn[3] * kPi;
  q[4] = K * pn[4] * m.pi.PI4third;
  q[5] = K * m.pi.PI5third * (pn[8] + pn[9] * Lc) - kPi / 4.;
  q[6] = K * m.pi.PIsquare * (pn[10] - pn[11] * Lc);
  q[7] = K * pn[7] * m.pi.PI7third;
  q[8] = m.l.sigma[1] * s.inv_eta;
  q[9] = (3. / 4.) * m.l.sigma[2] * s.inv_eta;
  q[10] = (3. / 5.) * m.l.sigma[3] * s.inv_eta;
  q[11] = (1. / 2.) * m.l.sigma[4] * s.inv_eta;
  double cp = 1.0 / ((cu * cu) * (cu * cu) * cu);  // cu^-5
  for (int j = 0; j < 12; j++) {
    x.qi[j] = q[j] * cp;
    cp *= cu;
  }
  x.bi0 = K * m.pi.PI5third * pn[9];
  x.bi1 = -K * m.pi.PIsquare * pn[11] * cu;
  x.pA = (m.l.beta[0] + m.l.beta[2] * (Lc - kLnPi)) * s.inv_eta;  // ln(M df)
  x.pB = m.l.beta[1] * Mdf * s.inv_eta;
  x.pC = m.l.beta[2] * s.inv_eta;
  x.pD = m.l.beta[3] * s.inv_eta * ((1. / 3.) * (iMdf * iMdf * iMdf));
  x.mA = m.l.alpha[0] * s.inv_eta;
  x.mB = m.l.alpha[1] * Mdf * s.inv_eta;
  x.mC = m.l.alpha[2] * s.inv_eta * iMdf;
  x.mD = (4. / 3.) * m.l.alpha[3] * sqrt(Mdf * sqrt(Mdf)) * s.inv_eta;
  x.mE = m.l.alpha[4] * s.inv_eta;
  x.nc = m.l.alpha[5] * s.fRD / df;
  x.inv_nw = df / s.fdamp;
  {
    const double *pa = m.pn_amp;
    double a[10] = {pa[0], pa[1] * m.pi.PIthird, pa[2] * m.pi.PI2third, pa[3] * kPi, pa[4] * m.pi.PI4third,
                    pa[5] * m.pi.PI5third, pa[6] * m.pi.PIsquare, m.l.rho[0], m.l.rho[1], m.l.rho[2]};
    double c = 1.0;
    for (int j = 0; j < 10; j++) {
      x.ai[j] = a[j] * c;
      c *= cu;
    }
  }
  {
    double h = floor(0.5 * (s.f1 + s.f3) / df);
    x.n_mid = (int)h;
    const double *d = m.deltas;
    double c0 = d[0], c1 = d[1] * Mdf, c2 = d[2] * Mdf * Mdf, c3 = d[3] * Mdf * Mdf * Mdf,
           c4 = d[4] * Mdf * Mdf * Mdf * Mdf;
    x.ei[4] = c4;
    x.ei[3] = c3 + 4 * c4 * h;
    x.ei[2] = c2 + 3 * c3 * h + 6 * c4 * h * h;
    x.ei[1] = c1 + 2 * c2 * h + 3 * c3 * h * h + 4 * c4 * h * h * h;
    x.ei[0] = c0 + c1 * h + c2 * h * h + c3 * h * h * h + c4 * h * h * h * h;
  }
  {
    double g1 = m.l.gamma[0], g2 = m.l.gamma[1], g3 = m.l.gamma[2];
    x.nrd = s.fRD / df;
    double w = g3 * s.fdamp / df;
    x.mrK = g1 * g3 * s.fdamp / (M * df * df);
    x.mrExp = g2 / w;
    x.mrG2 = w * w;
  }
  x.tcl = m.tcl;
  x.fref = m.fref;
  x.phic = m.phic;
}

// FP64 amplitude / A_scale and nonlinear phase at bin n (tables: t = n^(1/3),
// r = n^(-5/3), lnn = ln n, t34 = n^(3/4), m76 = n^(-7/6)).
// Amplitude of bin n alone (0 beyond the cut).
GW_HD double wave64_amp(const WaveF64 &x, int n, double t, double m76) {
  if (n > x.n_cut) return 0.0;
  double a;
  if (n < x.n_f1) {
    a = x.ai[9];
    for (int j = 8; j >= 0; j--) a = a * t + x.ai[j];
  } else if (n >= x.n_f3) {
    double xx = (double)n - x.nrd;
    a = x.mrK * exp(-x.mrExp * xx) / (xx * xx + x.mrG2);
  } else {
    double h = (double)(n - x.n_mid);
    a = (((x.ei[4] * h + x.ei[3]) * h + x.ei[2]) * h + x.ei[1]) * h + x.ei[0];
  }
  return a * m76;
}
// Phase of bin n alone (0 beyond the cut).
GW_HD double wave64_phase(const WaveF64 &x, int n, double t, double r, double lnn, double t34) {
  if (n > x.n_cut) return 0.0;
  double nd = (double)n;
  if (n < x.n_f1p) {
    double p = x.qi[11];
    for (int j = 10; j >= 0; j--) p = p * t + x.qi[j];
    return r * p + lnn * (x.bi0 + x.bi1 * t);
  }
  if (n >= x.n_f2p) return x.mA + x.mB * nd - x.mC * (r * t * t) + x.mD * t34 + x.mE * atan((nd - x.nc) * x.inv_nw);
  return x.pA + x.pB * nd + x.pC * lnn - x.pD * (r * r * t);
}
GW_HD void wave64_eval(const WaveF64 &x, int n, double t, double r, double lnn, double t34, double m76, double &amp,
                       double &phi) {
  amp = wave64_amp(x, n, t, m76);
  phi = wave64_phase(x, n, t, r, lnn, t34);
}
// A+ s+ - A- s- of the waveforms of a central difference at bin n (s: the
// amplitude scales relative to the centre).  Where both are in the ringdown
// amplitude region the difference is A- s- expm1(L) with L = ln(A+ s+ / (A- s-))
// = lk - (e+ x+ - e- x-) + ln(d- / d+) assembled from small differences
// (lk = ln(K+ s+ / (K- s-)) per source, x = n - n_rd, d = x^2 + G): one FP64
// exp and one division instead of two.
GW_HD double wave64_amp_diff(const WaveF64 &p, const WaveF64 &m, int n, double t, double m76, double sp, double sm,
                             double lk) {
  if (n >= p.n_f3 && n >= m.n_f3 && n <= p.n_cut && n <= m.n_cut) {
    const double xm = (double)n - m.nrd, xp = (double)n - p.nrd;
    const double dm = xm * xm + m.mrG2, dp = xp * xp + p.mrG2;
    const double u = ((p.nrd - m.nrd) * (xm + xp) + (m.mrG2 - p.mrG2)) / dp;  // (d- - d+) / d+
    const double L = lk - (p.mrExp * (m.nrd - p.nrd) + (p.mrExp - m.mrExp) * xm) +
                     u * (1.0 - u * (0.5 - u * (1.0 / 3.0)));  // log1p(u) to u^3
    if (fabs(u) < 1e-4 && fabs(L) < 1e-4) {
      const double am = m.mrK * exp(-m.mrExp * xm) / dm * m76;
      return am * sm * (L * (1.0 + L * (0.5 + L * (1.0 / 6.0))));  // expm1(L) to L^3
    }
  }
  return wave64_amp(p, n, t, m76) * sp - wave64_amp(m, n, t, m76) * sm;
}
// (phase+ - phic+) - (phase- - phic-) of the waveforms of a central
// difference at bin n.  Where both are in the ringdown region their atan terms
// are combined, mE+ atan(y+) - mE- atan(y-) = mE+ atan((y+ - y-)/(1 + y+ y-))
// + (mE+ - mE-) atan(y-): one FP64 atan instead of two, the first by its
// series (argument below 1e-3: y+ and y- differ by the step).
GW_HD double wave64_phase_diff(const WaveF64 &p, const WaveF64 &m, int n, double t, double r, double lnn,
                               double t34) {
  if (n >= p.n_f2p && n >= m.n_f2p && n <= p.n_cut && n <= m.n_cut) {
    const double nd = (double)n;
    const double yp = (nd - p.nc) * p.inv_nw, ym = (nd - m.nc) * m.inv_nw;
    const double z = (yp - ym) / (1.0 + yp * ym);
    if (fabs(z) < 1e-3) {
      const double z2 = z * z;
      const double datan = z * (1.0 - z2 * ((1.0 / 3.0) - z2 * 0.2));  // atan z to z^5
      const double rtt = r * t * t;
      const double bp = p.mA + p.mB * nd - p.mC * rtt + p.mD * t34;
      const double bm = m.mA + m.mB * nd - m.mC * rtt + m.mD * t34;
      return ((bp - p.phic) - (bm - m.phic)) + (p.mE * datan + (p.mE - m.mE) * atan(ym));
    }
  }
  return (wave64_phase(p, n, t, r, lnn, t34) - p.phic) - (wave64_phase(m, n, t, r, lnn, t34) - m.phic);
}

GW_HD void split_f(double v, float &hi, float &lo) {
  hi = (float)v;
  lo = (float)(v - (double)hi);
}

// Q64 turns helpers
GW_HD uint64_t turns_q64(double turns) {  // frac(turns) * 2^64
  double fr = turns - floor(turns);
  double v = fr * 18446744073709551616.0;
  if (v >= 18446744073709551616.0) return 0;
  return (uint64_t)v;
}

// Build the mixed constants of one request for a grid with spacing df and
// integer offset (f_n = n df).  Returns the status of the prologue.
// The mixed constants in parts (regions and scale, phase, amplitude, Pv2
// angles, detectors) so that the cooperative prologue can spread them over
// warps; mixed_prologue runs them in order.
// amplitude scale: A0eff * (M df)^(-7/6) [* 1/2 for the Pv2 amp/2]
GW_HD double mixed_a_scale(const Request &r, double df) {
  return r.m.A0eff * pow_m7_6(r.m.s.M * df) * (r.approximant == kPhenomPv2 ? 0.5 : 1.0);
}
GW_HD void mixed_regions(const Request &r, double df, MixedReq &x) {
  const ModelD &m = r.m;
  const Source &s = m.s;
  x.approximant = r.approximant;
  x.status = m.status;
  x.ndet = r.ndet;
  // region starts in n: first n with n*df >= boundary (strict "<" tests of build_amp/build_phase)
  x.n_f1 = grid_first(s.f1, df, false);          // amp: f < f1 inspiral
  x.n_f1p = grid_first(s.f1_phase, df, false);   // phase: f < f1_phase inspiral
  x.n_f3 = grid_first(s.f3, df, true);           // amp: f > f3 ringdown
  x.n_f2p = grid_first(s.f2_phase, df, true);
  x.n_cut = grid_first(m.fcut, df, true) - 1;    // last n with n df <= fcut
  x.A_scale = mixed_a_scale(r, df);
}
GW_HD void mixed_phase_coeffs(const Request &r, double df, MixedReq &x) {
  const ModelD &m = r.m;
  const Source &s = m.s;
  const double M = s.M, eta = s.eta, Mdf = M * df;
  (void)M;
  (void)eta;
  (void)Mdf;
  // ---------------- inspiral phase: u = (M f)^(1/3) = cu t, t = n^(1/3)
  const double cu = cbrt(Mdf), iMdf = 1. / Mdf;
  const double K = s.k_tf2 * m.pi.PIminus_5third;
  const double *pn = m.pn_phase;
  const double Lc = log(kPi * Mdf);  // ln(pi M f) = Lc + ln n
  double q[12];
  q[0] = K * pn[0];
  q[1] = K * pn[1] * m.pi.PIthird;
  q[2] = K * pn[2] * m.pi.PI2third;
  q[3] = K * pn[3] * kPi;
  q[4] = K * pn[4] * m.pi.PI4third;
  q[5] = K * m.pi.PI5third * (pn[8] + pn[9] * Lc) - kPi / 4.;
  q[6] = K * m.pi.PIsquare * (pn[10] - pn[11] * Lc);
  q[7] = K * pn[7] * m.pi.PI7third;
  q[8] = m.l.sigma[1] * s.inv_eta;
  q[9] = (3. / 4.) * m.l.sigma[2] * s.inv_eta;
  q[10] = (3. / 5.) * m.l.sigma[3] * s.inv_eta;
  q[11] = (1. / 2.) * m.l.sigma[4] * s.inv_eta;
  double cp = 1.0 / ((cu * cu) * (cu * cu) * cu);  // cu^-5
  for (int j = 0; j < 12; j++) {
    x.qi[j] = q[j] * cp;
    cp *= cu;
  }
  x.bi0 = K * m.pi.PI5third * pn[9];
  x.bi1 = -K * m.pi.PIsquare * pn[11] * cu;
  // ---------------- intermediate phase
  x.pA = (m.l.beta[0] + m.l.beta[2] * (Lc - kLnPi)) * s.inv_eta;  // ln(M df)
  x.pB = m.l.beta[1] * Mdf * s.inv_eta;
  x.pC = m.l.beta[2] * s.inv_eta;
  x.pD = m.l.beta[3] * s.inv_eta * ((1. / 3.) * (iMdf * iMdf * iMdf));
  // ---------------- ringdown phase
  x.mA = m.l.alpha[0] * s.inv_eta;
  x.mB = m.l.alpha[1] * Mdf * s.inv_eta;
  x.mC = m.l.alpha[2] * s.inv_eta * iMdf;
  x.mD = (4. / 3.) * m.l.alpha[3] * sqrt(Mdf * sqrt(Mdf)) * s.inv_eta;
  x.mE = m.l.alpha[4] * s.inv_eta;
  x.mEq = (float)(x.mE * (1.0 / (2.0 * 3.14159265358979323846)) * kSegFScale);
  {
    double nc = m.l.alpha[5] * s.fRD / df;
    double nci = floor(nc);
    x.n_c = (int)nci;
    x.ncfrac = (float)(nc - nci);
    x.inv_nw = (float)(df / s.fdamp);
  }
}
GW_HD void mixed_amp_coeffs(const Request &r, double df, MixedReq &x) {
  const ModelD &m = r.m;
  const Source &s = m.s;
  const double M = s.M, Mdf = M * df;
  const double cu = cbrt(Mdf);
  // ---------------- inspiral amplitude: sum_i pn_i (pi M f)^(i/3) + rho (Mf)^(7..9)/3
  {
    const double *pa = m.pn_amp;
    double a[10];
    a[0] = pa[0];
    a[1] = pa[1] * m.pi.PIthird;
    a[2] = pa[2] * m.pi.PI2third;
    a[3] = pa[3] * kPi;
    a[4] = pa[4] * m.pi.PI4third;
    a[5] = pa[5] * m.pi.PI5third;
    a[6] = pa[6] * m.pi.PIsquare;
    a[7] = m.l.rho[0];
    a[8] = m.l.rho[1];
    a[9] = m.l.rho[2];
    double c = 1.0;
    for (int j = 0; j < 10; j++) {
      split_f(a[j] * c, x.ai[j], x.ai_lo[j]);
      c *= cu;
    }
  }
  // ---------------- intermediate amplitude: quartic in Mf re-centred on n_mid
  {
    double nmid = floor(0.5 * (s.f1 + s.f3) / df);
    x.n_mid = (int)nmid;
    const double *d = m.deltas;
    double c0 = d[0], c1 = d[1] * Mdf, c2 = d[2] * Mdf * Mdf, c3 = d[3] * Mdf * Mdf * Mdf,
           c4 = d[4] * Mdf * Mdf * Mdf * Mdf;  // polynomial in n
    double h = nmid;  // p(n) = sum c_j n^j = sum e_j (n - h)^j
    split_f(c4, x.ei[4], x.ei_lo[4]);
    split_f(c3 + 4 * c4 * h, x.ei[3], x.ei_lo[3]);
    split_f(c2 + 3 * c3 * h + 6 * c4 * h * h, x.ei[2], x.ei_lo[2]);
    split_f(c1 + 2 * c2 * h + 3 * c3 * h * h + 4 * c4 * h * h * h, x.ei[1], x.ei_lo[1]);
    split_f(c0 + c1 * h + c2 * h * h + c3 * h * h * h + c4 * h * h * h * h, x.ei[0], x.ei_lo[0]);
  }
  // ---------------- ringdown amplitude: g1 g3 fdamp M exp(-g2 (f-fRD)/(g3 fdamp)) / (M^2 ((f-fRD)^2 + (g3 fdamp)^2))
  {
    double g1 = m.l.gamma[0], g2 = m.l.gamma[1], g3 = m.l.gamma[2];
    double nrd = s.fRD / df, nrdi = floor(nrd);
    x.n_rd = (int)nrdi;
    x.mrRDfrac = (float)(nrd - nrdi);
    double w = g3 * s.fdamp / df;  // in bins
    split_f(g1 * g3 * s.fdamp / (M * df * df), x.mrK, x.mrK_lo);
    split_f(g2 / w, x.mrExp, x.mrExp_lo);
    split_f(w * w, x.mrG2, x.mrG2_lo);
  }
}
GW_HD void mixed_pv2_coeffs(const Request &r, double df, MixedReq &x) {
  const ModelD &m = r.m;
  const Source &s = m.s;
  const double M = s.M, eta = s.eta, Mdf = M * df;
  (void)M;
  (void)eta;
  (void)Mdf;
  // ---------------- Pv2 angles
  {
    double cw = cbrt(kPi * Mdf);  // omega^(1/3) = cw t
    const double *a = r.p.ac, *e = r.p.ec;
    double Lw = log(kPi * Mdf);
    // alpha = a0/w + a1/w^(2/3) + a2/w^(1/3) + a3 ln w + a4 w^(1/3); w = pi Mdf n
    // with r = n^(-5/3): 1/n = r t^2, n^(-2/3) = r n, n^(-1/3) = r n t
    x.ea[0] = a[0] / (kPi * Mdf);
    x.ea[1] = a[1] / (cw * cw);
    x.ea[2] = a[2] / cw;
    x.ea[3] = a[3] * Lw + r.p.alpha_shift;
    x.ea[4] = a[4] * cw;
    x.ea[5] = a[3];
    x.ee[0] = e[0] / (kPi * Mdf);
    x.ee[1] = e[1] / (cw * cw);
    x.ee[2] = e[2] / cw;
    x.ee[3] = e[3] * Lw - r.p.eps_off;
    x.ee[4] = e[4] * cw;
    x.ee[5] = e[3];
    for (int k = 0; k < 5; k++) split_f(r.p.Y[k], x.Y[k], x.Y_lo[k]);
    // s = SP / (L + SL), L = eta (1 + l1 x + l2 x^2) / sqrt(x)  ->  1/s
    double l1 = 1.5 + eta / 6.0, l2 = 3.375 - (19.0 * eta) / 8. - eta * eta / 24.0;
    split_f(eta / s.SP, x.w[0], x.w_lo[0]);
    split_f(eta * l1 / s.SP, x.w[1], x.w_lo[1]);
    split_f(eta * l2 / s.SP, x.w[2], x.w_lo[2]);
    split_f(s.SL / s.SP, x.w[3], x.w_lo[3]);
    split_f(cw * cw, x.x2c, x.x2c_lo);  // L2PN x = (pi M f)^(2/3) = cw^2 t^2
  }
}
// The complex antenna factor G_d of the response r_d = G_d h (D: the
// inclination factors of h+ and hx folded in; Pv2: the 2 zeta rotation).
GW_HD void mixed_det_G(const Request &r, int d, double &Gre, double &Gim) {
  if (r.approximant == kPhenomPv2) {
    Gre = r.det[d].fp * r.p.c2z - r.det[d].fc * r.p.s2z;
    Gim = r.det[d].fp * r.p.s2z + r.det[d].fc * r.p.c2z;
  } else {
    const double ci = r.m.s.cos_incl;
    Gre = r.det[d].fp * .5 * (1 + ci * ci);
    Gim = -r.det[d].fc * ci;
  }
}
// Detectors in two independent parts: the linear phases and projections
// (needs the time shift), and the finalize factors (needs the amplitude
// scale).
GW_HD void mixed_det_phase(const Request &r, double df, MixedReq &x) {
  const ModelD &m = r.m;
  const bool pv2 = (r.approximant == kPhenomPv2);
  // ---------------- linear phase per detector, in turns (f = n df):
  // D:   psi_d = phi(f) - tcl (f - fref) - phic - tau_d f
  // Pv2: psi_d = phi(f) + 2 eps(f) - tcl (f - fref) - phic + 2 pi t_corr f - tau_d f
  const double inv2pi = 1.0 / (2.0 * kPi);
  double c0 = (m.tcl * m.fref - m.phic) * inv2pi;
  double c1 = -m.tcl * df * inv2pi;
  if (pv2) c1 += r.p.t_corr * df;
  for (int d = 0; d < r.ndet; d++) {
    x.det[d].L0 = turns_q64(c0);
    x.det[d].L1 = turns_q64(c1 - r.det[d].tau * df * inv2pi);
    mixed_det_G(r, d, x.det[d].Gre, x.det[d].Gim);
    // D: DH_d = A ds Re(conj(G) S) = A ds |G| Re(e^{-i arg G} S): the phase of
    // conj(G) joins the detector's fixed-point linear phase, so the bins
    // accumulate Re(S) only and |G| is applied in FP64 (mixed_det_factors_a)
    if (!pv2) x.det[d].L0 -= turns_q64(atan2(x.det[d].Gim, x.det[d].Gre) * inv2pi);
  }
}
// A: the amplitude scale (x.A_scale, passed so that a caller that has just
// computed it need not read it back).
GW_HD void mixed_det_factors_a(const Request &r, MixedReq &x, double A, const double *dscale, const double *wscale) {
  const bool pv2 = (r.approximant == kPhenomPv2);
  for (int d = 0; d < r.ndet; d++) {
    // HH = A^2 w |G h|^2 sums, DH = A d Re(G ...) sums; log L = -HH/2 + DH
    double G1, G2;
    mixed_det_G(r, d, G1, G2);
    const double w = wscale[d], ds = dscale[d];
    double *f = x.fc + d * kAccPerDet;
    if (pv2) {
      f[0] = -0.5 * A * A * w * G1 * G1;
      f[1] = -0.5 * A * A * w * G2 * G2;
      f[2] = -A * A * w * G1 * G2;
      f[3] = A * ds * G1;
      f[4] = A * ds * G2;
    } else {  // the phase of conj(G) is in the detector's linear phase (mixed_det_phase)
      f[0] = -0.5 * A * A * w * (G1 * G1 + G2 * G2);
      f[1] = A * ds * sqrt(G1 * G1 + G2 * G2);
      f[2] = 0.0;
      f[3] = 0.0;
      f[4] = 0.0;
    }
  }
  for (int d = r.ndet; d < kMaxDet; d++)
    for (int j = 0; j < kAccPerDet; j++) x.fc[d * kAccPerDet + j] = 0.0;
}
// Detectors whose whitening weights are the same array (the same PSD on the
// same grid) have the same weighted |h|^2 sums: their HH factors are added to
// detector 0's and the bin kernels accumulate those sums once (wshared).
GW_HD void mixed_fold_shared_weights(MixedReq &x, const unsigned long long *wkey, int ndet) {
  bool same = ndet > 1;
  for (int d = 1; d < ndet; d++) same = same && wkey[d] == wkey[0];
  x.wshared = same ? 1 : 0;
  if (!same) return;
  const int nh = x.approximant == kPhenomPv2 ? 3 : 1;  // the weighted sums: D |h|^2; Pv2 |h+|^2, |hx|^2, h+ hx*
  for (int d = 1; d < ndet; d++)
    for (int j = 0; j < nh; j++) {
      x.fc[j] += x.fc[d * kAccPerDet + j];
      x.fc[d * kAccPerDet + j] = 0.0;
    }
}
GW_HD void mixed_det_factors(const Request &r, MixedReq &x, const double *dscale, const double *wscale) {
  mixed_det_factors_a(r, x, x.A_scale, dscale, wscale);
}
GW_HD void mixed_det_coeffs(const Request &r, double df, MixedReq &x, const double *dscale, const double *wscale) {
  mixed_det_phase(r, df, x);
  mixed_det_factors(r, x, dscale, wscale);
}
GW_HDNI int mixed_prologue(const Request &r, double df, MixedReq &x, const double *dscale, const double *wscale) {
  mixed_regions(r, df, x);
  mixed_phase_coeffs(r, df, x);
  mixed_amp_coeffs(r, df, x);
  if (r.approximant == kPhenomPv2) mixed_pv2_coeffs(r, df, x);
  mixed_det_coeffs(r, df, x, dscale, wscale);
  return x.status;
}

// ------------------------------------------------------------ per-bin math
#if defined(__CUDA_ARCH__)
GW_HD float __int_as_float_h(int i) { return __int_as_float(i); }
GW_HD int __float_as_int_h(float f) { return __float_as_int(f); }
GW_HD int64_t gw_llrint(double x) { return __double2ll_rn(x); }
GW_HD int gw_f2i_rn(float x) { return __float2int_rn(x); }
GW_HD float gw_rsqrt_rn(float x) { return __frsqrt_rn(x); }  // 1/sqrt(x), correctly rounded
#else
inline float __int_as_float_h(int i) {
  float f;
  std::memcpy(&f, &i, 4);
  return f;
}
inline int __float_as_int_h(float f) {
  int i;
  std::memcpy(&i, &f, 4);
  return i;
}
GW_HD int64_t gw_llrint(double x) { return (int64_t)std::llrint(x); }
GW_HD int gw_f2i_rn(float x) { return (int)std::lrintf(x); }
GW_HD float gw_rsqrt_rn(float x) { return (float)(1.0 / std::sqrt((double)x)); }
#endif

// Kahan-compensated FP32 accumulator: value = s - c.
struct KSum {
  float s, c;
};
GW_HD void kadd(KSum &k, float v) {
  float y = v - k.c;
  float t = k.s + y;
  k.c = (t - k.s) - y;
  k.s = t;
}

// Phase of the D model at bin n (FP64, radians), without the linear terms.
// with_atan: include the ringdown atan term, evaluated in FP32 (its
// coefficient is about 1 rad, so the FP32 error stays near 1e-7 rad); the
// segment nodes leave it out and the bins add it in FP32.
GW_HD float mixed_atan(const MixedReq &x, int n) {
  return atanf(((float)(n - x.n_c) - x.ncfrac) * x.inv_nw);
}
GW_HD double mixed_phase_d(const MixedReq &x, int n, double t, double r, double lnn, double t34,
                           bool with_atan = true) {
  if (n < x.n_f1p) {
    const double *q = x.qi;
    double p = q[11];
    for (int j = 10; j >= 0; j--) p = p * t + q[j];
    return r * p + lnn * (x.bi0 + x.bi1 * t);
  }
  double nd = (double)n;
  if (n >= x.n_f2p) {
    double ph = x.mA + x.mB * nd - x.mC * (r * t * t) + x.mD * t34;
    return with_atan ? ph + x.mE * (double)mixed_atan(x, n) : ph;
  }
  return x.pA + x.pB * nd + x.pC * lnn - x.pD * (r * r * t);
}
// Round hi + lo (|lo| < ulp(hi)) to FP32 stochastically with a per-bin
// low-discrepancy dither u in [0, 1): the expectation over bins is hi + lo,
// so the lo parts of per-request coefficients are not lost to round-to-nearest.
GW_HD float sround(float hi, float lo, uint32_t u) {
  float ahi = fabsf(hi);
  float ulp = __int_as_float_h(__float_as_int_h(ahi) + 1) - ahi;  // a power of two
  float fu = (float)(u >> 8) * 5.9604644775390625e-08f;            // 2^-24
  // fu < |lo| / ulp without the division: fu * ulp is exact (24-bit fu times
  // a power of two) for every amplitude above 2^-100
  return (fu * ulp < fabsf(lo)) ? hi + copysignf(ulp, lo) : hi;
}
GW_HD uint32_t dither(int n) { return (uint32_t)n * 2654435769u; }  // Weyl sequence, golden ratio

// Amplitude / (A_scale) at bin n, FP32: hi part plus the lo part carried by
// the hi/lo coefficient pairs, stochastically rounded.
GW_HD float mixed_amp(const MixedReq &x, int n, float tf, float m76) {
  float hi, lo;
  if (n < x.n_f1) {
    const float *c = x.ai, *cl = x.ai_lo;
    hi = c[9];
    lo = cl[9];
#pragma unroll
    for (int j = 8; j >= 0; j--) {
      hi = fmaf(hi, tf, c[j]);
      lo = fmaf(lo, tf, cl[j]);
    }
  } else if (n >= x.n_f3) {
    float xx = (float)(n - x.n_rd) - x.mrRDfrac;
    float iden = 1.0f / fmaf(xx, xx, x.mrG2);
    float e = expf(-x.mrExp * xx) * iden;
    hi = x.mrK * e;
    lo = e * (x.mrK_lo - x.mrK * (x.mrExp_lo * xx + x.mrG2_lo * iden));
  } else {
    float h = (float)(n - x.n_mid);
    const float *e = x.ei, *el = x.ei_lo;
    hi = e[4];
    lo = el[4];
#pragma unroll
    for (int j = 3; j >= 0; j--) {
      hi = fmaf(hi, h, e[j]);
      lo = fmaf(lo, h, el[j]);
    }
  }
  return sround(hi, lo, dither(n)) * m76;
}
GW_HD uint64_t phase_q64(double phase_rad) {  // radians -> turns * 2^64 (2^-32 turn resolution)
  const double k = 4294967296.0 / (2.0 * 3.14159265358979323846);
  return ((uint64_t)gw_llrint(phase_rad * k)) << 32;
}
// sin and cos of 2 pi q / 2^64 in FP32: the top two bits of q pick the
// nearest quarter turn exactly, the rest is an angle |x| <= pi/4 for the
// Taylor series of sin (to x^9) and cos (to x^10), whose truncation errors
// there are below 2e-9; the result is within about 1e-7 of sin/cos, unbiased.
GW_HD void q64_sincospi(uint64_t q, float *s, float *c) {
  const uint32_t u = (uint32_t)(q >> 32);
  const uint32_t quad = (u + 0x20000000u) >> 30;
  const int32_t r = (int32_t)(u - (quad << 30));
  const float x = (float)r * 1.4629180792671596e-09f;  // 2 pi / 2^32
  const float x2 = x * x;
  const float sn =
      x * fmaf(x2, fmaf(x2, fmaf(x2, fmaf(x2, 1.0f / 362880.0f, -1.0f / 5040.0f), 1.0f / 120.0f), -1.0f / 6.0f), 1.0f);
  const float cs = fmaf(
      x2, fmaf(x2, fmaf(x2, fmaf(x2, fmaf(x2, -1.0f / 3628800.0f, 1.0f / 40320.0f), -1.0f / 720.0f), 1.0f / 24.0f), -0.5f),
      1.0f);
  const bool odd = quad & 1u;
  const float ss = odd ? cs : sn, cc = odd ? sn : cs;
  *s = (quad & 2u) ? -ss : ss;
  *c = ((quad + 1u) & 2u) ? -cc : cc;
}

// FP64 phase of bin n (radians; Pv2: phase + 2 epsilon) and the Pv2 Euler
// angle alpha, from the per-bin power tables t = n^(1/3), r = n^(-5/3),
// lnn = ln n, t34 = n^(3/4).
GW_HD double mixed_pv2_alpha(const MixedReq &x, int n, double t, double r, double lnn) {
  double nd = (double)n;
  return r * (x.ea[0] * t * t + x.ea[1] * nd + x.ea[2] * nd * t) + x.ea[3] + x.ea[4] * t + x.ea[5] * lnn;
}
GW_HD double mixed_pv2_eps(const MixedReq &x, int n, double t, double r, double lnn) {
  double nd = (double)n;
  return r * (x.ee[0] * t * t + x.ee[1] * nd + x.ee[2] * nd * t) + x.ee[3] + x.ee[4] * t + x.ee[5] * lnn;
}
GW_HD double mixed_phase_full(const MixedReq &x, int n, double t, double r, double lnn, double t34,
                              bool with_atan = true) {
  double ph = mixed_phase_d(x, n, t, r, lnn, t34, with_atan);
  if (x.approximant == kPhenomPv2) ph += 2.0 * mixed_pv2_eps(x, n, t, r, lnn);
  return ph;
}

// ----------------------------------------------------- segment polynomials
// Over a segment of kSegBins consecutive bins the FP64 phase (and the Pv2
// angle alpha) is replaced by its degree-8 interpolant in u = m / 128,
// m = n - n_c, through nine FP64 node values.  The coefficients of m^0..m^4
// are carried as exact fixed-point turns (uint64, modulo one turn: integer m
// keeps every product exact), those of u^5..u^8 in FP32; per bin this costs
// integer multiply-adds and four FP32 FMAs instead of the FP64 series.  Two
// check points between the outermost node pairs bound the interpolation
// error; a segment that fails them, whose FP32 part is not small enough to
// keep FP32 rounding near 1e-9 rad, that straddles a phase region boundary or
// leaves the grid is evaluated per bin in FP64.  The ringdown atan term is
// not part of the nodes; the bins add it in FP32 (mixed_atan).
constexpr int kSegBins = 256, kSegHalf = 128;
constexpr int kSegNodes = GWT_SEG_NODES, kSegEval = GWT_SEG_NODES + GWT_SEG_CHECKS;
constexpr int kSegQ = 5;                     // m^0 .. m^4 in fixed point
constexpr int kSegF = kSegNodes - kSegQ;     // u^5 .. u^8 in FP32
constexpr double kSegTolRad = 1e-8;          // interpolation error allowed at the check points
constexpr double kSegFMaxTurns = 0.02;       // bound on the FP32 part (sum of |coefficients|)

struct SegPoly {
  uint64_t q[kSegQ];  // coefficient of m^j, turns * 2^64
  float f[kSegF];     // coefficient of u^(kSegQ + j), turns * 2^28
  int direct;         // 1: per-bin FP64 phase in this segment
  int pad;
};

GW_HD int seg_offset(int j) { return GWT_T(gwt_seg_offsets)[j]; }

// The fit in steps, parallel over (segment, coefficient) or segments in the
// kernel: (1) coefficient j >= 1 of u^j (radians) from the node values
// v[0..kSegEval) (v[4] is the centre; coefficient 0 is v[4]);
GW_HD double seg_coef(const double *v, int j) {
  if (j == 0) return 0.0;
  double s = 0.0;
  for (int k = 0; k < kSegNodes; k++) s += GWT_T(gwt_seg_vinv)[j][k] * (v[k] - v[4]);
  return s;
}
// (2) the acceptance test (check points, size of the FP32 part): 0 when usable;
GW_HD int seg_check(const double *v, const double *c) {
  for (int k = kSegNodes; k < kSegEval; k++) {
    double u = seg_offset(k) * (1.0 / kSegHalf), y = c[kSegNodes - 1];
    for (int j = kSegNodes - 2; j >= 0; j--) y = y * u + c[j];
    if (!(fabs(y - (v[k] - v[4])) <= kSegTolRad)) return 1;
  }
  double bound = 0.0;
  for (int j = kSegQ; j < kSegNodes; j++) bound += fabs(c[j]);
  return bound * (1.0 / (2.0 * 3.14159265358979323846)) < kSegFMaxTurns ? 0 : 1;
}
// (3) coefficient j in its stored form.
GW_HD void seg_store(const double *v, const double *c, int j, SegPoly &p) {
  const double inv2pi = 1.0 / (2.0 * 3.14159265358979323846);
  if (j < kSegQ) {
    double sc = 1.0;
    for (int i = 0; i < j; i++) sc *= (1.0 / kSegHalf);
    p.q[j] = turns_q64((j == 0 ? v[4] : c[j] * sc) * inv2pi);
  } else {
    p.f[j - kSegQ] = (float)(c[j] * inv2pi * kSegFScale);
  }
}
// Whole fit of one segment (host use); returns 0 when usable.
GW_HD int seg_fit(const double *v, SegPoly &p) {
  double c[kSegNodes];
  for (int j = 0; j < kSegNodes; j++) c[j] = seg_coef(v, j);
  if (seg_check(v, c)) return 1;
  for (int j = 0; j < kSegNodes; j++) seg_store(v, c, j, p);
  return 0;
}

// Whether the segment of bins [kseg, kseg + kSegBins) of a grid of N bins
// (n = n0 + k) can carry a polynomial: inside the grid, below the cut, and
// not across a phase region boundary.
GW_HD bool seg_usable(const MixedReq &x, int n0, int N, int kseg) {
  if (kseg < 0 || kseg + kSegBins > N) return false;
  const int nlo = n0 + kseg, nhi = nlo + kSegBins - 1;
  if (nlo > x.n_cut) return false;
  if (nlo < x.n_f1p && nhi >= x.n_f1p) return false;
  if (nlo < x.n_f2p && nhi >= x.n_f2p) return false;
  return true;
}
// Bin n of node j of the segment starting at kseg.
GW_HD int seg_node_n(int n0, int kseg, int j) { return n0 + kseg + kSegHalf + seg_offset(j); }

// Phase of bin m of a fitted segment, turns * 2^64; extra (turns * 2^28) is
// added to the FP32 part before its conversion.
GW_HD uint64_t seg_eval(const SegPoly &p, int m, float extra = 0.0f) {
  const uint64_t mm = (uint64_t)(int64_t)m;
  uint64_t acc = p.q[kSegQ - 1];
#pragma unroll
  for (int j = kSegQ - 2; j >= 0; j--) acc = acc * mm + p.q[j];
  const float u = (float)m * (1.0f / kSegHalf), u2 = u * u;
  float r = fmaf(fmaf(fmaf(p.f[3], u, p.f[2]), u, p.f[1]), u, p.f[0]);
  r = fmaf(r, u2 * u2 * u, extra);
  return acc + ((uint64_t)(int64_t)gw_f2i_rn(r) << 36);
}
// The FP32 ringdown atan term of bin n in the units of seg_eval's extra.
GW_HD float seg_atan_extra(const MixedReq &x, int n) {
  return x.mEq * mixed_atan(x, n);
}

// The detector's linear phase (L0 + L1 n, turns * 2^64) as a rotation, in
// two factors: at the first bin n_s of a segment pass (shared by the pass) and
// at the offset j = n - n_s (shared by the item).  Each factor is exact to
// FP32 (fixed-point reduction); their product adds one complex rounding.
GW_HD void det_rot_seg(const MixedReq &x, int d, int n_s, float &c, float &s) {
  q64_sincospi(x.det[d].L0 + x.det[d].L1 * (uint64_t)n_s, &s, &c);
}
GW_HD void det_rot_off(const MixedReq &x, int d, int j, float &c, float &s) {
  q64_sincospi(x.det[d].L1 * (uint64_t)j, &s, &c);
}
GW_HD void cmulf(float ac, float as, float bc, float bs, float &c, float &s) {
  c = ac * bc - as * bs;
  s = as * bc + ac * bs;
}

// IMRPhenomD bin: two sums per detector at acc[d * STRIDE + 0] (weighted
// |h|^2; once for all detectors when they share a weight stream) and
// acc[d * STRIDE + 1] (Re d* h e^{i phi_d}).
template <int NDET, int STRIDE>
GW_HD void mixed_bin_d(const MixedReq &x, int n, uint64_t ph, float tf, float m76, const float *dre, const float *dim,
                       const float *w, const float *rotc, const float *rots, KSum *acc, bool wshared) {
  if (n > x.n_cut) return;
  const float a = mixed_amp(x, n, tf, m76);
  float sp, cp;
  q64_sincospi(ph, &sp, &cp);
  const float aa = a * a;
#pragma unroll
  for (int d = 0; d < NDET; d++) {
    float sn, cs;
    cmulf(cp, sp, rotc[d], rots[d], cs, sn);
    float ar = a * dre[d], ai = a * dim[d];
    if (d == 0 || !wshared) kadd(acc[d * STRIDE + 0], w[d] * aa);
    kadd(acc[d * STRIDE + 1], ar * cs - ai * sn);  // Re(a dhat e^{i (phase + linear phase - arg G)})
  }
}
// IMRPhenomPv2 bin: five sums per detector at acc[d * kAccPerDet + j], with
// the Euler angle alpha in fixed-point turns.
template <int NDET>
GW_HD void mixed_bin_p(const MixedReq &x, int n, uint64_t ph, uint64_t al, float tf, float m76, const float *dre,
                       const float *dim, const float *w, const float *rotc, const float *rots, KSum *acc,
                       bool wshared) {
  if (n > x.n_cut) return;
  float a = mixed_amp(x, n, tf, m76);
  float sp, cp;
  q64_sincospi(ph, &sp, &cp);
  // Pv2: twist-up (FP32) with alpha from its fixed-point turns
  float sa, ca;
  q64_sincospi(al, &sa, &ca);
  // WignerD from L2PN (IMRPhenomP.cpp:665-693, 1214-1220)
  float tf2 = tf * tf;
  float xx = fmaf(x.x2c, tf2, x.x2c_lo * tf2);
  float rs = gw_rsqrt_rn(xx);
  float ph_ = fmaf(fmaf(x.w[2], xx, x.w[1]), xx, x.w[0]);
  float pl_ = fmaf(fmaf(x.w_lo[2], xx, x.w_lo[1]), xx, x.w_lo[0]);
  float us = sround(fmaf(ph_, rs, x.w[3]), fmaf(pl_, rs, x.w_lo[3]), dither(n) ^ 0x9e3779b9u);  // 1/s
  // sin beta = 1/sqrt(1 + us^2); cos beta = |us| sin beta >= 0, also when L + SL < 0
  float sb = gw_rsqrt_rn(fmaf(us, us, 1.0f));
  float cb = fabsf(us) * sb;
  // half angles: sin(beta/2) = sin beta / (2 cos(beta/2)), without the
  // cancellation of 1 - cos beta near beta = 0
  float yh = (1.0f + cb) * 0.5f, rcbh = gw_rsqrt_rn(yh);
  float cbh = yh * rcbh, sbh = 0.5f * sb * rcbh;
  float c2 = cbh * cbh, s2 = sbh * sbh;
  float d2[5] = {s2 * s2, 2.f * cbh * s2 * sbh, 2.44948974278317788f * s2 * c2, 2.f * c2 * cbh * sbh, c2 * c2};
  // exp(i m alpha), m = -2..2
  float e2r = ca * ca - sa * sa, e2i = 2.f * ca * sa;
  float er[5] = {e2r, ca, 1.f, ca, e2r}, ei[5] = {-e2i, -sa, 0.f, sa, e2i};
  float hpr = 0.f, hpi = 0.f, hcr = 0.f, hci = 0.f;
#pragma unroll
  for (int m = -2; m <= 2; m++) {
    float dm = (m == -1 || m == 1) ? -d2[2 - m] : d2[2 - m];  // dm2[m+2] = (-1)^m d2[2-m]
    float y = x.Y[m + 2], yl = x.Y_lo[m + 2];
    float a1 = fmaf(dm, y, dm * yl), a2 = fmaf(d2[m + 2], y, d2[m + 2] * yl);
    float t2r = er[-m + 2] * a1, t2i = ei[-m + 2] * a1;  // T2m
    float tmr = er[m + 2] * a2, tmi = ei[m + 2] * a2;    // Tm2m
    hpr += t2r + tmr;
    hpi += t2i + tmi;
    hcr += -(t2i - tmi);
    hci += (t2r - tmr);
  }
  float aa = a * a;
  float spp = aa * (hpr * hpr + hpi * hpi), scc = aa * (hcr * hcr + hci * hci), spc = aa * (hpr * hcr + hpi * hci);
#pragma unroll
  for (int d = 0; d < NDET; d++) {
    float sn, cs;
    cmulf(cp, sp, rotc[d], rots[d], cs, sn);
    // a * dhat * exp(i psi)
    float qr = a * (dre[d] * cs - dim[d] * sn), qi = a * (dre[d] * sn + dim[d] * cs);
    if (d == 0 || !wshared) {
      kadd(acc[d * kAccPerDet + 0], w[d] * spp);
      kadd(acc[d * kAccPerDet + 1], w[d] * scc);
      kadd(acc[d * kAccPerDet + 2], w[d] * spc);
    }
    kadd(acc[d * kAccPerDet + 3], qr * hpr + qi * hpi);  // Re(q conj(hpf))
    kadd(acc[d * kAccPerDet + 4], qr * hcr + qi * hci);  // Re(q conj(hcf))
  }
}

// One bin of the mixed form, accumulated into acc[d * kAccPerDet + j], with
// the phase ph (Pv2: phase + 2 epsilon) and the Pv2 angle al in turns * 2^64.
// dre/dim/w: the detector streams at this bin; rotc/rots: the detector's linear
// phase rotation at this bin (cos, sin).  The detector phase is the angle sum
// of ph and that rotation.
template <int NDET>
GW_HD void mixed_bin_q(const MixedReq &x, int n, uint64_t ph, uint64_t al, float tf, float m76, const float *dre,
                       const float *dim, const float *w, const float *rotc, const float *rots, KSum *acc,
                       bool wshared) {
  if (x.approximant != kPhenomPv2)
    mixed_bin_d<NDET, kAccPerDet>(x, n, ph, tf, m76, dre, dim, w, rotc, rots, acc, wshared);
  else
    mixed_bin_p<NDET>(x, n, ph, al, tf, m76, dre, dim, w, rotc, rots, acc, wshared);
}

// The per-bin FP64 path: phase and alpha of bin n in fixed-point turns.
GW_HD void mixed_phase_direct(const MixedReq &x, int n, double t, double r, double lnn, double t34, uint64_t &ph,
                              uint64_t &al) {
  ph = phase_q64(mixed_phase_full(x, n, t, r, lnn, t34));
  al = x.approximant == kPhenomPv2 ? phase_q64(mixed_pv2_alpha(x, n, t, r, lnn)) : 0;
}

// log L of one request from its FP64 accumulated sums s[d * kAccPerDet + j].
GW_HD double mixed_finalize(const MixedReq &x, const double *s) {
  double ll = 0;
  for (int j = 0; j < kMaxDet * kAccPerDet; j++) ll += x.fc[j] * s[j];
  return ll;
}

}  // namespace gwt
