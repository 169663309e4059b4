/* Test-only stand-in for ADOL-C's adouble, used solely so that the reference's
 * IMRPhenomD.cpp / IMRPhenomP.cpp translation units compile for the oracle pin
 * build (oracle/Makefile).  It wraps a double; no taping is done.  The pin
 * build runs only the double instantiations of the reference classes; the
 * counting build (GWO_COUNT_OPS) runs the adouble ones to count operations. */
#ifndef GWO_SHIM_ADOUBLE_H
#define GWO_SHIM_ADOUBLE_H
#include <cmath>
#include <complex>
#include <iostream>
#include <vector>
#include <string>
#ifdef GWO_COUNT_OPS
/* Operation counter for the algorithmic-work measurement (oracle/count_ops.cpp):
 * every arithmetic operator and elementary function on adouble increments a
 * per-kind counter. */
enum { GWO_ADD, GWO_MUL, GWO_DIV, GWO_SQRT, GWO_EXP, GWO_LOG, GWO_POW, GWO_SIN, GWO_COS, GWO_ATAN, GWO_CBRT,
       GWO_OTHER, GWO_NKINDS };
extern long long gwo_opcount[GWO_NKINDS];
#define GWO_CNT(k) (++gwo_opcount[k])
#else
#define GWO_CNT(k) ((void)0)
#endif
class adouble {
 public:
  double v;
  adouble() : v(0) {}
  adouble(double x) : v(x) {}
  double value() const { return v; }
  double getValue() const { return v; }
  adouble &operator<<=(double x) { v = x; return *this; }
  adouble &operator>>=(double &x) { x = v; return *this; }
  adouble &operator=(double x) { v = x; return *this; }
  adouble &operator+=(const adouble &o) { GWO_CNT(GWO_ADD); v += o.v; return *this; }
  adouble &operator-=(const adouble &o) { GWO_CNT(GWO_ADD); v -= o.v; return *this; }
  adouble &operator*=(const adouble &o) { GWO_CNT(GWO_MUL); v *= o.v; return *this; }
  adouble &operator/=(const adouble &o) { GWO_CNT(GWO_DIV); v /= o.v; return *this; }
  adouble operator-() const { return adouble(-v); }
  adouble operator+() const { return *this; }
};
inline adouble operator+(const adouble &a, const adouble &b) { GWO_CNT(GWO_ADD); return adouble(a.v + b.v); }
inline adouble operator-(const adouble &a, const adouble &b) { GWO_CNT(GWO_ADD); return adouble(a.v - b.v); }
inline adouble operator*(const adouble &a, const adouble &b) { GWO_CNT(GWO_MUL); return adouble(a.v * b.v); }
inline adouble operator/(const adouble &a, const adouble &b) { GWO_CNT(GWO_DIV); return adouble(a.v / b.v); }
inline adouble operator+(const adouble &a, double b) { GWO_CNT(GWO_ADD); return adouble(a.v + b); }
inline adouble operator-(const adouble &a, double b) { GWO_CNT(GWO_ADD); return adouble(a.v - b); }
inline adouble operator*(const adouble &a, double b) { GWO_CNT(GWO_MUL); return adouble(a.v * b); }
inline adouble operator/(const adouble &a, double b) { GWO_CNT(GWO_DIV); return adouble(a.v / b); }
inline adouble operator+(double a, const adouble &b) { GWO_CNT(GWO_ADD); return adouble(a + b.v); }
inline adouble operator-(double a, const adouble &b) { GWO_CNT(GWO_ADD); return adouble(a - b.v); }
inline adouble operator*(double a, const adouble &b) { GWO_CNT(GWO_MUL); return adouble(a * b.v); }
inline adouble operator/(double a, const adouble &b) { GWO_CNT(GWO_DIV); return adouble(a / b.v); }
#define GWO_CMP(op)                                                                  \
  inline bool operator op(const adouble &a, const adouble &b) { return a.v op b.v; } \
  inline bool operator op(const adouble &a, double b) { return a.v op b; }           \
  inline bool operator op(double a, const adouble &b) { return a op b.v; }
GWO_CMP(<) GWO_CMP(>) GWO_CMP(<=) GWO_CMP(>=) GWO_CMP(==) GWO_CMP(!=)
#undef GWO_CMP
#define GWO_F1(fn, k) inline adouble fn(const adouble &a) { GWO_CNT(k); return adouble(std::fn(a.v)); }
GWO_F1(sqrt, GWO_SQRT) GWO_F1(exp, GWO_EXP) GWO_F1(log, GWO_LOG) GWO_F1(log10, GWO_LOG) GWO_F1(sin, GWO_SIN)
GWO_F1(cos, GWO_COS) GWO_F1(tan, GWO_OTHER) GWO_F1(atan, GWO_ATAN) GWO_F1(asin, GWO_OTHER) GWO_F1(acos, GWO_OTHER)
GWO_F1(cbrt, GWO_CBRT) GWO_F1(sinh, GWO_OTHER) GWO_F1(cosh, GWO_OTHER) GWO_F1(tanh, GWO_OTHER)
GWO_F1(erf, GWO_OTHER)
#undef GWO_F1
#define GWO_F0(fn) inline adouble fn(const adouble &a) { return adouble(std::fn(a.v)); }
GWO_F0(fabs) GWO_F0(abs) GWO_F0(floor) GWO_F0(ceil) GWO_F0(trunc)
#undef GWO_F0
inline adouble pow(const adouble &a, double b) { GWO_CNT(GWO_POW); return adouble(std::pow(a.v, b)); }
inline adouble pow(const adouble &a, const adouble &b) { GWO_CNT(GWO_POW); return adouble(std::pow(a.v, b.v)); }
inline adouble pow(double a, const adouble &b) { GWO_CNT(GWO_POW); return adouble(std::pow(a, b.v)); }
inline adouble atan2(const adouble &a, const adouble &b) { GWO_CNT(GWO_ATAN); return adouble(std::atan2(a.v, b.v)); }
inline adouble fmax(const adouble &a, const adouble &b) { return adouble(std::fmax(a.v, b.v)); }
inline adouble fmin(const adouble &a, const adouble &b) { return adouble(std::fmin(a.v, b.v)); }
inline adouble hypot(const adouble &a, const adouble &b) { GWO_CNT(GWO_SQRT); return adouble(std::hypot(a.v, b.v)); }
inline bool isnan(const adouble &a) { return std::isnan(a.v); }
inline bool isinf(const adouble &a) { return std::isinf(a.v); }
inline adouble condassign(adouble &r, const adouble &c, const adouble &a, const adouble &b) { r = (c.v > 0) ? a : b; return r; }
typedef adouble adub;
typedef adouble areal;
class advector {};
#endif
