/* Test-only stand-in for ADOL-C's adouble, used solely so that the reference's
 * IMRPhenomD.cpp / IMRPhenomP.cpp translation units compile for the oracle pin
 * build (oracle/ref_build.sh).  It wraps a double; no taping is done.  Only the
 * double instantiations of the reference classes are ever executed. */
#ifndef GWO_SHIM_ADOUBLE_H
#define GWO_SHIM_ADOUBLE_H
#include <cmath>
#include <complex>
#include <iostream>
#include <vector>
#include <string>
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
  adouble &operator+=(const adouble &o) { v += o.v; return *this; }
  adouble &operator-=(const adouble &o) { v -= o.v; return *this; }
  adouble &operator*=(const adouble &o) { v *= o.v; return *this; }
  adouble &operator/=(const adouble &o) { v /= o.v; return *this; }
  adouble operator-() const { return adouble(-v); }
  adouble operator+() const { return *this; }
};
inline adouble operator+(const adouble &a, const adouble &b) { return adouble(a.v + b.v); }
inline adouble operator-(const adouble &a, const adouble &b) { return adouble(a.v - b.v); }
inline adouble operator*(const adouble &a, const adouble &b) { return adouble(a.v * b.v); }
inline adouble operator/(const adouble &a, const adouble &b) { return adouble(a.v / b.v); }
inline adouble operator+(const adouble &a, double b) { return adouble(a.v + b); }
inline adouble operator-(const adouble &a, double b) { return adouble(a.v - b); }
inline adouble operator*(const adouble &a, double b) { return adouble(a.v * b); }
inline adouble operator/(const adouble &a, double b) { return adouble(a.v / b); }
inline adouble operator+(double a, const adouble &b) { return adouble(a + b.v); }
inline adouble operator-(double a, const adouble &b) { return adouble(a - b.v); }
inline adouble operator*(double a, const adouble &b) { return adouble(a * b.v); }
inline adouble operator/(double a, const adouble &b) { return adouble(a / b.v); }
#define GWO_CMP(op)                                                                  \
  inline bool operator op(const adouble &a, const adouble &b) { return a.v op b.v; } \
  inline bool operator op(const adouble &a, double b) { return a.v op b; }           \
  inline bool operator op(double a, const adouble &b) { return a op b.v; }
GWO_CMP(<) GWO_CMP(>) GWO_CMP(<=) GWO_CMP(>=) GWO_CMP(==) GWO_CMP(!=)
#undef GWO_CMP
#define GWO_F1(fn) inline adouble fn(const adouble &a) { return adouble(std::fn(a.v)); }
GWO_F1(sqrt) GWO_F1(exp) GWO_F1(log) GWO_F1(log10) GWO_F1(sin) GWO_F1(cos) GWO_F1(tan) GWO_F1(atan)
GWO_F1(asin) GWO_F1(acos) GWO_F1(fabs) GWO_F1(abs) GWO_F1(floor) GWO_F1(ceil) GWO_F1(cbrt) GWO_F1(sinh)
GWO_F1(cosh) GWO_F1(tanh) GWO_F1(erf) GWO_F1(trunc)
#undef GWO_F1
inline adouble pow(const adouble &a, double b) { return adouble(std::pow(a.v, b)); }
inline adouble pow(const adouble &a, const adouble &b) { return adouble(std::pow(a.v, b.v)); }
inline adouble pow(double a, const adouble &b) { return adouble(std::pow(a, b.v)); }
inline adouble atan2(const adouble &a, const adouble &b) { return adouble(std::atan2(a.v, b.v)); }
inline adouble fmax(const adouble &a, const adouble &b) { return adouble(std::fmax(a.v, b.v)); }
inline adouble fmin(const adouble &a, const adouble &b) { return adouble(std::fmin(a.v, b.v)); }
inline adouble hypot(const adouble &a, const adouble &b) { return adouble(std::hypot(a.v, b.v)); }
inline bool isnan(const adouble &a) { return std::isnan(a.v); }
inline bool isinf(const adouble &a) { return std::isinf(a.v); }
inline adouble condassign(adouble &r, const adouble &c, const adouble &a, const adouble &b) { r = (c.v > 0) ? a : b; return r; }
typedef adouble adub;
typedef adouble areal;
class advector {};
#endif
