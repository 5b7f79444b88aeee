// Op-counting FP64 scalar for the CPU oracle -- TEST / MEASUREMENT
// INFRASTRUCTURE, never part of the product.
//
// rg_opcount.cpp compiles the oracle's own sources a second time with every
// `double` replaced by rg_count::Real, a one-double struct whose arithmetic
// does the same IEEE operation and counts it.  The counts are the algorithmic
// FP64 work of the reference algorithm as the oracle restates it: each
// addition, subtraction, multiplication, division and square root written in
// the Fortran, plus calls of pow / log / exp (counted as calls), comparisons
// and min / max selections.  They are kept per phase of the cycle (the
// oracle marks its hexa element groups, shell element groups and nodal work
// with RG_OPCOUNT_PHASE), so a per-element figure is the count of a phase
// divided by the elements it processed.  Conversions and loads/stores are
// not counted.
#pragma once

#include <cmath>
#include <cstdint>

namespace rg_count {

enum Op { ADD = 0, MUL, DIV, SQRT, POW, LOG, EXP, TRIG, CMP, MINMAX, NOPS };
enum { NPHASE = 4 };  // 0 other, 1 hexa elements, 2 shell elements, 3 nodes

extern long long counts[NPHASE][NOPS];
extern int phase;

inline void tick(Op o) { counts[phase][o]++; }

struct Real {
  double v;
  Real() = default;
  constexpr Real(double x) : v(x) {}
  Real(float x) : v(x) {}
  Real(int x) : v(x) {}
  Real(long x) : v((double)x) {}
  Real(long long x) : v((double)x) {}
  Real(unsigned x) : v(x) {}
  Real(unsigned long x) : v((double)x) {}
  explicit operator int() const { return (int)v; }
  explicit operator long() const { return (long)v; }
  explicit operator long long() const { return (long long)v; }
  explicit operator float() const { return (float)v; }
  explicit operator bool() const { return v != 0.0; }
  // explicit only: every arithmetic use goes through a counted operator
  explicit operator double() const { return v; }
  Real &operator+=(Real b) { tick(ADD); v += b.v; return *this; }
  Real &operator-=(Real b) { tick(ADD); v -= b.v; return *this; }
  Real &operator*=(Real b) { tick(MUL); v *= b.v; return *this; }
  Real &operator/=(Real b) { tick(DIV); v /= b.v; return *this; }
  Real operator-() const { return Real(-v); }
  Real operator+() const { return *this; }
};
static_assert(sizeof(Real) == sizeof(double), "same layout as double");

inline Real operator+(Real a, Real b) { tick(ADD); return Real(a.v + b.v); }
inline Real operator-(Real a, Real b) { tick(ADD); return Real(a.v - b.v); }
inline Real operator*(Real a, Real b) { tick(MUL); return Real(a.v * b.v); }
inline Real operator/(Real a, Real b) { tick(DIV); return Real(a.v / b.v); }
inline bool operator<(Real a, Real b) { tick(CMP); return a.v < b.v; }
inline bool operator>(Real a, Real b) { tick(CMP); return a.v > b.v; }
inline bool operator<=(Real a, Real b) { tick(CMP); return a.v <= b.v; }
inline bool operator>=(Real a, Real b) { tick(CMP); return a.v >= b.v; }
inline bool operator==(Real a, Real b) { tick(CMP); return a.v == b.v; }
inline bool operator!=(Real a, Real b) { tick(CMP); return a.v != b.v; }

inline Real sqrt(Real a) { tick(SQRT); return Real(std::sqrt(a.v)); }
inline Real pow(Real a, Real b) { tick(POW); return Real(std::pow(a.v, b.v)); }
inline Real log(Real a) { tick(LOG); return Real(std::log(a.v)); }
inline Real exp(Real a) { tick(EXP); return Real(std::exp(a.v)); }
inline Real sin(Real a) { tick(TRIG); return Real(std::sin(a.v)); }
inline Real cos(Real a) { tick(TRIG); return Real(std::cos(a.v)); }
inline Real nearbyint(Real a) { return Real(std::nearbyint(a.v)); }
inline Real fabs(Real a) { return Real(std::fabs(a.v)); }
inline Real abs(Real a) { return Real(std::fabs(a.v)); }
inline Real copysign(Real a, Real b) { return Real(std::copysign(a.v, b.v)); }
inline Real fmax(Real a, Real b) { tick(MINMAX); return Real(std::fmax(a.v, b.v)); }
inline Real fmin(Real a, Real b) { tick(MINMAX); return Real(std::fmin(a.v, b.v)); }
inline bool isfinite(Real a) { return std::isfinite(a.v); }
inline bool isnan(Real a) { return std::isnan(a.v); }
// std::min / std::max semantics (first argument on ties), counted once
inline const Real &max(const Real &a, const Real &b) { tick(MINMAX); return (a.v < b.v) ? b : a; }
inline const Real &min(const Real &a, const Real &b) { tick(MINMAX); return (b.v < a.v) ? b : a; }

}  // namespace rg_count

// the oracle calls the std:: spellings: route them to the counted versions
namespace std {
using rg_count::copysign;
using rg_count::cos;
using rg_count::nearbyint;
using rg_count::sin;
using rg_count::exp;
using rg_count::fabs;
using rg_count::fmax;
using rg_count::fmin;
using rg_count::isfinite;
using rg_count::isnan;
using rg_count::log;
using rg_count::max;
using rg_count::min;
using rg_count::pow;
using rg_count::sqrt;
}  // namespace std
