// Operation-counting scalar for the oracle's FLOP-count build -- TEST
// INFRASTRUCTURE ONLY.  Force-included (g++ -include opcount.hpp) ahead of the
// oracle sources by `make opcount`: it pulls in every system header the oracle
// uses, then maps the type `double` onto opc::D, a standard-layout wrapper of
// one double whose arithmetic is plain IEEE double arithmetic (the same
// results bit for bit) and counts every operation: add / sub, mul, div, sqrt,
// exp, log, pow, trigonometric functions, comparisons.  FMA is never formed
// (-ffp-contract=off), so a multiply-add counts as two operations.  The counts
// are thread-local; OPC_PAUSE() / OPC_RESUME() suspend counting around work
// the algorithmic count excludes (the reference's redundant second SW
// two-stream pass).
#pragma once
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <map>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace opc {

enum { ADD, MUL, DIV, SQRT, EXP, LOG, POW, TRIG, CMP, NKIND };
inline thread_local unsigned long long g_count[NKIND] = {};
inline thread_local int g_paused = 0;
inline void tick(int k) {
  if (!g_paused) ++g_count[k];
}

struct D {
  double v;
  D() = default;
  constexpr D(double x) : v(x) {}
  template <class I, typename std::enable_if<std::is_integral<I>::value, int>::type = 0>
  constexpr D(I x) : v((double)x) {}
  explicit operator double() const { return v; }
  template <class I, typename std::enable_if<std::is_integral<I>::value, int>::type = 0>
  explicit operator I() const { return (I)v; }
  D& operator+=(D b) { tick(ADD); v += b.v; return *this; }
  D& operator-=(D b) { tick(ADD); v -= b.v; return *this; }
  D& operator*=(D b) { tick(MUL); v *= b.v; return *this; }
  D& operator/=(D b) { tick(DIV); v /= b.v; return *this; }
};
static_assert(sizeof(D) == sizeof(double) && std::is_standard_layout<D>::value, "D must be layout-compatible");
static_assert(std::is_trivially_copyable<D>::value, "D must be trivially copyable");

inline D operator+(D a, D b) { tick(ADD); return D(a.v + b.v); }
inline D operator-(D a, D b) { tick(ADD); return D(a.v - b.v); }
inline D operator*(D a, D b) { tick(MUL); return D(a.v * b.v); }
inline D operator/(D a, D b) { tick(DIV); return D(a.v / b.v); }
inline D operator-(D a) { return D(-a.v); }
inline D operator+(D a) { return a; }
inline bool operator<(D a, D b) { tick(CMP); return a.v < b.v; }
inline bool operator>(D a, D b) { tick(CMP); return a.v > b.v; }
inline bool operator<=(D a, D b) { tick(CMP); return a.v <= b.v; }
inline bool operator>=(D a, D b) { tick(CMP); return a.v >= b.v; }
inline bool operator==(D a, D b) { tick(CMP); return a.v == b.v; }
inline bool operator!=(D a, D b) { tick(CMP); return a.v != b.v; }

}  // namespace opc

// The oracle calls these qualified as std::; plain double arguments still
// reach the standard overloads.
namespace std {
inline opc::D exp(opc::D a) { opc::tick(opc::EXP); return opc::D(::exp(a.v)); }
inline opc::D log(opc::D a) { opc::tick(opc::LOG); return opc::D(::log(a.v)); }
inline opc::D sqrt(opc::D a) { opc::tick(opc::SQRT); return opc::D(::sqrt(a.v)); }
inline opc::D pow(opc::D a, opc::D b) { opc::tick(opc::POW); return opc::D(::pow(a.v, b.v)); }
inline opc::D sin(opc::D a) { opc::tick(opc::TRIG); return opc::D(::sin(a.v)); }
inline opc::D cos(opc::D a) { opc::tick(opc::TRIG); return opc::D(::cos(a.v)); }
inline opc::D asin(opc::D a) { opc::tick(opc::TRIG); return opc::D(::asin(a.v)); }
inline opc::D fmod(opc::D a, opc::D b) { opc::tick(opc::DIV); return opc::D(::fmod(a.v, b.v)); }
inline opc::D fabs(opc::D a) { return opc::D(::fabs(a.v)); }
inline opc::D abs(opc::D a) { return opc::D(::fabs(a.v)); }
inline bool isfinite(opc::D a) { return std::isfinite(a.v); }
// mixed (counting, plain double) arguments, e.g. std::min(x, 500.)
inline opc::D min(opc::D a, opc::D b) { opc::tick(opc::CMP); return b.v < a.v ? b : a; }
inline opc::D max(opc::D a, opc::D b) { opc::tick(opc::CMP); return a.v < b.v ? b : a; }
}  // namespace std

#define OPC_PAUSE() (++opc::g_paused)
#define OPC_RESUME() (--opc::g_paused)
#define double opc::D
