// Forward-mode dual numbers with two tangents, used by the adjoint to get the
// derivatives of one layer's optical quantities with respect to that layer's
// temperature (tangent t) and specific humidity (tangent q) from the same
// templated gas-optics code the forward path runs.  Comparisons, truncation to
// int and the branch structure follow the value, so the derivative is that of
// the branch the forward takes (piecewise-smooth functions, derivative from
// the active piece).
#pragma once
#include <cuda_runtime.h>

#include <cmath>
#include <type_traits>

namespace rrtmg {

// The dual overloads below live in this namespace; keep the plain ones visible.
using ::exp;
using ::expm1;
using ::fmin;
using ::log;
using ::pow;
using ::sqrt;

template <class R>
struct Dual {
  R v, t, q;  // value, d/dT(layer), d/dq(layer)
  __host__ __device__ Dual() : v(0), t(0), q(0) {}
  // constant (zero tangents) from any arithmetic value
  template <class T, typename std::enable_if<std::is_arithmetic<T>::value, int>::type = 0>
  __host__ __device__ Dual(T a) : v((R)a), t(0), q(0) {}
  __host__ __device__ Dual(R a, R dt, R dq) : v(a), t(dt), q(dq) {}
  __host__ __device__ explicit operator int() const { return (int)v; }
  __host__ __device__ explicit operator R() const { return v; }
  __host__ __device__ Dual& operator+=(const Dual& b) { v += b.v; t += b.t; q += b.q; return *this; }
  __host__ __device__ Dual& operator-=(const Dual& b) { v -= b.v; t -= b.t; q -= b.q; return *this; }
  __host__ __device__ Dual& operator*=(const Dual& b) { *this = *this * b; return *this; }
};

template <class R> __host__ __device__ inline Dual<R> operator-(const Dual<R>& a) { return {-a.v, -a.t, -a.q}; }
template <class R> __host__ __device__ inline Dual<R> operator+(const Dual<R>& a, const Dual<R>& b) { return {a.v + b.v, a.t + b.t, a.q + b.q}; }
template <class R> __host__ __device__ inline Dual<R> operator-(const Dual<R>& a, const Dual<R>& b) { return {a.v - b.v, a.t - b.t, a.q - b.q}; }
template <class R> __host__ __device__ inline Dual<R> operator*(const Dual<R>& a, const Dual<R>& b) {
  return {a.v * b.v, a.t * b.v + a.v * b.t, a.q * b.v + a.v * b.q};
}
// One reciprocal per dual division (the value is a.v * (1 / b.v), within an
// ulp of a.v / b.v); FP64 divides are sequences on the FP64 pipe.
template <class R> __host__ __device__ inline Dual<R> operator/(const Dual<R>& a, const Dual<R>& b) {
  const R inv = (R)1 / b.v;
  const R r = a.v * inv;
  return {r, (a.t - r * b.t) * inv, (a.q - r * b.q) * inv};
}
template <class R> __host__ __device__ inline Dual<R> operator+(const Dual<R>& a, R b) { return {a.v + b, a.t, a.q}; }
template <class R> __host__ __device__ inline Dual<R> operator+(R a, const Dual<R>& b) { return {a + b.v, b.t, b.q}; }
template <class R> __host__ __device__ inline Dual<R> operator-(const Dual<R>& a, R b) { return {a.v - b, a.t, a.q}; }
template <class R> __host__ __device__ inline Dual<R> operator-(R a, const Dual<R>& b) { return {a - b.v, -b.t, -b.q}; }
template <class R> __host__ __device__ inline Dual<R> operator*(const Dual<R>& a, R b) { return {a.v * b, a.t * b, a.q * b}; }
template <class R> __host__ __device__ inline Dual<R> operator*(R a, const Dual<R>& b) { return {a * b.v, a * b.t, a * b.q}; }
template <class R> __host__ __device__ inline Dual<R> operator/(const Dual<R>& a, R b) {
  const R inv = (R)1 / b;
  return {a.v * inv, a.t * inv, a.q * inv};
}
template <class R> __host__ __device__ inline Dual<R> operator/(R a, const Dual<R>& b) {
  const R inv = (R)1 / b.v;
  const R r = a * inv;
  return {r, -r * b.t * inv, -r * b.q * inv};
}
template <class R> __host__ __device__ inline bool operator<(const Dual<R>& a, const Dual<R>& b) { return a.v < b.v; }
template <class R> __host__ __device__ inline bool operator>(const Dual<R>& a, const Dual<R>& b) { return a.v > b.v; }
template <class R> __host__ __device__ inline bool operator<=(const Dual<R>& a, const Dual<R>& b) { return a.v <= b.v; }
template <class R> __host__ __device__ inline bool operator>=(const Dual<R>& a, const Dual<R>& b) { return a.v >= b.v; }
template <class R> __host__ __device__ inline bool operator==(const Dual<R>& a, const Dual<R>& b) { return a.v == b.v; }
template <class R> __host__ __device__ inline bool operator<(const Dual<R>& a, R b) { return a.v < b; }
template <class R> __host__ __device__ inline bool operator>(const Dual<R>& a, R b) { return a.v > b; }
template <class R> __host__ __device__ inline bool operator<=(const Dual<R>& a, R b) { return a.v <= b; }
template <class R> __host__ __device__ inline bool operator>=(const Dual<R>& a, R b) { return a.v >= b; }
template <class R> __host__ __device__ inline bool operator==(const Dual<R>& a, R b) { return a.v == b; }

template <class R> __device__ inline Dual<R> exp(const Dual<R>& a) {
  const R e = exp(a.v);
  return {e, e * a.t, e * a.q};
}
template <class R> __device__ inline Dual<R> expm1(const Dual<R>& a) {
  const R e = exp(a.v);
  return {expm1(a.v), e * a.t, e * a.q};
}
template <class R> __device__ inline Dual<R> log(const Dual<R>& a) {
  const R inv = (R)1 / a.v;
  return {log(a.v), a.t * inv, a.q * inv};
}
template <class R> __device__ inline Dual<R> sqrt(const Dual<R>& a) {
  const R s = sqrt(a.v);
  const R h = (R)0.5 / s;
  return {s, h * a.t, h * a.q};
}
// x^p for constant p
template <class R> __device__ inline Dual<R> pow(const Dual<R>& a, R p) {
  const R y = pow(a.v, p);
  const R d = p * pow(a.v, p - (R)1);
  return {y, d * a.t, d * a.q};
}
template <class R> __device__ inline Dual<R> fmin(const Dual<R>& a, R b) { return a.v <= b ? a : Dual<R>(b); }
template <class R> __device__ inline Dual<R> fmin(const Dual<R>& a, const Dual<R>& b) { return a.v <= b.v ? a : b; }

// Value of a plain or dual number.
template <class R> __host__ __device__ inline R val(const R& a) { return a; }
template <class R> __host__ __device__ inline R val(const Dual<R>& a) { return a.v; }

}  // namespace rrtmg
