// Forward-mode dual numbers for the FP64 derivative kernels.
//
// Dual<N> carries a value and N directional derivatives.  Arithmetic and
// the math functions the time step uses follow the chain rule; comparisons,
// isnan and isinf act on the value only, so an expression evaluated on duals
// takes exactly the branches the plain FP64 evaluation takes at the same
// point (limiter cases, wave-speed cases, floors).  At a kink the derivative
// of the branch taken is returned: e.g. max(a, b) differentiates the chosen
// argument.
#pragma once

#include <cmath>

// Host+device inline functions: the physics and its derivatives compile
// for the GPU and, in test harnesses, for the host.
#ifndef SPLASH_HD
#if defined(__CUDACC__)
#define SPLASH_HD __host__ __device__ __forceinline__
#else
#define SPLASH_HD inline
#endif
#endif

namespace splash {

template <int N>
struct Dual {
  double v;
  double d[N];

  SPLASH_HD Dual() : v(0.0) {
#pragma unroll
    for (int i = 0; i < N; ++i) d[i] = 0.0;
  }
  SPLASH_HD Dual(double x) : v(x) {  // NOLINT: constants promote
#pragma unroll
    for (int i = 0; i < N; ++i) d[i] = 0.0;
  }
  SPLASH_HD static Dual seed(double x, int dir) {
    Dual r(x);
    r.d[dir] = 1.0;
    return r;
  }
};

template <class T>
struct is_dual {
  static constexpr bool value = false;
};
template <int N>
struct is_dual<Dual<N>> {
  static constexpr bool value = true;
};

// value of a plain double or a dual (for branches)
SPLASH_HD double val(double x) { return x; }
template <int N>
SPLASH_HD double val(const Dual<N>& x) { return x.v; }

template <int N>
SPLASH_HD Dual<N> operator+(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v + b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i];
  return r;
}
template <int N>
SPLASH_HD Dual<N> operator-(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v - b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i];
  return r;
}
template <int N>
SPLASH_HD Dual<N> operator-(const Dual<N>& a) {
  Dual<N> r;
  r.v = -a.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = -a.d[i];
  return r;
}
template <int N>
SPLASH_HD Dual<N> operator*(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v * b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
  return r;
}
template <int N>
SPLASH_HD Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v / b.v;
  const double ib = 1.0 / b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
  return r;
}
// mixed double / dual forms
template <int N> SPLASH_HD Dual<N> operator+(double a, const Dual<N>& b) { return Dual<N>(a) + b; }
template <int N> SPLASH_HD Dual<N> operator+(const Dual<N>& a, double b) { return a + Dual<N>(b); }
template <int N> SPLASH_HD Dual<N> operator-(double a, const Dual<N>& b) { return Dual<N>(a) - b; }
template <int N> SPLASH_HD Dual<N> operator-(const Dual<N>& a, double b) { return a - Dual<N>(b); }
template <int N>
SPLASH_HD Dual<N> operator*(double a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a * b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a * b.d[i];
  return r;
}
template <int N> SPLASH_HD Dual<N> operator*(const Dual<N>& a, double b) { return b * a; }
template <int N>
SPLASH_HD Dual<N> operator/(const Dual<N>& a, double b) {
  // the value is a.v / b, exactly as the plain FP64 expression evaluates it
  Dual<N> r;
  r.v = a.v / b;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] / b;
  return r;
}
template <int N> SPLASH_HD Dual<N> operator/(double a, const Dual<N>& b) { return Dual<N>(a) / b; }
template <int N> SPLASH_HD Dual<N>& operator+=(Dual<N>& a, const Dual<N>& b) { return a = a + b; }
template <int N> SPLASH_HD Dual<N>& operator-=(Dual<N>& a, const Dual<N>& b) { return a = a - b; }

// comparisons on values
#define SPLASH_DUAL_CMP(op)                                                                            \
  template <int N> SPLASH_HD bool operator op(const Dual<N>& a, const Dual<N>& b) { return a.v op b.v; } \
  template <int N> SPLASH_HD bool operator op(const Dual<N>& a, double b) { return a.v op b; }           \
  template <int N> SPLASH_HD bool operator op(double a, const Dual<N>& b) { return a op b.v; }
SPLASH_DUAL_CMP(<)
SPLASH_DUAL_CMP(>)
SPLASH_DUAL_CMP(<=)
SPLASH_DUAL_CMP(>=)
#undef SPLASH_DUAL_CMP

// NaN / inf tests usable on doubles and duals alike (value only)
#if defined(__CUDA_ARCH__)
SPLASH_HD bool is_nan(double x) { return ::isnan(x); }
SPLASH_HD bool is_inf(double x) { return ::isinf(x); }
#else
SPLASH_HD bool is_nan(double x) { return std::isnan(x); }
SPLASH_HD bool is_inf(double x) { return std::isinf(x); }
#endif
template <int N> SPLASH_HD bool is_nan(const Dual<N>& a) { return is_nan(a.v); }
template <int N> SPLASH_HD bool is_inf(const Dual<N>& a) { return is_inf(a.v); }

// the double overloads next to the dual ones, so unqualified calls in
// templated code resolve for both
using ::exp;
using ::expm1;
using ::log;
using ::sqrt;
using ::tanh;

template <int N>
SPLASH_HD Dual<N> chain(const Dual<N>& a, double fv, double dfdx) {
  Dual<N> r;
  r.v = fv;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = dfdx * a.d[i];
  return r;
}
template <int N>
SPLASH_HD Dual<N> sqrt(const Dual<N>& a) {
  const double s = ::sqrt(a.v);
  // at 0 (a zero velocity's norm) the one-sided derivative is taken as 0
  return chain(a, s, (s > 0.0) ? 0.5 / s : 0.0);
}
template <int N>
SPLASH_HD Dual<N> exp(const Dual<N>& a) {
  const double e = ::exp(a.v);
  return chain(a, e, e);
}
template <int N>
SPLASH_HD Dual<N> expm1(const Dual<N>& a) {
  const double e = ::expm1(a.v);
  // saturated (e = inf): the derivative e + 1 is inf as well; keep the chain
  return chain(a, e, e + 1.0);
}
template <int N>
SPLASH_HD Dual<N> log(const Dual<N>& a) {
  return chain(a, ::log(a.v), 1.0 / a.v);
}
template <int N>
SPLASH_HD Dual<N> tanh(const Dual<N>& a) {
  const double t = ::tanh(a.v);
  const double dt = 1.0 - t * t;
  // saturated: the derivative is 0 even where the argument's is not finite
  if (dt == 0.0) return Dual<N>(t);
  return chain(a, t, dt);
}

}  // namespace splash
