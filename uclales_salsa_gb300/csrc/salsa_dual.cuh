// salsa_dual.cuh -- forward-mode dual numbers for the gradient kernels.
//
// Dual<N> carries a value and N tangent components.  The collision-kernel
// templates (bin_props, coag_pair, terminal_vel) instantiate with Dual<2> to give
// dK/d(d_i) and dK/d(d_j) for the adjoint, and the chain step instantiates with
// Dual<1> for the tangent-linear model.  Derivatives follow the elementary rules;
// min/max/abs take the branch of the value (one-sided at ties).  The value parts round
// exactly as the plain FP64 code (no contraction); the tangent parts use fused
// multiply-adds, which only changes their last bits.
#pragma once
#include <cuda_runtime.h>

namespace salsa {

// keep the double forms visible next to the dual overloads below
using ::fabs;
using ::fmin;
using ::fmax;

template <int N>
struct Dual {
  double v;
  double d[N];
  __device__ __forceinline__ Dual() : v(0.) {
#pragma unroll
    for (int i = 0; i < N; i++) d[i] = 0.;
  }
  __device__ __forceinline__ Dual(double x) : v(x) {   // constants: zero tangent
#pragma unroll
    for (int i = 0; i < N; i++) d[i] = 0.;
  }
  __device__ __forceinline__ explicit operator double() const { return v; }
};

// chain rule helper: f(a) with f'(a) = g
template <int N>
__device__ __forceinline__ Dual<N> d_apply(const Dual<N> &a, double f, double g) {
  Dual<N> r;
  r.v = f;
#pragma unroll
  for (int i = 0; i < N; i++) r.d[i] = g * a.d[i];
  return r;
}

template <int N> __device__ __forceinline__ Dual<N> operator+(const Dual<N> &a, const Dual<N> &b) {
  Dual<N> r; r.v = a.v + b.v;
#pragma unroll
  for (int i = 0; i < N; i++) r.d[i] = a.d[i] + b.d[i];
  return r;
}
template <int N> __device__ __forceinline__ Dual<N> operator-(const Dual<N> &a, const Dual<N> &b) {
  Dual<N> r; r.v = a.v - b.v;
#pragma unroll
  for (int i = 0; i < N; i++) r.d[i] = a.d[i] - b.d[i];
  return r;
}
template <int N> __device__ __forceinline__ Dual<N> operator-(const Dual<N> &a) {
  Dual<N> r; r.v = -a.v;
#pragma unroll
  for (int i = 0; i < N; i++) r.d[i] = -a.d[i];
  return r;
}
template <int N> __device__ __forceinline__ Dual<N> operator*(const Dual<N> &a, const Dual<N> &b) {
  Dual<N> r; r.v = a.v * b.v;
#pragma unroll
  for (int i = 0; i < N; i++) r.d[i] = __fma_rn(a.d[i], b.v, a.v * b.d[i]);
  return r;
}
template <int N> __device__ __forceinline__ Dual<N> operator/(const Dual<N> &a, const Dual<N> &b) {
  Dual<N> r; r.v = a.v / b.v;
  const double ib = 1. / b.v;
#pragma unroll
  for (int i = 0; i < N; i++) r.d[i] = __fma_rn(-r.v, b.d[i], a.d[i]) * ib;
  return r;
}
template <int N> __device__ __forceinline__ Dual<N> operator+(const Dual<N> &a, double b) { return a + Dual<N>(b); }
template <int N> __device__ __forceinline__ Dual<N> operator+(double a, const Dual<N> &b) { return Dual<N>(a) + b; }
template <int N> __device__ __forceinline__ Dual<N> operator-(const Dual<N> &a, double b) { return a - Dual<N>(b); }
template <int N> __device__ __forceinline__ Dual<N> operator-(double a, const Dual<N> &b) { return Dual<N>(a) - b; }
template <int N> __device__ __forceinline__ Dual<N> operator*(const Dual<N> &a, double b) {
  Dual<N> r; r.v = a.v * b;
#pragma unroll
  for (int i = 0; i < N; i++) r.d[i] = a.d[i] * b;
  return r;
}
template <int N> __device__ __forceinline__ Dual<N> operator*(double a, const Dual<N> &b) { return b * a; }
template <int N> __device__ __forceinline__ Dual<N> operator/(const Dual<N> &a, double b) { return a / Dual<N>(b); }
template <int N> __device__ __forceinline__ Dual<N> operator/(double a, const Dual<N> &b) { return Dual<N>(a) / b; }
template <int N> __device__ __forceinline__ Dual<N> &operator+=(Dual<N> &a, const Dual<N> &b) { a = a + b; return a; }
template <int N> __device__ __forceinline__ Dual<N> &operator-=(Dual<N> &a, const Dual<N> &b) { a = a - b; return a; }
template <int N> __device__ __forceinline__ Dual<N> &operator*=(Dual<N> &a, const Dual<N> &b) { a = a * b; return a; }

#define SALSA_DUAL_CMP(op)                                                                                    \
  template <int N> __device__ __forceinline__ bool operator op(const Dual<N> &a, const Dual<N> &b) { return a.v op b.v; } \
  template <int N> __device__ __forceinline__ bool operator op(const Dual<N> &a, double b) { return a.v op b; }           \
  template <int N> __device__ __forceinline__ bool operator op(double a, const Dual<N> &b) { return a op b.v; }
SALSA_DUAL_CMP(<)
SALSA_DUAL_CMP(<=)
SALSA_DUAL_CMP(>)
SALSA_DUAL_CMP(>=)
#undef SALSA_DUAL_CMP

template <int N> __device__ __forceinline__ Dual<N> sq(const Dual<N> &a) { return a * a; }
template <int N> __device__ __forceinline__ Dual<N> cube(const Dual<N> &a) { return a * a * a; }
template <int N> __device__ __forceinline__ Dual<N> fabs(const Dual<N> &a) { return a.v < 0. ? -a : a; }
template <int N> __device__ __forceinline__ Dual<N> fmin(const Dual<N> &a, const Dual<N> &b) { return b.v < a.v ? b : a; }
template <int N> __device__ __forceinline__ Dual<N> fmax(const Dual<N> &a, const Dual<N> &b) { return b.v > a.v ? b : a; }
template <int N> __device__ __forceinline__ Dual<N> fmin(const Dual<N> &a, double b) { return fmin(a, Dual<N>(b)); }
template <int N> __device__ __forceinline__ Dual<N> fmax(const Dual<N> &a, double b) { return fmax(a, Dual<N>(b)); }
template <int N> __device__ __forceinline__ Dual<N> fmin(double a, const Dual<N> &b) { return fmin(Dual<N>(a), b); }
template <int N> __device__ __forceinline__ Dual<N> fmax(double a, const Dual<N> &b) { return fmax(Dual<N>(a), b); }
template <int N> __device__ __forceinline__ Dual<N> d_exp(const Dual<N> &a) { double e = exp(a.v); return d_apply(a, e, e); }
template <int N> __device__ __forceinline__ Dual<N> d_log(const Dual<N> &a) { return d_apply(a, log(a.v), 1. / a.v); }
template <int N> __device__ __forceinline__ Dual<N> d_sqrt(const Dual<N> &a) {
  double s = sqrt(a.v);
  return d_apply(a, s, s > 0. ? 0.5 / s : 0.);
}
template <int N> __device__ __forceinline__ Dual<N> d_cbrt(const Dual<N> &a) {
  double c = cbrt(a.v);
  return d_apply(a, c, c != 0. ? 1. / (3. * c * c) : 0.);
}
template <int N> __device__ __forceinline__ Dual<N> d_pow(const Dual<N> &a, const Dual<N> &b) {
  Dual<N> r;
  r.v = pow(a.v, b.v);
  const double la = a.v > 0. ? log(a.v) : 0.;
  const double ga = a.v != 0. ? b.v * r.v / a.v : 0., rl = r.v * la;
#pragma unroll
  for (int i = 0; i < N; i++) r.d[i] = __fma_rn(ga, a.d[i], rl * b.d[i]);
  return r;
}

// warp shuffles of every component
template <int N> __device__ __forceinline__ Dual<N> shfl_xor(const Dual<N> &a, int m) {
  Dual<N> r;
  r.v = __shfl_xor_sync(0xffffffffu, a.v, m);
#pragma unroll
  for (int i = 0; i < N; i++) r.d[i] = __shfl_xor_sync(0xffffffffu, a.d[i], m);
  return r;
}
template <int N> __device__ __forceinline__ Dual<N> shfl_idx(const Dual<N> &a, int l) {
  Dual<N> r;
  r.v = __shfl_sync(0xffffffffu, a.v, l);
#pragma unroll
  for (int i = 0; i < N; i++) r.d[i] = __shfl_sync(0xffffffffu, a.d[i], l);
  return r;
}
__device__ __forceinline__ double shfl_xor(double a, int m) { return __shfl_xor_sync(0xffffffffu, a, m); }
__device__ __forceinline__ double shfl_idx(double a, int l) { return __shfl_sync(0xffffffffu, a, l); }

// the float-only flux-matching form is never taken by dual numbers (is_f32 is false)
template <int N> __device__ __forceinline__ Dual<N> flux_match_stable(const Dual<N> &, const Dual<N> &) { return Dual<N>(0.); }

// value part of either type
__device__ __forceinline__ double val(double a) { return a; }
template <int N> __device__ __forceinline__ double val(const Dual<N> &a) { return a.v; }

}  // namespace salsa
