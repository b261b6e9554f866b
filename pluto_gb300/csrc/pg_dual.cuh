// Forward-mode dual numbers for the differentiated paths.
//
// Dual<N> carries a value and N directional derivatives.  Every branch of
// the point physics (limiters, HLLD region selection, floors, MIN/MAX)
// compares values only, so a dual evaluation differentiates exactly the
// branch the plain evaluation takes.  Used (a) with N = 1 to run the whole
// FP64 step as a tangent-linear model, and (b) to form the local Jacobians
// of point kernels that the adjoint kernels apply transposed.
#pragma once
#include <cmath>

namespace pg {

template <int N>
struct Dual {
  double v;
  double d[N];
  __host__ __device__ Dual() : v(0.0) {
#pragma unroll
    for (int k = 0; k < N; k++) d[k] = 0.0;
  }
  __host__ __device__ Dual(double x) : v(x) {  // constants have no derivative
#pragma unroll
    for (int k = 0; k < N; k++) d[k] = 0.0;
  }
  __host__ __device__ static Dual seed(double x, int k) {
    Dual r(x);
    r.d[k] = 1.0;
    return r;
  }
};

#define PG_DUAL_BIN(OP, VEXPR, DEXPR)                                                   \
  template <int N>                                                                      \
  __host__ __device__ __forceinline__ Dual<N> operator OP(const Dual<N>& a, const Dual<N>& b) { \
    Dual<N> r;                                                                          \
    r.v = VEXPR;                                                                        \
    _Pragma("unroll") for (int k = 0; k < N; k++) r.d[k] = DEXPR;                       \
    return r;                                                                           \
  }
PG_DUAL_BIN(+, a.v + b.v, a.d[k] + b.d[k])
PG_DUAL_BIN(-, a.v - b.v, a.d[k] - b.d[k])
PG_DUAL_BIN(*, a.v * b.v, a.d[k] * b.v + a.v * b.d[k])
#undef PG_DUAL_BIN

template <int N>
__host__ __device__ __forceinline__ Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v / b.v;
  const double ib = 1.0 / b.v;
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = (a.d[k] - r.v * b.d[k]) * ib;
  return r;
}

template <int N>
__host__ __device__ __forceinline__ Dual<N> operator-(const Dual<N>& a) {
  Dual<N> r;
  r.v = -a.v;
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = -a.d[k];
  return r;
}

template <int N>
__host__ __device__ __forceinline__ Dual<N> operator+(const Dual<N>& a) {
  return a;
}

// mixed Dual/double operands (a double is a constant)
template <int N> __host__ __device__ __forceinline__ Dual<N> operator+(const Dual<N>& a, double b) { return a + Dual<N>(b); }
template <int N> __host__ __device__ __forceinline__ Dual<N> operator+(double a, const Dual<N>& b) { return Dual<N>(a) + b; }
template <int N> __host__ __device__ __forceinline__ Dual<N> operator-(const Dual<N>& a, double b) { return a - Dual<N>(b); }
template <int N> __host__ __device__ __forceinline__ Dual<N> operator-(double a, const Dual<N>& b) { return Dual<N>(a) - b; }
template <int N> __host__ __device__ __forceinline__ Dual<N> operator*(const Dual<N>& a, double b) {
  Dual<N> r;
  r.v = a.v * b;
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = a.d[k] * b;
  return r;
}
template <int N> __host__ __device__ __forceinline__ Dual<N> operator*(double a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a * b.v;
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = a * b.d[k];
  return r;
}
template <int N> __host__ __device__ __forceinline__ Dual<N> operator/(const Dual<N>& a, double b) { return a / Dual<N>(b); }
template <int N> __host__ __device__ __forceinline__ Dual<N> operator/(double a, const Dual<N>& b) { return Dual<N>(a) / b; }

template <int N> __host__ __device__ __forceinline__ Dual<N>& operator+=(Dual<N>& a, const Dual<N>& b) { return a = a + b; }
template <int N> __host__ __device__ __forceinline__ Dual<N>& operator-=(Dual<N>& a, const Dual<N>& b) { return a = a - b; }
template <int N> __host__ __device__ __forceinline__ Dual<N>& operator*=(Dual<N>& a, const Dual<N>& b) { return a = a * b; }
template <int N> __host__ __device__ __forceinline__ Dual<N>& operator/=(Dual<N>& a, const Dual<N>& b) { return a = a / b; }

// Distance to the nearest branch switch along the tangent direction.  With
// recording on (pg_tangent_kink), every comparison of a Dual<1> (limiter
// signs, MIN/MAX, Riemann-fan regions, floors, |x|) notes |a - b| / |a' - b'|,
// the perturbation size at which, to first order, its outcome would flip;
// the minimum over a run bounds the step h of central differences that cross
// no kink.  Each translation unit has its own copy of these two variables.
static __device__ int g_pg_kink_on;
static __device__ unsigned long long g_pg_kink_bits;  // non-negative double bits: ordered as integers

template <int N>
__host__ __device__ __forceinline__ void kink_note(double dv, double dd) {
#ifdef __CUDA_ARCH__
  if (N != 1 || !g_pg_kink_on) return;
  const double ad = ::fabs(dd);
  if (!(ad > 0.0)) return;
  const unsigned long long b = (unsigned long long)__double_as_longlong(::fabs(dv) / ad);
  if (b < *(volatile unsigned long long*)&g_pg_kink_bits) atomicMin(&g_pg_kink_bits, b);
#else
  (void)dv;
  (void)dd;
#endif
}

#define PG_DUAL_CMP(OP)                                                                         \
  template <int N>                                                                              \
  __host__ __device__ __forceinline__ bool operator OP(const Dual<N>& a, const Dual<N>& b) {    \
    kink_note<N>(a.v - b.v, a.d[0] - b.d[0]);                                                   \
    return a.v OP b.v;                                                                          \
  }                                                                                             \
  template <int N>                                                                              \
  __host__ __device__ __forceinline__ bool operator OP(const Dual<N>& a, double b) {            \
    kink_note<N>(a.v - b, a.d[0]);                                                              \
    return a.v OP b;                                                                            \
  }                                                                                             \
  template <int N>                                                                              \
  __host__ __device__ __forceinline__ bool operator OP(double a, const Dual<N>& b) {            \
    kink_note<N>(a - b.v, -b.d[0]);                                                             \
    return a OP b.v;                                                                            \
  }
PG_DUAL_CMP(<)
PG_DUAL_CMP(>)
PG_DUAL_CMP(<=)
PG_DUAL_CMP(>=)
PG_DUAL_CMP(==)
PG_DUAL_CMP(!=)
#undef PG_DUAL_CMP

template <int N>
__host__ __device__ __forceinline__ Dual<N> fabs(const Dual<N>& a) {
  kink_note<N>(a.v, a.d[0]);
  return a.v < 0.0 ? -a : a;  // derivative of the branch taken (sign(+0) = +)
}

template <int N>
__host__ __device__ __forceinline__ Dual<N> sqrt(const Dual<N>& a) {
  Dual<N> r;
  r.v = ::sqrt(a.v);
  const double h = 0.5 / r.v;
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = a.d[k] * h;
  return r;
}

// value part (for reductions and bit tests)
__host__ __device__ __forceinline__ double value_of(double x) { return x; }
template <int N> __host__ __device__ __forceinline__ double value_of(const Dual<N>& x) { return x.v; }

}  // namespace pg
