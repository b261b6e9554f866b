// Double-double numbers (an unevaluated sum hi + lo of two doubles, about
// 106 significant bits) for the extended-precision FP64 step, PG_FP64_DD.
//
// Its purpose is verification: central differences of the step in this
// precision can use perturbations far smaller than the distance to the
// nearest limiter or Riemann-branch switch (about 1e-10 along a random
// direction for 256 steps of a 128^2 problem), where plain FP64 differences
// drown in round-off; they then check the adjoint of the branch taken.
//
// The arithmetic is the double-word algorithms of M. Joldes, J.-M. Muller,
// V. Popescu, "Tight and rigorous error bounds for basic building blocks of
// double-word arithmetic", ACM TOMS 44(2), 2017, on doubles: TwoSum
// (Knuth), Fast2Sum (Dekker), 2Prod with an FMA, AccurateDWPlusDW (Alg. 6),
// DWTimesFP3 (Alg. 9), DWTimesDW3 (Alg. 12), DWDivDW2 (Alg. 17); the square
// root is the double root corrected by one Newton step in double-double.
// Translation units that use it are compiled without multiply-add
// contraction, so every operation rounds as written.
#pragma once
#include <cmath>

namespace pg {

struct DD {
  double hi, lo;
  __host__ __device__ DD() : hi(0.0), lo(0.0) {}
  __host__ __device__ DD(double x) : hi(x), lo(0.0) {}  // NOLINT: constants convert implicitly
  __host__ __device__ DD(double h, double l) : hi(h), lo(l) {}
};

__host__ __device__ __forceinline__ DD dd_two_sum(double a, double b) {
  const double s = a + b;
  const double bb = s - a;
  return DD(s, (a - (s - bb)) + (b - bb));
}

__host__ __device__ __forceinline__ DD dd_fast_two_sum(double a, double b) {  // |a| >= |b| (or a == 0)
  const double s = a + b;
  return DD(s, b - (s - a));
}

__host__ __device__ __forceinline__ DD dd_two_prod(double a, double b) {
  const double p = a * b;
  return DD(p, fma(a, b, -p));
}

__host__ __device__ __forceinline__ DD operator+(const DD& x, const DD& y) {  // AccurateDWPlusDW
  const DD s = dd_two_sum(x.hi, y.hi);
  const DD t = dd_two_sum(x.lo, y.lo);
  const DD v = dd_fast_two_sum(s.hi, s.lo + t.hi);
  return dd_fast_two_sum(v.hi, t.lo + v.lo);
}

__host__ __device__ __forceinline__ DD operator-(const DD& x) { return DD(-x.hi, -x.lo); }
__host__ __device__ __forceinline__ DD operator+(const DD& x) { return x; }
__host__ __device__ __forceinline__ DD operator-(const DD& x, const DD& y) { return x + (-y); }

__host__ __device__ __forceinline__ DD dd_times_d(const DD& x, double y) {  // DWTimesFP3
  const DD c = dd_two_prod(x.hi, y);
  return dd_fast_two_sum(c.hi, fma(x.lo, y, c.lo));
}

__host__ __device__ __forceinline__ DD operator*(const DD& x, const DD& y) {  // DWTimesDW3
  const DD c = dd_two_prod(x.hi, y.hi);
  const double tl1 = fma(x.hi, y.lo, x.lo * y.lo);
  const double cl2 = fma(x.lo, y.hi, tl1);
  return dd_fast_two_sum(c.hi, c.lo + cl2);
}

__host__ __device__ __forceinline__ DD operator/(const DD& x, const DD& y) {  // DWDivDW2
  const double th = x.hi / y.hi;
  const DD r = dd_times_d(y, th);
  const double d = (x.hi - r.hi) + (x.lo - r.lo);
  return dd_fast_two_sum(th, d / y.hi);
}

// mixed operands: a double is a double-double with a zero low part
__host__ __device__ __forceinline__ DD operator+(const DD& a, double b) { return a + DD(b); }
__host__ __device__ __forceinline__ DD operator+(double a, const DD& b) { return DD(a) + b; }
__host__ __device__ __forceinline__ DD operator-(const DD& a, double b) { return a - DD(b); }
__host__ __device__ __forceinline__ DD operator-(double a, const DD& b) { return DD(a) - b; }
__host__ __device__ __forceinline__ DD operator*(const DD& a, double b) { return dd_times_d(a, b); }
__host__ __device__ __forceinline__ DD operator*(double a, const DD& b) { return dd_times_d(b, a); }
__host__ __device__ __forceinline__ DD operator/(const DD& a, double b) { return a / DD(b); }
__host__ __device__ __forceinline__ DD operator/(double a, const DD& b) { return DD(a) / b; }

__host__ __device__ __forceinline__ DD& operator+=(DD& a, const DD& b) { return a = a + b; }
__host__ __device__ __forceinline__ DD& operator-=(DD& a, const DD& b) { return a = a - b; }
__host__ __device__ __forceinline__ DD& operator*=(DD& a, const DD& b) { return a = a * b; }
__host__ __device__ __forceinline__ DD& operator/=(DD& a, const DD& b) { return a = a / b; }

// Ordering of normalised pairs (|lo| <= ulp(hi)/2): by hi, ties by lo.
__host__ __device__ __forceinline__ int dd_cmp(const DD& a, const DD& b) {
  if (a.hi < b.hi) return -1;
  if (a.hi > b.hi) return 1;
  if (a.lo < b.lo) return -1;
  if (a.lo > b.lo) return 1;
  return (a.hi == b.hi && a.lo == b.lo) ? 0 : 2;  // 2: unordered (NaN)
}
#define PG_DD_CMP(OP, TEST)                                                                              \
  __host__ __device__ __forceinline__ bool operator OP(const DD& a, const DD& b) {                     \
    const int c = dd_cmp(a, b);                                                                        \
    return TEST;                                                                                       \
  }                                                                                                    \
  __host__ __device__ __forceinline__ bool operator OP(const DD& a, double b) { return a OP DD(b); }   \
  __host__ __device__ __forceinline__ bool operator OP(double a, const DD& b) { return DD(a) OP b; }
PG_DD_CMP(<, c == -1)
PG_DD_CMP(>, c == 1)
PG_DD_CMP(<=, c == -1 || c == 0)
PG_DD_CMP(>=, c == 1 || c == 0)
PG_DD_CMP(==, c == 0)
PG_DD_CMP(!=, c != 0)
#undef PG_DD_CMP

__host__ __device__ __forceinline__ DD fabs(const DD& a) { return a < 0.0 ? -a : a; }

// sqrt(x) = s + (x - s^2) / (2 s) with s the double root (one Newton step)
__host__ __device__ __forceinline__ DD sqrt(const DD& x) {
  if (!(x.hi > 0.0)) return DD(::sqrt(x.hi));
  const double s = ::sqrt(x.hi);
  const DD p = dd_two_prod(s, s);
  const double r = ((x.hi - p.hi) - p.lo + x.lo) / (2.0 * s);
  return dd_fast_two_sum(s, r);
}

__host__ __device__ __forceinline__ double value_of(const DD& x) { return x.hi; }

}  // namespace pg
