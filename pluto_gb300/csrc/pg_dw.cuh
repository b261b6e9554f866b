// Double-word ("double-float") arithmetic on FP32 pairs, used by the
// mixed-precision path where it needs more than FP32 but the GB300's FP64
// pipe (1/58 of the FP32 rate) would dominate the step.
//
// Algorithms are the error-free transformations and double-word operators
// of M. Joldes, J.-M. Muller, V. Popescu, "Tight and rigorous error bounds for
// basic building blocks of double-word arithmetic", ACM TOMS 44(2), 2017:
//   TwoSum (Knuth), Fast2Sum (Dekker), 2Prod via FMA,
//   DWPlusDW ("AccurateDWPlusDW", Alg. 6, relative error <= 3u^2),
//   DWTimesFP (Alg. 9), DWTimesDW (Alg. 12), DWDivDW (Alg. 17).
// All FP32 operations use the explicit _rn intrinsics so that the compiler
// can neither contract nor reassociate them.
#pragma once

namespace pg {

struct dw {
  float hi, lo;
};

__device__ __forceinline__ dw two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}

__device__ __forceinline__ dw fast_two_sum(float a, float b) {  // |a| >= |b|
  float s = __fadd_rn(a, b);
  float e = __fsub_rn(b, __fsub_rn(s, a));
  return {s, e};
}

__device__ __forceinline__ dw two_prod(float a, float b) {
  float p = __fmul_rn(a, b);
  float e = __fmaf_rn(a, b, -p);
  return {p, e};
}

__device__ __forceinline__ dw dw_from(float a) { return {a, 0.f}; }

__device__ __forceinline__ dw operator+(dw x, dw y) {
  dw s = two_sum(x.hi, y.hi);
  dw t = two_sum(x.lo, y.lo);
  float c = __fadd_rn(s.lo, t.hi);
  dw v = fast_two_sum(s.hi, c);
  float w = __fadd_rn(t.lo, v.lo);
  return fast_two_sum(v.hi, w);
}

__device__ __forceinline__ dw operator-(dw y) { return {-y.hi, -y.lo}; }
__device__ __forceinline__ dw operator-(dw x, dw y) { return x + (-y); }

__device__ __forceinline__ dw operator+(dw x, float y) {  // DWPlusFP (Alg. 4)
  dw s = two_sum(x.hi, y);
  float v = __fadd_rn(x.lo, s.lo);
  return fast_two_sum(s.hi, v);
}

__device__ __forceinline__ dw operator*(dw x, float y) {  // DWTimesFP3 (Alg. 9)
  dw c = two_prod(x.hi, y);
  float cl3 = __fmaf_rn(x.lo, y, c.lo);
  return fast_two_sum(c.hi, cl3);
}

__device__ __forceinline__ dw operator*(dw x, dw y) {  // DWTimesDW3 (Alg. 12)
  dw c = two_prod(x.hi, y.hi);
  float tl0 = __fmul_rn(x.lo, y.lo);
  float tl1 = __fmaf_rn(x.hi, y.lo, tl0);
  float cl2 = __fmaf_rn(x.lo, y.hi, tl1);
  float cl3 = __fadd_rn(c.lo, cl2);
  return fast_two_sum(c.hi, cl3);
}

__device__ __forceinline__ dw dw_div(dw x, dw y) {  // DWDivDW2 (Alg. 17)
  float th = __fdiv_rn(x.hi, y.hi);
  dw r = y * th;
  float pih = __fsub_rn(x.hi, r.hi);
  float dl = __fsub_rn(x.lo, r.lo);
  float d = __fadd_rn(pih, dl);
  float tl = __fdiv_rn(d, y.hi);
  return fast_two_sum(th, tl);
}

__device__ __forceinline__ float dw_to_float(dw x) { return __fadd_rn(x.hi, x.lo); }

// Exact float -> double from the IEEE-754 fields with integer operations:
// sign kept, exponent rebiased (127 -> 1023), the 23 fraction bits shifted to
// the top of the 52.  GB300 issues the hardware conversion on its FP64 pipe
// (about as costly as a DADD there); this form issues on the integer pipes.
// Subnormal inputs take the hardware conversion.  NaN payloads are kept.
__device__ __forceinline__ double widen(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu, frac = u & 0x7fffffu;
  if (e == 0u && frac != 0u) return (double)f;
  const unsigned ex = e == 0u ? 0u : (e == 0xffu ? 0x7ffu : e + 896u);
  const unsigned hi = (u & 0x80000000u) | (ex << 20) | (frac >> 3);
  return __hiloint2double((int)hi, (int)(u << 29));
}

// double -> float with round-to-nearest-even, from the fields: for results
// whose exponent lies in the normal float range the top 23 fraction bits are
// kept and the 29 dropped bits decide the rounding (above half, or exactly
// half with an odd last bit, adds one ulp; the carry may step the exponent,
// up to infinity).  Zero, subnormal, out-of-range and non-finite values take
// the hardware conversion.
__device__ __forceinline__ float narrow(double d) {
  const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
  const unsigned e = (hi >> 20) & 0x7ffu;
  if (e - 897u > 253u) return (float)d;
  unsigned r = (hi & 0x80000000u) | ((e - 896u) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
  const unsigned rest = lo & 0x1fffffffu;
  r += (rest > 0x10000000u || (rest == 0x10000000u && (r & 1u))) ? 1u : 0u;
  return __uint_as_float(r);
}

// Accumulator traits: the mixed path is instantiated with native double or
// with dw; both expose the same handful of operations.
template <class A> struct Acc;

template <> struct Acc<double> {
  using T = double;
  // conversions through widen / narrow (same values as the hardware ones)
  static __device__ __forceinline__ T from(float a) { return widen(a); }
  static __device__ __forceinline__ T prod(float a, float b) { return widen(a) * widen(b); }
  static __device__ __forceinline__ T add(T a, T b) { return a + b; }
  static __device__ __forceinline__ T addf(T a, float b) { return a + widen(b); }
  static __device__ __forceinline__ T sub(T a, T b) { return a - b; }
  static __device__ __forceinline__ T mulf(T a, float b) { return a * widen(b); }
  static __device__ __forceinline__ T mul(T a, T b) { return a * b; }
  // a/b through an FP32 reciprocal refined by one Newton step in FP64
  // (relative error ~1e-14), three FP64 operations instead of a full division.
  static __device__ __forceinline__ T div(T a, T b) {
    double r = widen(__frcp_rn(narrow(b)));
    r = fma(r, fma(-b, r, 1.0), r);
    return a * r;
  }
  static __device__ __forceinline__ float tof(T a) { return narrow(a); }
  static __device__ __forceinline__ bool neg(T a) { return a < 0.0; }
  static __device__ __forceinline__ T konst(double hi, float, float) { return hi; }
};

template <> struct Acc<dw> {
  using T = dw;
  static __device__ __forceinline__ T from(float a) { return {a, 0.f}; }
  static __device__ __forceinline__ T prod(float a, float b) { return two_prod(a, b); }
  static __device__ __forceinline__ T add(T a, T b) { return a + b; }
  static __device__ __forceinline__ T addf(T a, float b) { return a + b; }
  static __device__ __forceinline__ T sub(T a, T b) { return a - b; }
  static __device__ __forceinline__ T mulf(T a, float b) { return a * b; }
  static __device__ __forceinline__ T mul(T a, T b) { return a * b; }
  static __device__ __forceinline__ T div(T a, T b) { return dw_div(a, b); }
  static __device__ __forceinline__ float tof(T a) { return dw_to_float(a); }
  static __device__ __forceinline__ bool neg(T a) { return a.hi < 0.f || (a.hi == 0.f && a.lo < 0.f); }
  static __device__ __forceinline__ T konst(double, float hi, float lo) { return {hi, lo}; }
};

}  // namespace pg
