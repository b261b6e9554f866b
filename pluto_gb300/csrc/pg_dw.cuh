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

// Exact float -> double from the IEEE-754 fields with integer operations
// only: sign kept; a normal number has its exponent rebiased (127 -> 1023)
// and its 23 fraction bits moved to the top of the 52; a subnormal one,
// frac * 2^-149 with its leading one at bit p, becomes the normal double
// 2^(p-149) * 1.f (exponent field p + 874, the bits below p shifted up to
// the top of the fraction); zero stays zero; Inf/NaN keep the all-ones
// exponent and the fraction bits.  GB300 issues the hardware conversion on
// its FP64 pipe (about as costly as a DADD there); every case here is
// integer work and the compiler turns the cases into selects.
__device__ __forceinline__ double widen(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned sign = u & 0x80000000u;
  const unsigned e = (u >> 23) & 0xffu, frac = u & 0x7fffffu;
  unsigned hi, lo;
  if (e - 1u < 254u) {  // normal
    hi = sign | ((e + 896u) << 20) | (frac >> 3);
    lo = frac << 29;
  } else if (e == 0xffu) {  // Inf / NaN
    hi = sign | 0x7ff00000u | (frac >> 3);
    lo = frac << 29;
  } else if (frac == 0u) {  // zero
    hi = sign;
    lo = 0u;
  } else {  // subnormal
    const unsigned p = 31u - (unsigned)__clz((int)frac);
    const unsigned long long m = (unsigned long long)(frac ^ (1u << p)) << (52u - p);
    hi = sign | ((p + 874u) << 20) | (unsigned)(m >> 32);
    lo = (unsigned)m;
  }
  return __hiloint2double((int)hi, (int)lo);
}

// double -> float with round-to-nearest-even from the fields, integer
// operations only.  Normal results (double exponent 897..1150): the top 23
// fraction bits are kept and the 29 dropped bits round (above half, or
// exactly half with an odd last bit, adds one ulp; the carry may step the
// exponent, up to infinity).  Smaller magnitudes: the 53-bit significand
// shifted to units of 2^-149 and rounded the same way gives the subnormal
// (or zero, or smallest normal) encoding directly.  Exponents above the float
// range give infinity; Inf stays Inf and NaN gives a quiet NaN.
__device__ __forceinline__ float narrow(double d) {
  const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
  const unsigned sign = hi & 0x80000000u;
  const unsigned e = (hi >> 20) & 0x7ffu;
  unsigned r;
  if (e - 897u <= 253u) {  // normal float result
    r = ((e - 896u) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
    const unsigned rest = lo & 0x1fffffffu;
    r += (rest > 0x10000000u || (rest == 0x10000000u && (r & 1u))) ? 1u : 0u;
  } else if (e == 0x7ffu) {  // Inf / NaN
    r = ((hi & 0xfffffu) | lo) ? 0x7fc00000u : 0x7f800000u;
  } else if (e > 1150u) {  // overflow
    r = 0x7f800000u;
  } else if (e == 0u) {  // zero or double subnormal: far below half the smallest float
    r = 0u;
  } else {  // subnormal float result (or a round-up to the smallest normal)
    const unsigned long long s = (1ull << 52) | ((unsigned long long)(hi & 0xfffffu) << 32) | lo;
    const unsigned sh = 926u - e;  // >= 30
    if (sh > 63u) {
      r = 0u;
    } else {
      const unsigned long long q = s >> sh, rem = s & ((1ull << sh) - 1ull), half = 1ull << (sh - 1u);
      r = (unsigned)q + ((rem > half || (rem == half && (q & 1ull))) ? 1u : 0u);
    }
  }
  return __uint_as_float(sign | r);
}

// widen(f) / 2 exactly: a double made from a float is zero or normal with an
// exponent far above 1, so halving is one step down of the exponent field.
__device__ __forceinline__ double widen_half(float f) {
  const double w = widen(f);
  const long long b = __double_as_longlong(w);
  return (b & 0x7fffffffffffffffll) == 0 ? w : __longlong_as_double(b - (1ll << 52));
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
  // 1/b the same way (two FP64 operations)
  static __device__ __forceinline__ T rcp(T b) {
    const double r = widen(__frcp_rn(narrow(b)));
    return fma(r, fma(-b, r, 1.0), r);
  }
  // a*b + c with one rounding, and e - k/2 with one rounding
  static __device__ __forceinline__ T fmadd(T a, T b, T c) { return fma(a, b, c); }
  static __device__ __forceinline__ T sub_half(T e, T k) { return fma(k, -0.5, e); }
  static __device__ __forceinline__ float tof(T a) { return narrow(a); }
  // a < 0 from the bits (integer compare; a DSETP would take an FP64-pipe
  // slot): sign set, not -0, not NaN
  static __device__ __forceinline__ bool neg(T a) {
    const long long b = __double_as_longlong(a);
    return b < 0 && (b & 0x7fffffffffffffffll) != 0 && (b & 0x7fffffffffffffffll) <= 0x7ff0000000000000ll;
  }
  static __device__ __forceinline__ T konst(double hi, float, float) { return hi; }
  // (x + y) / 2 of two floats: one FMA, the same value as 0.5 * (x + y)
  // (halving commutes with rounding)
  static __device__ __forceinline__ T avg2(float x, float y) { return fma(0.5, widen(x), widen_half(y)); }
  // RK2 corrector (u0 + u + d) / 2 with one FMA after the sum
  static __device__ __forceinline__ T half_sum3(T u0, T u, float d) { return fma(0.5, u0 + u, widen_half(d)); }
  // u0 + (d0 + d1) / 2 with the two floats summed exactly (their exponents
  // within 29 of each other; else one rounding) and one FMA
  static __device__ __forceinline__ T add_half_sum(T u0, float d0, float d1) {
    return fma(0.5, widen(d0) + widen(d1), u0);
  }
  // element q of a resident accumulator array
  static __device__ __forceinline__ T ld(const void* p, long long q) { return ((const double*)p)[q]; }
  static __device__ __forceinline__ void st(void* p, long long q, T v) { ((double*)p)[q] = v; }
};

// FP64 accumulators with the hardware conversions, for kernels that are not
// bound by the FP64 pipe (the batched tubes): there the integer forms only
// add issue slots and registers.
struct f64hw {};
template <> struct Acc<f64hw> : Acc<double> {
  static __device__ __forceinline__ T from(float a) { return (double)a; }
  static __device__ __forceinline__ T prod(float a, float b) { return (double)a * (double)b; }
  static __device__ __forceinline__ T addf(T a, float b) { return a + (double)b; }
  static __device__ __forceinline__ T mulf(T a, float b) { return a * (double)b; }
  static __device__ __forceinline__ T div(T a, T b) {
    double r = (double)__frcp_rn((float)b);
    r = fma(r, fma(-b, r, 1.0), r);
    return a * r;
  }
  static __device__ __forceinline__ float tof(T a) { return (float)a; }
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
  static __device__ __forceinline__ T rcp(T b) { return dw_div(dw{1.f, 0.f}, b); }
  static __device__ __forceinline__ T fmadd(T a, T b, T c) { return a * b + c; }
  static __device__ __forceinline__ T sub_half(T e, T k) { return e - k * 0.5f; }
  static __device__ __forceinline__ float tof(T a) { return dw_to_float(a); }
  static __device__ __forceinline__ bool neg(T a) { return a.hi < 0.f || (a.hi == 0.f && a.lo < 0.f); }
  static __device__ __forceinline__ T konst(double, float hi, float lo) { return {hi, lo}; }
  static __device__ __forceinline__ T avg2(float x, float y) { return (dw{x, 0.f} + y) * 0.5f; }
  static __device__ __forceinline__ T half_sum3(T u0, T u, float d) { return ((u + d) + u0) * 0.5f; }
  static __device__ __forceinline__ T add_half_sum(T u0, float d0, float d1) {
    return u0 + two_sum(d0, d1) * 0.5f;
  }
  static __device__ __forceinline__ T ld(const void* p, long long q) {
    const float2 f = ((const float2*)p)[q];
    return {f.x, f.y};
  }
  static __device__ __forceinline__ void st(void* p, long long q, T v) { ((float2*)p)[q] = make_float2(v.hi, v.lo); }
};

}  // namespace pg
