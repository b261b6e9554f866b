// Point-wise ideal-MHD physics (device code; also callable on the host), templated on the arithmetic
// type.  Every expression keeps the operand order of PLUTO 4.3 so that the
// FP64 instantiation, compiled without multiply-add contraction, reproduces
// the reference C code bit for bit.  References are to files in the PLUTO
// source tree.
#pragma once
#include <cstdint>

namespace pg {

enum : int { RHO = 0, VX1 = 1, VX2 = 2, VX3 = 3, BX1 = 4, BX2 = 5, BX3 = 6, PRS = 7, NV = 8 };
constexpr int MX1 = VX1, ENG = PRS;
constexpr unsigned char FLAG_CONS2PRIM_FAIL = 64;  // Src/pluto.h:200

// FlipSign, Src/boundary.c:318-437: +1 or -1 for variable nv (BX1+d for a
// face component) mirrored across a REFLECTIVE / EQTSYMMETRIC side of axis d.
__host__ __device__ __forceinline__ int bc_flip(int d, int type, int nv, int components) {
  if (type != 2 && type != 3) return 1;  // PG_REFLECTIVE, PG_EQTSYMMETRIC
  if (nv == 1 + d) return -1;            // normal velocity
  if (type == 3) {
    if (nv == 4 + d) return 1;
    return (nv >= 4 && nv <= 6 && nv - 4 < components) ? -1 : 1;
  }
  return nv == 4 + d ? -1 : 1;           // normal field
}
// An axis's boundary types packed as beginning | end << 4 (the reference sets
// them per side, pluto.ini X*-beg / X*-end; PERIODIC on both sides is 0), and
// the type of one side.
__host__ __device__ __forceinline__ int bc_pack(int lo, int hi) { return lo | (hi << 4); }
__host__ __device__ __forceinline__ int bc_side(int packed, bool end_side) {
  return end_side ? (packed >> 4) & 15 : packed & 15;
}
// mirror / image / edge zone that ghost x copies from (Src/boundary.c:439-560)
__host__ __device__ __forceinline__ int bc_src(int x, int beg, int end, int n, int packed) {
  if (x < beg) {
    const int type = packed & 15;
    return type == 0 ? x + n : (type == 1 ? beg : 2 * beg - x - 1);
  }
  if (x > end) {
    const int type = (packed >> 4) & 15;
    return type == 0 ? x - n : (type == 1 ? end : 2 * end - x + 1);
  }
  return x;
}

template <class T> __host__ __device__ __forceinline__ T pmax(T a, T b) { return a >= b ? a : b; }  // macros.h MAX
template <class T> __host__ __device__ __forceinline__ T pmin(T a, T b) { return a <= b ? a : b; }  // macros.h MIN
template <class T> __host__ __device__ __forceinline__ T abs_min(T a, T b) { return fabs(a) < fabs(b) ? a : b; }
template <class T> __host__ __device__ __forceinline__ T minmod(T a, T b) {
  return a * b > T(0) ? (fabs(a) < fabs(b) ? a : b) : T(0);
}

// Normal/tangent/bitangent rotation, Src/set_indexes.c:49-124.
template <int DIR> struct Rot;
template <> struct Rot<0> { static constexpr int vn = VX1, vt = VX2, vb = VX3, bn = BX1, bt = BX2, bb = BX3; };
template <> struct Rot<1> { static constexpr int vn = VX2, vt = VX1, vb = VX3, bn = BX2, bt = BX1, bb = BX3; };
template <> struct Rot<2> { static constexpr int vn = VX3, vt = VX1, vb = VX2, bn = BX3, bt = BX1, bb = BX2; };

// Src/MHD/mappers.c:25-86
template <class T>
__host__ __device__ __forceinline__ void prim_to_cons(const T* v, T* u, T gmm1) {
  T kinb2;
  u[RHO] = v[RHO];
  u[MX1] = v[RHO] * v[VX1];
  u[MX1 + 1] = v[RHO] * v[VX2];
  u[MX1 + 2] = v[RHO] * v[VX3];
  u[BX1] = v[BX1];
  u[BX2] = v[BX2];
  u[BX3] = v[BX3];
  kinb2 = v[VX1] * v[VX1] + v[VX2] * v[VX2] + v[VX3] * v[VX3];
  kinb2 = v[RHO] * kinb2 + v[BX1] * v[BX1] + v[BX2] * v[BX2] + v[BX3] * v[BX3];
  kinb2 *= T(0.5);
  u[ENG] = kinb2 + v[PRS] / gmm1;
}

// Src/MHD/mappers.c:88-254 (ideal EOS): floors modify u in place.
template <class T>
__host__ __device__ __forceinline__ int cons_to_prim(T* u, T* v, T gmm1, T small_rho, T small_p,
                                            unsigned char* flag) {
  T tau, kinb2, m2, b2;
  int ifail = 0;
  m2 = u[MX1] * u[MX1] + u[MX1 + 1] * u[MX1 + 1] + u[MX1 + 2] * u[MX1 + 2];
  b2 = u[BX1] * u[BX1] + u[BX2] * u[BX2] + u[BX3] * u[BX3];
  if (u[RHO] < T(0)) {
    u[RHO] = small_rho;
    *flag |= FLAG_CONS2PRIM_FAIL;
    ifail = 1;
  }
  v[RHO] = u[RHO];
  tau = T(1) / u[RHO];
  v[VX1] = u[MX1] * tau;
  v[VX2] = u[MX1 + 1] * tau;
  v[VX3] = u[MX1 + 2] * tau;
  v[BX1] = u[BX1];
  v[BX2] = u[BX2];
  v[BX3] = u[BX3];
  kinb2 = T(0.5) * (m2 * tau + b2);
  if (u[ENG] < T(0)) {
    u[ENG] = small_p / gmm1 + kinb2;
    *flag |= FLAG_CONS2PRIM_FAIL;
    ifail = 1;
  }
  v[PRS] = gmm1 * (u[ENG] - kinb2);
  if (v[PRS] < T(0)) {
    v[PRS] = small_p;
    u[ENG] = v[PRS] / gmm1 + kinb2;
    *flag |= FLAG_CONS2PRIM_FAIL;
    ifail = 1;
  }
  return ifail;
}

// Src/MHD/fluxes.c:110-249
template <int DIR, class T>
__host__ __device__ __forceinline__ void flux(const T* v, const T* u, T* fx, T& ptot) {
  using R = Rot<DIR>;
  T Bmag2 = v[BX1] * v[BX1] + v[BX2] * v[BX2] + v[BX3] * v[BX3];
  ptot = v[PRS] + T(0.5) * Bmag2;
  T vB = v[VX1] * v[BX1] + v[VX2] * v[BX2] + v[VX3] * v[BX3];
  fx[RHO] = u[R::vn];
  fx[MX1] = v[R::vn] * u[MX1] - v[R::bn] * v[BX1];
  fx[MX1 + 1] = v[R::vn] * u[MX1 + 1] - v[R::bn] * v[BX2];
  fx[MX1 + 2] = v[R::vn] * u[MX1 + 2] - v[R::bn] * v[BX3];
  fx[R::bn] = T(0);
  fx[R::bt] = v[R::vn] * v[R::bt] - v[R::bn] * v[R::vt];
  fx[R::bb] = v[R::vn] * v[R::bb] - v[R::bn] * v[R::vb];
  fx[ENG] = (u[ENG] + ptot) * v[R::vn] - v[R::bn] * vB;
}

// Src/MHD/eigenv.c:35-104 (ideal EOS)
template <int DIR, class T>
__host__ __device__ __forceinline__ void max_signal_speed(const T* v, T gamma, T& cmin, T& cmax) {
  using R = Rot<DIR>;
  T gpr = gamma * v[PRS];
  T b1 = v[R::bn], b2 = v[R::bt], b3 = v[R::bb];
  T Btmag2 = b2 * b2 + b3 * b3;
  T Bmag2 = b1 * b1 + Btmag2;
  T cf = gpr - Bmag2;
  cf = gpr + Bmag2 + sqrt(cf * cf + T(4) * gpr * Btmag2);
  cf = sqrt(T(0.5) * cf / v[RHO]);
  cmin = v[R::vn] - cf;
  cmax = v[R::vn] + cf;
}

template <class T> struct Iface {
  T f[NV];
  T press, SL, SR, cmax;
};

// Src/MHD/hll_speed.c:23-108 (DAVIS_ESTIMATE); Mach estimate only on request.
template <int DIR, bool MACH, class T>
__host__ __device__ __forceinline__ void hll_speed(const T* vL, const T* vR, T gamma, T& SL, T& SR, T& mach) {
  using R = Rot<DIR>;
  T slmin, slmax, srmin, srmax;
  max_signal_speed<DIR>(vL, gamma, slmin, slmax);
  max_signal_speed<DIR>(vR, gamma, srmin, srmax);
  SL = pmin(slmin, srmin);
  SR = pmax(slmax, srmax);
  if (MACH) {
    T a2L = gamma * vL[PRS] / vL[RHO];
    T a2R = gamma * vR[PRS] / vR[RHO];
    T scrh = fabs(vL[R::vn]) + fabs(vR[R::vn]);
    scrh /= sqrt(a2L) + sqrt(a2R);
    mach = scrh;
  }
}

// Src/MHD/hll.c:30-166
template <int DIR, bool MACH, class T>
__host__ __device__ __forceinline__ void hll_solver(const T* vL, const T* uL, const T* vR, const T* uR, T gamma,
                                           Iface<T>& o, T& mach) {
  T fL[NV], fR[NV], ptL, ptR, SL, SR, scrh;
  flux<DIR>(vL, uL, fL, ptL);
  flux<DIR>(vR, uR, fR, ptR);
  hll_speed<DIR, MACH>(vL, vR, gamma, SL, SR, mach);
  o.SL = SL;
  o.SR = SR;
  o.cmax = pmax(fabs(SL), fabs(SR));
  if (SL > T(0)) {
#pragma unroll
    for (int nv = 0; nv < NV; nv++) o.f[nv] = fL[nv];
    o.press = ptL;
  } else if (SR < T(0)) {
#pragma unroll
    for (int nv = 0; nv < NV; nv++) o.f[nv] = fR[nv];
    o.press = ptR;
  } else {
    scrh = T(1) / (SR - SL);
#pragma unroll
    for (int nv = 0; nv < NV; nv++) {
      o.f[nv] = SL * SR * (uR[nv] - uL[nv]) + SR * fL[nv] - SL * fR[nv];
      o.f[nv] *= scrh;
    }
    o.press = (SR * ptL - SL * ptR) * scrh;
  }
}

// Src/MHD/roe.c:53-799: linearised solver of Cargo & Gallice (1997), ideal
// EOS, no background field, HLL hybridisation off, entropy fix delta = 1e-6.
// Waves in the order of the KWAVES enumeration (Src/MHD/mod_defs.h:54-72):
// fast-, fast+, entropy, div.B (zero jump), slow-, slow+ and, with three
// components, Alfven-, Alfven+.  The upwind sum skips the structurally zero
// eigenvector entries (adding them changes no bit).  bad = 1 when the Roe
// sound speed squared is negative (the reference stops the run there).
template <int DIR, bool MACH, class T>
__host__ __device__ __forceinline__ void roe_solver(const T* vL, const T* uL, const T* vR, const T* uR, T gamma, bool c3,
                                           Iface<T>& o, T& mach, int& bad) {
  using R = Rot<DIR>;
  constexpr int vn = R::vn, vt = R::vt, vb = R::vb, bn = R::bn, bt = R::bt, bb = R::bb;
  const T delta = T(1.e-6), g1 = gamma - T(1);
  T fL[NV], fR[NV], ptL, ptR, dV[NV], dU[NV];
  flux<DIR>(vL, uL, fL, ptL);
  flux<DIR>(vR, uR, fR, ptR);
#pragma unroll
  for (int nv = 0; nv < NV; nv++) {
    dV[nv] = vR[nv] - vL[nv];
    dU[nv] = uR[nv] - uL[nv];
  }
  // Roe averages
  const T srL = sqrt(vL[RHO]), srR = sqrt(vR[RHO]);
  const T sl = srL / (srL + srR), sr = srR / (srL + srR);
  const T rho = sr * vL[RHO] + sl * vR[RHO];
  const T sqrt_rho = sqrt(rho);
  const T u = sl * vL[vn] + sr * vR[vn];
  const T v = sl * vL[vt] + sr * vR[vt];
  const T w = sl * vL[vb] + sr * vR[vb];
  const T Bx = sr * vL[bn] + sl * vR[bn];
  const T By = sr * vL[bt] + sl * vR[bt];
  const T Bz = sr * vL[bb] + sl * vR[bb];
  const T sBx = Bx >= T(0) ? T(1) : T(-1);
  const T bx = Bx / sqrt_rho, by = By / sqrt_rho, bz = Bz / sqrt_rho;
  const T bt2 = T(0) + by * by + bz * bz;
  const T b2 = bx * bx + bt2;
  const T Btmag = sqrt(bt2 * rho);
  T X = dV[bn] * dV[bn] + dV[bt] * dV[bt] + dV[bb] * dV[bb];
  X /= (srL + srR) * (srL + srR) * T(2);
  const T vdm = u * dU[vn] + v * dU[vt] + w * dU[vb];
  const T BdB = Bx * dU[bn] + By * dU[bt] + Bz * dU[bb];
  // enthalpy and sound speed
  const T vel2 = u * u + v * v + w * w;
  dV[PRS] = g1 * ((T(0.5) * vel2 - X) * dV[RHO] - vdm + dU[ENG] - BdB);
  const T HL = (uL[ENG] + ptL) / vL[RHO];
  const T HR = (uR[ENG] + ptR) / vR[RHO];
  const T H = sl * HL + sr * HR;
  const T Hgas = H - b2;
  T a2 = (T(2) - gamma) * X + g1 * (Hgas - T(0.5) * vel2);
  if (a2 < T(0)) {
    bad = 1;
    a2 = sqrt(gamma * (vL[PRS] + vR[PRS]) / (vL[RHO] + vR[RHO]));
  }
  // fast and slow speeds
  T scrh = a2 - b2;
  const T ca2 = bx * bx;
  scrh = scrh * scrh + T(4) * bt2 * a2;
  scrh = sqrt(scrh);
  const T cf2 = T(0.5) * (a2 + b2 + scrh);
  const T cs2 = a2 * ca2 / cf2;
  const T cf = sqrt(cf2), cs = sqrt(cs2), ca = sqrt(ca2), a = sqrt(a2);
  T af, as;
  if (cf == cs) {
    af = T(1);
    as = T(0);
  } else if (a <= cs) {
    af = T(0);
    as = T(1);
  } else if (cf <= a) {
    af = T(1);
    as = T(0);
  } else {
    scrh = T(1) / (cf2 - cs2);
    af = (a2 - cs2) * scrh;
    as = (cf2 - a2) * scrh;
    af = pmax(T(0), af);
    as = pmax(T(0), as);
    af = sqrt(af);
    as = sqrt(as);
  }
  T beta_y, beta_z;
  if (Btmag > T(1.e-9)) {
    if (c3) {
      beta_y = By / Btmag;
      beta_z = Bz / Btmag;
    } else {
      beta_y = By >= T(0) ? T(1) : T(-1);
      beta_z = T(0);
    }
  } else {
    beta_y = c3 ? T(0.70710678118654752440) : T(1);
    beta_z = c3 ? T(0.70710678118654752440) : T(0);
  }
  const T beta_dv = T(0) + beta_y * dV[vt] + beta_z * dV[vb];
  const T beta_dB = T(0) + beta_y * dV[bt] + beta_z * dV[bb];
  const T beta_v = T(0) + beta_y * v + beta_z * w;
  const T h2 = T(0.5) / a2;

  // fast waves (eigenvector rows: rho, m_n, m_t, m_b, B_t, B_b, energy)
  scrh = as * cs * sBx;
  const T l0 = u - cf, l1 = u + cf;
  const T f_mt0 = af * v + scrh * beta_y, f_mb0 = af * w + scrh * beta_z;
  const T f_mt1 = af * v - scrh * beta_y, f_mb1 = af * w - scrh * beta_z;
  const T f_bt = as * a * beta_y / sqrt_rho, f_bb = as * a * beta_z / sqrt_rho;
  const T f_e0 = af * (Hgas - u * cf) + scrh * beta_v + as * a * Btmag / sqrt_rho;
  const T f_e1 = af * (Hgas + u * cf) - scrh * beta_v + as * a * Btmag / sqrt_rho;
  T eta0 = af * (X * dV[RHO] + dV[PRS]) + rho * scrh * beta_dv - rho * af * cf * dV[vn] +
           sqrt_rho * as * a * beta_dB;
  eta0 *= h2;
  T eta1 = af * (X * dV[RHO] + dV[PRS]) - rho * scrh * beta_dv + rho * af * cf * dV[vn] +
           sqrt_rho * as * a * beta_dB;
  eta1 *= h2;
  // entropy wave
  const T e_en = T(0.5) * vel2 + (gamma - T(2)) / g1 * X;
  const T eta2 = ((a2 - X) * dV[RHO] - dV[PRS]) / a2;
  // slow waves
  scrh = af * cf * sBx;
  const T l4 = u - cs, l5 = u + cs;
  const T s_mt4 = as * v - scrh * beta_y, s_mb4 = as * w - scrh * beta_z;
  const T s_mt5 = as * v + scrh * beta_y, s_mb5 = as * w + scrh * beta_z;
  const T s_bt = -af * a * beta_y / sqrt_rho, s_bb = -af * a * beta_z / sqrt_rho;
  const T s_e4 = as * (Hgas - u * cs) - scrh * beta_v - af * a * Btmag / sqrt_rho;
  const T s_e5 = as * (Hgas + u * cs) + scrh * beta_v - af * a * Btmag / sqrt_rho;
  T eta4 = as * (X * dV[RHO] + dV[PRS]) - rho * scrh * beta_dv - rho * as * cs * dV[vn] -
           sqrt_rho * af * a * beta_dB;
  eta4 *= h2;
  T eta5 = as * (X * dV[RHO] + dV[PRS]) + rho * scrh * beta_dv + rho * as * cs * dV[vn] -
           sqrt_rho * af * a * beta_dB;
  eta5 *= h2;

  o.cmax = fabs(u) + cf;
  if (MACH) mach = fabs(u / a);
  // |lambda| with the entropy fix on the fast and slow waves
  auto fix = [&](T l) -> T {
    T al = fabs(l);
    if (al < T(0.5) * delta) al = l * l / delta + T(0.25) * delta;
    return al;
  };
  const T c0 = fix(l0) * eta0, c1 = fix(l1) * eta1, c2 = fabs(u) * eta2;
  const T c4 = fix(l4) * eta4, c5 = fix(l5) * eta5;
  T s_rho = T(0) + c0 * af + c1 * af + c2 * T(1) + c4 * as + c5 * as;
  T s_mn = T(0) + c0 * (af * l0) + c1 * (af * l1) + c2 * u + c4 * (as * l4) + c5 * (as * l5);
  T s_mt = T(0) + c0 * f_mt0 + c1 * f_mt1 + c2 * v + c4 * s_mt4 + c5 * s_mt5;
  T s_mb = T(0) + c0 * f_mb0 + c1 * f_mb1 + c2 * w + c4 * s_mb4 + c5 * s_mb5;
  T s_bt2 = T(0) + c0 * f_bt + c1 * f_bt + c4 * s_bt + c5 * s_bt;
  T s_bb2 = T(0) + c0 * f_bb + c1 * f_bb + c4 * s_bb + c5 * s_bb;
  T s_en = T(0) + c0 * f_e0 + c1 * f_e1 + c2 * e_en + c4 * s_e4 + c5 * s_e5;
  if (c3) {  // Alfven waves
    const T l6 = u - ca, l7 = u + ca;
    const T a_mt = -rho * beta_z, a_mb = +rho * beta_y;
    const T a_bt = -sBx * sqrt_rho * beta_z, a_bb = sBx * sqrt_rho * beta_y;
    const T a_en = -rho * (v * beta_z - w * beta_y);
    T eta6 = +beta_y * dV[vb] - beta_z * dV[vt] + sBx / sqrt_rho * (beta_y * dV[bb] - beta_z * dV[bt]);
    eta6 *= T(0.5);
    T eta7 = -beta_y * dV[vb] + beta_z * dV[vt] + sBx / sqrt_rho * (beta_y * dV[bb] - beta_z * dV[bt]);
    eta7 *= T(0.5);
    const T c6 = fabs(l6) * eta6, c7 = fabs(l7) * eta7;
    s_mt = s_mt + c6 * a_mt + c7 * (-a_mt);
    s_mb = s_mb + c6 * a_mb + c7 * (-a_mb);
    s_bt2 = s_bt2 + c6 * a_bt + c7 * a_bt;
    s_bb2 = s_bb2 + c6 * a_bb + c7 * a_bb;
    s_en = s_en + c6 * a_en + c7 * (-a_en);
  }
  o.f[RHO] = T(0.5) * (fL[RHO] + fR[RHO] - s_rho);
  o.f[vn] = T(0.5) * (fL[vn] + fR[vn] - s_mn);
  o.f[vt] = T(0.5) * (fL[vt] + fR[vt] - s_mt);
  o.f[vb] = T(0.5) * (fL[vb] + fR[vb] - s_mb);
  o.f[bn] = T(0.5) * (fL[bn] + fR[bn] - T(0));
  o.f[bt] = T(0.5) * (fL[bt] + fR[bt] - s_bt2);
  o.f[bb] = T(0.5) * (fL[bb] + fR[bb] - s_bb2);
  o.f[ENG] = T(0.5) * (fL[ENG] + fR[ENG] - s_en);
  o.press = T(0.5) * (ptL + ptR);
  o.SL = l0;
  o.SR = l1;
}

// Src/MHD/hlld.c:44-452 (ideal EOS, no background field)
template <int DIR, bool MACH, class T>
__host__ __device__ __forceinline__ void hlld_solver(const T* vL, const T* uL, const T* vR, const T* uR, T gamma,
                                            Iface<T>& o, T& mach) {
  using R = Rot<DIR>;
  constexpr int MXn = R::vn, MXt = R::vt, MXb = R::vb;
  constexpr int VXn = R::vn, VXt = R::vt, VXb = R::vb;
  constexpr int BXn = R::bn, BXt = R::bt, BXb = R::bb;
  T fL[NV], fR[NV], ptL, ptR, SL, SR, scrh;
  flux<DIR>(vL, uL, fL, ptL);
  flux<DIR>(vR, uR, fR, ptR);
  hll_speed<DIR, MACH>(vL, vR, gamma, SL, SR, mach);
  o.SL = SL;
  o.SR = SR;
  o.cmax = pmax(fabs(SL), fabs(SR));

  if (SL >= T(0)) {
#pragma unroll
    for (int nv = 0; nv < NV; nv++) o.f[nv] = fL[nv];
    o.press = ptL;
    return;
  }
  if (SR <= T(0)) {
#pragma unroll
    for (int nv = 0; nv < NV; nv++) o.f[nv] = fR[nv];
    o.press = ptR;
    return;
  }
  T usL[NV], usR[NV];
  T Bx, Bx1, sBx, duL, duR, SM, pts, sqrL, sqrR, S1L, S1R, scrhL, scrhR, vsL, vsR, wsL, wsR;
  scrh = T(1) / (SR - SL);
  Bx1 = Bx = (SR * vR[BXn] - SL * vL[BXn]) * scrh;
  sBx = (Bx > T(0) ? T(1) : T(-1));
  duL = SL - vL[VXn];
  duR = SR - vR[VXn];
  scrh = T(1) / (duR * uR[RHO] - duL * uL[RHO]);
  SM = (duR * uR[MXn] - duL * uL[MXn] - ptR + ptL) * scrh;
  pts = duR * uR[RHO] * ptL - duL * uL[RHO] * ptR + vL[RHO] * vR[RHO] * duR * duL * (vR[VXn] - vL[VXn]);
  pts *= scrh;
  usL[RHO] = uL[RHO] * duL / (SL - SM);
  usR[RHO] = uR[RHO] * duR / (SR - SM);
  sqrL = sqrt(usL[RHO]);
  sqrR = sqrt(usR[RHO]);
  S1L = SM - fabs(Bx) / sqrL;
  S1R = SM + fabs(Bx) / sqrR;

  bool revert_to_hllc = false;
  if ((S1L - SL) < T(1.e-4) * (SM - SL)) revert_to_hllc = true;
  if ((S1R - SR) > -T(1.e-4) * (SR - SM)) revert_to_hllc = true;

  if (revert_to_hllc) {
    scrh = T(1) / (SR - SL);
    T Un = (SR * uR[BXn] - SL * uL[BXn] + fL[BXn] - fR[BXn]) * scrh;
    T Ut = (SR * uR[BXt] - SL * uL[BXt] + fL[BXt] - fR[BXt]) * scrh;
    T Ub = (SR * uR[BXb] - SL * uL[BXb] + fL[BXb] - fR[BXb]) * scrh;
    usL[BXn] = usR[BXn] = Un;
    usL[BXt] = usR[BXt] = Ut;
    usL[BXb] = usR[BXb] = Ub;
    S1L = S1R = SM;
  } else {
    scrhL = (uL[RHO] * duL * duL - Bx * Bx) / (uL[RHO] * duL * (SL - SM) - Bx * Bx);
    scrhR = (uR[RHO] * duR * duR - Bx * Bx) / (uR[RHO] * duR * (SR - SM) - Bx * Bx);
    usL[BXn] = Bx1;
    usL[BXt] = uL[BXt] * scrhL;
    usL[BXb] = uL[BXb] * scrhL;
    usR[BXn] = Bx1;
    usR[BXt] = uR[BXt] * scrhR;
    usR[BXb] = uR[BXb] * scrhR;
  }
  scrhL = Bx / (uL[RHO] * duL);
  scrhR = Bx / (uR[RHO] * duR);
  vsL = vL[VXt] - scrhL * (usL[BXt] - uL[BXt]);
  vsR = vR[VXt] - scrhR * (usR[BXt] - uR[BXt]);
  wsL = vL[VXb] - scrhL * (usL[BXb] - uL[BXb]);
  wsR = vR[VXb] - scrhR * (usR[BXb] - uR[BXb]);
  usL[MXn] = usL[RHO] * SM;
  usR[MXn] = usR[RHO] * SM;
  usL[MXt] = usL[RHO] * vsL;
  usR[MXt] = usR[RHO] * vsR;
  usL[MXb] = usL[RHO] * wsL;
  usR[MXb] = usR[RHO] * wsR;

  scrhL = vL[VXn] * Bx1 + vL[VXt] * uL[BXt] + vL[VXb] * uL[BXb];
  scrhL -= SM * Bx1 + vsL * usL[BXt] + wsL * usL[BXb];
  usL[ENG] = duL * uL[ENG] - ptL * vL[VXn] + pts * SM + Bx * scrhL;
  usL[ENG] /= SL - SM;
  scrhR = vR[VXn] * Bx1 + vR[VXt] * uR[BXt] + vR[VXb] * uR[BXb];
  scrhR -= SM * Bx1 + vsR * usR[BXt] + wsR * usR[BXb];
  usR[ENG] = duR * uR[ENG] - ptR * vR[VXn] + pts * SM + Bx * scrhR;
  usR[ENG] /= SR - SM;

  if (S1L >= T(0)) {
#pragma unroll
    for (int nv = 0; nv < NV; nv++) o.f[nv] = fL[nv] + SL * (usL[nv] - uL[nv]);
    o.press = ptL;
  } else if (S1R <= T(0)) {
#pragma unroll
    for (int nv = 0; nv < NV; nv++) o.f[nv] = fR[nv] + SR * (usR[nv] - uR[nv]);
    o.press = ptR;
  } else {
    T ussl[NV], ussr[NV];
    ussl[RHO] = usL[RHO];
    ussr[RHO] = usR[RHO];
    T vss = sqrL * vsL + sqrR * vsR + (usR[BXt] - usL[BXt]) * sBx;
    vss /= sqrL + sqrR;
    T wss = sqrL * wsL + sqrR * wsR + (usR[BXb] - usL[BXb]) * sBx;
    wss /= sqrL + sqrR;
    ussl[MXn] = ussl[RHO] * SM;
    ussr[MXn] = ussr[RHO] * SM;
    ussl[MXt] = ussl[RHO] * vss;
    ussr[MXt] = ussr[RHO] * vss;
    ussl[MXb] = ussl[RHO] * wss;
    ussr[MXb] = ussr[RHO] * wss;
    ussl[BXn] = ussr[BXn] = Bx1;
    ussl[BXt] = sqrL * usR[BXt] + sqrR * usL[BXt] + sqrL * sqrR * (vsR - vsL) * sBx;
    ussl[BXt] /= sqrL + sqrR;
    ussr[BXt] = ussl[BXt];
    ussl[BXb] = sqrL * usR[BXb] + sqrR * usL[BXb] + sqrL * sqrR * (wsR - wsL) * sBx;
    ussl[BXb] /= sqrL + sqrR;
    ussr[BXb] = ussl[BXb];
    scrhL = SM * Bx1 + vsL * usL[BXt] + wsL * usL[BXb];
    scrhL -= SM * Bx1 + vss * ussl[BXt] + wss * ussl[BXb];
    scrhR = SM * Bx1 + vsR * usR[BXt] + wsR * usR[BXb];
    scrhR -= SM * Bx1 + vss * ussr[BXt] + wss * ussr[BXb];
    ussl[ENG] = usL[ENG] - sqrL * scrhL * sBx;
    ussr[ENG] = usR[ENG] + sqrR * scrhR * sBx;
    if (SM >= T(0)) {
#pragma unroll
      for (int nv = 0; nv < NV; nv++) o.f[nv] = fL[nv] + S1L * (ussl[nv] - usL[nv]) + SL * (usL[nv] - uL[nv]);
      o.press = ptL;
    } else {
#pragma unroll
      for (int nv = 0; nv < NV; nv++) o.f[nv] = fR[nv] + S1R * (ussr[nv] - usR[nv]) + SR * (usR[nv] - uR[nv]);
      o.press = ptR;
    }
  }
}

// Limiters, Src/States/plm_coeffs.h:72-175 (uniform Cartesian forms);
// DEFAULT mix from Src/States/plm_states.c:180-213.
enum : int { LIM_FLAT = 0, LIM_MINMOD = 1, LIM_VANLEER = 2, LIM_MC = 3, LIM_DEFAULT = 4 };

template <class T>
__host__ __device__ __forceinline__ T limit(int lim, int nv, T dvp, T dvm) {
  if (lim == LIM_DEFAULT) lim = (nv == RHO) ? LIM_MC : (nv == PRS ? LIM_MINMOD : LIM_VANLEER);
  switch (lim) {
    case LIM_FLAT: return T(0);
    case LIM_MINMOD: return dvp * dvm > T(0) ? abs_min(dvp, dvm) : T(0);
    case LIM_VANLEER: return dvp * dvm > T(0) ? T(2) * dvp * dvm / (dvp + dvm) : T(0);
    default:
      if (dvp * dvm > T(0)) {
        T qc = T(0.5) * (dvm + dvp), scrh = T(2) * abs_min(dvp, dvm);
        return abs_min(qc, scrh);
      }
      return T(0);
  }
}

// PPM interface value with minmod clip, ppm_states.c:131-143 (PPM_ORDER 4,
// Cartesian coefficients ppm_coeffs.c:478-520).
template <class T>
__host__ __device__ __forceinline__ T ppm_iface(T vm1, T v0, T vp1, T vp2) {
  const T w_1 = T(-1.0 / 12.0), w0 = T(7.0 / 12.0), w1 = T(7.0 / 12.0), w2 = T(-1.0 / 12.0);
  T vp = w_1 * vm1 + w0 * v0 + w1 * vp1 + w2 * vp2;
  T dv = vp1 - v0;
  T dvp = vp - v0;
  return v0 + minmod(dvp, dv);
}

// Parabolic limiter, ppm_states.c:146-207 with hp = hm = 3 (cp = cm = 2).
template <class T>
__host__ __device__ __forceinline__ void ppm_limit(T v, T& vp, T& vm) {
  const T cm = (T(3) + T(1)) / (T(3) - T(1));
  const T cp = (T(3) + T(1)) / (T(3) - T(1));
  T dvp = vp - v, dvm = vm - v;
  if (dvp * dvm >= T(0)) dvp = dvm = T(0);
  else {
    if (fabs(dvp) >= cm * fabs(dvm)) dvp = -cm * dvm;
    else if (fabs(dvm) >= cp * fabs(dvp)) dvm = -cp * dvp;
  }
  vp = v + dvp;
  vm = v + dvm;
}

// Src/MHD/CT/ct_stag_slopes.c:92-105
template <class T>
__host__ __device__ __forceinline__ T mc_lim2(T dp, T dm) {
  if (dp * dm < T(0)) return T(0);
  T dc = T(0.5) * (dp + dm);
  T scrh = T(2) * (fabs(dp) < fabs(dm) ? dp : dm);
  return fabs(dc) < fabs(scrh) ? dc : scrh;
}

// Combination of the 2D HLL edge formula, ct_emf_average.c:262-289.
template <class T>
__host__ __device__ __forceinline__ T uct_hll_combine(T a_xp, T a_xm, T a_yp, T a_ym, T eSW, T eSE, T eNE, T eNW, T bS,
                                             T bN, T bW, T bE) {
  T e = a_xp * a_yp * eSW + a_xm * a_yp * eSE + a_xm * a_ym * eNE + a_xp * a_ym * eNW;
  e /= (a_xp + a_xm) * (a_yp + a_ym);
  e -= a_yp * a_ym * (bN - bS) / (a_yp + a_ym);
  e += a_xp * a_xm * (bE - bW) / (a_xp + a_xm);
  return e;
}

}  // namespace pg
