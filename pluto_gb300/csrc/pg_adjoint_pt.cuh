// Point functions of the adjoint: the forward point evaluations the adjoint
// kernels differentiate (written over a small input vector), and hand-derived
// reverse-mode (transposed-Jacobian) versions of the HLL and HLLD Riemann
// outputs and of the edge EMF.
//
// A reverse function recomputes the forward point evaluation in FP64 with
// the forward's own expressions (so, compiled like the forward without
// multiply-add contraction, it takes the same branches bit for bit), then
// runs the chain rule backwards through the branch taken and returns
// J^T lambda for all inputs at once.  It replaces one Dual<1> evaluation per
// input (16 per interface, 40 per edge); the Dual<1> evaluation of the same
// point function stays the check of each derivative (the host harness
// tests/adjoint_rev_check.cu compares the two on random states that visit
// every branch).  Everything here also compiles for the host.
#pragma once
#include <cmath>

#include "pluto_gb300.h"
// the physics templates first: their calls of fabs / sqrt on a double bind
// to the C library functions, with the Dual<N> overloads found by ADL
#include "pg_physics.cuh"
#include "pg_dual.cuh"

namespace pg {

// States of one zone from w[0..4] = v[c-2..c+2] (as k_recon).
template <class T>
__host__ __device__ __forceinline__ void recon_pt(int recon, int lim, int nv, const T* w, T& vp, T& vm) {
  if (recon == PG_LINEAR) {
    T v0 = w[2];
    T dvp = w[3] - v0;
    T dvm = v0 - w[1];
    T dv = limit(lim, nv, dvp, dvm);
    vp = v0 + dv * 0.5;
    vm = v0 - dv * 0.5;
  } else {
    T v0 = w[2];
    T p = ppm_iface(w[1], v0, w[3], w[4]);
    T m = ppm_iface(w[0], w[1], v0, w[3]);
    ppm_limit(v0, p, m);
    vp = p;
    vm = m;
  }
}

// Riemann outputs at one interface (as k_riemann):
// out[0..7] flux, out[8] total pressure, out[9] max(0,-SL), out[10] max(0,SR).
constexpr int kRiemannOut = NV + 3;
template <class T, int DIR>
__host__ __device__ __forceinline__ void riemann_pt(int solver, double gamma, bool c3, const T* vL, const T* vR,
                                                    T* out) {
  T uL[NV], uR[NV], mach = T(0.0);
  const T gmm1 = T(gamma - 1.0);
  prim_to_cons(vL, uL, gmm1);
  prim_to_cons(vR, uR, gmm1);
  Iface<T> o;
  if (solver == PG_HLL) {
    hll_solver<DIR, false>(vL, uL, vR, uR, T(gamma), o, mach);
  } else if (solver == PG_ROE) {
    int bad = 0;
    roe_solver<DIR, false>(vL, uL, vR, uR, T(gamma), c3, o, mach, bad);
  } else {
    hlld_solver<DIR, false>(vL, uL, vR, uR, T(gamma), o, mach);
  }
#pragma unroll
  for (int nv = 0; nv < NV; nv++) out[nv] = o.f[nv];
  out[NV] = o.press;
  out[NV + 1] = pmax(T(0.0), -o.SL);
  out[NV + 2] = pmax(T(0.0), o.SR);
}

// Edge EMF from its 40 inputs (as uct_edge):
//  in[0..7]   SR_x(c00) SR_x(c0y) SL_x(c00) SL_x(c0y) SR_y(c00) SR_y(cx0) SL_y(c00) SL_y(cx0)
//  in[8..11]  x-face field at c00-sy, c00, c0y, c0y+sy
//  in[12..15] y-face field at c00-sx, c00, cx0, cx0+sx
//  in[16..39] per zone q of (c00, cx0, c0y, cxy): vy, vx, dvy_dx, dvy_dy, dvx_dx, dvx_dy
constexpr int kEdgeIn = 40;
template <class T>
__host__ __device__ __forceinline__ T emf_pt(const T* in) {
  T a_xp = pmax(in[0], in[1]);
  T a_xm = pmax(in[2], in[3]);
  T a_yp = pmax(in[4], in[5]);
  T a_ym = pmax(in[6], in[7]);
  T sbS = mc_lim2(in[10] - in[9], in[9] - in[8]);
  T sbN = mc_lim2(in[11] - in[10], in[10] - in[9]);
  T sbW = mc_lim2(in[14] - in[13], in[13] - in[12]);
  T sbE = mc_lim2(in[15] - in[14], in[14] - in[13]);
  T bS = in[9] + 0.5 * sbS;
  T bW = in[13] + 0.5 * sbW;
  T bN = in[10] - 0.5 * sbN;
  T bE = in[14] - 0.5 * sbE;
  const T* q0 = in + 16;  // c00
  const T* q1 = in + 22;  // cx0
  const T* q2 = in + 28;  // c0y
  const T* q3 = in + 34;  // cxy
  T eSW = (q0[0] + 0.5 * (q0[2] + q0[3])) * bS - (q0[1] + 0.5 * (q0[4] + q0[5])) * bW;
  T eSE = (q1[0] - 0.5 * (q1[2] - q1[3])) * bS - (q1[1] - 0.5 * (q1[4] - q1[5])) * bE;
  T eNE = (q3[0] - 0.5 * (q3[2] + q3[3])) * bN - (q3[1] - 0.5 * (q3[4] + q3[5])) * bE;
  T eNW = (q2[0] + 0.5 * (q2[2] - q2[3])) * bN - (q2[1] + 0.5 * (q2[4] - q2[5])) * bW;
  return uct_hll_combine(a_xp, a_xm, a_yp, a_ym, eSW, eSE, eNE, eNW, bS, bN, bW, bE);
}

// ---------------------------------------------------------------------------
// reverse-mode building blocks: each adds (d out / d in)^T a_out into a_in
// ---------------------------------------------------------------------------

// prim_to_cons (Src/MHD/mappers.c:25-86): a_v += (du/dv)^T a_u
__host__ __device__ __forceinline__ void p2c_rev(const double* v, double gmm1, const double* au, double* av) {
  const double k1 = v[VX1] * v[VX1] + v[VX2] * v[VX2] + v[VX3] * v[VX3];
  const double e = au[ENG];
  av[RHO] += au[RHO] + au[MX1] * v[VX1] + au[MX1 + 1] * v[VX2] + au[MX1 + 2] * v[VX3] + 0.5 * e * k1;
#pragma unroll
  for (int i = 0; i < 3; i++) {
    av[VX1 + i] += v[RHO] * (au[MX1 + i] + e * v[VX1 + i]);
    av[BX1 + i] += au[BX1 + i] + e * v[BX1 + i];
  }
  av[PRS] += e / gmm1;
}

// cons_to_prim (Src/MHD/mappers.c:88-254) transposed, floors included: lu
// = (dv/du)^T lv on the branch the forward takes.  A floored density is the
// constant small_rho (the velocities and kinetic energy still depend on the
// momenta through tau = 1/small_rho); a floored energy gives the pressure
// small_p's value, independent of u, and so does a floored pressure.
__host__ __device__ __forceinline__ void c2p_rev(const double* u, double gmm1, double small_rho, const double* lv,
                                                 double* lu) {
  const double m2 = u[MX1] * u[MX1] + u[MX1 + 1] * u[MX1 + 1] + u[MX1 + 2] * u[MX1 + 2];
  const double b2 = u[BX1] * u[BX1] + u[BX2] * u[BX2] + u[BX3] * u[BX3];
  const bool rho_fl = u[RHO] < 0.0;
  const double tau = 1.0 / (rho_fl ? small_rho : u[RHO]);
  const double kinb2 = 0.5 * (m2 * tau + b2);
  const bool p_dep = !(u[ENG] < 0.0) && !(gmm1 * (u[ENG] - kinb2) < 0.0);
#pragma unroll
  for (int nv = 0; nv < NV; nv++) lu[nv] = 0.0;
  double atau = 0.0;
#pragma unroll
  for (int i = 0; i < 3; i++) {  // v = m tau, B = B
    lu[MX1 + i] = lv[VX1 + i] * tau;
    atau += lv[VX1 + i] * u[MX1 + i];
    lu[BX1 + i] = lv[BX1 + i];
  }
  if (p_dep) {  // p = (g-1) (E - (m2 tau + b2)/2)
    const double akin = -gmm1 * lv[PRS];
    lu[ENG] = gmm1 * lv[PRS];
    atau += 0.5 * m2 * akin;
#pragma unroll
    for (int i = 0; i < 3; i++) {
      lu[MX1 + i] += u[MX1 + i] * tau * akin;
      lu[BX1 + i] += u[BX1 + i] * akin;
    }
  }
  if (!rho_fl) lu[RHO] = lv[RHO] - tau * tau * atau;
}

// flux (Src/MHD/fluxes.c:110-249): a_v, a_u += J^T (a_f, a_ptot)
template <int DIR>
__host__ __device__ __forceinline__ void flux_rev(const double* v, const double* u, const double* af, double apt,
                                                  double* av, double* au) {
  using R = Rot<DIR>;
  const double vn = v[R::vn], bn = v[R::bn];
  const double Bmag2 = v[BX1] * v[BX1] + v[BX2] * v[BX2] + v[BX3] * v[BX3];
  const double ptot = v[PRS] + 0.5 * Bmag2;
  const double vB = v[VX1] * v[BX1] + v[VX2] * v[BX2] + v[VX3] * v[BX3];
  au[R::vn] += af[RHO];
#pragma unroll
  for (int i = 0; i < 3; i++) {  // fx[MXi] = vn u[MXi] - bn B_i
    const double a = af[MX1 + i];
    av[R::vn] += a * u[MX1 + i];
    au[MX1 + i] += a * vn;
    av[R::bn] -= a * v[BX1 + i];
    av[BX1 + i] -= a * bn;
  }
  {  // fx[bt] = vn bt - bn vt
    const double a = af[R::bt];
    av[R::vn] += a * v[R::bt];
    av[R::bt] += a * vn;
    av[R::bn] -= a * v[R::vt];
    av[R::vt] -= a * bn;
  }
  {  // fx[bb] = vn bb - bn vb
    const double a = af[R::bb];
    av[R::vn] += a * v[R::bb];
    av[R::bb] += a * vn;
    av[R::bn] -= a * v[R::vb];
    av[R::vb] -= a * bn;
  }
  // fx[ENG] = (u[ENG] + ptot) vn - bn vB
  const double e = af[ENG];
  au[ENG] += e * vn;
  const double apt_tot = apt + e * vn;
  av[R::vn] += e * (u[ENG] + ptot);
  av[R::bn] -= e * vB;
  const double avB = -e * bn;
#pragma unroll
  for (int i = 0; i < 3; i++) {
    av[VX1 + i] += avB * v[BX1 + i];
    av[BX1 + i] += avB * v[VX1 + i] + apt_tot * v[BX1 + i];
  }
  av[PRS] += apt_tot;
}

// max_signal_speed (Src/MHD/eigenv.c:35-104): a_v += J^T (a_cmin, a_cmax)
template <int DIR>
__host__ __device__ __forceinline__ void signal_rev(const double* v, double gamma, double acmin, double acmax,
                                                    double* av) {
  using R = Rot<DIR>;
  if (acmin == 0.0 && acmax == 0.0) return;
  const double gpr = gamma * v[PRS];
  const double b1 = v[R::bn], b2 = v[R::bt], b3 = v[R::bb];
  const double Bt2 = b2 * b2 + b3 * b3;
  const double B2 = b1 * b1 + Bt2;
  const double cf0 = gpr - B2;
  const double sq = ::sqrt(cf0 * cf0 + 4.0 * gpr * Bt2);
  const double cf1 = gpr + B2 + sq;
  const double w = 0.5 * cf1 / v[RHO];
  const double cf = ::sqrt(w);
  av[R::vn] += acmin + acmax;
  const double aw = (acmax - acmin) * (0.5 / cf);
  const double acf1 = aw * 0.5 / v[RHO];
  av[RHO] -= aw * w / v[RHO];
  const double as = acf1 * (0.5 / sq);
  const double acf0 = as * 2.0 * cf0;
  const double agpr = acf1 + as * 4.0 * Bt2 + acf0;
  const double aB2 = acf1 - acf0;
  const double aBt2 = as * 4.0 * gpr + aB2;
  av[R::bn] += aB2 * 2.0 * b1;
  av[R::bt] += aBt2 * 2.0 * b2;
  av[R::bb] += aBt2 * 2.0 * b3;
  av[PRS] += agpr * gamma;
}

// The parts both solvers share: states, fluxes and the Davis speed
// estimate (hll_speed), recomputed as the forward computes them.
template <int DIR>
struct RiemannBase {
  double uL[NV], uR[NV], fL[NV], fR[NV], ptL, ptR, slmin, slmax, srmin, srmax, SL, SR;
  __host__ __device__ __forceinline__ RiemannBase(const double* vL, const double* vR, double gamma) {
    const double gmm1 = gamma - 1.0;
    prim_to_cons(vL, uL, gmm1);
    prim_to_cons(vR, uR, gmm1);
    flux<DIR>(vL, uL, fL, ptL);
    flux<DIR>(vR, uR, fR, ptR);
    max_signal_speed<DIR>(vL, gamma, slmin, slmax);
    max_signal_speed<DIR>(vR, gamma, srmin, srmax);
    SL = pmin(slmin, srmin);
    SR = pmax(slmax, srmax);
  }
  // a_SL, a_SR, a_fL/R, a_ptL/R, a_uL/R -> a_vL, a_vR (the latter hold the
  // direct uses already)
  __host__ __device__ __forceinline__ void finish(const double* vL, const double* vR, double gamma, double aSL,
                                                  double aSR, const double* afL, const double* afR, double aptL,
                                                  double aptR, double* auL, double* auR, double* aL,
                                                  double* aR) const {
    // SL = MIN(slmin, srmin), SR = MAX(slmax, srmax): the operand selected
    const bool lmin = slmin <= srmin, lmax = slmax >= srmax;
    signal_rev<DIR>(vL, gamma, lmin ? aSL : 0.0, lmax ? aSR : 0.0, aL);
    signal_rev<DIR>(vR, gamma, lmin ? 0.0 : aSL, lmax ? 0.0 : aSR, aR);
    flux_rev<DIR>(vL, uL, afL, aptL, aL, auL);
    flux_rev<DIR>(vR, uR, afR, aptR, aR, auR);
    p2c_rev(vL, gamma - 1.0, auL, aL);
    p2c_rev(vR, gamma - 1.0, auR, aR);
  }
};

// a_SL, a_SR from the outputs max(0,-SL), max(0,SR)
__host__ __device__ __forceinline__ void speed_out_rev(double SL, double SR, const double* lam, double& aSL,
                                                       double& aSR) {
  aSL = (0.0 >= -SL) ? 0.0 : -lam[NV + 1];
  aSR = (0.0 >= SR) ? 0.0 : lam[NV + 2];
}

// HLL (Src/MHD/hll.c:30-166): gL, gR = J^T lam for the outputs of riemann_pt
template <int DIR>
__host__ __device__ __forceinline__ void hll_rev(const double* vL, const double* vR, double gamma, const double* lam,
                                                 double* gL, double* gR) {
  const RiemannBase<DIR> b(vL, vR, gamma);
  double afL[NV], afR[NV], auL[NV], auR[NV], aSL, aSR, aptL = 0.0, aptR = 0.0;
#pragma unroll
  for (int nv = 0; nv < NV; nv++) {
    afL[nv] = afR[nv] = auL[nv] = auR[nv] = 0.0;
    gL[nv] = gR[nv] = 0.0;
  }
  speed_out_rev(b.SL, b.SR, lam, aSL, aSR);
  if (b.SL > 0.0) {
#pragma unroll
    for (int nv = 0; nv < NV; nv++) afL[nv] = lam[nv];
    aptL = lam[NV];
  } else if (b.SR < 0.0) {
#pragma unroll
    for (int nv = 0; nv < NV; nv++) afR[nv] = lam[nv];
    aptR = lam[NV];
  } else {
    // f = (SL SR (uR - uL) + SR fL - SL fR) s, press = (SR ptL - SL ptR) s, s = 1 / (SR - SL)
    const double SL = b.SL, SR = b.SR, s = 1.0 / (SR - SL);
    double as = 0.0;
#pragma unroll
    for (int nv = 0; nv < NV; nv++) {
      const double du = b.uR[nv] - b.uL[nv];
      const double N = SL * SR * du + SR * b.fL[nv] - SL * b.fR[nv];
      const double aN = lam[nv] * s;
      as += lam[nv] * N;
      aSL += aN * (SR * du - b.fR[nv]);
      aSR += aN * (SL * du + b.fL[nv]);
      auR[nv] += aN * SL * SR;
      auL[nv] -= aN * SL * SR;
      afL[nv] += aN * SR;
      afR[nv] -= aN * SL;
    }
    const double Np = SR * b.ptL - SL * b.ptR, aNp = lam[NV] * s;
    as += lam[NV] * Np;
    aSR += aNp * b.ptL;
    aptL += aNp * SR;
    aSL -= aNp * b.ptR;
    aptR -= aNp * SL;
    aSR -= as * s * s;
    aSL += as * s * s;
  }
  b.finish(vL, vR, gamma, aSL, aSR, afL, afR, aptL, aptR, auL, auR, gL, gR);
}

// HLLD (Src/MHD/hlld.c:44-452, ideal EOS, no background field): gL, gR =
// J^T lam for the outputs of riemann_pt.  The forward part repeats
// hlld_solver's expressions (values decide the branch); the reverse part
// goes back through the region selected (L / R flux, single-star state,
// double-star state, the HLLC reversion), each intermediate's adjoint
// complete before its definition is undone.
template <int DIR>
__host__ __device__ __forceinline__ void hlld_rev(const double* vL, const double* vR, double gamma, const double* lam,
                                                  double* gL, double* gR) {
  using R = Rot<DIR>;
  constexpr int MXn = R::vn, MXt = R::vt, MXb = R::vb;
  constexpr int VXn = R::vn, VXt = R::vt, VXb = R::vb;
  constexpr int BXn = R::bn, BXt = R::bt, BXb = R::bb;
  const RiemannBase<DIR> b(vL, vR, gamma);
  const double* uL = b.uL;
  const double* uR = b.uR;
  const double SL = b.SL, SR = b.SR, ptL = b.ptL, ptR = b.ptR;
  double afL[NV], afR[NV], auL[NV], auR[NV], aSL, aSR, aptL = 0.0, aptR = 0.0;
#pragma unroll
  for (int nv = 0; nv < NV; nv++) {
    afL[nv] = afR[nv] = auL[nv] = auR[nv] = 0.0;
    gL[nv] = gR[nv] = 0.0;
  }
  speed_out_rev(SL, SR, lam, aSL, aSR);

  if (SL >= 0.0) {
#pragma unroll
    for (int nv = 0; nv < NV; nv++) afL[nv] = lam[nv];
    aptL = lam[NV];
  } else if (SR <= 0.0) {
#pragma unroll
    for (int nv = 0; nv < NV; nv++) afR[nv] = lam[nv];
    aptR = lam[NV];
  } else {
    // ---- forward: the single-star states ----
    const double s0 = 1.0 / (SR - SL);
    const double NB = SR * vR[BXn] - SL * vL[BXn];
    const double Bx = NB * s0;  // Bx1 is the same value
    const double sBx = (Bx > 0.0 ? 1.0 : -1.0);
    const double duL = SL - vL[VXn];
    const double duR = SR - vR[VXn];
    const double D = duR * uR[RHO] - duL * uL[RHO];
    const double s1 = 1.0 / D;
    const double NSM = duR * uR[MXn] - duL * uL[MXn] - ptR + ptL;
    const double SM = NSM * s1;
    const double dvn = vR[VXn] - vL[VXn];
    const double pts0 = duR * uR[RHO] * ptL - duL * uL[RHO] * ptR + vL[RHO] * vR[RHO] * duR * duL * dvn;
    const double pts = pts0 * s1;
    const double tL = uL[RHO] * duL, tR = uR[RHO] * duR;
    const double dLm = SL - SM, dRm = SR - SM;
    const double rsL = tL / dLm, rsR = tR / dRm;
    const double sqrL = ::sqrt(rsL), sqrR = ::sqrt(rsR);
    const double aBxm = ::fabs(Bx);
    double S1L = SM - aBxm / sqrL;
    double S1R = SM + aBxm / sqrR;
    bool revert = false;
    if ((S1L - SL) < 1.e-4 * (SM - SL)) revert = true;
    if ((S1R - SR) > -1.e-4 * (SR - SM)) revert = true;
    double usL[NV], usR[NV];
    double s2 = 0.0, Nc[3] = {0.0, 0.0, 0.0};
    double nL = 0.0, mL = 1.0, hL = 0.0, nR = 0.0, mR = 1.0, hR = 0.0;
    if (revert) {
      s2 = 1.0 / (SR - SL);
      Nc[0] = SR * uR[BXn] - SL * uL[BXn] + b.fL[BXn] - b.fR[BXn];
      Nc[1] = SR * uR[BXt] - SL * uL[BXt] + b.fL[BXt] - b.fR[BXt];
      Nc[2] = SR * uR[BXb] - SL * uL[BXb] + b.fL[BXb] - b.fR[BXb];
      usL[BXn] = usR[BXn] = Nc[0] * s2;
      usL[BXt] = usR[BXt] = Nc[1] * s2;
      usL[BXb] = usR[BXb] = Nc[2] * s2;
      S1L = S1R = SM;
    } else {
      nL = uL[RHO] * duL * duL - Bx * Bx;
      mL = uL[RHO] * duL * dLm - Bx * Bx;
      hL = nL / mL;
      nR = uR[RHO] * duR * duR - Bx * Bx;
      mR = uR[RHO] * duR * dRm - Bx * Bx;
      hR = nR / mR;
      usL[BXn] = Bx;
      usL[BXt] = uL[BXt] * hL;
      usL[BXb] = uL[BXb] * hL;
      usR[BXn] = Bx;
      usR[BXt] = uR[BXt] * hR;
      usR[BXb] = uR[BXb] * hR;
    }
    const double qL = Bx / tL, qR = Bx / tR;
    const double vsL = vL[VXt] - qL * (usL[BXt] - uL[BXt]);
    const double vsR = vR[VXt] - qR * (usR[BXt] - uR[BXt]);
    const double wsL = vL[VXb] - qL * (usL[BXb] - uL[BXb]);
    const double wsR = vR[VXb] - qR * (usR[BXb] - uR[BXb]);
    usL[RHO] = rsL;
    usR[RHO] = rsR;
    usL[MXn] = rsL * SM;
    usR[MXn] = rsR * SM;
    usL[MXt] = rsL * vsL;
    usR[MXt] = rsR * vsR;
    usL[MXb] = rsL * wsL;
    usR[MXb] = rsR * wsR;
    double eL2 = vL[VXn] * Bx + vL[VXt] * uL[BXt] + vL[VXb] * uL[BXb];
    eL2 -= SM * Bx + vsL * usL[BXt] + wsL * usL[BXb];
    const double EL = duL * uL[ENG] - ptL * vL[VXn] + pts * SM + Bx * eL2;
    usL[ENG] = EL / dLm;
    double eR2 = vR[VXn] * Bx + vR[VXt] * uR[BXt] + vR[VXb] * uR[BXb];
    eR2 -= SM * Bx + vsR * usR[BXt] + wsR * usR[BXb];
    const double ER = duR * uR[ENG] - ptR * vR[VXn] + pts * SM + Bx * eR2;
    usR[ENG] = ER / dRm;

    // ---- reverse: the flux of the region taken ----
    double ausL[NV], ausR[NV];
#pragma unroll
    for (int nv = 0; nv < NV; nv++) ausL[nv] = ausR[nv] = 0.0;
    double aSM = 0.0, aBx = 0.0, asqrL = 0.0, asqrR = 0.0, aS1L = 0.0, aS1R = 0.0;
    double avsL = 0.0, avsR = 0.0, awsL = 0.0, awsR = 0.0, arsL = 0.0, arsR = 0.0;
    if (S1L >= 0.0) {  // f = fL + SL (usL - uL)
#pragma unroll
      for (int nv = 0; nv < NV; nv++) {
        const double l = lam[nv];
        afL[nv] += l;
        aSL += l * (usL[nv] - uL[nv]);
        ausL[nv] += l * SL;
        auL[nv] -= l * SL;
      }
      aptL += lam[NV];
    } else if (S1R <= 0.0) {  // f = fR + SR (usR - uR)
#pragma unroll
      for (int nv = 0; nv < NV; nv++) {
        const double l = lam[nv];
        afR[nv] += l;
        aSR += l * (usR[nv] - uR[nv]);
        ausR[nv] += l * SR;
        auR[nv] -= l * SR;
      }
      aptR += lam[NV];
    } else {
      // forward: the double-star state
      const double den = sqrL + sqrR;
      const double Mv = sqrL * vsL + sqrR * vsR + (usR[BXt] - usL[BXt]) * sBx;
      const double vss = Mv / den;
      const double Mw = sqrL * wsL + sqrR * wsR + (usR[BXb] - usL[BXb]) * sBx;
      const double wss = Mw / den;
      const double dv = (vsR - vsL) * sBx, dw = (wsR - wsL) * sBx;
      const double Nt = sqrL * usR[BXt] + sqrR * usL[BXt] + sqrL * sqrR * (vsR - vsL) * sBx;
      const double btss = Nt / den;
      const double Nb = sqrL * usR[BXb] + sqrR * usL[BXb] + sqrL * sqrR * (wsR - wsL) * sBx;
      const double bbss = Nb / den;
      const double gss = vss * btss + wss * bbss;
      const double gLs = vsL * usL[BXt] + wsL * usL[BXb] - gss;  // the SM Bx1 terms cancel
      const double gRs = vsR * usR[BXt] + wsR * usR[BXb] - gss;
      double uss[NV];  // ussl (SM >= 0) or ussr
      const bool left = SM >= 0.0;
      const double rs = left ? rsL : rsR;
      uss[RHO] = rs;
      uss[MXn] = rs * SM;
      uss[MXt] = rs * vss;
      uss[MXb] = rs * wss;
      uss[BXn] = Bx;
      uss[BXt] = btss;
      uss[BXb] = bbss;
      uss[ENG] = left ? usL[ENG] - sqrL * gLs * sBx : usR[ENG] + sqrR * gRs * sBx;
      // f = fX + S1X (ussX - usX) + SX (usX - uX)
      double auss[NV];
      const double S1 = left ? S1L : S1R, S = left ? SL : SR;
      double aS1 = 0.0, aS = 0.0;
#pragma unroll
      for (int nv = 0; nv < NV; nv++) {
        const double l = lam[nv];
        const double us = left ? usL[nv] : usR[nv];
        const double u = left ? uL[nv] : uR[nv];
        aS1 += l * (uss[nv] - us);
        auss[nv] = l * S1;
        aS += l * (us - u);
        if (left) {
          afL[nv] += l;
          ausL[nv] += l * (S - S1);
          auL[nv] -= l * S;
        } else {
          afR[nv] += l;
          ausR[nv] += l * (S - S1);
          auR[nv] -= l * S;
        }
      }
      if (left) {
        aS1L += aS1;
        aSL += aS;
        aptL += lam[NV];
      } else {
        aS1R += aS1;
        aSR += aS;
        aptR += lam[NV];
      }
      // ussX[ENG] = usX[ENG] -/+ sqrX gX sBx
      double agL = 0.0, agR = 0.0;
      if (left) {
        ausL[ENG] += auss[ENG];
        asqrL -= auss[ENG] * gLs * sBx;
        agL = -auss[ENG] * sqrL * sBx;
      } else {
        ausR[ENG] += auss[ENG];
        asqrR += auss[ENG] * gRs * sBx;
        agR = auss[ENG] * sqrR * sBx;
      }
      avsL += agL * usL[BXt];
      ausL[BXt] += agL * vsL;
      awsL += agL * usL[BXb];
      ausL[BXb] += agL * wsL;
      avsR += agR * usR[BXt];
      ausR[BXt] += agR * vsR;
      awsR += agR * usR[BXb];
      ausR[BXb] += agR * wsR;
      const double ag = agL + agR;
      double avss = -ag * btss, awss = -ag * bbss, abtss = -ag * vss, abbss = -ag * wss;
      // the components of ussX
      if (left) arsL += auss[RHO] + auss[MXn] * SM + auss[MXt] * vss + auss[MXb] * wss;
      else arsR += auss[RHO] + auss[MXn] * SM + auss[MXt] * vss + auss[MXb] * wss;
      aSM += auss[MXn] * rs;
      avss += auss[MXt] * rs;
      awss += auss[MXb] * rs;
      aBx += auss[BXn];
      abtss += auss[BXt];
      abbss += auss[BXb];
      // btss = Nt / den, bbss = Nb / den, vss = Mv / den, wss = Mw / den
      const double aNt = abtss / den, aNb = abbss / den, aMv = avss / den, aMw = awss / den;
      const double aden = -(abtss * btss + abbss * bbss + avss * vss + awss * wss) / den;
      asqrL += aNt * (usR[BXt] + sqrR * dv) + aNb * (usR[BXb] + sqrR * dw);
      asqrR += aNt * (usL[BXt] + sqrL * dv) + aNb * (usL[BXb] + sqrL * dw);
      ausR[BXt] += aNt * sqrL;
      ausL[BXt] += aNt * sqrR;
      ausR[BXb] += aNb * sqrL;
      ausL[BXb] += aNb * sqrR;
      const double pq = sqrL * sqrR * sBx;
      avsR += aNt * pq;
      avsL -= aNt * pq;
      awsR += aNb * pq;
      awsL -= aNb * pq;
      asqrL += aMv * vsL + aMw * wsL + aden;
      asqrR += aMv * vsR + aMw * wsR + aden;
      avsL += aMv * sqrL;
      avsR += aMv * sqrR;
      awsL += aMw * sqrL;
      awsR += aMw * sqrR;
      ausR[BXt] += aMv * sBx;
      ausL[BXt] -= aMv * sBx;
      ausR[BXb] += aMw * sBx;
      ausL[BXb] -= aMw * sBx;
    }

    // ---- reverse: the single-star states ----
    double aduL = 0.0, aduR = 0.0, apts = 0.0;
    {  // usL[ENG] = EL / (SL - SM), EL = duL uL[ENG] - ptL vnL + pts SM + Bx eL2
      const double aE = ausL[ENG] / dLm, q = ausL[ENG] * usL[ENG] / dLm;
      aSL -= q;
      aSM += q;
      aduL += aE * uL[ENG];
      auL[ENG] += aE * duL;
      aptL -= aE * vL[VXn];
      gL[VXn] -= aE * ptL;
      apts += aE * SM;
      aSM += aE * pts;
      aBx += aE * eL2;
      const double ae = aE * Bx;  // eL2 = vnL Bx + vtL uL[BXt] + vbL uL[BXb] - (SM Bx + vsL usL[BXt] + wsL usL[BXb])
      gL[VXn] += ae * Bx;
      aBx += ae * (vL[VXn] - SM);
      gL[VXt] += ae * uL[BXt];
      auL[BXt] += ae * vL[VXt];
      gL[VXb] += ae * uL[BXb];
      auL[BXb] += ae * vL[VXb];
      aSM -= ae * Bx;
      avsL -= ae * usL[BXt];
      ausL[BXt] -= ae * vsL;
      awsL -= ae * usL[BXb];
      ausL[BXb] -= ae * wsL;
    }
    {
      const double aE = ausR[ENG] / dRm, q = ausR[ENG] * usR[ENG] / dRm;
      aSR -= q;
      aSM += q;
      aduR += aE * uR[ENG];
      auR[ENG] += aE * duR;
      aptR -= aE * vR[VXn];
      gR[VXn] -= aE * ptR;
      apts += aE * SM;
      aSM += aE * pts;
      aBx += aE * eR2;
      const double ae = aE * Bx;
      gR[VXn] += ae * Bx;
      aBx += ae * (vR[VXn] - SM);
      gR[VXt] += ae * uR[BXt];
      auR[BXt] += ae * vR[VXt];
      gR[VXb] += ae * uR[BXb];
      auR[BXb] += ae * vR[VXb];
      aSM -= ae * Bx;
      avsR -= ae * usR[BXt];
      ausR[BXt] -= ae * vsR;
      awsR -= ae * usR[BXb];
      ausR[BXb] -= ae * wsR;
    }
    // usX[RHO] = rsX, usX[MXn] = rsX SM, usX[MXt] = rsX vsX, usX[MXb] = rsX wsX
    arsL += ausL[RHO] + ausL[MXn] * SM + ausL[MXt] * vsL + ausL[MXb] * wsL;
    arsR += ausR[RHO] + ausR[MXn] * SM + ausR[MXt] * vsR + ausR[MXb] * wsR;
    aSM += ausL[MXn] * rsL + ausR[MXn] * rsR;
    avsL += ausL[MXt] * rsL;
    awsL += ausL[MXb] * rsL;
    avsR += ausR[MXt] * rsR;
    awsR += ausR[MXb] * rsR;
    // vsX = vtX - qX (usX[BXt] - uX[BXt]), wsX = vbX - qX (usX[BXb] - uX[BXb])
    gL[VXt] += avsL;
    gL[VXb] += awsL;
    gR[VXt] += avsR;
    gR[VXb] += awsR;
    const double aqL = -avsL * (usL[BXt] - uL[BXt]) - awsL * (usL[BXb] - uL[BXb]);
    const double aqR = -avsR * (usR[BXt] - uR[BXt]) - awsR * (usR[BXb] - uR[BXb]);
    ausL[BXt] -= avsL * qL;
    auL[BXt] += avsL * qL;
    ausL[BXb] -= awsL * qL;
    auL[BXb] += awsL * qL;
    ausR[BXt] -= avsR * qR;
    auR[BXt] += avsR * qR;
    ausR[BXb] -= awsR * qR;
    auR[BXb] += awsR * qR;
    // qX = Bx / tX
    aBx += aqL / tL + aqR / tR;
    double atL = -aqL * qL / tL, atR = -aqR * qR / tR;
    if (revert) {
      // usL = usR = (SR uR - SL uL + fL - fR) / (SR - SL) on the field; S1X = SM
      aSM += aS1L + aS1R;
      constexpr int bi[3] = {BXn, BXt, BXb};
      double as2 = 0.0;
#pragma unroll
      for (int t = 0; t < 3; t++) {
        const int q = bi[t];
        const double aU = ausL[q] + ausR[q];
        const double aN = aU * s2;
        as2 += aU * Nc[t];
        aSR += aN * uR[q];
        auR[q] += aN * SR;
        aSL -= aN * uL[q];
        auL[q] -= aN * SL;
        if (t > 0) {  // the normal flux of the normal field is the constant 0
          afL[q] += aN;
          afR[q] -= aN;
        }
      }
      aSR -= as2 * s2 * s2;
      aSL += as2 * s2 * s2;
    } else {
      // usX[BXn] = Bx1, usX[BXt,BXb] = uX[BXt,BXb] hX, hX = nX / mX
      aBx += ausL[BXn] + ausR[BXn];
      auL[BXt] += ausL[BXt] * hL;
      auL[BXb] += ausL[BXb] * hL;
      auR[BXt] += ausR[BXt] * hR;
      auR[BXb] += ausR[BXb] * hR;
      const double ahL = ausL[BXt] * uL[BXt] + ausL[BXb] * uL[BXb];
      const double ahR = ausR[BXt] * uR[BXt] + ausR[BXb] * uR[BXb];
      const double anL = ahL / mL, amL = -ahL * hL / mL;
      const double anR = ahR / mR, amR = -ahR * hR / mR;
      // nX = uX[RHO] duX duX - Bx^2, mX = uX[RHO] duX (SX - SM) - Bx^2
      auL[RHO] += anL * duL * duL + amL * duL * dLm;
      aduL += anL * 2.0 * uL[RHO] * duL + amL * uL[RHO] * dLm;
      aSL += amL * tL;
      aSM -= amL * tL;
      auR[RHO] += anR * duR * duR + amR * duR * dRm;
      aduR += anR * 2.0 * uR[RHO] * duR + amR * uR[RHO] * dRm;
      aSR += amR * tR;
      aSM -= amR * tR;
      aBx -= 2.0 * Bx * (anL + amL + anR + amR);
      // S1L = SM - |Bx| / sqrL, S1R = SM + |Bx| / sqrR
      aSM += aS1L + aS1R;
      const double aab = -aS1L / sqrL + aS1R / sqrR;
      asqrL += aS1L * aBxm / (sqrL * sqrL);
      asqrR -= aS1R * aBxm / (sqrR * sqrR);
      aBx += Bx < 0.0 ? -aab : aab;
    }
    // sqrX = ::sqrt(rsX)
    arsL += asqrL * (0.5 / sqrL);
    arsR += asqrR * (0.5 / sqrR);
    // rsX = tX / (SX - SM)
    {
      const double r = arsL * rsL / dLm;
      atL += arsL / dLm;
      aSL -= r;
      aSM += r;
    }
    {
      const double r = arsR * rsR / dRm;
      atR += arsR / dRm;
      aSR -= r;
      aSM += r;
    }
    // tX = uX[RHO] duX
    auL[RHO] += atL * duL;
    aduL += atL * uL[RHO];
    auR[RHO] += atR * duR;
    aduR += atR * uR[RHO];
    // pts = pts0 s1
    const double apts0 = apts * s1;
    double as1 = apts * pts0;
    const double rr = vL[RHO] * vR[RHO];
    aduR += apts0 * (uR[RHO] * ptL + rr * duL * dvn);
    auR[RHO] += apts0 * duR * ptL;
    aptL += apts0 * duR * uR[RHO];
    aduL += apts0 * (rr * duR * dvn - uL[RHO] * ptR);
    auL[RHO] -= apts0 * duL * ptR;
    aptR -= apts0 * duL * uL[RHO];
    gL[RHO] += apts0 * vR[RHO] * duR * duL * dvn;
    gR[RHO] += apts0 * vL[RHO] * duR * duL * dvn;
    const double advn = apts0 * rr * duR * duL;
    gR[VXn] += advn;
    gL[VXn] -= advn;
    // SM = NSM s1
    const double aNSM = aSM * s1;
    as1 += aSM * NSM;
    aduR += aNSM * uR[MXn];
    auR[MXn] += aNSM * duR;
    aduL -= aNSM * uL[MXn];
    auL[MXn] -= aNSM * duL;
    aptR -= aNSM;
    aptL += aNSM;
    // s1 = 1 / (duR uR[RHO] - duL uL[RHO])
    const double aD = -as1 * s1 * s1;
    aduR += aD * uR[RHO];
    auR[RHO] += aD * duR;
    aduL -= aD * uL[RHO];
    auL[RHO] -= aD * duL;
    // duX = SX - vnX
    aSL += aduL;
    gL[VXn] -= aduL;
    aSR += aduR;
    gR[VXn] -= aduR;
    // Bx = (SR bnR - SL bnL) s0, s0 = 1 / (SR - SL)
    const double aNB = aBx * s0, as0 = aBx * NB;
    aSR += aNB * vR[BXn];
    gR[BXn] += aNB * SR;
    aSL -= aNB * vL[BXn];
    gL[BXn] -= aNB * SL;
    aSR -= as0 * s0 * s0;
    aSL += as0 * s0 * s0;
  }
  b.finish(vL, vR, gamma, aSL, aSR, afL, afR, aptL, aptR, auL, auR, gL, gR);
}

// J^T lam of riemann_pt for HLL and HLLD; false for the Roe solver (whose
// adjoint keeps the per-input Dual<1> evaluations).
template <int DIR>
__host__ __device__ __forceinline__ bool riemann_rev(int solver, double gamma, const double* vL, const double* vR,
                                                     const double* lam, double* gL, double* gR) {
  if (solver == PG_HLLD) {
    hlld_rev<DIR>(vL, vR, gamma, lam, gL, gR);
    return true;
  }
  if (solver == PG_HLL) {
    hll_rev<DIR>(vL, vR, gamma, lam, gL, gR);
    return true;
  }
  return false;
}

// Partial derivatives (pp, pm) of limit(lim, nv, dvp, dvm) with respect to
// dvp and dvm, on the branch limit takes (Src/States/plm_coeffs.h:72-175).
__host__ __device__ __forceinline__ void limit_partials(int lim, int nv, double dvp, double dvm, double& pp,
                                                        double& pm) {
  pp = pm = 0.0;
  if (lim == LIM_DEFAULT) lim = (nv == RHO) ? LIM_MC : (nv == PRS ? LIM_MINMOD : LIM_VANLEER);
  if (lim == LIM_FLAT || !(dvp * dvm > 0.0)) return;
  const bool pmin = ::fabs(dvp) < ::fabs(dvm);  // abs_min(dvp, dvm) selects dvp
  if (lim == LIM_MINMOD) {
    (pmin ? pp : pm) = 1.0;
  } else if (lim == LIM_VANLEER) {  // 2 dvp dvm / (dvp + dvm)
    const double s = dvp + dvm, r = 2.0 * dvp * dvm / s;
    pp = (2.0 * dvm - r) / s;
    pm = (2.0 * dvp - r) / s;
  } else {  // MC: abs_min(0.5 (dvm + dvp), 2 abs_min(dvp, dvm))
    const double qc = 0.5 * (dvm + dvp), scrh = 2.0 * (pmin ? dvp : dvm);
    if (::fabs(qc) < ::fabs(scrh)) pp = pm = 0.5;
    else (pmin ? pp : pm) = 2.0;
  }
}

// PLM states of one zone transposed (recon_pt with PG_LINEAR): vp = v0 +
// dv/2, vm = v0 - dv/2, dv = limit(w3 - v0, v0 - w1); g[0..2] = the adjoint
// on w1, v0, w3 from the adjoints lp, lm on vp, vm.
__host__ __device__ __forceinline__ void plm_rev(int lim, int nv, double w1, double v0, double w3, double lp,
                                                 double lm, double* g) {
  double pp, pm;
  limit_partials(lim, nv, w3 - v0, v0 - w1, pp, pm);
  const double adv = 0.5 * (lp - lm);
  g[0] = -adv * pm;
  g[1] = lp + lm + adv * (pm - pp);
  g[2] = adv * pp;
}

// ppm_iface transposed: out = v0 + minmod(S - v0, vp1 - v0) with S the
// four-point interface value; adds a_out's share into g[0..3] (the
// adjoints on vm1, v0, vp1, vp2).
__host__ __device__ __forceinline__ void ppm_iface_rev(double vm1, double v0, double vp1, double vp2, double a,
                                                       double* g) {
  const double w_1 = -1.0 / 12.0, w0 = 7.0 / 12.0, w1 = 7.0 / 12.0, w2 = -1.0 / 12.0;
  const double S = w_1 * vm1 + w0 * v0 + w1 * vp1 + w2 * vp2;  // as ppm_iface
  const double dv = vp1 - v0, dvp = S - v0;
  g[1] += a;
  if (!(dvp * dv > 0.0)) return;  // minmod: 0
  if (::fabs(dvp) < ::fabs(dv)) {  // the interface value's slope: a_S
    g[0] += w_1 * a;
    g[1] += w0 * a - a;
    g[2] += w1 * a;
    g[3] += w2 * a;
  } else {  // the one-sided difference vp1 - v0
    g[2] += a;
    g[1] -= a;
  }
}

// PPM states of one zone transposed (recon_pt with PG_PARABOLIC, the
// parabolic limiter of ppm_states.c:146-207 with cp = cm = 2): g[0..4] =
// the adjoint on w[0..4] = v[c-2..c+2] from lp, lm on vp, vm.
__host__ __device__ __forceinline__ void ppm_rev(const double* w, double lp, double lm, double* g) {
#pragma unroll
  for (int t = 0; t < 5; t++) g[t] = 0.0;
  const double v0 = w[2];
  double p = ppm_iface(w[1], v0, w[3], w[4]);
  double m = ppm_iface(w[0], w[1], v0, w[3]);
  const double cm = (3.0 + 1.0) / (3.0 - 1.0), cp = cm;
  const double dvp = p - v0, dvm = m - v0;
  // vp = v0 + dvp', vm = v0 + dvm' with (dvp', dvm') of the branch taken
  g[2] += lp + lm;
  double adp = 0.0, adm = 0.0;  // adjoints on dvp, dvm
  if (dvp * dvm >= 0.0) {
    // dvp' = dvm' = 0
  } else if (::fabs(dvp) >= cm * ::fabs(dvm)) {  // dvp' = -cm dvm
    adm = lm - cm * lp;
  } else if (::fabs(dvm) >= cp * ::fabs(dvp)) {  // dvm' = -cp dvp
    adp = lp - cp * lm;
  } else {
    adp = lp;
    adm = lm;
  }
  g[2] -= adp + adm;  // dvp = p - v0, dvm = m - v0
  double gp[4] = {0.0, 0.0, 0.0, 0.0}, gm[4] = {0.0, 0.0, 0.0, 0.0};
  ppm_iface_rev(w[1], v0, w[3], w[4], adp, gp);  // p from w1, v0, w3, w4
  ppm_iface_rev(w[0], w[1], v0, w[3], adm, gm);  // m from w0, w1, v0, w3
  g[1] += gp[0];
  g[2] += gp[1];
  g[3] += gp[2];
  g[4] += gp[3];
  g[0] += gm[0];
  g[1] += gm[1];
  g[2] += gm[2];
  g[3] += gm[3];
}

// mc_lim2 (Src/MHD/CT/ct_stag_slopes.c:92-105) transposed: a_dp, a_dm
__host__ __device__ __forceinline__ void mc_lim2_rev(double dp, double dm, double a, double& adp, double& adm) {
  adp = adm = 0.0;
  if (dp * dm < 0.0) return;
  const double dc = 0.5 * (dp + dm);
  const bool pfirst = ::fabs(dp) < ::fabs(dm);
  const double scrh = 2.0 * (pfirst ? dp : dm);
  if (::fabs(dc) < ::fabs(scrh)) {
    adp = adm = 0.5 * a;
  } else if (pfirst) {
    adp = 2.0 * a;
  } else {
    adm = 2.0 * a;
  }
}

// g = lam * d emf_pt / d in (all 40 inputs)
__host__ __device__ __forceinline__ void emf_rev(const double* in, double lam, double* g) {
#pragma unroll
  for (int q = 0; q < kEdgeIn; q++) g[q] = 0.0;
  const int ixp = in[0] >= in[1] ? 0 : 1, ixm = in[2] >= in[3] ? 2 : 3;
  const int iyp = in[4] >= in[5] ? 4 : 5, iym = in[6] >= in[7] ? 6 : 7;
  const double a_xp = in[ixp], a_xm = in[ixm], a_yp = in[iyp], a_ym = in[iym];
  const double sbS = mc_lim2(in[10] - in[9], in[9] - in[8]);
  const double sbN = mc_lim2(in[11] - in[10], in[10] - in[9]);
  const double sbW = mc_lim2(in[14] - in[13], in[13] - in[12]);
  const double sbE = mc_lim2(in[15] - in[14], in[14] - in[13]);
  const double bS = in[9] + 0.5 * sbS;
  const double bW = in[13] + 0.5 * sbW;
  const double bN = in[10] - 0.5 * sbN;
  const double bE = in[14] - 0.5 * sbE;
  const double* q0 = in + 16;  // c00
  const double* q1 = in + 22;  // cx0
  const double* q2 = in + 28;  // c0y
  const double* q3 = in + 34;  // cxy
  const double AS = q0[0] + 0.5 * (q0[2] + q0[3]), BS = q0[1] + 0.5 * (q0[4] + q0[5]);
  const double AE = q1[0] - 0.5 * (q1[2] - q1[3]), BE = q1[1] - 0.5 * (q1[4] - q1[5]);
  const double AN = q3[0] - 0.5 * (q3[2] + q3[3]), BN = q3[1] - 0.5 * (q3[4] + q3[5]);
  const double AW = q2[0] + 0.5 * (q2[2] - q2[3]), BW = q2[1] + 0.5 * (q2[4] - q2[5]);
  const double eSW = AS * bS - BS * bW;
  const double eSE = AE * bS - BE * bE;
  const double eNE = AN * bN - BN * bE;
  const double eNW = AW * bN - BW * bW;
  // uct_hll_combine (ct_emf_average.c:262-289)
  const double X = a_xp + a_xm, Y = a_yp + a_ym, P = X * Y;
  const double Nn = a_xp * a_yp * eSW + a_xm * a_yp * eSE + a_xm * a_ym * eNE + a_xp * a_ym * eNW;
  const double e1 = Nn / P;
  const double aNn = lam / P;
  double aX = -lam * e1 / P * Y, aY = -lam * e1 / P * X;
  const double aeSW = aNn * a_xp * a_yp, aeSE = aNn * a_xm * a_yp;
  const double aeNE = aNn * a_xm * a_ym, aeNW = aNn * a_xp * a_ym;
  double aaxp = aNn * (a_yp * eSW + a_ym * eNW), aaxm = aNn * (a_yp * eSE + a_ym * eNE);
  double aayp = aNn * (a_xp * eSW + a_xm * eSE), aaym = aNn * (a_xm * eNE + a_xp * eNW);
  // - a_yp a_ym (bN - bS) / Y
  const double t2 = a_yp * a_ym * (bN - bS) / Y, aT2 = -lam / Y;
  aY += lam * t2 / Y;
  aayp += aT2 * a_ym * (bN - bS);
  aaym += aT2 * a_yp * (bN - bS);
  double abN = aT2 * a_yp * a_ym, abS = -aT2 * a_yp * a_ym;
  // + a_xp a_xm (bE - bW) / X
  const double t3 = a_xp * a_xm * (bE - bW) / X, aT3 = lam / X;
  aX -= lam * t3 / X;
  aaxp += aT3 * a_xm * (bE - bW);
  aaxm += aT3 * a_xp * (bE - bW);
  double abE = aT3 * a_xp * a_xm, abW = -aT3 * a_xp * a_xm;
  aaxp += aX;
  aaxm += aX;
  aayp += aY;
  aaym += aY;
  g[ixp] += aaxp;
  g[ixm] += aaxm;
  g[iyp] += aayp;
  g[iym] += aaym;
  // corner EMFs
  abS += aeSW * AS + aeSE * AE;
  abW -= aeSW * BS + aeNW * BW;
  abE -= aeSE * BE + aeNE * BN;
  abN += aeNE * AN + aeNW * AW;
  {
    const double aA = aeSW * bS, aB = -aeSW * bW;
    g[16 + 0] += aA;
    g[16 + 2] += 0.5 * aA;
    g[16 + 3] += 0.5 * aA;
    g[16 + 1] += aB;
    g[16 + 4] += 0.5 * aB;
    g[16 + 5] += 0.5 * aB;
  }
  {
    const double aA = aeSE * bS, aB = -aeSE * bE;
    g[22 + 0] += aA;
    g[22 + 2] -= 0.5 * aA;
    g[22 + 3] += 0.5 * aA;
    g[22 + 1] += aB;
    g[22 + 4] -= 0.5 * aB;
    g[22 + 5] += 0.5 * aB;
  }
  {
    const double aA = aeNE * bN, aB = -aeNE * bE;
    g[34 + 0] += aA;
    g[34 + 2] -= 0.5 * aA;
    g[34 + 3] -= 0.5 * aA;
    g[34 + 1] += aB;
    g[34 + 4] -= 0.5 * aB;
    g[34 + 5] -= 0.5 * aB;
  }
  {
    const double aA = aeNW * bN, aB = -aeNW * bW;
    g[28 + 0] += aA;
    g[28 + 2] += 0.5 * aA;
    g[28 + 3] -= 0.5 * aA;
    g[28 + 1] += aB;
    g[28 + 4] += 0.5 * aB;
    g[28 + 5] -= 0.5 * aB;
  }
  // bS = in9 + sbS / 2, bN = in10 - sbN / 2, bW = in13 + sbW / 2, bE = in14 - sbE / 2
  g[9] += abS;
  g[10] += abN;
  g[13] += abW;
  g[14] += abE;
  double adp, adm;
  mc_lim2_rev(in[10] - in[9], in[9] - in[8], 0.5 * abS, adp, adm);
  g[10] += adp;
  g[9] += adm - adp;
  g[8] -= adm;
  mc_lim2_rev(in[11] - in[10], in[10] - in[9], -0.5 * abN, adp, adm);
  g[11] += adp;
  g[10] += adm - adp;
  g[9] -= adm;
  mc_lim2_rev(in[14] - in[13], in[13] - in[12], 0.5 * abW, adp, adm);
  g[14] += adp;
  g[13] += adm - adp;
  g[12] -= adm;
  mc_lim2_rev(in[15] - in[14], in[14] - in[13], -0.5 * abE, adp, adm);
  g[15] += adp;
  g[14] += adm - adp;
  g[13] -= adm;
}

}  // namespace pg
