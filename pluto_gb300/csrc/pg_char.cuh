// Characteristic decomposition of ideal MHD in primitive variables on the
// plain FP64 path: PrimEigenvectors, PrimToChar, the characteristic-limited
// PLM states (CHAR_LIMITING YES) and CharTracingStep (TIME_STEPPING
// CHARACTERISTIC_TRACING).  Double only: the eigenvector formulas take square
// roots of values that are often exactly zero, where a dual-number
// derivative is infinite, so the tangent-linear build does not use them.
#pragma once
#include "pg_physics.cuh"

namespace pg {

// PrimEigenvectors (Src/MHD/eigenv.c:190-688, ideal EOS, no 8-wave / GLM):
// eigenvalues and left/right primitive eigenvectors along DIR in the wave
// order fast-, fast+, entropy, div-B, slow-, slow+, Alfven-, Alfven+
// (Src/MHD/mod_defs.h:54-71).  L[wave][var], R[var][wave] start at zero;
// the zero entries take part in the tracing sums below like in the
// reference's dense loops.
enum : int { WFM = 0, WFP, WEN, WDB, WSM, WSP, WAM, WAP };
template <int DIR>
__device__ __forceinline__ void prim_eigen(const double* q, double a2, bool c3, int dims, double L[8][8],
                                           double R[8][8], double* lambda) {
  using Rt = Rot<DIR>;
  constexpr int vn = Rt::vn, vt = Rt::vt, vb = Rt::vb, bn = Rt::bn, bt = Rt::bt, bb = Rt::bb;
  const double sqrt_1_2 = 0.70710678118654752440;
#pragma unroll
  for (int a = 0; a < 8; a++) {
    lambda[a] = 0.0;
#pragma unroll
    for (int b = 0; b < 8; b++) L[a][b] = R[a][b] = 0.0;
  }
  const double u = q[vn], tau = 1.0 / q[RHO], sqrt_rho = ::sqrt(q[RHO]);
  double scrh0, scrh1, scrh2, scrh3, scrh4;
  scrh2 = q[bn] * q[bn];
  scrh3 = c3 ? 0.0 + q[bt] * q[bt] + q[bb] * q[bb] : 0.0 + q[bt] * q[bt];
  const double b2 = scrh2 + scrh3, ca2 = scrh2 * tau, A2 = b2 * tau, At2 = scrh3 * tau;
  scrh1 = a2 - A2;
  scrh0 = ::sqrt(scrh1 * scrh1 + 4.0 * a2 * At2);
  const double cf2 = 0.5 * (a2 + A2 + scrh0), cs2 = a2 * ca2 / cf2;
  const double cf = ::sqrt(cf2), cs = ::sqrt(cs2), ca = ::sqrt(ca2), a = ::sqrt(a2);
  double alpha_f, alpha_s;
  if (cf == cs) {
    alpha_f = 1.0;
    alpha_s = 0.0;
  } else {
    scrh0 = 1.0 / scrh0;
    alpha_f = ::sqrt(pmax(0.0, (a2 - cs2) * scrh0));
    alpha_s = ::sqrt(pmax(0.0, (cf2 - a2) * scrh0));
  }
  double beta_y, beta_z = 0.0;
  scrh0 = ::sqrt(scrh3);
  if (scrh0 > 1.e-9) {
    if (c3) {
      beta_y = q[bt] / scrh0;
      beta_z = q[bb] / scrh0;
    } else {
      beta_y = q[bt] >= 0.0 ? 1.0 : -1.0;
    }
  } else {
    beta_y = c3 ? sqrt_1_2 : 1.0;
    if (c3) beta_z = sqrt_1_2;
  }
  const double S = q[bn] >= 0.0 ? 1.0 : -1.0;
  // fast waves
  lambda[WFM] = u - cf;
  scrh0 = alpha_s * cs * S;
  scrh1 = alpha_s * sqrt_rho * a;
  scrh2 = 0.5 / a2;
  scrh3 = scrh2 * tau;
  R[RHO][WFM] = q[RHO] * alpha_f;
  R[vn][WFM] = -cf * alpha_f;
  R[vt][WFM] = scrh0 * beta_y;
  R[bt][WFM] = scrh1 * beta_y;
  if (c3) {
    R[vb][WFM] = scrh0 * beta_z;
    R[bb][WFM] = scrh1 * beta_z;
  }
  R[PRS][WFM] = alpha_f * a2 * q[RHO];
  L[WFM][vn] = R[vn][WFM] * scrh2;
  L[WFM][vt] = R[vt][WFM] * scrh2;
  L[WFM][bt] = R[bt][WFM] * scrh3;
  if (c3) {
    L[WFM][vb] = R[vb][WFM] * scrh2;
    L[WFM][bb] = R[bb][WFM] * scrh3;
  }
  L[WFM][PRS] = alpha_f * scrh3;
  lambda[WFP] = u + cf;
#pragma unroll
  for (int v = 0; v < 8; v++) {
    const bool odd = v == vn || v == vt || v == vb;  // velocities flip sign
    R[v][WFP] = odd ? -R[v][WFM] : R[v][WFM];
    L[WFP][v] = odd ? -L[WFM][v] : L[WFM][v];
  }
  // entropy and div-B waves
  lambda[WEN] = u;
  R[RHO][WEN] = 1.0;
  L[WEN][RHO] = 1.0;
  L[WEN][PRS] = -1.0 / a2;
  lambda[WDB] = 0.0;
  // slow waves
  lambda[WSM] = u - cs;
  scrh0 = alpha_f * cf * S;
  scrh1 = alpha_f * sqrt_rho * a;
  R[RHO][WSM] = q[RHO] * alpha_s;
  R[vn][WSM] = -cs * alpha_s;
  R[vt][WSM] = -scrh0 * beta_y;
  R[bt][WSM] = -scrh1 * beta_y;
  if (c3) {
    R[vb][WSM] = -scrh0 * beta_z;
    R[bb][WSM] = -scrh1 * beta_z;
  }
  scrh4 = alpha_s * a2 * q[RHO];
  R[PRS][WSM] = scrh4;
  L[WSM][vn] = R[vn][WSM] * scrh2;
  L[WSM][vt] = R[vt][WSM] * scrh2;
  L[WSM][bt] = R[bt][WSM] * scrh3;
  if (c3) {
    L[WSM][vb] = R[vb][WSM] * scrh2;
    L[WSM][bb] = R[bb][WSM] * scrh3;
  }
  L[WSM][PRS] = alpha_s * scrh3;
  lambda[WSP] = u + cs;
#pragma unroll
  for (int v = 0; v < 8; v++) {
    const bool odd = v == vn || v == vt || v == vb;
    R[v][WSP] = odd ? -R[v][WSM] : R[v][WSM];
    L[WSP][v] = odd ? -L[WSM][v] : L[WSM][v];
  }
  // Alfven waves (three components)
  if (c3) {
    lambda[WAM] = u - ca;
    scrh2 = beta_y * sqrt_1_2;
    scrh3 = beta_z * sqrt_1_2;
    R[vt][WAM] = -scrh3;
    R[vb][WAM] = scrh2;
    R[bt][WAM] = -scrh3 * sqrt_rho * S;
    R[bb][WAM] = scrh2 * sqrt_rho * S;
    L[WAM][vt] = R[vt][WAM];
    L[WAM][vb] = R[vb][WAM];
    L[WAM][bt] = R[bt][WAM] * tau;
    L[WAM][bb] = R[bb][WAM] * tau;
    lambda[WAP] = u + ca;
    R[vt][WAP] = R[vt][WAM];
    R[vb][WAP] = R[vb][WAM];
    R[bt][WAP] = -R[bt][WAM];
    R[bb][WAP] = -R[bb][WAM];
    L[WAP][vt] = L[WAM][vt];
    L[WAP][vb] = L[WAM][vb];
    L[WAP][bt] = -L[WAM][bt];
    L[WAP][bb] = -L[WAM][bb];
    if (dims <= 2 && q[bn] == 0 && q[bt] == 0.0)  // eigenv.c:528-531
#pragma unroll
      for (int k = 0; k < 8; k++) R[bt][k] = 0.0;
  }
}

// PrimToChar, Src/MHD/eigenv.c:1310-1380: w = L . v over the nonzero
// entries of the left eigenvectors, in the reference's grouping.
template <int DIR>
__device__ __forceinline__ void prim_to_char(const double L[8][8], const double* dv, bool c3, double* dw) {
  using Rt = Rot<DIR>;
  constexpr int vn = Rt::vn, vt = Rt::vt, vb = Rt::vb, bt = Rt::bt, bb = Rt::bb;
  double wv, wB;
  wv = c3 ? L[WFM][vn] * dv[vn] + L[WFM][vt] * dv[vt] + L[WFM][vb] * dv[vb]
          : L[WFM][vn] * dv[vn] + L[WFM][vt] * dv[vt];
  wB = c3 ? L[WFM][PRS] * dv[PRS] + L[WFM][bt] * dv[bt] + L[WFM][bb] * dv[bb]
          : L[WFM][PRS] * dv[PRS] + L[WFM][bt] * dv[bt];
  dw[WFM] = wv + wB;
  dw[WFP] = -wv + wB;
  dw[WEN] = L[WEN][RHO] * dv[RHO] + L[WEN][PRS] * dv[PRS];
  dw[WDB] = 0.0;
  wv = c3 ? L[WSM][vn] * dv[vn] + L[WSM][vt] * dv[vt] + L[WSM][vb] * dv[vb]
          : L[WSM][vn] * dv[vn] + L[WSM][vt] * dv[vt];
  wB = c3 ? L[WSM][PRS] * dv[PRS] + L[WSM][bt] * dv[bt] + L[WSM][bb] * dv[bb]
          : L[WSM][PRS] * dv[PRS] + L[WSM][bt] * dv[bt];
  dw[WSM] = wv + wB;
  dw[WSP] = -wv + wB;
  wv = L[WAM][vt] * dv[vt] + L[WAM][vb] * dv[vb];
  wB = L[WAM][bt] * dv[bt] + L[WAM][bb] * dv[bb];
  dw[WAM] = wv + wB;
  dw[WAP] = wv - wB;
}

// States with CHAR_LIMITING YES (Src/States/plm_states.c:446-705, uniform
// Cartesian grid: cp = cm = 2, dp = dm = 0.5) for the zone with neighbours
// vl, v0, vr along DIR: the undivided differences projected on the left
// eigenvectors, limited per characteristic family (LIMITER DEFAULT: the
// generalised minmod SET_GM_LIMITER with steepness 1 for the fast and slow
// families, 2 otherwise), summed back over the right eigenvectors in wave
// order and clipped by MINMOD against twice the primitive differences.
// With two components the third velocity / field slots keep the centre value.
template <int DIR>
__device__ __forceinline__ void plm_char(const double* vl, const double* v0, const double* vr, double gamma, int lim,
                                         bool c3, int dims, double* vp, double* vm) {
  double L[8][8], R[8][8], lambda[8], dvp[8], dvm[8], dwp[8], dwm[8], dwl[8];
  const double a2 = gamma * v0[PRS] / v0[RHO];  // SoundSpeed2, Src/EOS/Ideal/eos.c:33
  prim_eigen<DIR>(v0, a2, c3, dims, L, R, lambda);
#pragma unroll
  for (int v = 0; v < 8; v++) {
    dvp[v] = vr[v] - v0[v];
    dvm[v] = v0[v] - vl[v];
  }
  prim_to_char<DIR>(L, dvm, c3, dwm);
  prim_to_char<DIR>(L, dvp, c3, dwp);
  const int nflx = c3 ? 8 : 6;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    if (lim == LIM_DEFAULT) {
      const double ck = (k == WFM || k == WFP || k == WSM || k == WSP) ? 1.0 : 2.0;
      if (dwp[k] * dwm[k] > 0.0) {
        const double qc = 0.5 * (dwm[k] + dwp[k]), scrh = abs_min(dwp[k] * ck, dwm[k] * ck);
        dwl[k] = abs_min(qc, scrh);
      } else {
        dwl[k] = 0.0;
      }
    } else {
      dwl[k] = limit(lim, -1, dwp[k], dwm[k]);
    }
  }
#pragma unroll
  for (int v = 0; v < 8; v++) {
    if (!c3 && (v == VX3 || v == BX3)) {
      vp[v] = vm[v] = v0[v];
      continue;
    }
    double dc = 0.0;
#pragma unroll
    for (int k = 0; k < 8; k++)
      if (k < nflx) dc += dwl[k] * R[v][k];
    double dvl = 0.0;
    if (dvp[v] * dvm[v] > 0.0) dvl = minmod(abs_min(2.0 * dvp[v], 2.0 * dvm[v]), dc);
    vp[v] = v0[v] + dvl * 0.5;
    vm[v] = v0[v] - dvl * 0.5;
  }
}

// CharTracingStep (Src/States/char_tracing.c:280-573; LINEAR, reference
// state 3, uniform Cartesian grid, no passive scalars): the PLM states vp, vm
// of the zone with centre value vc are replaced by their characteristic
// traces over dt/2.  PrimSource is zero here (Src/MHD/prim_eqn.c:120-210
// without geometry, gravity or div-B terms) and is added as +0.  With two
// components the third velocity and field slots are left alone.
template <int DIR>
__device__ __forceinline__ void char_tracing(const double* vc, double* vp, double* vm, double gamma, double dtdx,
                                             double dt, bool c3, int dims) {
  using Rt = Rot<DIR>;
  constexpr int vn = Rt::vn, vt = Rt::vt, vb = Rt::vb, bt = Rt::bt, bb = Rt::bb;
  double L[8][8], R[8][8], lambda[8];
  const double a2 = gamma * vc[PRS] / vc[RHO];  // SoundSpeed2, Src/EOS/Ideal/eos.c:33
  prim_eigen<DIR>(vc, a2, c3, dims, L, R, lambda);
  const int nflx = c3 ? 8 : 6;
  double nu[8], dv[8], dw[8];
#pragma unroll
  for (int k = 0; k < 8; k++) nu[k] = dtdx * lambda[k];
  const double nu_max = pmax(nu[1], 0.0), nu_min = pmin(nu[0], 0.0);
#pragma unroll
  for (int v = 0; v < 8; v++) dv[v] = vp[v] - vm[v];
  prim_to_char<DIR>(L, dv, c3, dw);
#pragma unroll
  for (int v = 0; v < 8; v++) {
    if (!c3 && (v == VX3 || v == BX3)) continue;
    vp[v] = vc[v] + 0.5 * dv[v] * (1.0 - nu_max);
    vm[v] = vc[v] - 0.5 * dv[v] * (1.0 + nu_min);
  }
#pragma unroll
  for (int k = 0; k < 8; k++) {
    if (k >= nflx) break;
    const bool right = nu[k] >= 0.0;
    const double w = dw[k] * (right ? 0.5 * (nu_max - nu[k]) : 0.5 * (nu_min - nu[k]));
#pragma unroll
    for (int v = 0; v < 8; v++) {
      if (!c3 && (v == VX3 || v == BX3)) continue;
      if (right) vp[v] += w * R[v][k];
      else vm[v] += w * R[v][k];
    }
  }
  const double src = 0.0;
#pragma unroll
  for (int v = 0; v < 8; v++) {
    if (!c3 && (v == VX3 || v == BX3)) continue;
    vp[v] += 0.5 * dt * src;
    vm[v] += 0.5 * dt * src;
  }
}


// CharTracingStep for parabolic states (Src/States/char_tracing.c:46-279,
// uniform Cartesian grid): with reference state 3 (no CHAR_LIMITING) the
// states first move to the PPM reference state of the fastest wave towards
// each interface; then (states 3 and 2) each family's parabola averaged over
// its domain of dependence is added on the side it reaches; PrimSource is
// zero (+0).
template <int DIR>
__device__ __forceinline__ void char_tracing_ppm(const double* vc, double* vp, double* vm, double gamma,
                                                 double dtdx, double dt, bool c3, int dims, int ref_state) {
  double L[8][8], R[8][8], lambda[8], nu[8], dvp[8], dvm[8], dwp[8], dwm[8];
  const double a2 = gamma * vc[PRS] / vc[RHO];  // SoundSpeed2, Src/EOS/Ideal/eos.c:33
  prim_eigen<DIR>(vc, a2, c3, dims, L, R, lambda);
  const int nflx = c3 ? 8 : 6;
#pragma unroll
  for (int k = 0; k < 8; k++) nu[k] = dtdx * lambda[k];
#pragma unroll
  for (int v = 0; v < 8; v++) {
    dvp[v] = vp[v] - vc[v];
    dvm[v] = vm[v] - vc[v];
  }
  prim_to_char<DIR>(L, dvp, c3, dwp);
  prim_to_char<DIR>(L, dvm, c3, dwm);
  const double nup = pmax(nu[1], 0.0), num = pmin(nu[0], 0.0);
#pragma unroll
  for (int v = 0; v < 8; v++) {
    if (ref_state != 3 || (!c3 && (v == VX3 || v == BX3))) continue;
    const double dwh = vp[v] - vm[v], d2w = vp[v] + vm[v] - 2.0 * vc[v];
    vp[v] -= 0.5 * nup * (dwh + d2w * (3.0 - 2.0 * nup));
    vm[v] -= 0.5 * num * (dwh - d2w * (3.0 + 2.0 * num));
  }
#pragma unroll
  for (int k = 0; k < 8; k++) {
    if (k >= nflx) break;
    const double dwh = dwp[k] - dwm[k], d2w = dwp[k] + dwm[k];
    const bool right = nu[k] >= 0.0;
    double S;
    if (ref_state == 3)
      S = right ? -0.5 * (nu[k] - nup) * (dwh + 3.0 * d2w) + (nu[k] * nu[k] - nup * nup) * d2w
                : -0.5 * (nu[k] - num) * (dwh - 3.0 * d2w) + (nu[k] * nu[k] - num * num) * d2w;
    else  // reference state 2 (with CHAR_LIMITING, char_tracing.c:35-43)
      S = right ? -0.5 * nu[k] * (dwh + d2w * (3.0 - 2.0 * nu[k])) : -0.5 * nu[k] * (dwh - d2w * (3.0 + 2.0 * nu[k]));
#pragma unroll
    for (int v = 0; v < 8; v++) {
      if (!c3 && (v == VX3 || v == BX3)) continue;
      if (right) vp[v] += S * R[v][k];
      else vm[v] += S * R[v][k];
    }
  }
  const double src = 0.0;
#pragma unroll
  for (int v = 0; v < 8; v++) {
    if (!c3 && (v == VX3 || v == BX3)) continue;
    const double dwh = 0.5 * dt * src;
    vp[v] += dwh;
    vm[v] += dwh;
  }
}


// States with RECONSTRUCTION PARABOLIC and CHAR_LIMITING YES
// (Src/States/ppm_states.c:258-560; PPM_ORDER 4, PARABOLIC_LIM 1, uniform
// Cartesian: hp = hm = 3, cp = cm = 2) for the zone v0 with neighbours
// w2 w1 | e1 e2 along DIR: the unlimited interface values projected on the
// left eigenvectors and clipped by MINMOD against the projected neighbour
// differences, summed back over the right eigenvectors in wave order, the
// parabolic limiter on the primitive increments, and linear density /
// pressure where a state came out negative.
template <int DIR>
__device__ __forceinline__ void ppm_char(const double* w2, const double* w1, const double* v0, const double* e1,
                                         const double* e2, double gamma, bool c3, int dims, double* vp, double* vm) {
  const double q_1 = -1.0 / 12.0, q0 = 7.0 / 12.0, q1 = 7.0 / 12.0, q2 = -1.0 / 12.0;
  double L[8][8], R[8][8], lambda[8], dvp[8], dvm[8], dvF0[8], dvF1[8], dwp[8], dwm[8], dwp1[8], dwm1[8];
  const double a2 = gamma * v0[PRS] / v0[RHO];  // SoundSpeed2
  prim_eigen<DIR>(v0, a2, c3, dims, L, R, lambda);
#pragma unroll
  for (int v = 0; v < 8; v++) {
    const double ip = q_1 * w1[v] + q0 * v0[v] + q1 * e1[v] + q2 * e2[v];
    const double im = q_1 * w2[v] + q0 * w1[v] + q1 * v0[v] + q2 * e1[v];
    dvp[v] = ip - v0[v];
    dvm[v] = im - v0[v];
    dvF1[v] = e1[v] - v0[v];
    dvF0[v] = v0[v] - w1[v];
  }
  prim_to_char<DIR>(L, dvp, c3, dwp);
  prim_to_char<DIR>(L, dvm, c3, dwm);
  prim_to_char<DIR>(L, dvF0, c3, dwm1);
  prim_to_char<DIR>(L, dvF1, c3, dwp1);
  const int nflx = c3 ? 8 : 6;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    dwp[k] = minmod(dwp[k], dwp1[k]);
    dwm[k] = minmod(dwm[k], -dwm1[k]);
  }
  const double cm = (3.0 + 1.0) / (3.0 - 1.0), cp = (3.0 + 1.0) / (3.0 - 1.0);
#pragma unroll
  for (int v = 0; v < 8; v++) {
    if (!c3 && (v == VX3 || v == BX3)) {
      vp[v] = vm[v] = v0[v];
      continue;
    }
    double dp = 0.0, dm = 0.0;
#pragma unroll
    for (int k = 0; k < 8; k++)
      if (k < nflx) {
        dp += dwp[k] * R[v][k];
        dm += dwm[k] * R[v][k];
      }
    if (dp * dm >= 0.0) {
      dp = dm = 0.0;
    } else {
      if (::fabs(dp) >= cm * ::fabs(dm)) dp = -cm * dm;
      else if (::fabs(dm) >= cp * ::fabs(dp)) dm = -cp * dp;
    }
    vp[v] = v0[v] + dp;
    vm[v] = v0[v] + dm;
  }
  if (vp[RHO] < 0.0 || vm[RHO] < 0.0) {
    const double d = 0.5 * (minmod(dvF1[RHO], dvF0[RHO]));
    vp[RHO] = v0[RHO] + d;
    vm[RHO] = v0[RHO] + (-d);
  }
  if (vp[PRS] < 0.0 || vm[PRS] < 0.0) {
    const double d = 0.5 * (minmod(dvF1[PRS], dvF0[PRS]));
    vp[PRS] = v0[PRS] + d;
    vm[PRS] = v0[PRS] + (-d);
  }
}

}  // namespace pg
