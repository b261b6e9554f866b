/*
 * CPU oracle: plain-C restatement of PLUTO 4.3's unsplit RK + CT ideal-MHD
 * step.  TEST INFRASTRUCTURE ONLY -- see mhd_oracle.h.
 *
 * Each function names the reference routine it restates (file:line, paths
 * inside the PLUTO source tree).  Expressions keep the reference's operand
 * order so that, built with -ffp-contract=off, results match the reference
 * binary bit for bit.
 */
#include "mhd_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NV OC_NVAR
#define RHO OC_RHO
#define VX1 OC_VX1
#define VX2 OC_VX2
#define VX3 OC_VX3
#define BX1 OC_BX1
#define BX2 OC_BX2
#define BX3 OC_BX3
#define PRS OC_PRS
#define ENG OC_PRS
#define MX1 OC_VX1

/* Src/macros.h:140-151 */
#define MAX(a, b) ((a) >= (b) ? (a) : (b))
#define MIN(a, b) ((a) <= (b) ? (a) : (b))
#define ABS_MIN(a, b) (fabs(a) < fabs(b) ? (a) : (b))
#define MINMOD(a, b) ((a) * (b) > 0.0 ? (fabs(a) < fabs(b) ? (a) : (b)) : 0.0)

#define SMALL_DENSITY 1.e-12  /* Src/globals.h:113 */
#define SMALL_PRESSURE 1.e-12 /* Src/globals.h:114 */
#define FLAG_CONS2PRIM_FAIL 64 /* Src/pluto.h:200 */
#define FLAG_INTERNAL_BOUNDARY 32 /* Src/pluto.h:197 */

struct oc_problem {
  oc_config c;
  oc_userdef_fn ud_fn;     /* USERDEF sides */
  void *ud_user;
  int internal;            /* INTERNAL_BOUNDARY */
  int bstage;              /* boundary fills so far in the step */
  int ng, nt[3], beg[3], end[3];
  size_t ncell, nface[3];
  double inv_dx[3];
  double *vc[NV], *uc[NV], *u0[NV];
  double *bs[3], *bs0[3];
  double *sl[3], *sr[3];   /* max(0,-SL), max(0,SR) per interface, emf->S?L/R */
  double *dv[3][3];        /* dv[d][c]: slope of velocity c along d, emf->dv?_d? */
  double *ex, *ey, *ez;    /* edge EMFs */
  double *cdt;             /* C_dt, update_stage.c:81 */
  unsigned char *flag;
  int64_t nfail;
  double max_mach;
  int roe_bad;           /* Roe: negative a^2 met (the reference stops there) */
  /* CTU (TIME_STEPPING HANCOCK) work arrays, ctu_step.c:195-221 */
  double *up_s[3][NV], *um_s[3][NV], *rhs_s[3][NV], *uh[NV];
  double *eface[6];        /* face EMFs: ezi, ezj, eyi, eyk, exj, exk (ct_emf.c:29-100) */
  signed char *sv[3];      /* sign of the mass flux at each face (UCT_CONTACT) */
  double *ecc[3];          /* cell-centred EMF (CT_ComputeCenterEMF) */
  int emf_lo[3], emf_hi[3];/* emf->ibeg.. set by CT_StoreUpwindEMF */
};

/* ------------------------------------------------------------------ */
/* indexing                                                             */
/* ------------------------------------------------------------------ */
static inline size_t CI(const oc_problem *p, int k, int j, int i) {
  return ((size_t)k * p->nt[1] + j) * p->nt[0] + i;
}
/* face array d, reference index with -1 origin along d
   (Src/initialize.c:448-453) */
static inline size_t FI(const oc_problem *p, int d, int k, int j, int i) {
  int sx = p->nt[0] + (d == 0), sy = p->nt[1] + (d == 1);
  return ((size_t)(k + (d == 2)) * sy + (j + (d == 1))) * sx + (i + (d == 0));
}

/* ------------------------------------------------------------------ */
/* Physics kernels on one point                                        */
/* ------------------------------------------------------------------ */

/* Src/MHD/mappers.c:25-86 (IDEAL EOS) */
static void prim_to_cons(const double *v, double *u, double gmm1) {
  double kinb2;
  u[RHO] = v[RHO];
  u[MX1] = v[RHO] * v[VX1];
  u[MX1 + 1] = v[RHO] * v[VX2];
  u[MX1 + 2] = v[RHO] * v[VX3];
  u[BX1] = v[BX1];
  u[BX2] = v[BX2];
  u[BX3] = v[BX3];
  kinb2 = v[VX1] * v[VX1] + v[VX2] * v[VX2] + v[VX3] * v[VX3];
  kinb2 = v[RHO] * kinb2 + v[BX1] * v[BX1] + v[BX2] * v[BX2] + v[BX3] * v[BX3];
  kinb2 *= 0.5;
  u[ENG] = kinb2 + v[PRS] / gmm1;
}

/* Src/MHD/mappers.c:88-254 (IDEAL EOS, no entropy switch).  The floors
   modify u in place exactly as the reference does. */
static int cons_to_prim(double *u, double *v, double gmm1, unsigned char *flag) {
  double tau, rho, kinb2, m2, b2;
  int ifail = 0;
  m2 = u[MX1] * u[MX1] + u[MX1 + 1] * u[MX1 + 1] + u[MX1 + 2] * u[MX1 + 2];
  b2 = u[BX1] * u[BX1] + u[BX2] * u[BX2] + u[BX3] * u[BX3];
  if (u[RHO] < 0.0) {
    u[RHO] = SMALL_DENSITY;
    *flag |= FLAG_CONS2PRIM_FAIL;
    ifail = 1;
  }
  v[RHO] = rho = u[RHO];
  tau = 1.0 / u[RHO];
  v[VX1] = u[MX1] * tau;
  v[VX2] = u[MX1 + 1] * tau;
  v[VX3] = u[MX1 + 2] * tau;
  v[BX1] = u[BX1];
  v[BX2] = u[BX2];
  v[BX3] = u[BX3];
  kinb2 = 0.5 * (m2 * tau + b2);
  if (u[ENG] < 0.0) {
    u[ENG] = SMALL_PRESSURE / gmm1 + kinb2;
    *flag |= FLAG_CONS2PRIM_FAIL;
    ifail = 1;
  }
  v[PRS] = gmm1 * (u[ENG] - kinb2);
  if (v[PRS] < 0.0) {
    v[PRS] = SMALL_PRESSURE;
    u[ENG] = v[PRS] / gmm1 + kinb2;
    *flag |= FLAG_CONS2PRIM_FAIL;
    ifail = 1;
  }
  (void)rho;
  return ifail;
}

/* Normal / tangent / bitangent rotation, Src/set_indexes.c:49-124 */
typedef struct { int vn, vt, vb, bn, bt, bb; } Rot;
static Rot rot_for(int dir) {
  Rot r;
  if (dir == 0) { r.vn = VX1; r.vt = VX2; r.vb = VX3; }
  else if (dir == 1) { r.vn = VX2; r.vt = VX1; r.vb = VX3; }
  else { r.vn = VX3; r.vt = VX1; r.vb = VX2; }
  r.bn = r.vn + 3; r.bt = r.vt + 3; r.bb = r.vb + 3;
  return r;
}

/* Src/MHD/fluxes.c:110-249 (ideal MHD, no background field) */
static void flux(const double *v, const double *u, double *fx, double *ptot_out,
                 const Rot *r) {
  double Bmag2, ptot, vB;
  Bmag2 = v[BX1] * v[BX1] + v[BX2] * v[BX2] + v[BX3] * v[BX3];
  ptot = v[PRS] + 0.5 * Bmag2;
  vB = v[VX1] * v[BX1] + v[VX2] * v[BX2] + v[VX3] * v[BX3];
  fx[RHO] = u[r->vn];
  fx[MX1] = v[r->vn] * u[MX1] - v[r->bn] * v[BX1];
  fx[MX1 + 1] = v[r->vn] * u[MX1 + 1] - v[r->bn] * v[BX2];
  fx[MX1 + 2] = v[r->vn] * u[MX1 + 2] - v[r->bn] * v[BX3];
  fx[r->bn] = 0.0;
  fx[r->bt] = v[r->vn] * v[r->bt] - v[r->bn] * v[r->vt];
  fx[r->bb] = v[r->vn] * v[r->bb] - v[r->bn] * v[r->vb];
  fx[ENG] = (u[ENG] + ptot) * v[r->vn] - v[r->bn] * vB;
  *ptot_out = ptot;
}

/* Src/MHD/eigenv.c:35-104 (IDEAL EOS) */
static void max_signal_speed(const double *v, double gamma, const Rot *r,
                             double *cmin, double *cmax) {
  double gpr, b1, b2, b3, Btmag2, Bmag2, cf;
  gpr = gamma * v[PRS];
  b1 = v[r->bn];
  b2 = v[r->bt];
  b3 = v[r->bb];
  Btmag2 = b2 * b2 + b3 * b3;
  Bmag2 = b1 * b1 + Btmag2;
  cf = gpr - Bmag2;
  cf = gpr + Bmag2 + sqrt(cf * cf + 4.0 * gpr * Btmag2);
  cf = sqrt(0.5 * cf / v[RHO]);
  *cmin = v[r->vn] - cf;
  *cmax = v[r->vn] + cf;
}

/* Riemann interface record */
typedef struct { double f[NV], press, SL, SR, cmax; } Iface;

/* Src/MHD/hll_speed.c:23-108 (DAVIS_ESTIMATE) + Src/EOS/Ideal/eos.c:16-42 */
static double hll_speed(const double *vL, const double *vR, double gamma,
                        const Rot *r, double *SL, double *SR) {
  double slmin, slmax, srmin, srmax, a2L, a2R, scrh;
  max_signal_speed(vL, gamma, r, &slmin, &slmax);
  max_signal_speed(vR, gamma, r, &srmin, &srmax);
  *SL = MIN(slmin, srmin);
  *SR = MAX(slmax, srmax);
  a2L = gamma * vL[PRS] / vL[RHO];
  a2R = gamma * vR[PRS] / vR[RHO];
  scrh = fabs(vL[r->vn]) + fabs(vR[r->vn]);
  scrh /= sqrt(a2L) + sqrt(a2R);
  return scrh;
}

/* Src/MHD/hll.c:30-166 */
static void hll_solver(const double *vL, const double *uL, const double *vR,
                       const double *uR, double gamma, const Rot *r, Iface *o,
                       double *mach) {
  double fL[NV], fR[NV], ptL, ptR, SL, SR, scrh;
  int nv;
  flux(vL, uL, fL, &ptL, r);
  flux(vR, uR, fR, &ptR, r);
  *mach = hll_speed(vL, vR, gamma, r, &SL, &SR);
  o->SL = SL;
  o->SR = SR;
  scrh = MAX(fabs(SL), fabs(SR));
  o->cmax = scrh;
  if (SL > 0.0) {
    for (nv = 0; nv < NV; nv++) o->f[nv] = fL[nv];
    o->press = ptL;
  } else if (SR < 0.0) {
    for (nv = 0; nv < NV; nv++) o->f[nv] = fR[nv];
    o->press = ptR;
  } else {
    scrh = 1.0 / (SR - SL);
    for (nv = 0; nv < NV; nv++) {
      o->f[nv] = SL * SR * (uR[nv] - uL[nv]) + SR * fL[nv] - SL * fR[nv];
      o->f[nv] *= scrh;
    }
    o->press = (SR * ptL - SL * ptR) * scrh;
  }
}

/* Src/MHD/roe.c:53-799: linearised solver of Cargo & Gallice (1997), ideal
   EOS, no background field, HLL hybridisation off, entropy fix with
   delta = 1e-6.  Waves in the order of the KWAVES enumeration
   (Src/MHD/mod_defs.h:54-72): fast-, fast+, entropy, div.B, slow-, slow+
   and, with three components, Alfven-, Alfven+.  Returns 1 when the Roe
   sound speed squared is negative (the reference stops there). */
static int roe_solver(const double *vL, const double *uL, const double *vR,
                      const double *uR, double gamma, int c3, const Rot *r,
                      Iface *o, double *mach) {
  const int vn = r->vn, vt = r->vt, vb = r->vb, bn = r->bn, bt = r->bt, bb = r->bb;
  const double delta = 1.e-6, g1 = gamma - 1.0;
  double fL[NV], fR[NV], ptL, ptR, dV[NV], dU[NV];
  double srL, srR, sl, sr, rho, sqrt_rho, u, v, w, Bx, By, Bz, sBx, bx, by, bz;
  double bt2, b2, Btmag, X, vdm, BdB, vel2, HL, HR, H, Hgas, a2, scrh, ca2, cf2, cs2;
  double cf, cs, ca, a, af, as, beta_y, beta_z, beta_dv, beta_dB, beta_v;
  double lam[8], eta[8], al[8], c[8];
  double Rf[8], Rs[8], Ra[8], Rfp[8], Rsp[8], Rap[8], Re[8];
  int bad = 0, nv, k;
  flux(vL, uL, fL, &ptL, r);
  flux(vR, uR, fR, &ptR, r);
  for (nv = 0; nv < NV; nv++) {
    dV[nv] = vR[nv] - vL[nv];
    dU[nv] = uR[nv] - uL[nv];
  }
  /* Roe averages */
  srL = sqrt(vL[RHO]);
  srR = sqrt(vR[RHO]);
  sl = srL / (srL + srR);
  sr = srR / (srL + srR);
  rho = sr * vL[RHO] + sl * vR[RHO];
  sqrt_rho = sqrt(rho);
  u = sl * vL[vn] + sr * vR[vn];
  v = sl * vL[vt] + sr * vR[vt];
  w = sl * vL[vb] + sr * vR[vb];
  Bx = sr * vL[bn] + sl * vR[bn];
  By = sr * vL[bt] + sl * vR[bt];
  Bz = sr * vL[bb] + sl * vR[bb];
  sBx = (Bx >= 0.0 ? 1.0 : -1.0);
  bx = Bx / sqrt_rho;
  by = By / sqrt_rho;
  bz = Bz / sqrt_rho;
  bt2 = 0.0 + by * by + bz * bz;
  b2 = bx * bx + bt2;
  Btmag = sqrt(bt2 * rho);
  X = dV[bn] * dV[bn] + dV[bt] * dV[bt] + dV[bb] * dV[bb];
  X /= (srL + srR) * (srL + srR) * 2.0;
  vdm = u * dU[vn] + v * dU[vt] + w * dU[vb];
  BdB = Bx * dU[bn] + By * dU[bt] + Bz * dU[bb];
  /* enthalpy and sound speed */
  vel2 = u * u + v * v + w * w;
  dV[PRS] = g1 * ((0.5 * vel2 - X) * dV[RHO] - vdm + dU[ENG] - BdB);
  HL = (uL[ENG] + ptL) / vL[RHO];
  HR = (uR[ENG] + ptR) / vR[RHO];
  H = sl * HL + sr * HR;
  Hgas = H - b2;
  a2 = (2.0 - gamma) * X + g1 * (Hgas - 0.5 * vel2);
  if (a2 < 0.0) {
    bad = 1;
    a2 = sqrt(gamma * (vL[PRS] + vR[PRS]) / (vL[RHO] + vR[RHO]));
  }
  /* fast and slow speeds */
  scrh = a2 - b2;
  ca2 = bx * bx;
  scrh = scrh * scrh + 4.0 * bt2 * a2;
  scrh = sqrt(scrh);
  cf2 = 0.5 * (a2 + b2 + scrh);
  cs2 = a2 * ca2 / cf2;
  cf = sqrt(cf2);
  cs = sqrt(cs2);
  ca = sqrt(ca2);
  a = sqrt(a2);
  if (cf == cs) {
    af = 1.0;
    as = 0.0;
  } else if (a <= cs) {
    af = 0.0;
    as = 1.0;
  } else if (cf <= a) {
    af = 1.0;
    as = 0.0;
  } else {
    scrh = 1.0 / (cf2 - cs2);
    af = (a2 - cs2) * scrh;
    as = (cf2 - a2) * scrh;
    af = MAX(0.0, af);
    as = MAX(0.0, as);
    af = sqrt(af);
    as = sqrt(as);
  }
  if (Btmag > 1.e-9) {
    if (c3) {
      beta_y = By / Btmag;
      beta_z = Bz / Btmag;
    } else {
      beta_y = (By >= 0.0 ? 1.0 : -1.0);
      beta_z = 0.0;
    }
  } else {
    beta_y = c3 ? 0.70710678118654752440 : 1.0;
    beta_z = c3 ? 0.70710678118654752440 : 0.0;
  }
  beta_dv = 0.0 + beta_y * dV[vt] + beta_z * dV[vb];
  beta_dB = 0.0 + beta_y * dV[bt] + beta_z * dV[bb];
  beta_v = 0.0 + beta_y * v + beta_z * w;

  /* eigenvector entries by row role: 0 rho, 1 m_n, 2 m_t, 3 m_b, 4 B_t,
     5 B_b, 6 energy (the B_n row is zero for every wave) */
  /* fast waves */
  scrh = as * cs * sBx;
  lam[0] = u - cf;
  Rf[0] = af;
  Rf[1] = af * lam[0];
  Rf[2] = af * v + scrh * beta_y;
  Rf[3] = af * w + scrh * beta_z;
  Rf[4] = as * a * beta_y / sqrt_rho;
  Rf[5] = as * a * beta_z / sqrt_rho;
  Rf[6] = af * (Hgas - u * cf) + scrh * beta_v + as * a * Btmag / sqrt_rho;
  eta[0] = af * (X * dV[RHO] + dV[PRS]) + rho * scrh * beta_dv - rho * af * cf * dV[vn] +
           sqrt_rho * as * a * beta_dB;
  eta[0] *= 0.5 / a2;
  lam[1] = u + cf;
  Rfp[0] = af;
  Rfp[1] = af * lam[1];
  Rfp[2] = af * v - scrh * beta_y;
  Rfp[3] = af * w - scrh * beta_z;
  Rfp[4] = Rf[4];
  Rfp[5] = Rf[5];
  Rfp[6] = af * (Hgas + u * cf) - scrh * beta_v + as * a * Btmag / sqrt_rho;
  eta[1] = af * (X * dV[RHO] + dV[PRS]) - rho * scrh * beta_dv + rho * af * cf * dV[vn] +
           sqrt_rho * as * a * beta_dB;
  eta[1] *= 0.5 / a2;
  /* entropy wave */
  lam[2] = u;
  Re[0] = 1.0;
  Re[1] = u;
  Re[2] = v;
  Re[3] = w;
  Re[6] = 0.5 * vel2 + (gamma - 2.0) / g1 * X;
  eta[2] = ((a2 - X) * dV[RHO] - dV[PRS]) / a2;
  /* div.B wave: zero jump */
  lam[3] = u;
  eta[3] = 0.0;
  /* slow waves */
  scrh = af * cf * sBx;
  lam[4] = u - cs;
  Rs[0] = as;
  Rs[1] = as * lam[4];
  Rs[2] = as * v - scrh * beta_y;
  Rs[3] = as * w - scrh * beta_z;
  Rs[4] = -af * a * beta_y / sqrt_rho;
  Rs[5] = -af * a * beta_z / sqrt_rho;
  Rs[6] = as * (Hgas - u * cs) - scrh * beta_v - af * a * Btmag / sqrt_rho;
  eta[4] = as * (X * dV[RHO] + dV[PRS]) - rho * scrh * beta_dv - rho * as * cs * dV[vn] -
           sqrt_rho * af * a * beta_dB;
  eta[4] *= 0.5 / a2;
  lam[5] = u + cs;
  Rsp[0] = as;
  Rsp[1] = as * lam[5];
  Rsp[2] = as * v + scrh * beta_y;
  Rsp[3] = as * w + scrh * beta_z;
  Rsp[4] = Rs[4];
  Rsp[5] = Rs[5];
  Rsp[6] = as * (Hgas + u * cs) + scrh * beta_v - af * a * Btmag / sqrt_rho;
  eta[5] = as * (X * dV[RHO] + dV[PRS]) + rho * scrh * beta_dv + rho * as * cs * dV[vn] -
           sqrt_rho * af * a * beta_dB;
  eta[5] *= 0.5 / a2;
  /* Alfven waves (three components only) */
  lam[6] = u - ca;
  lam[7] = u + ca;
  Ra[2] = -rho * beta_z;
  Ra[3] = +rho * beta_y;
  Ra[4] = -sBx * sqrt_rho * beta_z;
  Ra[5] = sBx * sqrt_rho * beta_y;
  Ra[6] = -rho * (v * beta_z - w * beta_y);
  Rap[2] = -Ra[2];
  Rap[3] = -Ra[3];
  Rap[4] = Ra[4];
  Rap[5] = Ra[5];
  Rap[6] = -Ra[6];
  eta[6] = +beta_y * dV[vb] - beta_z * dV[vt] + sBx / sqrt_rho * (beta_y * dV[bb] - beta_z * dV[bt]);
  eta[6] *= 0.5;
  eta[7] = -beta_y * dV[vb] + beta_z * dV[vt] + sBx / sqrt_rho * (beta_y * dV[bb] - beta_z * dV[bt]);
  eta[7] *= 0.5;

  o->cmax = fabs(u) + cf;
  *mach = fabs(u / a);
  for (k = 0; k < 8; k++) al[k] = fabs(lam[k]);
  /* entropy fix */
  if (al[0] < 0.5 * delta) al[0] = lam[0] * lam[0] / delta + 0.25 * delta;
  if (al[1] < 0.5 * delta) al[1] = lam[1] * lam[1] / delta + 0.25 * delta;
  if (al[4] < 0.5 * delta) al[4] = lam[4] * lam[4] / delta + 0.25 * delta;
  if (al[5] < 0.5 * delta) al[5] = lam[5] * lam[5] / delta + 0.25 * delta;
  for (k = 0; k < 8; k++) c[k] = al[k] * eta[k];
  /* upwind sum over the waves in enumeration order (zero entries skipped) */
  {
    double s_rho, s_mn, s_mt, s_mb, s_bt, s_bb, s_en;
    s_rho = 0.0 + c[0] * Rf[0] + c[1] * Rfp[0] + c[2] * Re[0] + c[4] * Rs[0] + c[5] * Rsp[0];
    s_mn = 0.0 + c[0] * Rf[1] + c[1] * Rfp[1] + c[2] * Re[1] + c[4] * Rs[1] + c[5] * Rsp[1];
    s_mt = 0.0 + c[0] * Rf[2] + c[1] * Rfp[2] + c[2] * Re[2] + c[4] * Rs[2] + c[5] * Rsp[2];
    s_mb = 0.0 + c[0] * Rf[3] + c[1] * Rfp[3] + c[2] * Re[3] + c[4] * Rs[3] + c[5] * Rsp[3];
    s_bt = 0.0 + c[0] * Rf[4] + c[1] * Rfp[4] + c[4] * Rs[4] + c[5] * Rsp[4];
    s_bb = 0.0 + c[0] * Rf[5] + c[1] * Rfp[5] + c[4] * Rs[5] + c[5] * Rsp[5];
    s_en = 0.0 + c[0] * Rf[6] + c[1] * Rfp[6] + c[2] * Re[6] + c[4] * Rs[6] + c[5] * Rsp[6];
    if (c3) {
      s_mt = s_mt + c[6] * Ra[2] + c[7] * Rap[2];
      s_mb = s_mb + c[6] * Ra[3] + c[7] * Rap[3];
      s_bt = s_bt + c[6] * Ra[4] + c[7] * Rap[4];
      s_bb = s_bb + c[6] * Ra[5] + c[7] * Rap[5];
      s_en = s_en + c[6] * Ra[6] + c[7] * Rap[6];
    }
    o->f[RHO] = 0.5 * (fL[RHO] + fR[RHO] - s_rho);
    o->f[vn] = 0.5 * (fL[vn] + fR[vn] - s_mn);
    o->f[vt] = 0.5 * (fL[vt] + fR[vt] - s_mt);
    o->f[vb] = 0.5 * (fL[vb] + fR[vb] - s_mb);
    o->f[bn] = 0.5 * (fL[bn] + fR[bn] - 0.0);
    o->f[bt] = 0.5 * (fL[bt] + fR[bt] - s_bt);
    o->f[bb] = 0.5 * (fL[bb] + fR[bb] - s_bb);
    o->f[ENG] = 0.5 * (fL[ENG] + fR[ENG] - s_en);
  }
  o->press = 0.5 * (ptL + ptR);
  o->SL = lam[0];
  o->SR = lam[1];
  return bad;
}

/* Src/MHD/hlld.c:44-452 (IDEAL EOS, no background field) */
static void hlld_solver(const double *vL, const double *uL, const double *vR,
                        const double *uR, double gamma, const Rot *r, Iface *o,
                        double *mach) {
  const int MXn = r->vn, MXt = r->vt, MXb = r->vb;
  const int VXn = r->vn, VXt = r->vt, VXb = r->vb;
  const int BXn = r->bn, BXt = r->bt, BXb = r->bb;
  double fL[NV], fR[NV], ptL, ptR, SL, SR, scrh, Uhll[NV];
  double usL[NV], ussl[NV], usR[NV], ussr[NV];
  double vsL, wsL, scrhL, S1L, sqrL, duL;
  double vsR, wsR, scrhR, S1R, sqrR, duR;
  double Bx, Bx1, SM, sBx, pts, vss, wss;
  int nv, revert_to_hllc;

  flux(vL, uL, fL, &ptL, r);
  flux(vR, uR, fR, &ptR, r);
  *mach = hll_speed(vL, vR, gamma, r, &SL, &SR);
  o->SL = SL;
  o->SR = SR;
  scrh = MAX(fabs(SL), fabs(SR));
  o->cmax = scrh;

  if (SL >= 0.0) {
    for (nv = NV; nv--;) o->f[nv] = fL[nv];
    o->press = ptL;
  } else if (SR <= 0.0) {
    for (nv = NV; nv--;) o->f[nv] = fR[nv];
    o->press = ptR;
  } else {
    scrh = 1.0 / (SR - SL);
    Bx1 = Bx = (SR * vR[BXn] - SL * vL[BXn]) * scrh;
    sBx = (Bx > 0.0 ? 1.0 : -1.0);
    duL = SL - vL[VXn];
    duR = SR - vR[VXn];
    scrh = 1.0 / (duR * uR[RHO] - duL * uL[RHO]);
    SM = (duR * uR[MXn] - duL * uL[MXn] - ptR + ptL) * scrh;
    pts = duR * uR[RHO] * ptL - duL * uL[RHO] * ptR +
          vL[RHO] * vR[RHO] * duR * duL * (vR[VXn] - vL[VXn]);
    pts *= scrh;
    usL[RHO] = uL[RHO] * duL / (SL - SM);
    usR[RHO] = uR[RHO] * duR / (SR - SM);
    sqrL = sqrt(usL[RHO]);
    sqrR = sqrt(usR[RHO]);
    S1L = SM - fabs(Bx) / sqrL;
    S1R = SM + fabs(Bx) / sqrR;

    revert_to_hllc = 0;
    if ((S1L - SL) < 1.e-4 * (SM - SL)) revert_to_hllc = 1;
    if ((S1R - SR) > -1.e-4 * (SR - SM)) revert_to_hllc = 1;

    if (revert_to_hllc) {
      scrh = 1.0 / (SR - SL);
      for (nv = NV; nv--;) {
        Uhll[nv] = SR * uR[nv] - SL * uL[nv] + fL[nv] - fR[nv];
        Uhll[nv] *= scrh;
      }
      usL[BXn] = usR[BXn] = Uhll[BXn];
      usL[BXt] = usR[BXt] = Uhll[BXt];
      usL[BXb] = usR[BXb] = Uhll[BXb];
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

    if (S1L >= 0.0) {
      for (nv = NV; nv--;) o->f[nv] = fL[nv] + SL * (usL[nv] - uL[nv]);
      o->press = ptL;
    } else if (S1R <= 0.0) {
      for (nv = NV; nv--;) o->f[nv] = fR[nv] + SR * (usR[nv] - uR[nv]);
      o->press = ptR;
    } else {
      ussl[RHO] = usL[RHO];
      ussr[RHO] = usR[RHO];
      vss = sqrL * vsL + sqrR * vsR + (usR[BXt] - usL[BXt]) * sBx;
      vss /= sqrL + sqrR;
      wss = sqrL * wsL + sqrR * wsR + (usR[BXb] - usL[BXb]) * sBx;
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

      if (SM >= 0.0) {
        for (nv = NV; nv--;)
          o->f[nv] = fL[nv] + S1L * (ussl[nv] - usL[nv]) + SL * (usL[nv] - uL[nv]);
        o->press = ptL;
      } else {
        for (nv = NV; nv--;)
          o->f[nv] = fR[nv] + S1R * (ussr[nv] - usR[nv]) + SR * (usR[nv] - uR[nv]);
        o->press = ptR;
      }
    }
  }
}

/* ------------------------------------------------------------------ */
/* Reconstruction                                                       */
/* ------------------------------------------------------------------ */

/* Src/States/plm_coeffs.h:72-175 (uniform Cartesian forms) */
static inline double limit(int lim, int nv, double dvp, double dvm) {
  double dv;
  if (lim == OC_DEFAULT_LIM) { /* plm_states.c:180-213 */
    if (nv == RHO) lim = OC_MC_LIM;
    else if (nv == PRS) lim = OC_MINMOD_LIM;
    else lim = OC_VANLEER_LIM;
  }
  switch (lim) {
    case OC_FLAT_LIM: dv = 0.0; break;
    case OC_MINMOD_LIM: dv = (dvp * dvm > 0.0 ? ABS_MIN(dvp, dvm) : 0.0); break;
    case OC_VANLEER_LIM: dv = (dvp * dvm > 0.0 ? 2.0 * dvp * dvm / (dvp + dvm) : 0.0); break;
    default:
      if (dvp * dvm > 0.0) {
        double qc = 0.5 * (dvm + dvp), scrh = 2.0 * ABS_MIN(dvp, dvm);
        dv = ABS_MIN(qc, scrh);
      } else dv = 0.0;
  }
  return dv;
}

/* Src/States/plm_states.c:80-312: PLM on primitive variables for cells
   beg..end of a pencil; vp/vm indexed by cell. */
static void plm_states(double (*v)[NV], double (*vp)[NV], double (*vm)[NV],
                       int beg, int end, int lim) {
  int i, nv;
  for (i = beg; i <= end; i++) {
    for (nv = 0; nv < NV; nv++) {
      double dvp = v[i + 1][nv] - v[i][nv];
      double dvm = v[i][nv] - v[i - 1][nv];
      double dv = limit(lim, nv, dvp, dvm);
      vp[i][nv] = v[i][nv] + dv * 0.5;
      vm[i][nv] = v[i][nv] - dv * 0.5;
    }
  }
}

/* Src/States/ppm_states.c:68-253 with PPM_ORDER 4, Cartesian uniform
   coefficients (ppm_coeffs.c:478-520, Q6 hp = hm = 3 at :528-556). */
static void ppm_states(double (*v)[NV], double (*vp)[NV], double (*vm)[NV],
                       int beg, int end) {
  const double w_1 = -1.0 / 12.0, w0 = 7.0 / 12.0, w1 = 7.0 / 12.0, w2 = -1.0 / 12.0;
  const double hp = 3.0, hm = 3.0;
  int i, nv;
  for (i = beg - 1; i <= end; i++) {
    for (nv = 0; nv < NV; nv++) {
      double dv, dvp;
      vp[i][nv] = w_1 * v[i - 1][nv] + w0 * v[i][nv] + w1 * v[i + 1][nv] + w2 * v[i + 2][nv];
      dv = v[i + 1][nv] - v[i][nv];
      dvp = vp[i][nv] - v[i][nv];
      vp[i][nv] = v[i][nv] + MINMOD(dvp, dv);
    }
  }
  for (i = beg; i <= end; i++)
    for (nv = 0; nv < NV; nv++) vm[i][nv] = vp[i - 1][nv];
  for (i = beg; i <= end; i++) {
    double cm = (hm + 1.0) / (hp - 1.0);
    double cp = (hp + 1.0) / (hm - 1.0);
    for (nv = 0; nv < NV; nv++) {
      double dvp = vp[i][nv] - v[i][nv];
      double dvm = vm[i][nv] - v[i][nv];
      if (dvp * dvm >= 0.0) dvp = dvm = 0.0;
      else {
        if (fabs(dvp) >= cm * fabs(dvm)) dvp = -cm * dvm;
        else if (fabs(dvm) >= cp * fabs(dvp)) dvm = -cp * dvp;
      }
      vp[i][nv] = v[i][nv] + dvp;
      vm[i][nv] = v[i][nv] + dvm;
    }
  }
}

/* ------------------------------------------------------------------ */
/* Boundary conditions, Src/boundary.c:41-303, 318-565                 */
/* ------------------------------------------------------------------ */

/* FlipSign, Src/boundary.c:318-437 (REFLECTIVE and EQTSYMMETRIC): sign of
   variable nv (or of face component BX1+fd) mirrored across a side of axis d */
static int flip_sign(int d, int type, int nv, int components) {
  const int vn = VX1 + d, bn = BX1 + d;
  if (nv == vn) return -1;
  if (type == OC_EQTSYMMETRIC) {
    if (nv == bn) return 1;
    if (nv >= BX1 && nv <= BX3 && nv - BX1 < components) return -1; /* EXPAND(Bn, Bp, Bt) */
    return 1;
  }
  return nv == bn ? -1 : 1;
}

static void bound_box(oc_problem *p, double *q, int face_dir, int ib, int ie,
                      int jb, int je, int kb, int ke, int side, int type, int sgn) {
  /* q is a cell array (face_dir < 0) or face array face_dir.  Loops run
     over the box in increasing order; the copies read interior or
     already-assigned points only. */
  int i, j, k;
  int lo_i = ib < ie ? ib : ie, hi_i = ib < ie ? ie : ib;
  int lo_j = jb < je ? jb : je, hi_j = jb < je ? je : jb;
  int lo_k = kb < ke ? kb : ke, hi_k = kb < ke ? ke : kb;
  int NX1 = p->c.nx[0], NX2 = p->c.nx[1], NX3 = p->c.nx[2];
#define IDX(kk, jj, ii) (face_dir < 0 ? CI(p, kk, jj, ii) : FI(p, face_dir, kk, jj, ii))
  /* BOX_LOOP direction follows the box's own ordering (Src/macros.h:91). */
  int di = ib <= ie ? 1 : -1, dj = jb <= je ? 1 : -1, dk = kb <= ke ? 1 : -1;
  (void)lo_i; (void)hi_i; (void)lo_j; (void)hi_j; (void)lo_k; (void)hi_k;
  for (k = kb; dk * k <= dk * ke; k += dk)
    for (j = jb; dj * j <= dj * je; j += dj)
      for (i = ib; di * i <= di * ie; i += di) {
        size_t dst = IDX(k, j, i), src;
        if (type == OC_REFLECTIVE || type == OC_EQTSYMMETRIC) { /* ReflectiveBound, boundary.c:523-560 */
          if (side == 0) src = IDX(k, j, 2 * p->beg[0] - i - 1);
          else if (side == 1) src = IDX(k, j, 2 * p->end[0] - i + 1);
          else if (side == 2) src = IDX(k, 2 * p->beg[1] - j - 1, i);
          else if (side == 3) src = IDX(k, 2 * p->end[1] - j + 1, i);
          else if (side == 4) src = IDX(2 * p->beg[2] - k - 1, j, i);
          else src = IDX(2 * p->end[2] - k + 1, j, i);
          q[dst] = sgn * q[src];
          continue;
        } else if (type == OC_PERIODIC) {
          if (side == 0) src = IDX(k, j, i + NX1);
          else if (side == 1) src = IDX(k, j, i - NX1);
          else if (side == 2) src = IDX(k, j + NX2, i);
          else if (side == 3) src = IDX(k, j - NX2, i);
          else if (side == 4) src = IDX(k + NX3, j, i);
          else src = IDX(k - NX3, j, i);
        } else {
          if (side == 0) src = IDX(k, j, p->beg[0]);
          else if (side == 1) src = IDX(k, j, p->end[0]);
          else if (side == 2) src = IDX(k, p->beg[1], i);
          else if (side == 3) src = IDX(k, p->end[1], i);
          else if (side == 4) src = IDX(p->beg[2], j, i);
          else src = IDX(p->end[2], j, i);
        }
        q[dst] = q[src];
      }
#undef IDX
}

/* Face areas of a uniform Cartesian grid, Src/set_geometry.c:139-210:
   A1 = 1*dx2(*dx3), A2 = dx1*1(*dx3), A3 = dx1*dx2*1 (D_EXPAND over DIMENSIONS). */
static void face_areas(const oc_problem *p, double A[3]) {
  const double *dx = p->c.dx;
  if (p->c.dims == 2) {
    A[0] = 1.0 * dx[1];
    A[1] = dx[0] * 1.0;
    A[2] = 0.0;
  } else {
    A[0] = 1.0 * dx[1] * dx[2];
    A[1] = dx[0] * 1.0 * dx[2];
    A[2] = dx[0] * dx[1] * 1.0;
  }
}

/* FillMagneticField, Src/MHD/CT/ct_fill_mag_field.c:38-180 (Cartesian): the
   staggered component normal to an outflow side is recovered in the ghost
   faces from div B = 0, marching away from the boundary face. */
static void fill_magnetic_field(oc_problem *p, int side) {
  const int dims = p->c.dims;
  int ibeg = 0, iend = p->nt[0] - 1, di = 1;
  int jbeg = 0, jend = p->nt[1] - 1, dj = 1;
  int kbeg = 0, kend = p->nt[2] - 1, dk = 1;
  int i, j, k;
  double A[3];
  double *bx = p->bs[0], *by = p->bs[1], *bz = dims == 3 ? p->bs[2] : NULL;
  face_areas(p, A);
  if (dims < 3) { kbeg = kend = 0; dk = 1; }
  if (side == 0) { ibeg = p->beg[0] - 1; iend = 0; di = -1; }
  if (side == 1) ibeg = p->end[0] + 1;
  if (side == 2) { jbeg = p->beg[1] - 1; jend = 0; dj = -1; }
  if (side == 3) jbeg = p->end[1] + 1;
  if (side == 4) { kbeg = p->beg[2] - 1; kend = 0; dk = -1; }
  if (side == 5) kbeg = p->end[2] + 1;
  for (k = kbeg; dk * k <= dk * kend; k += dk)
    for (j = jbeg; dj * j <= dj * jend; j += dj)
      for (i = ibeg; di * i <= di * iend; i += di) {
        double bxp = bx[FI(p, 0, k, j, i)], bxm = bx[FI(p, 0, k, j, i - 1)];
        double byp = by[FI(p, 1, k, j, i)], bym = by[FI(p, 1, k, j - 1, i)];
        double bzp = 0.0, bzm = 0.0;
        double dBx = 0.0, dBy = 0.0, dBz = 0.0;
        if (dims == 3) {
          bzp = bz[FI(p, 2, k, j, i)];
          bzm = bz[FI(p, 2, k - 1, j, i)];
        }
        dBx = (A[0] * bxp - A[0] * bxm);
        dBy = (A[1] * byp - A[1] * bym);
        if (dims == 3) dBz = (A[2] * bzp - A[2] * bzm);
        if (side == 0) bx[FI(p, 0, k, j, i - 1)] = (A[0] * bxp + dBy + dBz) / A[0];
        else if (side == 1) bx[FI(p, 0, k, j, i)] = (A[0] * bxm - (dBy + dBz)) / A[0];
        else if (side == 2) by[FI(p, 1, k, j - 1, i)] = (A[1] * byp + dBx + dBz) / A[1];
        else if (side == 3) by[FI(p, 1, k, j, i)] = (A[1] * bym - (dBx + dBz)) / A[1];
        else if (side == 4) bz[FI(p, 2, k - 1, j, i)] = (A[2] * bzp + dBx + dBy) / A[2];
        else bz[FI(p, 2, k, j, i)] = (A[2] * bzm - (dBx + dBy)) / A[2];
      }
}

/* CT_AverageNormalMagField, Src/MHD/CT/ct_field_average.c:134-275
   (Cartesian): normal cell-centred field in the ghost zones of one side. */
static void ct_average_normal(oc_problem *p, int side) {
  const int d = side / 2;
  int i, j, k;
  int lo[3] = {0, 0, 0}, hi[3] = {p->nt[0] - 1, p->nt[1] - 1, p->nt[2] - 1};
  double *B = p->vc[BX1 + d], *b = p->bs[d];
  if (side % 2 == 0) { lo[d] = 0; hi[d] = p->beg[d] - 1; }
  else { lo[d] = p->end[d] + 1; hi[d] = p->nt[d] - 1; }
  for (k = lo[2]; k <= hi[2]; k++)
    for (j = lo[1]; j <= hi[1]; j++)
      for (i = lo[0]; i <= hi[0]; i++) {
        int o[3] = {0, 0, 0};
        o[d] = 1;
        B[CI(p, k, j, i)] = 0.5 * (b[FI(p, d, k, j, i)] + b[FI(p, d, k - o[2], j - o[1], i - o[0])]);
      }
}

/* CT_AverageTransverseMagField, Src/MHD/CT/ct_field_average.c:275-440
   (Cartesian): the transverse cell-centred field in the ghost zones of side
   is from the staggered components. */
static void ct_average_transverse(oc_problem *p, int is) {
  int d = is / 2, i, j, k, fd;
  int lo[3] = {0, 0, 0}, hi[3] = {p->nt[0] - 1, p->nt[1] - 1, p->nt[2] - 1};
  if (is & 1) lo[d] = p->end[d] + 1;
  else hi[d] = p->beg[d] - 1;
  for (k = lo[2]; k <= hi[2]; k++)
    for (j = lo[1]; j <= hi[1]; j++)
      for (i = lo[0]; i <= hi[0]; i++)
        for (fd = 0; fd < p->c.dims; fd++) {
          int o[3] = {0, 0, 0};
          if (fd == d) continue;
          o[fd] = 1;
          p->vc[BX1 + fd][CI(p, k, j, i)] =
              0.5 * (p->bs[fd][FI(p, fd, k, j, i)] + p->bs[fd][FI(p, fd, k - o[2], j - o[1], i - o[0])]);
        }
}

static void boundary(oc_problem *p) {
  int is, nv;
  int dims = p->c.dims;
  /* INTERNAL_BOUNDARY: UserDefBoundary (d, NULL, 0, grid), Src/boundary.c:90-92 */
  if (p->internal && p->ud_fn) p->ud_fn(p->ud_user, 6, 0, p->bstage + 1);
  for (is = 0; is < 2 * dims; is++) {
    int d = is / 2, type = (is & 1) ? p->c.bc_hi[d] : p->c.bc[d]; /* X*_BEG, X*_END */
    int ib = 0, ie = p->nt[0] - 1, jb = 0, je = p->nt[1] - 1, kb = 0, ke = p->nt[2] - 1;
    if (is == 0) { ib = p->beg[0] - 1; ie = 0; }
    else if (is == 1) { ib = p->end[0] + 1; ie = p->nt[0] - 1; }
    else if (is == 2) { jb = p->beg[1] - 1; je = 0; }
    else if (is == 3) { jb = p->end[1] + 1; je = p->nt[1] - 1; }
    else if (is == 4) { kb = p->beg[2] - 1; ke = 0; }
    else { kb = p->end[2] + 1; ke = p->nt[2] - 1; }
    if (type == OC_USERDEF) { /* Src/boundary.c:258-288 */
      int fd;
      if (p->ud_fn) {
        p->ud_fn(p->ud_user, is, 0, p->bstage + 1);
        if (p->c.ct)
          for (fd = 0; fd < dims; fd++) p->ud_fn(p->ud_user, is, 1 + fd, p->bstage + 1);
      }
      if (p->c.ct) { /* Src/boundary.c:287-289 */
        fill_magnetic_field(p, is);
        ct_average_normal(p, is);
        ct_average_transverse(p, is);
      }
      continue;
    }
    for (nv = 0; nv < NV; nv++)
      bound_box(p, p->vc[nv], -1, ib, ie, jb, je, kb, ke, is, type, flip_sign(d, type, nv, p->c.components));
    if (p->c.ct) {
      int fd;
      for (fd = 0; fd < dims; fd++) {
        int fib = ib, fie = ie, fjb = jb, fje = je, fkb = kb, fke = ke;
        /* face boxes, Src/boundary.c:141-149 */
        if (fd == 0) { if (ib < ie) fib = ib - 1; else fie = ie - 1; }
        if (fd == 1) { if (jb < je) fjb = jb - 1; else fje = je - 1; }
        if (fd == 2) { if (kb < ke) fkb = kb - 1; else fke = ke - 1; }
        if (type == OC_PERIODIC) {
          bound_box(p, p->bs[fd], fd, fib, fie, fjb, fje, fkb, fke, is, type, 1);
        } else if (fd != d) {
          bound_box(p, p->bs[fd], fd, fib, fie, fjb, fje, fkb, fke, is, type,
                    flip_sign(d, type, BX1 + fd, p->c.components));
        }
      }
      /* outflow: the normal staggered component from div B = 0, then its
         cell average (Src/boundary.c:171-190) */
      if (type == OC_OUTFLOW) {
        fill_magnetic_field(p, is);
        ct_average_normal(p, is);
      } else if (type == OC_REFLECTIVE || type == OC_EQTSYMMETRIC) {
        fill_magnetic_field(p, is); /* no normal averaging here (boundary.c:192-207) */
      }
    }
  }
  p->bstage++;
}

/* ------------------------------------------------------------------ */
/* One directional sweep of UpdateStage, Src/Time_Stepping/update_stage.c  */
/* ------------------------------------------------------------------ */

typedef struct {
  double (*v)[NV], (*vp)[NV], (*vm)[NV], (*up)[NV], (*um)[NV], (*rhs)[NV];
  double *bn;
  Iface *ifc;
} Pencil;

static void pencil_alloc(Pencil *w, int n) {
  w->v = malloc(sizeof(double[NV]) * n);
  w->vp = malloc(sizeof(double[NV]) * n);
  w->vm = malloc(sizeof(double[NV]) * n);
  w->up = malloc(sizeof(double[NV]) * n);
  w->um = malloc(sizeof(double[NV]) * n);
  w->rhs = malloc(sizeof(double[NV]) * n);
  w->bn = malloc(sizeof(double) * n);
  w->ifc = malloc(sizeof(Iface) * n);
}
static void pencil_free(Pencil *w) {
  free(w->v); free(w->vp); free(w->vm); free(w->up); free(w->um);
  free(w->rhs); free(w->bn); free(w->ifc);
}

static void plm_char_states(double (*v)[NV], double (*vp)[NV], double (*vm)[NV], int beg, int end, int lim,
                            double gamma, const Rot *r, int c3, int dims);
static void ppm_char_states(double (*v)[NV], double (*vp)[NV], double (*vm)[NV], int beg, int end, double gamma,
                            const Rot *r, int c3, int dims);

/* face-EMF slots of eface[] */
enum { EZI = 0, EZJ, EYI, EYK, EXJ, EXK };

static void sweep(oc_problem *p, int dir, double dt, int stage, double *inv_dt_1d,
                  double *mach_out) {
  const int dims = p->c.dims;
  const int td = dir == 0 ? 1 : 0, bd = dir == 2 ? 1 : 2; /* rbox.c:52-80 */
  const Rot r = rot_for(dir);
  int nbeg = p->beg[dir], nend = p->end[dir];
  int tbeg = p->beg[td], tend = p->end[td], bbeg = p->beg[bd], bend = p->end[bd];
  int ntot = p->nt[dir];
  const double gmm1 = p->c.gamma - 1.0;
  const double inv_dl = p->inv_dx[dir];
  const double dxd = p->c.dx[dir];
  double mach_max = 0.0, invdt1 = 0.0;
  long npencil, ip;
  int tn, roe_bad = 0;

  if (p->c.ct) { /* update_stage.c:144-148 */
    if (dims >= 2) { tbeg--; tend++; }
    if (dims == 3) { bbeg--; bend++; }
  }
  tn = tend - tbeg + 1;
  npencil = (long)tn * (bend - bbeg + 1);

#pragma omp parallel reduction(max : mach_max, invdt1) reduction(| : roe_bad)
  {
    Pencil w;
    pencil_alloc(&w, ntot + 2);
#pragma omp for schedule(static)
    for (ip = 0; ip < npencil; ip++) {
      int t = tbeg + (int)(ip % tn), b = bbeg + (int)(ip / tn);
      int i, nv, ijk[3];
      ijk[td] = t;
      ijk[bd] = b;
      /* gather, update_stage.c:158-164 */
      for (i = 0; i < ntot; i++) {
        size_t c;
        ijk[dir] = i;
        c = CI(p, ijk[2], ijk[1], ijk[0]);
        for (nv = 0; nv < NV; nv++) w.v[i][nv] = p->vc[nv][c];
        if (p->c.ct) w.bn[i] = p->bs[dir][FI(p, dir, ijk[2], ijk[1], ijk[0])];
      }
      /* States, update_stage.c:193 with beg = nbeg-1, end = nend+1 */
      {
        int beg = nbeg - 1, end = nend + 1;
        if (p->c.recon == OC_LINEAR && p->c.char_limiting)
          plm_char_states(w.v, w.vp, w.vm, beg, end, p->c.limiter, p->c.gamma, &r, p->c.components == 3, dims);
        else if (p->c.char_limiting)
          ppm_char_states(w.v, w.vp, w.vm, beg, end, p->c.gamma, &r, p->c.components == 3, dims);
        else if (p->c.recon == OC_LINEAR) plm_states(w.v, w.vp, w.vm, beg, end, p->c.limiter);
        else ppm_states(w.v, w.vp, w.vm, beg, end);
        if (p->c.ct) { /* plm_states.c:271-275 */
          for (i = beg - 1; i <= end; i++) {
            w.vp[i][r.bn] = w.bn[i];
            w.vm[i + 1][r.bn] = w.bn[i];
          }
        }
        for (i = beg; i <= end; i++) {
          prim_to_cons(w.vp[i], w.up[i], gmm1);
          prim_to_cons(w.vm[i], w.um[i], gmm1);
        }
      }
      /* Riemann, update_stage.c:194 on interfaces nbeg-1..nend; interface
         i lies between cell i (vp) and cell i+1 (vm). */
      for (i = nbeg - 1; i <= nend; i++) {
        double m;
        if (p->c.solver == OC_HLL)
          hll_solver(w.vp[i], w.up[i], w.vm[i + 1], w.um[i + 1], p->c.gamma, &r, &w.ifc[i], &m);
        else if (p->c.solver == OC_ROE)
          roe_bad |= roe_solver(w.vp[i], w.up[i], w.vm[i + 1], w.um[i + 1], p->c.gamma,
                                p->c.components == 3, &r, &w.ifc[i], &m);
        else
          hlld_solver(w.vp[i], w.up[i], w.vm[i + 1], w.um[i + 1], p->c.gamma, &r, &w.ifc[i], &m);
        mach_max = MAX(m, mach_max);
      }
      /* CT_StoreUpwindEMF, ct_emf.c:104-207 (UCT_HLL) + CT_StoreVelSlopes */
      if (p->c.ct) {
        for (i = nbeg - 1; i <= nend; i++) {
          size_t c;
          ijk[dir] = i;
          c = CI(p, ijk[2], ijk[1], ijk[0]);
          p->sl[dir][c] = MAX(0.0, -w.ifc[i].SL);
          p->sr[dir][c] = MAX(0.0, w.ifc[i].SR);
          if (p->c.emf != OC_UCT_HLL) { /* the other averages: face EMFs and mass-flux signs */
            const double *F = w.ifc[i].f;
            if (dir == 0) {
              p->eface[EZI][c] = -F[BX2];
              if (dims == 3) p->eface[EYI][c] = F[BX3];
            } else if (dir == 1) {
              p->eface[EZJ][c] = F[BX1];
              if (dims == 3) p->eface[EXJ][c] = -F[BX3];
            } else {
              p->eface[EYK][c] = -F[BX1];
              p->eface[EXK][c] = F[BX2];
            }
            p->sv[dir][c] = F[RHO] > 1.e-6 ? 1 : (F[RHO] < -1.e-6 ? -1 : 0);
          }
        }
        for (i = nbeg - 1; i <= nend + 1; i++) {
          size_t c;
          int comp;
          ijk[dir] = i;
          c = CI(p, ijk[2], ijk[1], ijk[0]);
          for (comp = 0; comp < dims; comp++)
            p->dv[dir][comp][c] = w.vp[i][VX1 + comp] - w.vm[i][VX1 + comp];
        }
      }
      /* RightHandSide (Src/MHD/rhs.c:193-201, Cartesian, USE_PRS_GRADIENT) */
      for (i = nbeg; i <= nend; i++) {
        double scrh = dt / dxd;
        for (nv = 0; nv < NV; nv++)
          w.rhs[i][nv] = -scrh * (w.ifc[i].f[nv] - w.ifc[i - 1].f[nv]);
        w.rhs[i][r.vn] -= scrh * (w.ifc[i].press - w.ifc[i - 1].press);
      }
      /* U += rhs, update_stage.c:214-216; dt bookkeeping :229-241 */
      for (i = nbeg; i <= nend; i++) {
        size_t c;
        ijk[dir] = i;
        c = CI(p, ijk[2], ijk[1], ijk[0]);
        /* InternalBoundaryReset, Src/int_bound_reset.c:33-37 */
        if (p->internal && (p->flag[c] & FLAG_INTERNAL_BOUNDARY))
          for (nv = 0; nv < NV; nv++) w.rhs[i][nv] = 0.0;
        for (nv = 0; nv < NV; nv++) p->uc[nv][c] += w.rhs[i][nv];
        if (dims > 1 && stage == 1)
          p->cdt[c] += 0.5 * (w.ifc[i - 1].cmax + w.ifc[i].cmax) * inv_dl;
      }
      if (dims == 1)
        for (i = nbeg - 1; i <= nend; i++) invdt1 = MAX(invdt1, w.ifc[i].cmax * inv_dl);
    }
    pencil_free(&w);
  }
  if (*mach_out < mach_max) *mach_out = mach_max;
  if (roe_bad) p->roe_bad = 1;
  *inv_dt_1d = MAX(*inv_dt_1d, invdt1);
}

/* ------------------------------------------------------------------ */
/* Constrained transport                                                */
/* ------------------------------------------------------------------ */

/* Src/MHD/CT/ct_stag_slopes.c:92-105 */
static double mc_lim2(double dp, double dm) {
  double dc, scrh;
  if (dp * dm < 0.0) return 0.0;
  dc = 0.5 * (dp + dm);
  scrh = 2.0 * (fabs(dp) < fabs(dm) ? dp : dm);
  return (fabs(dc) < fabs(scrh) ? dc : scrh);
}

/* Staggered slope of face field fd along direction a at reference index
   (k,j,i): CT_GetStagSlopes, ct_stag_slopes.c:51-89. */
static double bslope(const oc_problem *p, int fd, int a, int k, int j, int i) {
  int o[3] = {0, 0, 0};
  double b0, bp, bm;
  o[a] = 1;
  b0 = p->bs[fd][FI(p, fd, k, j, i)];
  bp = p->bs[fd][FI(p, fd, k + o[2], j + o[1], i + o[0])];
  bm = p->bs[fd][FI(p, fd, k - o[2], j - o[1], i - o[0])];
  return mc_lim2(bp - b0, b0 - bm);
}

/* Edge EMF along axis e from the 2D HLL solver of Londrillo & Del Zanna:
   CT_EMF_HLL_Solver, Src/MHD/CT/ct_emf_average.c:179-352.  (x,y) is the
   ordered pair of in-plane axes: e = z -> (x,y); e = x -> (y,z);
   e = y -> (z,x). */
static double uct_hll_edge(const oc_problem *p, int e, int k, int j, int i) {
  const int ax = e == 2 ? 0 : (e == 0 ? 1 : 2);
  const int ay = e == 2 ? 1 : (e == 0 ? 2 : 0);
  int c[3] = {i, j, k}, cx[3], cy[3], cxy[3];
  double a_xp, a_xm, a_yp, a_ym, bS, bN, bW, bE, eSW, eSE, eNE, eNW, ez;
  double *vxa = p->vc[VX1 + ax], *vya = p->vc[VX1 + ay];
  size_t c00, cx0, c0y, cxy_;
  memcpy(cx, c, sizeof c); cx[ax]++;
  memcpy(cy, c, sizeof c); cy[ay]++;
  memcpy(cxy, c, sizeof c); cxy[ax]++; cxy[ay]++;
  c00 = CI(p, c[2], c[1], c[0]);
  cx0 = CI(p, cx[2], cx[1], cx[0]);
  c0y = CI(p, cy[2], cy[1], cy[0]);
  cxy_ = CI(p, cxy[2], cxy[1], cxy[0]);

  /* Speeds on faces normal to x (stored at cells c and c+y) and to y. */
  a_xp = MAX(p->sr[ax][c00], p->sr[ax][c0y]);
  a_xm = MAX(p->sl[ax][c00], p->sl[ax][c0y]);
  a_yp = MAX(p->sr[ay][c00], p->sr[ay][cx0]);
  a_ym = MAX(p->sl[ay][c00], p->sl[ay][cx0]);

  /* bS, bN: x-face field dP/dM along y; bW, bE: y-face field along x */
  bS = p->bs[ax][FI(p, ax, c[2], c[1], c[0])] + 0.5 * bslope(p, ax, ay, c[2], c[1], c[0]);
  bW = p->bs[ay][FI(p, ay, c[2], c[1], c[0])] + 0.5 * bslope(p, ay, ax, c[2], c[1], c[0]);
  bN = p->bs[ax][FI(p, ax, cy[2], cy[1], cy[0])] - 0.5 * bslope(p, ax, ay, cy[2], cy[1], cy[0]);
  bE = p->bs[ay][FI(p, ay, cx[2], cx[1], cx[0])] - 0.5 * bslope(p, ay, ax, cx[2], cx[1], cx[0]);

#define DV(comp, dir, cc) (p->dv[dir][comp][cc])
  /* dPP, dMP, dMM, dPM macros, ct_emf_average.c:198-213 */
  eSW = (vya[c00] + 0.5 * (DV(ay, ax, c00) + DV(ay, ay, c00))) * bS -
        (vxa[c00] + 0.5 * (DV(ax, ax, c00) + DV(ax, ay, c00))) * bW;
  eSE = (vya[cx0] - 0.5 * (DV(ay, ax, cx0) - DV(ay, ay, cx0))) * bS -
        (vxa[cx0] - 0.5 * (DV(ax, ax, cx0) - DV(ax, ay, cx0))) * bE;
  eNE = (vya[cxy_] - 0.5 * (DV(ay, ax, cxy_) + DV(ay, ay, cxy_))) * bN -
        (vxa[cxy_] - 0.5 * (DV(ax, ax, cxy_) + DV(ax, ay, cxy_))) * bE;
  eNW = (vya[c0y] + 0.5 * (DV(ay, ax, c0y) - DV(ay, ay, c0y))) * bN -
        (vxa[c0y] + 0.5 * (DV(ax, ax, c0y) - DV(ax, ay, c0y))) * bW;
#undef DV
  ez = a_xp * a_yp * eSW + a_xm * a_yp * eSE + a_xm * a_ym * eNE + a_xp * a_ym * eNW;
  ez /= (a_xp + a_xm) * (a_yp + a_ym);
  ez -= a_yp * a_ym * (bN - bS) / (a_yp + a_ym);
  ez += a_xp * a_xm * (bE - bW) / (a_xp + a_xm);
  return ez;
}

/* CT_ComputeEMF (UCT_HLL): edges over the emf ranges set by the sweeps,
   ct_emf.c:130-131 etc.: i in [IBEG-1, IEND], likewise j, k. */
static void compute_emf(oc_problem *p) {
  const int dims = p->c.dims;
  int kb = dims == 3 ? p->beg[2] - 1 : 0, ke = dims == 3 ? p->end[2] : 0;
  int jb = p->beg[1] - 1, je = p->end[1];
  int ib = p->beg[0] - 1, ie = p->end[0];
  long nj = je - jb + 1, ni = ie - ib + 1, n = (long)(ke - kb + 1) * nj * ni, q;
#pragma omp parallel for schedule(static)
  for (q = 0; q < n; q++) {
    int i = ib + (int)(q % ni), j = jb + (int)((q / ni) % nj), k = kb + (int)(q / (ni * nj));
    size_t c = CI(p, k, j, i);
    p->ez[c] = uct_hll_edge(p, 2, k, j, i);
    if (dims == 3) {
      p->ex[c] = uct_hll_edge(p, 0, k, j, i);
      p->ey[c] = uct_hll_edge(p, 1, k, j, i);
    }
  }
}

/* CT_Update, Src/MHD/CT/ct_update.c:29-220 (Cartesian). */
static void ct_update(oc_problem *p, double dt) {
  const int dims = p->c.dims;
  const int KO = dims == 3;
  int kb = dims == 3 ? p->beg[2] - 1 : 0, ke = dims == 3 ? p->end[2] : 0;
  int jb = p->beg[1] - 1, je = p->end[1];
  int ib = p->beg[0] - 1, ie = p->end[0];
  double dx1 = p->c.dx[0], dx2 = p->c.dx[1], dx3 = p->c.dx[2];
  int i, j, k;
  for (k = kb + KO; k <= ke; k++)
    for (j = jb + 1; j <= je; j++)
      for (i = ib; i <= ie; i++) {
        double rhs_x;
        if (dims == 2)
          rhs_x = 0.0 - dt / dx2 * (p->ez[CI(p, k, j, i)] - p->ez[CI(p, k, j - 1, i)]);
        else
          rhs_x = 0.0 - dt / dx2 * (p->ez[CI(p, k, j, i)] - p->ez[CI(p, k, j - 1, i)]) +
                  dt / dx3 * (p->ey[CI(p, k, j, i)] - p->ey[CI(p, k - 1, j, i)]);
        p->bs[0][FI(p, 0, k, j, i)] = p->bs[0][FI(p, 0, k, j, i)] + rhs_x;
      }
  for (k = kb + KO; k <= ke; k++)
    for (j = jb; j <= je; j++)
      for (i = ib + 1; i <= ie; i++) {
        double rhs_y;
        if (dims == 2)
          rhs_y = dt / dx1 * (p->ez[CI(p, k, j, i)] - p->ez[CI(p, k, j, i - 1)]);
        else
          rhs_y = dt / dx1 * (p->ez[CI(p, k, j, i)] - p->ez[CI(p, k, j, i - 1)]) -
                  dt / dx3 * (p->ex[CI(p, k, j, i)] - p->ex[CI(p, k - 1, j, i)]);
        p->bs[1][FI(p, 1, k, j, i)] = p->bs[1][FI(p, 1, k, j, i)] + rhs_y;
      }
  if (dims == 3)
    for (k = kb; k <= ke; k++)
      for (j = jb + 1; j <= je; j++)
        for (i = ib + 1; i <= ie; i++) {
          double rhs_z = -dt / dx1 * (p->ey[CI(p, k, j, i)] - p->ey[CI(p, k, j, i - 1)]) +
                         dt / dx2 * (p->ex[CI(p, k, j, i)] - p->ex[CI(p, k, j - 1, i)]);
          p->bs[2][FI(p, 2, k, j, i)] = p->bs[2][FI(p, 2, k, j, i)] + rhs_z;
        }
}

/* CT_AverageMagneticField, Src/MHD/CT/ct_field_average.c:13-132 (Cartesian,
   CT_EN_CORRECTION NO): domain plus one ghost layer. */
static void ct_average(oc_problem *p) {
  const int dims = p->c.dims;
  int ko = dims == 3, d, i, j, k;
  for (k = p->beg[2] - ko; k <= p->end[2] + ko; k++)
    for (j = p->beg[1] - 1; j <= p->end[1] + 1; j++)
      for (i = p->beg[0] - 1; i <= p->end[0] + 1; i++) {
        size_t c = CI(p, k, j, i);
        for (d = 0; d < dims; d++) {
          int o[3] = {0, 0, 0};
          o[d] = 1;
          p->uc[BX1 + d][c] = 0.5 * (p->bs[d][FI(p, d, k, j, i)] +
                                     p->bs[d][FI(p, d, k - o[2], j - o[1], i - o[0])]);
        }
      }
}

/* ------------------------------------------------------------------ */
/* Stage driver                                                         */
/* ------------------------------------------------------------------ */

#define DOM_LOOP(p, k, j, i)                          \
  for (k = (p)->beg[2]; k <= (p)->end[2]; k++)         \
    for (j = (p)->beg[1]; j <= (p)->end[1]; j++)       \
      for (i = (p)->beg[0]; i <= (p)->end[0]; i++)

static void cons_to_prim_3d(oc_problem *p) {
  const double gmm1 = p->c.gamma - 1.0;
  int64_t nf = 0;
  long nk = p->end[2] - p->beg[2] + 1, nj = p->end[1] - p->beg[1] + 1;
  long ni = p->end[0] - p->beg[0] + 1, n = nk * nj * ni, q;
#pragma omp parallel for schedule(static) reduction(+ : nf)
  for (q = 0; q < n; q++) {
    int i = p->beg[0] + (int)(q % ni), j = p->beg[1] + (int)((q / ni) % nj);
    int k = p->beg[2] + (int)(q / (ni * nj));
    size_t c = CI(p, k, j, i);
    double u[NV], v[NV];
    int nv;
    for (nv = 0; nv < NV; nv++) u[nv] = p->uc[nv][c];
    nf += cons_to_prim(u, v, gmm1, &p->flag[c]);
    for (nv = 0; nv < NV; nv++) { p->uc[nv][c] = u[nv]; p->vc[nv][c] = v[nv]; }
  }
  p->nfail += nf;
}

static void ctu_compute_emf(oc_problem *p, int stage);

/* UpdateStage, update_stage.c:37-314 */
static void update_stage(oc_problem *p, double dt, int stage, double *inv_dt,
                         double *inv_dt_1d) {
  int dir;
  if (p->c.dims > 1 && stage == 1) memset(p->cdt, 0, p->ncell * sizeof(double));
  for (dir = 0; dir < p->c.dims; dir++) sweep(p, dir, dt, stage, inv_dt_1d, &p->max_mach);
  if (p->c.ct) {
    if (p->c.emf == OC_UCT_HLL) {
      compute_emf(p);
    } else { /* edges over i in [IBEG-1, IEND] etc. (ct_emf.c:130-131) */
      int d;
      for (d = 0; d < 3; d++) {
        p->emf_lo[d] = d < p->c.dims ? p->beg[d] - 1 : 0;
        p->emf_hi[d] = d < p->c.dims ? p->end[d] : 0;
      }
      ctu_compute_emf(p, 2);
    }
    ct_update(p, dt);
  }
  if (p->c.dims > 1 && stage == 1) { /* :308-312 */
    int i, j, k;
    double m = *inv_dt;
    DOM_LOOP(p, k, j, i) m = MAX(m, p->cdt[CI(p, k, j, i)]);
    m /= (double)p->c.dims;
    *inv_dt = m;
  }
}


/* ------------------------------------------------------------------ */
/* Corner Transport Upwind (TIME_STEPPING HANCOCK), ctu_step.c:140-727  */
/* ------------------------------------------------------------------ */

/* PrimRHS, Src/MHD/prim_eqn.c:29-112 (ideal EOS, no 8-wave / GLM terms) */
static void prim_rhs(const double *v, const double *dv, double gamma, const Rot *r, int c3,
                     double *Adv) {
  const int vn = r->vn, vt = r->vt, vb = r->vb, bn = r->bn, bt = r->bt, bb = r->bb;
  double tau = 1.0 / v[RHO], scrh;
  int nv;
  for (nv = 0; nv < NV; nv++) Adv[nv] = 0.0;
  Adv[RHO] = v[vn] * dv[RHO] + v[RHO] * dv[vn];
  scrh = c3 ? 0.0 + v[bt] * dv[bt] + v[bb] * dv[bb] : 0.0 + v[bt] * dv[bt];
  Adv[vn] = v[vn] * dv[vn] + tau * (dv[PRS] + scrh);
  Adv[vt] = v[vn] * dv[vt] - tau * v[bn] * dv[bt];
  if (c3) Adv[vb] = v[vn] * dv[vb] - tau * v[bn] * dv[bb];
  Adv[bn] = 0.0;
  Adv[bt] = v[bt] * dv[vn] - v[bn] * dv[vt] + v[vn] * dv[bt];
  if (c3) Adv[bb] = v[bb] * dv[vn] - v[bn] * dv[vb] + v[vn] * dv[bb];
  Adv[PRS] = gamma * v[PRS] * dv[vn] + v[vn] * dv[PRS];
}


/* PrimEigenvectors, Src/MHD/eigenv.c:190-688: primitive eigenvalues and
   eigenvectors of ideal MHD along the sweep (no 8-wave / GLM terms: the div-B
   wave has lambda 0 and no vectors).  Waves in the order of
   Src/MHD/mod_defs.h:54-71; L[wave][slot], R[slot][wave] over this file's 8
   variable slots; entries not set stay zero.  dims: DIMENSIONS (the 2D
   Alfven hot fix, eigenv.c:528-531). */
enum { WFM = 0, WFP, WEN, WDB, WSM, WSP, WAM, WAP };
static void prim_eigen(const double *q, double a2, const Rot *r, int c3, int dims, double L[8][8],
                       double R[8][8], double *lambda) {
  const int vn = r->vn, vt = r->vt, vb = r->vb, bn = r->bn, bt = r->bt, bb = r->bb;
  const double sqrt_1_2 = 0.70710678118654752440;
  double u, tau, sqrt_rho, scrh0, scrh1, scrh2, scrh3, scrh4, b2, ca2, A2, At2, cf2, cs2, cf, cs, ca, a;
  double alpha_f, alpha_s, beta_y, beta_z = 0.0, S;
  int k;
  memset(L, 0, sizeof(double[8][8]));
  memset(R, 0, sizeof(double[8][8]));
  u = q[vn];
  tau = 1.0 / q[RHO];
  sqrt_rho = sqrt(q[RHO]);
  scrh2 = q[bn] * q[bn];
  scrh3 = c3 ? 0.0 + q[bt] * q[bt] + q[bb] * q[bb] : 0.0 + q[bt] * q[bt];
  b2 = scrh2 + scrh3;
  ca2 = scrh2 * tau;
  A2 = b2 * tau;
  At2 = scrh3 * tau;
  scrh1 = a2 - A2;
  scrh0 = sqrt(scrh1 * scrh1 + 4.0 * a2 * At2);
  cf2 = 0.5 * (a2 + A2 + scrh0);
  cs2 = a2 * ca2 / cf2;
  cf = sqrt(cf2);
  cs = sqrt(cs2);
  ca = sqrt(ca2);
  a = sqrt(a2);
  if (cf == cs) {
    alpha_f = 1.0;
    alpha_s = 0.0;
  } else {
    scrh0 = 1.0 / scrh0;
    alpha_f = (a2 - cs2) * scrh0;
    alpha_s = (cf2 - a2) * scrh0;
    alpha_f = MAX(0.0, alpha_f);
    alpha_s = MAX(0.0, alpha_s);
    alpha_f = sqrt(alpha_f);
    alpha_s = sqrt(alpha_s);
  }
  scrh0 = sqrt(scrh3);
  if (scrh0 > 1.e-9) {
    if (c3) {
      beta_y = q[bt] / scrh0;
      beta_z = q[bb] / scrh0;
    } else {
      beta_y = (q[bt] >= 0.0 ? 1.0 : -1.0);
    }
  } else {
    if (c3) beta_z = beta_y = sqrt_1_2;
    else beta_y = 1.0;
  }
  S = (q[bn] >= 0.0 ? 1.0 : -1.0);

  k = WFM; /* fast wave, u - c_f */
  lambda[k] = u - cf;
  scrh0 = alpha_s * cs * S;
  scrh1 = alpha_s * sqrt_rho * a;
  scrh2 = 0.5 / a2;
  scrh3 = scrh2 * tau;
  R[RHO][k] = q[RHO] * alpha_f;
  R[vn][k] = -cf * alpha_f;
  R[vt][k] = scrh0 * beta_y;
  if (c3) R[vb][k] = scrh0 * beta_z;
  R[bt][k] = scrh1 * beta_y;
  if (c3) R[bb][k] = scrh1 * beta_z;
  scrh4 = alpha_f * a2 * q[RHO];
  R[PRS][k] = scrh4;
  L[k][vn] = R[vn][k] * scrh2;
  L[k][vt] = R[vt][k] * scrh2;
  if (c3) L[k][vb] = R[vb][k] * scrh2;
  L[k][bt] = R[bt][k] * scrh3;
  if (c3) L[k][bb] = R[bb][k] * scrh3;
  L[k][PRS] = alpha_f * scrh3;

  k = WFP; /* fast wave, u + c_f */
  lambda[k] = u + cf;
  R[RHO][k] = R[RHO][WFM];
  R[vn][k] = -R[vn][WFM];
  R[vt][k] = -R[vt][WFM];
  if (c3) R[vb][k] = -R[vb][WFM];
  R[bt][k] = R[bt][WFM];
  if (c3) R[bb][k] = R[bb][WFM];
  R[PRS][k] = R[PRS][WFM];
  L[k][vn] = -L[WFM][vn];
  L[k][vt] = -L[WFM][vt];
  if (c3) L[k][vb] = -L[WFM][vb];
  L[k][bt] = L[WFM][bt];
  if (c3) L[k][bb] = L[WFM][bb];
  L[k][PRS] = L[WFM][PRS];

  k = WEN; /* entropy wave, u */
  lambda[k] = u;
  R[RHO][k] = 1.0;
  L[k][RHO] = 1.0;
  L[k][PRS] = -1.0 / a2;

  lambda[WDB] = 0.0; /* div-B wave (no 8-wave control) */

  k = WSM; /* slow wave, u - c_s */
  lambda[k] = u - cs;
  scrh0 = alpha_f * cf * S;
  scrh1 = alpha_f * sqrt_rho * a;
  R[RHO][k] = q[RHO] * alpha_s;
  R[vn][k] = -cs * alpha_s;
  R[vt][k] = -scrh0 * beta_y;
  if (c3) R[vb][k] = -scrh0 * beta_z;
  R[bt][k] = -scrh1 * beta_y;
  if (c3) R[bb][k] = -scrh1 * beta_z;
  scrh4 = alpha_s * a2 * q[RHO];
  R[PRS][k] = scrh4;
  L[k][vn] = R[vn][k] * scrh2;
  L[k][vt] = R[vt][k] * scrh2;
  if (c3) L[k][vb] = R[vb][k] * scrh2;
  L[k][bt] = R[bt][k] * scrh3;
  if (c3) L[k][bb] = R[bb][k] * scrh3;
  L[k][PRS] = alpha_s * scrh3;

  k = WSP; /* slow wave, u + c_s */
  lambda[k] = u + cs;
  R[RHO][k] = R[RHO][WSM];
  R[vn][k] = -R[vn][WSM];
  R[vt][k] = -R[vt][WSM];
  if (c3) R[vb][k] = -R[vb][WSM];
  R[bt][k] = R[bt][WSM];
  if (c3) R[bb][k] = R[bb][WSM];
  R[PRS][k] = scrh4;
  L[k][vn] = -L[WSM][vn];
  L[k][vt] = -L[WSM][vt];
  if (c3) L[k][vb] = -L[WSM][vb];
  L[k][bt] = L[WSM][bt];
  if (c3) L[k][bb] = L[WSM][bb];
  L[k][PRS] = L[WSM][PRS];

  if (c3) {
    k = WAM; /* Alfven wave, u - c_a */
    lambda[k] = u - ca;
    scrh2 = beta_y * sqrt_1_2;
    scrh3 = beta_z * sqrt_1_2;
    R[vt][k] = -scrh3;
    R[vb][k] = scrh2;
    R[bt][k] = -scrh3 * sqrt_rho * S;
    R[bb][k] = scrh2 * sqrt_rho * S;
    L[k][vt] = R[vt][k];
    L[k][vb] = R[vb][k];
    L[k][bt] = R[bt][k] * tau;
    L[k][bb] = R[bb][k] * tau;

    k = WAP; /* Alfven wave, u + c_a */
    lambda[k] = u + ca;
    R[vt][k] = R[vt][WAM];
    R[vb][k] = R[vb][WAM];
    R[bt][k] = -R[bt][WAM];
    R[bb][k] = -R[bb][WAM];
    L[k][vt] = L[WAM][vt];
    L[k][vb] = L[WAM][vb];
    L[k][bt] = -L[WAM][bt];
    L[k][bb] = -L[WAM][bb];
    if (dims <= 2 && q[bn] == 0 && q[bt] == 0.0)
      for (k = 0; k < 8; k++) R[bt][k] = 0.0;
  }
}

/* PrimToChar, Src/MHD/eigenv.c:1310-1380: w = L . v from the nonzero entries */
static void prim_to_char(double L[8][8], const double *v, const Rot *r, int c3, double *w) {
  const int vn = r->vn, vt = r->vt, vb = r->vb, bt = r->bt, bb = r->bb;
  const double *l = L[WFM];
  double wv, wB;
  wv = c3 ? l[vn] * v[vn] + l[vt] * v[vt] + l[vb] * v[vb] : l[vn] * v[vn] + l[vt] * v[vt];
  wB = c3 ? l[PRS] * v[PRS] + l[bt] * v[bt] + l[bb] * v[bb] : l[PRS] * v[PRS] + l[bt] * v[bt];
  w[WFM] = wv + wB;
  w[WFP] = -wv + wB;
  l = L[WEN];
  w[WEN] = l[RHO] * v[RHO] + l[PRS] * v[PRS];
  w[WDB] = 0.0;
  l = L[WSM];
  wv = c3 ? l[vn] * v[vn] + l[vt] * v[vt] + l[vb] * v[vb] : l[vn] * v[vn] + l[vt] * v[vt];
  wB = c3 ? l[PRS] * v[PRS] + l[bt] * v[bt] + l[bb] * v[bb] : l[PRS] * v[PRS] + l[bt] * v[bt];
  w[WSM] = wv + wB;
  w[WSP] = -wv + wB;
  if (c3) {
    l = L[WAM];
    wv = l[vt] * v[vt] + l[vb] * v[vb];
    wB = l[bt] * v[bt] + l[bb] * v[bb];
    w[WAM] = wv + wB;
    w[WAP] = wv - wB;
  }
}

/* CharTracingStep, Src/States/char_tracing.c:280-573 (LINEAR reconstruction,
   CHTR_REF_STATE 3, Cartesian, no passive scalars; PrimSource is zero for
   ideal Cartesian MHD without body forces, prim_eqn.c:202, and is still
   added as +0).  vc: cell-centre state; vp, vm: its PLM states, updated in
   place.  Variables of COMPONENTS 2 problems skip the third component slots. */
static void char_tracing(const double *vc, double *vp, double *vm, double gamma, double dtdx, double dt,
                         const Rot *r, int c3, int dims) {
  double L[8][8], R[8][8], lambda[8], nu[8], dv[NV], dw[8], nu_max, nu_min;
  const int nflx = c3 ? 8 : 6;
  const double a2 = gamma * vc[PRS] / vc[RHO]; /* SoundSpeed2, Src/EOS/Ideal/eos.c:22 */
  const double src = 0.0;
  int k, nv;
  prim_eigen(vc, a2, r, c3, dims, L, R, lambda);
  for (k = 0; k < nflx; k++) nu[k] = dtdx * lambda[k];
  nu_max = MAX(nu[1], 0.0);
  nu_min = MIN(nu[0], 0.0);
  for (nv = NV; nv--;) dv[nv] = vp[nv] - vm[nv];
  prim_to_char(L, dv, r, c3, dw);
  for (nv = NV; nv--;) {
    if (!c3 && (nv == VX3 || nv == BX3)) continue;
    vp[nv] = vc[nv] + 0.5 * dv[nv] * (1.0 - nu_max);
    vm[nv] = vc[nv] - 0.5 * dv[nv] * (1.0 + nu_min);
  }
  for (k = 0; k < nflx; k++) {
    if (nu[k] >= 0.0) {
      dw[k] *= 0.5 * (nu_max - nu[k]);
      for (nv = 0; nv < NV; nv++)
        if (c3 || (nv != VX3 && nv != BX3)) vp[nv] += dw[k] * R[nv][k];
    } else {
      dw[k] *= 0.5 * (nu_min - nu[k]);
      for (nv = 0; nv < NV; nv++)
        if (c3 || (nv != VX3 && nv != BX3)) vm[nv] += dw[k] * R[nv][k];
    }
  }
  for (nv = NV; nv--;) {
    if (!c3 && (nv == VX3 || nv == BX3)) continue;
    vp[nv] += 0.5 * dt * src;
    vm[nv] += 0.5 * dt * src;
  }
}


/* States with CHAR_LIMITING YES, Src/States/plm_states.c:446-705 (uniform
   Cartesian grid: cp = cm = 2, dp = dm = 0.5): per cell the undivided
   differences projected on the left eigenvectors of PrimEigenvectors, limited
   per characteristic family (LIMITER DEFAULT: the generalised minmod with
   steepness kstp 1 for fast and slow waves, 2 otherwise), projected back on
   the right eigenvectors and clipped by MINMOD against twice the primitive
   differences. */
static void plm_char_states(double (*v)[NV], double (*vp)[NV], double (*vm)[NV], int beg, int end, int lim,
                            double gamma, const Rot *r, int c3, int dims) {
  const int nflx = c3 ? 8 : 6;
  int i, k, nv;
  for (i = beg; i <= end; i++) {
    double L[8][8], R[8][8], lambda[8], dvp[NV], dvm[NV], dwp[8], dwm[8], dwl[8];
    const double a2 = gamma * v[i][PRS] / v[i][RHO]; /* SoundSpeed2 */
    prim_eigen(v[i], a2, r, c3, dims, L, R, lambda);
    for (nv = 0; nv < NV; nv++) {
      dvp[nv] = v[i + 1][nv] - v[i][nv];
      dvm[nv] = v[i][nv] - v[i - 1][nv];
    }
    prim_to_char(L, dvm, r, c3, dwm);
    prim_to_char(L, dvp, r, c3, dwp);
    for (k = nflx; k--;) {
      if (lim == OC_DEFAULT_LIM) { /* SET_GM_LIMITER, plm_coeffs.h:96-100 */
        const double ck = (k == WFM || k == WFP || k == WSM || k == WSP) ? 1.0 : 2.0;
        if (dwp[k] * dwm[k] > 0.0) {
          double qc = 0.5 * (dwm[k] + dwp[k]), scrh = ABS_MIN(dwp[k] * ck, dwm[k] * ck);
          dwl[k] = ABS_MIN(qc, scrh);
        } else dwl[k] = 0.0;
      } else {
        dwl[k] = limit(lim, -1, dwp[k], dwm[k]);
      }
    }
    for (nv = NV; nv--;) {
      double dc = 0.0, dvl;
      if (!c3 && (nv == VX3 || nv == BX3)) {
        vp[i][nv] = vm[i][nv] = v[i][nv];
        continue;
      }
      for (k = 0; k < nflx; k++) dc += dwl[k] * R[nv][k];
      if (dvp[nv] * dvm[nv] > 0.0) {
        double d2v = ABS_MIN(2.0 * dvp[nv], 2.0 * dvm[nv]);
        dvl = MINMOD(d2v, dc);
      } else dvl = 0.0;
      vp[i][nv] = v[i][nv] + dvl * 0.5;
      vm[i][nv] = v[i][nv] - dvl * 0.5;
    }
  }
}


/* CharTracingStep for parabolic states, Src/States/char_tracing.c:46-279
   (CHTR_REF_STATE 3 without CHAR_LIMITING, uniform Cartesian grid, no passive
   scalars): the PPM reference state of the fastest wave towards each
   interface, then each family's parabola integrated over its domain of
   dependence added on the side it reaches; PrimSource zero (+0). */
static void char_tracing_ppm(const double *vc, double *vp, double *vm, double gamma, double dtdx, double dt,
                             const Rot *r, int c3, int dims, int ref_state) {
  double L[8][8], R[8][8], lambda[8], nu[8], dvp[NV], dvm[NV], dwp[8], dwm[8], nup, num, dwh, d2w;
  const int nflx = c3 ? 8 : 6;
  const double a2 = gamma * vc[PRS] / vc[RHO];
  const double src = 0.0;
  int k, nv;
  prim_eigen(vc, a2, r, c3, dims, L, R, lambda);
  for (k = 0; k < nflx; k++) nu[k] = dtdx * lambda[k];
  for (nv = NV; nv--;) {
    dvp[nv] = vp[nv] - vc[nv];
    dvm[nv] = vm[nv] - vc[nv];
  }
  prim_to_char(L, dvp, r, c3, dwp);
  prim_to_char(L, dvm, r, c3, dwm);
  nup = MAX(nu[1], 0.0);
  num = MIN(nu[0], 0.0);
  for (nv = NV; nv--;) {
    if (ref_state != 3 || (!c3 && (nv == VX3 || nv == BX3))) continue;
    dwh = vp[nv] - vm[nv];
    d2w = vp[nv] + vm[nv] - 2.0 * vc[nv];
    vp[nv] -= 0.5 * nup * (dwh + d2w * (3.0 - 2.0 * nup));
    vm[nv] -= 0.5 * num * (dwh - d2w * (3.0 + 2.0 * num));
  }
  for (k = 0; k < nflx; k++) {
    dwh = dwp[k] - dwm[k];
    d2w = dwp[k] + dwm[k];
    if (nu[k] >= 0.0) {
      double Spp = ref_state == 3 ? -0.5 * (nu[k] - nup) * (dwh + 3.0 * d2w) + (nu[k] * nu[k] - nup * nup) * d2w
                                  : -0.5 * nu[k] * (dwh + d2w * (3.0 - 2.0 * nu[k]));
      for (nv = NV; nv--;)
        if (c3 || (nv != VX3 && nv != BX3)) vp[nv] += Spp * R[nv][k];
    } else {
      double Smm = ref_state == 3 ? -0.5 * (nu[k] - num) * (dwh - 3.0 * d2w) + (nu[k] * nu[k] - num * num) * d2w
                                  : -0.5 * nu[k] * (dwh - d2w * (3.0 + 2.0 * nu[k]));
      for (nv = NV; nv--;)
        if (c3 || (nv != VX3 && nv != BX3)) vm[nv] += Smm * R[nv][k];
    }
  }
  for (nv = NV; nv--;) {
    if (!c3 && (nv == VX3 || nv == BX3)) continue;
    dwh = 0.5 * dt * src;
    vp[nv] += dwh;
    vm[nv] += dwh;
  }
}


/* States with RECONSTRUCTION PARABOLIC and CHAR_LIMITING YES,
   Src/States/ppm_states.c:258-560 (PPM_ORDER 4, PARABOLIC_LIM 1, uniform
   Cartesian coefficients: hp = hm = 3, so cp = cm = 2): the unlimited
   fourth-order interface values projected on the left eigenvectors and
   clipped by MINMOD against the projected neighbour differences, summed back
   over the right eigenvectors, the parabolic limiter on the primitive
   increments, and linear density / pressure where a state came out negative. */
static void ppm_char_states(double (*v)[NV], double (*vp)[NV], double (*vm)[NV], int beg, int end, double gamma,
                            const Rot *r, int c3, int dims) {
  const double w_1 = -1.0 / 12.0, w0 = 7.0 / 12.0, w1 = 7.0 / 12.0, w2 = -1.0 / 12.0;
  const double hp = 3.0, hm = 3.0;
  const int nflx = c3 ? 8 : 6;
  int i, k, nv;
  for (i = beg; i <= end; i++) {
    double L[8][8], R[8][8], lambda[8], dvp[NV], dvm[NV], dvF0[NV], dvF1[NV];
    double dwp[8], dwm[8], dwp1[8], dwm1[8], cp, cm;
    const double a2 = gamma * v[i][PRS] / v[i][RHO]; /* SoundSpeed2 */
    prim_eigen(v[i], a2, r, c3, dims, L, R, lambda);
    for (nv = 0; nv < NV; nv++) {
      double ip = w_1 * v[i - 1][nv] + w0 * v[i][nv] + w1 * v[i + 1][nv] + w2 * v[i + 2][nv];
      double im = w_1 * v[i - 2][nv] + w0 * v[i - 1][nv] + w1 * v[i][nv] + w2 * v[i + 1][nv];
      dvp[nv] = ip - v[i][nv];
      dvm[nv] = im - v[i][nv];
      dvF1[nv] = v[i + 1][nv] - v[i][nv];
      dvF0[nv] = v[i][nv] - v[i - 1][nv];
    }
    prim_to_char(L, dvp, r, c3, dwp);
    prim_to_char(L, dvm, r, c3, dwm);
    prim_to_char(L, dvF0, r, c3, dwm1);
    prim_to_char(L, dvF1, r, c3, dwp1);
    for (k = 0; k < nflx; k++) {
      dwp[k] = MINMOD(dwp[k], dwp1[k]);
      dwm[k] = MINMOD(dwm[k], -dwm1[k]);
    }
    cm = (hm + 1.0) / (hp - 1.0);
    cp = (hp + 1.0) / (hm - 1.0);
    for (nv = 0; nv < NV; nv++) {
      double dp = 0.0, dm = 0.0;
      if (!c3 && (nv == VX3 || nv == BX3)) {
        vp[i][nv] = vm[i][nv] = v[i][nv];
        continue;
      }
      for (k = 0; k < nflx; k++) {
        dp += dwp[k] * R[nv][k];
        dm += dwm[k] * R[nv][k];
      }
      if (dp * dm >= 0.0) dp = dm = 0.0;
      else {
        if (fabs(dp) >= cm * fabs(dm)) dp = -cm * dm;
        else if (fabs(dm) >= cp * fabs(dp)) dm = -cp * dp;
      }
      vp[i][nv] = v[i][nv] + dp;
      vm[i][nv] = v[i][nv] + dm;
    }
    if (vp[i][RHO] < 0.0 || vm[i][RHO] < 0.0) {
      double d = 0.5 * (MINMOD(dvF1[RHO], dvF0[RHO]));
      vp[i][RHO] = v[i][RHO] + d;
      vm[i][RHO] = v[i][RHO] + (-d);
    }
    if (vp[i][PRS] < 0.0 || vm[i][PRS] < 0.0) {
      double d = 0.5 * (MINMOD(dvF1[PRS], dvF0[PRS]));
      vp[i][PRS] = v[i][PRS] + d;
      vm[i][PRS] = v[i][PRS] + (-d);
    }
  }
}

/* face-EMF slot of (dir, component): ezi, ezj, eyi, eyk, exj, exk */

/* One CTU sweep.  stage 1: normal predictors (PLM + primitive Hancock,
   hancock.c:36-172, CheckPrimStates check_states.c:18-70), Riemann
   problems, rhs with dt/2 and CTU_CT_Source (ctu_step.c:731-816), stored in
   up_s/um_s/rhs_s (ctu_step.c:286-450).  stage 2: corner-coupled states
   U +- + sum of the other directions' rhs, face normal field, ConsToPrim,
   Riemann problems and U += rhs with dt (ctu_step.c:533-645). */
static void ctu_sweep(oc_problem *p, int dir, double dt, int stage, double *inv_dt) {
  const int dims = p->c.dims, ct = p->c.ct, c3 = p->c.components == 3;
  const int td = dir == 0 ? 1 : 0, bd = dir == 2 ? 1 : 2;
  const Rot r = rot_for(dir);
  int nbeg = p->beg[dir], nend = p->end[dir];
  int tbeg = p->beg[td], tend = p->end[td], bbeg = p->beg[bd], bend = p->end[bd];
  const int ntot = p->nt[dir];
  const double gmm1 = p->c.gamma - 1.0, inv_dl = p->inv_dx[dir], dxd = p->c.dx[dir];
  const double dt2 = 0.5 * dt;
  double invdt = *inv_dt;
  long npencil, ip;
  int tn;
  if (stage == 1) {
    if (dims >= 2) { tbeg--; tend++; }
    if (dims == 3) { bbeg--; bend++; }
    if (ct) {
      nbeg--; nend++;
      if (dims >= 2) { tbeg--; tend++; }
      if (dims == 3) { bbeg--; bend++; }
    }
  } else if (ct) {
    if (dims >= 2) { tbeg--; tend++; }
    if (dims == 3) { bbeg--; bend++; }
  }
  if (ct) { p->emf_lo[dir] = nbeg - 1; p->emf_hi[dir] = nend; }
  tn = tend - tbeg + 1;
  npencil = (long)tn * (bend - bbeg + 1);

#pragma omp parallel reduction(max : invdt)
  {
    Pencil w;
    double (*vn)[NV] = malloc(sizeof(double[NV]) * (ntot + 2));
    pencil_alloc(&w, ntot + 2);
#pragma omp for schedule(static)
    for (ip = 0; ip < npencil; ip++) {
      int t = tbeg + (int)(ip % tn), b = bbeg + (int)(ip / tn);
      int i, nv, ijk[3];
      ijk[td] = t;
      ijk[bd] = b;
      for (i = 0; i < ntot; i++) {
        size_t c;
        ijk[dir] = i;
        c = CI(p, ijk[2], ijk[1], ijk[0]);
        for (nv = 0; nv < NV; nv++) w.v[i][nv] = vn[i][nv] = p->vc[nv][c];
        if (ct) w.bn[i] = p->bs[dir][FI(p, dir, ijk[2], ijk[1], ijk[0])];
      }
      if (stage == 1) {
        if (p->c.recon == OC_PARABOLIC && p->c.char_limiting)
          ppm_char_states(w.v, w.vp, w.vm, nbeg - 1, nend + 1, p->c.gamma, &r, c3, dims);
        else if (p->c.recon == OC_PARABOLIC)
          ppm_states(w.v, w.vp, w.vm, nbeg - 1, nend + 1);
        else if (p->c.char_limiting)
          plm_char_states(w.v, w.vp, w.vm, nbeg - 1, nend + 1, p->c.limiter, p->c.gamma, &r, c3, dims);
        else
          plm_states(w.v, w.vp, w.vm, nbeg - 1, nend + 1, p->c.limiter);
        if (ct)
          for (i = nbeg - 2; i <= nend + 1; i++) {
            w.vp[i][r.bn] = w.bn[i];
            w.vm[i + 1][r.bn] = w.bn[i];
          }
        if (p->c.stepping == OC_CHARTR) { /* CharTracingStep, then its face field */
          for (i = nbeg - 1; i <= nend + 1; i++)
            if (p->c.recon == OC_PARABOLIC)
              char_tracing_ppm(w.v[i], w.vp[i], w.vm[i], p->c.gamma, dt / dxd, dt, &r, c3, dims,
                               p->c.char_limiting ? 2 : 3); /* char_tracing.c:35-43 */
            else
              char_tracing(w.v[i], w.vp[i], w.vm[i], p->c.gamma, dt / dxd, dt, &r, c3, dims);
          if (ct)
            for (i = nbeg - 2; i <= nend + 1; i++) {
              w.vp[i][r.bn] = w.bn[i];
              w.vm[i + 1][r.bn] = w.bn[i];
            }
        } else if (p->c.stepping == OC_HANCOCK_CONS) {
          /* conservative Hancock step (PRIMITIVE_HANCOCK NO), hancock.c:159-434:
             each zone's own interface states evolved by dt/2 with the
             difference of their fluxes; where U^{n+1/2} fails ConsToPrim the
             zone falls back to first order */
          const double dtdx = dt2 / dxd;
          for (i = nbeg - 1; i <= nend + 1; i++) {
            double uc[NV], uL[NV], uR[NV], fp[NV], fm[NV], uh[NV], vh[NV], pp, pm;
            unsigned char fl = 0;
            prim_to_cons(w.v[i], uc, gmm1);
            prim_to_cons(w.vp[i], uL, gmm1);
            prim_to_cons(w.vm[i], uR, gmm1);
            flux(w.vp[i], uL, fp, &pp, &r);
            flux(w.vm[i], uR, fm, &pm, &r);
            for (nv = 0; nv < NV; nv++) {
              double rhs = -dtdx * (fp[nv] - fm[nv]);
              if (nv == r.vn) rhs -= dtdx * (pp - pm);
              uh[nv] = uc[nv] + rhs;
            }
            cons_to_prim(uh, vh, gmm1, &fl);
            if (fl) {
              for (nv = 0; nv < NV; nv++) vh[nv] = w.vp[i][nv] = w.vm[i][nv] = w.v[i][nv];
              if (ct) { w.vp[i][r.bn] = w.bn[i]; w.vm[i][r.bn] = w.bn[i - 1]; }
            }
            for (nv = 0; nv < NV; nv++) {
              double P1 = w.vp[i][nv] - w.vm[i][nv], dvp, dvm;
              dvp = dvm = vh[nv] - w.v[i][nv];
              dvp += 0.5 * P1;
              dvm -= 0.5 * P1;
              w.vp[i][nv] = w.v[i][nv] + dvp;
              w.vm[i][nv] = w.v[i][nv] + dvm;
            }
          }
          if (ct)
            for (i = nbeg - 2; i <= nend + 1; i++) {
              w.vp[i][r.bn] = w.bn[i];
              w.vm[i + 1][r.bn] = w.bn[i];
            }
        } else {
          for (i = nbeg - 1; i <= nend + 1; i++) { /* primitive Hancock step */
            double dv[NV], Adv[NV];
            for (nv = 0; nv < NV; nv++) dv[nv] = w.vp[i][nv] - w.vm[i][nv];
            prim_rhs(w.v[i], dv, p->c.gamma, &r, c3, Adv);
            for (nv = NV - 1; nv >= 0; nv--) {
              double scrh = dt2 * (inv_dl * Adv[nv] - 0.0);
              w.vp[i][nv] -= scrh;
              w.vm[i][nv] -= scrh;
            }
          }
        }
        for (i = nbeg - 1; i <= nend + 1; i++) { /* CheckPrimStates */
          int sw = (w.vp[i][PRS] < 0.0) || (w.vm[i][PRS] < 0.0);
          sw = sw || (w.vp[i][RHO] < 0.0) || (w.vm[i][RHO] < 0.0);
          if (sw) {
            double sp = w.vp[i][r.bn], sm = w.vm[i][r.bn];
            for (nv = 0; nv < NV; nv++) w.vm[i][nv] = w.vp[i][nv] = w.v[i][nv];
            if (ct) { w.vp[i][r.bn] = sp; w.vm[i][r.bn] = sm; }
          }
        }
        for (i = nbeg - 1; i <= nend + 1; i++) {
          prim_to_cons(w.vp[i], w.up[i], gmm1);
          prim_to_cons(w.vm[i], w.um[i], gmm1);
        }
      } else {
        for (i = nbeg - 1; i <= nend + 1; i++) {
          size_t c;
          ijk[dir] = i;
          c = CI(p, ijk[2], ijk[1], ijk[0]);
          for (nv = 0; nv < NV; nv++) {
            double dU;
            if (dir == 0) dU = dims == 1 ? 0.0 : (dims == 2 ? 0.0 + p->rhs_s[1][nv][c]
                                                            : 0.0 + p->rhs_s[1][nv][c] + p->rhs_s[2][nv][c]);
            else if (dir == 1) dU = dims == 2 ? p->rhs_s[0][nv][c] + 0.0
                                              : p->rhs_s[0][nv][c] + 0.0 + p->rhs_s[2][nv][c];
            else dU = p->rhs_s[0][nv][c] + p->rhs_s[1][nv][c];
            w.up[i][nv] = p->up_s[dir][nv][c] + dU;
            w.um[i][nv] = p->um_s[dir][nv][c] + dU;
          }
        }
        if (ct)
          for (i = nbeg - 2; i <= nend + 1; i++) {
            if (i >= nbeg - 1) w.up[i][r.bn] = w.bn[i];
            if (i + 1 <= nend + 1) w.um[i + 1][r.bn] = w.bn[i];
          }
        for (i = nbeg - 1; i <= nend + 1; i++) {
          unsigned char fm = 0, fp = 0;
          cons_to_prim(w.um[i], w.vm[i], gmm1, &fm);
          cons_to_prim(w.up[i], w.vp[i], gmm1, &fp);
        }
      }
      /* Riemann problems on interfaces nbeg-1 .. nend */
      for (i = nbeg - 1; i <= nend; i++) {
        double m;
        if (p->c.solver == OC_HLL)
          hll_solver(w.vp[i], w.up[i], w.vm[i + 1], w.um[i + 1], p->c.gamma, &r, &w.ifc[i], &m);
        else if (p->c.solver == OC_ROE)
          roe_solver(w.vp[i], w.up[i], w.vm[i + 1], w.um[i + 1], p->c.gamma, c3, &r, &w.ifc[i], &m);
        else
          hlld_solver(w.vp[i], w.up[i], w.vm[i + 1], w.um[i + 1], p->c.gamma, &r, &w.ifc[i], &m);
      }
      /* CT_StoreUpwindEMF, ct_emf.c:104-207 */
      if (ct)
        for (i = nbeg - 1; i <= nend; i++) {
          size_t c;
          const double *F = w.ifc[i].f;
          ijk[dir] = i;
          c = CI(p, ijk[2], ijk[1], ijk[0]);
          if (dir == 0) {
            p->eface[EZI][c] = -F[BX2];
            if (dims == 3) p->eface[EYI][c] = F[BX3];
          } else if (dir == 1) {
            p->eface[EZJ][c] = F[BX1];
            if (dims == 3) p->eface[EXJ][c] = -F[BX3];
          } else {
            p->eface[EYK][c] = -F[BX1];
            p->eface[EXK][c] = F[BX2];
          }
          p->sv[dir][c] = F[RHO] > 1.e-6 ? 1 : (F[RHO] < -1.e-6 ? -1 : 0);
        }
      /* RightHandSide with dt/2 (predictor) or dt (corrector) */
      for (i = nbeg; i <= nend; i++) {
        double scrh = (stage == 1 ? dt2 : dt) / dxd;
        for (nv = 0; nv < NV; nv++) w.rhs[i][nv] = -scrh * (w.ifc[i].f[nv] - w.ifc[i - 1].f[nv]);
        w.rhs[i][r.vn] -= scrh * (w.ifc[i].press - w.ifc[i - 1].press);
      }
      if (stage == 1) {
        if (ct && p->c.stepping != OC_HANCOCK_CONS) { /* CTU_CT_Source (ctu_step.c:122-133) */
          const double dt2_dx = dt2 / dxd;
          for (i = nbeg - 1; i <= nend + 1; i++) {
            double db = dt2_dx * (w.up[i][r.bn] - w.um[i][r.bn]), scrh;
            w.up[i][MX1] += vn[i][BX1] * db;
            w.um[i][MX1] += vn[i][BX1] * db;
            w.up[i][MX1 + 1] += vn[i][BX2] * db;
            w.um[i][MX1 + 1] += vn[i][BX2] * db;
            if (c3) {
              w.up[i][MX1 + 2] += vn[i][BX3] * db;
              w.um[i][MX1 + 2] += vn[i][BX3] * db;
            }
            w.up[i][r.bt] += vn[i][r.vt] * db;
            w.um[i][r.bt] += vn[i][r.vt] * db;
            if (c3) {
              w.up[i][r.bb] += vn[i][r.vb] * db;
              w.um[i][r.bb] += vn[i][r.vb] * db;
            }
            scrh = c3 ? vn[i][VX1] * vn[i][BX1] + vn[i][VX2] * vn[i][BX2] + vn[i][VX3] * vn[i][BX3]
                      : vn[i][VX1] * vn[i][BX1] + vn[i][VX2] * vn[i][BX2];
            w.up[i][ENG] += scrh * db;
            w.um[i][ENG] += scrh * db;
          }
        }
        for (i = nbeg - 1; i <= nend + 1; i++) {
          size_t c;
          ijk[dir] = i;
          c = CI(p, ijk[2], ijk[1], ijk[0]);
          for (nv = 0; nv < NV; nv++) {
            p->up_s[dir][nv][c] = w.up[i][nv];
            p->um_s[dir][nv][c] = w.um[i][nv];
            if (i >= nbeg && i <= nend) p->rhs_s[dir][nv][c] = w.rhs[i][nv];
          }
        }
      } else {
        for (i = nbeg; i <= nend; i++) {
          size_t c;
          ijk[dir] = i;
          c = CI(p, ijk[2], ijk[1], ijk[0]);
          for (nv = 0; nv < NV; nv++) p->uc[nv][c] += w.rhs[i][nv];
        }
      }
      for (i = nbeg; i <= nend; i++) invdt = MAX(invdt, w.ifc[i].cmax * inv_dl);
    }
    pencil_free(&w);
    free(vn);
  }
  *inv_dt = invdt;
}

/* CT_ComputeEMF for ARITHMETIC, UCT0 and UCT_CONTACT (ct_emf.c:210-291,
   ct_emf_average.c:13-164); CT_ComputeCenterEMF (ct_emf.c:348-388).
   stage 1 = CTU predictor (no corner integration, ct_emf_average.c:89-91);
   the RK stages and the CTU corrector pass 2. */
static void ctu_compute_emf(oc_problem *p, int stage) {
  const int dims = p->c.dims, uct = p->c.emf == OC_UCT_CONTACT, uct0 = p->c.emf == OC_UCT0;
  const double w = uct ? 1.0 : 0.25;
  const int ib = p->emf_lo[0], ie = p->emf_hi[0], jb = p->emf_lo[1], je = p->emf_hi[1];
  const int kb = dims == 3 ? p->emf_lo[2] : 0, ke = dims == 3 ? p->emf_hi[2] : 0;
  const int KO = dims == 3;
  double *ezi = p->eface[EZI], *ezj = p->eface[EZJ], *eyi = p->eface[EYI], *eyk = p->eface[EYK];
  double *exj = p->eface[EXJ], *exk = p->eface[EXK];
  double *Ex1 = p->ecc[0], *Ex2 = p->ecc[1], *Ex3 = p->ecc[2];
  int i, j, k;
  if (uct || uct0) {
    size_t c;
    for (c = 0; c < p->ncell; c++) {
      double vx1 = p->vc[VX1][c], vx2 = p->vc[VX2][c], vx3 = p->vc[VX3][c];
      double Bx1 = p->vc[BX1][c], Bx2 = p->vc[BX2][c], Bx3 = p->vc[BX3][c];
      Ex1[c] = (vx3 * Bx2 - vx2 * Bx3);
      Ex2[c] = (vx1 * Bx3 - vx3 * Bx1);
      Ex3[c] = (vx2 * Bx1 - vx1 * Bx2);
    }
  }
#define E3(a, kk, jj, ii) (a[CI(p, kk, jj, ii)])
  if (uct0) /* face EMFs minus the centred ones, in place (ct_emf.c:261-282) */
    for (k = kb; k <= ke + KO; k++)
      for (j = jb; j <= je + 1; j++)
        for (i = ib; i <= ie + 1; i++) {
          if (dims == 3) {
            E3(exj, k, j, i) *= 2.0;
            E3(exk, k, j, i) *= 2.0;
            E3(eyi, k, j, i) *= 2.0;
            E3(eyk, k, j, i) *= 2.0;
            E3(exj, k, j, i) -= 0.5 * (E3(Ex1, k, j, i) + E3(Ex1, k, j + 1, i));
            E3(exk, k, j, i) -= 0.5 * (E3(Ex1, k, j, i) + E3(Ex1, k + 1, j, i));
            E3(eyi, k, j, i) -= 0.5 * (E3(Ex2, k, j, i) + E3(Ex2, k, j, i + 1));
            E3(eyk, k, j, i) -= 0.5 * (E3(Ex2, k, j, i) + E3(Ex2, k + 1, j, i));
          }
          E3(ezi, k, j, i) *= 2.0;
          E3(ezj, k, j, i) *= 2.0;
          E3(ezi, k, j, i) -= 0.5 * (E3(Ex3, k, j, i) + E3(Ex3, k, j, i + 1));
          E3(ezj, k, j, i) -= 0.5 * (E3(Ex3, k, j, i) + E3(Ex3, k, j + 1, i));
        }
  for (k = kb; k <= ke; k++)
    for (j = jb; j <= je; j++)
      for (i = ib; i <= ie; i++) {
        if (dims == 3) {
          E3(p->ex, k, j, i) = w * (E3(exk, k, j, i) + E3(exk, k, j + 1, i) + E3(exj, k, j, i) + E3(exj, k + 1, j, i));
          E3(p->ey, k, j, i) = w * (E3(eyi, k, j, i) + E3(eyi, k + 1, j, i) + E3(eyk, k, j, i) + E3(eyk, k, j, i + 1));
        }
        E3(p->ez, k, j, i) = w * (E3(ezi, k, j, i) + E3(ezi, k, j + 1, i) + E3(ezj, k, j, i) + E3(ezj, k, j, i + 1));
      }
  if (uct && stage == 2) { /* CT_EMF_IntegrateToCorner */
#define DEX_DYP(kk, jj, ii) (E3(exj, kk, jj, ii) - E3(Ex1, kk, jj, ii))
#define DEX_DZP(kk, jj, ii) (E3(exk, kk, jj, ii) - E3(Ex1, kk, jj, ii))
#define DEY_DXP(kk, jj, ii) (E3(eyi, kk, jj, ii) - E3(Ex2, kk, jj, ii))
#define DEY_DZP(kk, jj, ii) (E3(eyk, kk, jj, ii) - E3(Ex2, kk, jj, ii))
#define DEZ_DXP(kk, jj, ii) (E3(ezi, kk, jj, ii) - E3(Ex3, kk, jj, ii))
#define DEZ_DYP(kk, jj, ii) (E3(ezj, kk, jj, ii) - E3(Ex3, kk, jj, ii))
#define DEX_DYM(kk, jj, ii) (E3(Ex1, kk, jj, ii) - E3(exj, kk, jj - 1, ii))
#define DEX_DZM(kk, jj, ii) (E3(Ex1, kk, jj, ii) - E3(exk, kk - 1, jj, ii))
#define DEY_DXM(kk, jj, ii) (E3(Ex2, kk, jj, ii) - E3(eyi, kk, jj, ii - 1))
#define DEY_DZM(kk, jj, ii) (E3(Ex2, kk, jj, ii) - E3(eyk, kk - 1, jj, ii))
#define DEZ_DXM(kk, jj, ii) (E3(Ex3, kk, jj, ii) - E3(ezi, kk, jj, ii - 1))
#define DEZ_DYM(kk, jj, ii) (E3(Ex3, kk, jj, ii) - E3(ezj, kk, jj - 1, ii))
    for (k = kb; k <= ke + KO; k++)
      for (j = jb; j <= je + 1; j++)
        for (i = ib; i <= ie + 1; i++) {
          int sx = p->sv[0][CI(p, k, j, i)], sy = p->sv[1][CI(p, k, j, i)];
          int sz = dims == 3 ? p->sv[2][CI(p, k, j, i)] : 0;
          int iu = sx > 0 ? i : i + 1, ju = sy > 0 ? j : j + 1, ku = sz > 0 ? k : k + 1;
          if (sx == 0) {
            E3(p->ez, k, j, i) += 0.5 * (DEZ_DYP(k, j, i) + DEZ_DYP(k, j, i + 1));
            E3(p->ez, k, j - 1, i) -= 0.5 * (DEZ_DYM(k, j, i) + DEZ_DYM(k, j, i + 1));
            if (dims == 3) {
              E3(p->ey, k, j, i) += 0.5 * (DEY_DZP(k, j, i) + DEY_DZP(k, j, i + 1));
              E3(p->ey, k - 1, j, i) -= 0.5 * (DEY_DZM(k, j, i) + DEY_DZM(k, j, i + 1));
            }
          } else {
            E3(p->ez, k, j, i) += DEZ_DYP(k, j, iu);
            E3(p->ez, k, j - 1, i) -= DEZ_DYM(k, j, iu);
            if (dims == 3) {
              E3(p->ey, k, j, i) += DEY_DZP(k, j, iu);
              E3(p->ey, k - 1, j, i) -= DEY_DZM(k, j, iu);
            }
          }
          if (sy == 0) {
            E3(p->ez, k, j, i) += 0.5 * (DEZ_DXP(k, j, i) + DEZ_DXP(k, j + 1, i));
            E3(p->ez, k, j, i - 1) -= 0.5 * (DEZ_DXM(k, j, i) + DEZ_DXM(k, j + 1, i));
            if (dims == 3) {
              E3(p->ex, k, j, i) += 0.5 * (DEX_DZP(k, j, i) + DEX_DZP(k, j + 1, i));
              E3(p->ex, k - 1, j, i) -= 0.5 * (DEX_DZM(k, j, i) + DEX_DZM(k, j + 1, i));
            }
          } else {
            E3(p->ez, k, j, i) += DEZ_DXP(k, ju, i);
            E3(p->ez, k, j, i - 1) -= DEZ_DXM(k, ju, i);
            if (dims == 3) {
              E3(p->ex, k, j, i) += DEX_DZP(k, ju, i);
              E3(p->ex, k - 1, j, i) -= DEX_DZM(k, ju, i);
            }
          }
          if (dims == 3) {
            if (sz == 0) {
              E3(p->ex, k, j, i) += 0.5 * (DEX_DYP(k, j, i) + DEX_DYP(k + 1, j, i));
              E3(p->ex, k, j - 1, i) -= 0.5 * (DEX_DYM(k, j, i) + DEX_DYM(k + 1, j, i));
              E3(p->ey, k, j, i) += 0.5 * (DEY_DXP(k, j, i) + DEY_DXP(k + 1, j, i));
              E3(p->ey, k, j, i - 1) -= 0.5 * (DEY_DXM(k, j, i) + DEY_DXM(k + 1, j, i));
            } else {
              E3(p->ex, k, j, i) += DEX_DYP(ku, j, i);
              E3(p->ex, k, j - 1, i) -= DEX_DYM(ku, j, i);
              E3(p->ey, k, j, i) += DEY_DXP(ku, j, i);
              E3(p->ey, k, j, i - 1) -= DEY_DXM(ku, j, i);
            }
          }
        }
#undef DEX_DYP
#undef DEX_DZP
#undef DEY_DXP
#undef DEY_DZP
#undef DEZ_DXP
#undef DEZ_DYP
#undef DEX_DYM
#undef DEX_DZM
#undef DEY_DXM
#undef DEY_DZM
#undef DEZ_DXM
#undef DEZ_DYM
  }
  if (uct)
    for (k = kb; k <= ke; k++)
      for (j = jb; j <= je; j++)
        for (i = ib; i <= ie; i++) {
          if (dims == 3) {
            E3(p->ex, k, j, i) *= 0.25;
            E3(p->ey, k, j, i) *= 0.25;
          }
          E3(p->ez, k, j, i) *= 0.25;
        }
#undef E3
}

/* CT_Update over the emf ranges (ct_update.c:29-220): Vs = base + dt curl E */
static void ct_update_ranges(oc_problem *p, double *const base[3], double dt) {
  const int dims = p->c.dims;
  const int KO = dims == 3;
  const int kb = dims == 3 ? p->emf_lo[2] : 0, ke = dims == 3 ? p->emf_hi[2] : 0;
  const int jb = p->emf_lo[1], je = p->emf_hi[1], ib = p->emf_lo[0], ie = p->emf_hi[0];
  const double dx1 = p->c.dx[0], dx2 = p->c.dx[1], dx3 = p->c.dx[2];
  int i, j, k;
  for (k = kb + KO; k <= ke; k++)
    for (j = jb + 1; j <= je; j++)
      for (i = ib; i <= ie; i++) {
        double rhs_x;
        if (dims == 2)
          rhs_x = 0.0 - dt / dx2 * (p->ez[CI(p, k, j, i)] - p->ez[CI(p, k, j - 1, i)]);
        else
          rhs_x = 0.0 - dt / dx2 * (p->ez[CI(p, k, j, i)] - p->ez[CI(p, k, j - 1, i)]) +
                  dt / dx3 * (p->ey[CI(p, k, j, i)] - p->ey[CI(p, k - 1, j, i)]);
        p->bs[0][FI(p, 0, k, j, i)] = base[0][FI(p, 0, k, j, i)] + rhs_x;
      }
  for (k = kb + KO; k <= ke; k++)
    for (j = jb; j <= je; j++)
      for (i = ib + 1; i <= ie; i++) {
        double rhs_y;
        if (dims == 2)
          rhs_y = dt / dx1 * (p->ez[CI(p, k, j, i)] - p->ez[CI(p, k, j, i - 1)]);
        else
          rhs_y = dt / dx1 * (p->ez[CI(p, k, j, i)] - p->ez[CI(p, k, j, i - 1)]) -
                  dt / dx3 * (p->ex[CI(p, k, j, i)] - p->ex[CI(p, k - 1, j, i)]);
        p->bs[1][FI(p, 1, k, j, i)] = base[1][FI(p, 1, k, j, i)] + rhs_y;
      }
  if (dims == 3)
    for (k = kb; k <= ke; k++)
      for (j = jb + 1; j <= je; j++)
        for (i = ib + 1; i <= ie; i++) {
          double rhs_z = -dt / dx1 * (p->ey[CI(p, k, j, i)] - p->ey[CI(p, k, j, i - 1)]) +
                         dt / dx2 * (p->ex[CI(p, k, j, i)] - p->ex[CI(p, k, j - 1, i)]);
          p->bs[2][FI(p, 2, k, j, i)] = base[2][FI(p, 2, k, j, i)] + rhs_z;
        }
}

/* CT_AverageMagneticField into an arbitrary conserved array (domain + 1) */
static void ct_average_into(oc_problem *p, double *const U[NV]) {
  const int dims = p->c.dims;
  int ko = dims == 3, d, i, j, k;
  for (k = p->beg[2] - ko; k <= p->end[2] + ko; k++)
    for (j = p->beg[1] - 1; j <= p->end[1] + 1; j++)
      for (i = p->beg[0] - 1; i <= p->end[0] + 1; i++) {
        size_t c = CI(p, k, j, i);
        for (d = 0; d < dims; d++) {
          int o[3] = {0, 0, 0};
          o[d] = 1;
          U[BX1 + d][c] = 0.5 * (p->bs[d][FI(p, d, k, j, i)] + p->bs[d][FI(p, d, k - o[2], j - o[1], i - o[0])]);
        }
      }
}

/* AdvanceStep for CTU, ctu_step.c:140-727 (no parabolic terms) */
static int oc_advance_ctu(oc_problem *p, double dt, double *inv_dt_hyp, double *max_mach,
                          int64_t *nfail) {
  const double gmm1 = p->c.gamma - 1.0;
  const int dims = p->c.dims, ct = p->c.ct;
  double inv_dt = 0.0;
  int i, j, k, nv, d, lo[3], hi[3];
  size_t c;

  p->nfail = 0;
  p->max_mach = 0.0;
  p->roe_bad = 0;
  memset(p->flag, 0, p->ncell);
  boundary(p);
  if (ct)
    for (d = 0; d < dims; d++) memcpy(p->bs0[d], p->bs[d], p->nface[d] * sizeof(double));
  for (c = 0; c < p->ncell; c++) { /* PrimToCons3D over the whole grid */
    double v[NV], u[NV];
    for (nv = 0; nv < NV; nv++) v[nv] = p->vc[nv][c];
    prim_to_cons(v, u, gmm1);
    for (nv = 0; nv < NV; nv++) p->uc[nv][c] = u[nv];
  }
  /* predictor */
  for (d = 0; d < dims; d++) ctu_sweep(p, d, dt, 1, &inv_dt);
  for (d = 0; d < 3; d++) {
    int e = (ct && d < dims) ? 1 : 0;
    lo[d] = p->beg[d] - e;
    hi[d] = p->end[d] + e;
  }
  for (k = lo[2]; k <= hi[2]; k++)
    for (j = lo[1]; j <= hi[1]; j++)
      for (i = lo[0]; i <= hi[0]; i++) {
        c = CI(p, k, j, i);
        for (nv = 0; nv < NV; nv++) {
          double dU = dims == 1 ? p->rhs_s[0][nv][c]
                    : (dims == 2 ? p->rhs_s[0][nv][c] + p->rhs_s[1][nv][c]
                                 : p->rhs_s[0][nv][c] + p->rhs_s[1][nv][c] + p->rhs_s[2][nv][c]);
          p->uh[nv][c] = p->uc[nv][c] + dU;
        }
      }
  if (ct) {
    ctu_compute_emf(p, 1);
    ct_update_ranges(p, p->bs, 0.5 * dt);
    ct_average_into(p, p->uh);
  }
  for (k = lo[2]; k <= hi[2]; k++)
    for (j = lo[1]; j <= hi[1]; j++)
      for (i = lo[0]; i <= hi[0]; i++) {
        double u[NV], v[NV];
        c = CI(p, k, j, i);
        for (nv = 0; nv < NV; nv++) u[nv] = p->uh[nv][c];
        cons_to_prim(u, v, gmm1, &p->flag[c]);
        for (nv = 0; nv < NV; nv++) { p->uh[nv][c] = u[nv]; p->vc[nv][c] = v[nv]; }
      }
  /* corrector */
  for (d = 0; d < dims; d++) ctu_sweep(p, d, dt, 2, &inv_dt);
  if (ct) {
    ctu_compute_emf(p, 2);
    ct_update_ranges(p, p->bs0, dt);
    ct_average(p);
  }
  cons_to_prim_3d(p);
  if (inv_dt_hyp) *inv_dt_hyp = inv_dt;
  if (max_mach) *max_mach = p->max_mach;
  if (nfail) *nfail = p->nfail;
  return p->roe_bad ? 1 : 0;
}

/* AdvanceStep, Src/Time_Stepping/rk_step.c:27-254 */
int oc_advance(oc_problem *p, double dt, double *inv_dt_hyp, double *max_mach,
               int64_t *nfail) {
  const double gmm1 = p->c.gamma - 1.0;
  const double w0 = p->c.stepping == OC_RK3 ? 0.75 : 0.5;
  const double wc = p->c.stepping == OC_RK3 ? 0.25 : 0.5;
  static const double one_third = 1.0 / 3.0;
  double inv_dt = 0.0, inv_dt_1d = 0.0;
  int i, j, k, nv, d;
  size_t c;

  p->bstage = 0;
  if (IS_CTU(p->c.stepping)) return oc_advance_ctu(p, dt, inv_dt_hyp, max_mach, nfail);

  p->nfail = 0;
  p->max_mach = 0.0;
  p->roe_bad = 0;
  memset(p->flag, 0, p->ncell);
  /* stage 1 */
  boundary(p);
  DOM_LOOP(p, k, j, i) {
    double v[NV], u[NV];
    c = CI(p, k, j, i);
    for (nv = 0; nv < NV; nv++) v[nv] = p->vc[nv][c];
    prim_to_cons(v, u, gmm1);
    for (nv = 0; nv < NV; nv++) p->uc[nv][c] = p->u0[nv][c] = u[nv];
  }
  if (p->c.ct)
    for (d = 0; d < p->c.dims; d++) memcpy(p->bs0[d], p->bs[d], p->nface[d] * sizeof(double));
  update_stage(p, dt, 1, &inv_dt, &inv_dt_1d);
  if (p->c.ct) ct_average(p);
  cons_to_prim_3d(p);
  if (p->c.stepping == OC_EULER) goto done; /* the predictor alone, rk_step.c:145 */

  /* stage 2 */
  boundary(p);
  update_stage(p, dt, 2, &inv_dt, &inv_dt_1d);
  DOM_LOOP(p, k, j, i) {
    c = CI(p, k, j, i);
    for (nv = 0; nv < NV; nv++) p->uc[nv][c] = w0 * p->u0[nv][c] + wc * p->uc[nv][c];
  }
  if (p->c.ct) {
    for (d = 0; d < p->c.dims; d++) {
      size_t f;
      for (f = 0; f < p->nface[d]; f++) p->bs[d][f] = w0 * p->bs0[d][f] + wc * p->bs[d][f];
    }
    ct_average(p);
  }
  cons_to_prim_3d(p);

  if (p->c.stepping == OC_RK3) {
    boundary(p);
    update_stage(p, dt, 3, &inv_dt, &inv_dt_1d);
    DOM_LOOP(p, k, j, i) {
      c = CI(p, k, j, i);
      for (nv = 0; nv < NV; nv++)
        p->uc[nv][c] = one_third * (p->u0[nv][c] + 2.0 * p->uc[nv][c]);
    }
    if (p->c.ct) {
      for (d = 0; d < p->c.dims; d++) {
        size_t f;
        for (f = 0; f < p->nface[d]; f++) p->bs[d][f] = (p->bs0[d][f] + 2.0 * p->bs[d][f]) / 3.0;
      }
      ct_average(p);
    }
    cons_to_prim_3d(p);
  }
done:
  if (p->c.dims == 1) inv_dt = inv_dt_1d;
  if (inv_dt_hyp) *inv_dt_hyp = inv_dt;
  if (max_mach) *max_mach = p->max_mach;
  if (nfail) *nfail = p->nfail;
  return p->roe_bad ? 1 : 0;
}

/* Main loop dt logic, Src/main.c:143-151, 215, 236, 389-575 */
int oc_run(oc_problem *p, int nsteps, double first_dt, double cfl,
           double cfl_max_var, double *dts, double *t_final) {
  double g_dt = first_dt, g_time = 0.0;
  int s;
  for (s = 0; s < nsteps; s++) {
    double inv_dt, dt_hyp, dtnext;
    if (dts) dts[s] = g_dt;
    if (oc_advance(p, g_dt, &inv_dt, NULL, NULL)) return 1;
    g_time += g_dt;
    dt_hyp = 1.0 / inv_dt;
    dt_hyp *= cfl;
    dtnext = dt_hyp;
    dtnext = MIN(dtnext, cfl_max_var * g_dt);
    g_dt = dtnext;
  }
  if (t_final) *t_final = g_time;
  return 0;
}

/* ------------------------------------------------------------------ */
/* Allocation and state transfer                                        */
/* ------------------------------------------------------------------ */

oc_problem *oc_create(const oc_config *cfg) {
  oc_problem *p = calloc(1, sizeof *p);
  int d, nv;
  p->c = *cfg;
  if (cfg->ct && cfg->dims < 2) { free(p); return NULL; }
  for (d = 0; d < 3; d++) {
    if (cfg->bc[d] < OC_PERIODIC || cfg->bc[d] > OC_USERDEF) { free(p); return NULL; }
    if (cfg->bc_hi[d] < OC_PERIODIC || cfg->bc_hi[d] > OC_USERDEF) { free(p); return NULL; }
    if ((cfg->bc[d] == OC_PERIODIC) != (cfg->bc_hi[d] == OC_PERIODIC)) { free(p); return NULL; }
  }
  p->ng = cfg->recon == OC_PARABOLIC ? 3 : 2; /* Src/get_nghost.c:28-104 */
  if (IS_CTU(cfg->stepping)) {
    /* hancock.c:64-67; characteristic tracing takes parabolic states too */
    if (cfg->recon != OC_LINEAR && cfg->stepping != OC_CHARTR) { free(p); return NULL; }
    /* ct_emf.c:196-200: UCT_HLL needs the RK sweeps */
    if (cfg->ct && cfg->emf != OC_ARITHMETIC && cfg->emf != OC_UCT0 && cfg->emf != OC_UCT_CONTACT) {
      free(p);
      return NULL;
    }
    if (cfg->ct) p->ng++;                                    /* get_nghost.c:84-90 */
  }
  for (d = 0; d < 3; d++) {
    int active = d < cfg->dims;
    p->nt[d] = active ? cfg->nx[d] + 2 * p->ng : 1;
    p->beg[d] = active ? p->ng : 0;
    p->end[d] = active ? p->ng + cfg->nx[d] - 1 : 0;
    p->inv_dx[d] = 1.0 / cfg->dx[d]; /* set_geometry.c:244 */
    if (!active) p->c.nx[d] = 1;
  }
  p->ncell = (size_t)p->nt[0] * p->nt[1] * p->nt[2];
  for (d = 0; d < 3; d++)
    p->nface[d] = (size_t)(p->nt[0] + (d == 0)) * (p->nt[1] + (d == 1)) * (p->nt[2] + (d == 2));
  for (nv = 0; nv < NV; nv++) {
    p->vc[nv] = calloc(p->ncell, sizeof(double));
    p->uc[nv] = calloc(p->ncell, sizeof(double));
    p->u0[nv] = calloc(p->ncell, sizeof(double));
  }
  for (d = 0; d < 3; d++) {
    int c;
    p->bs[d] = calloc(p->nface[d], sizeof(double));
    p->bs0[d] = calloc(p->nface[d], sizeof(double));
    p->sl[d] = calloc(p->ncell, sizeof(double));
    p->sr[d] = calloc(p->ncell, sizeof(double));
    for (c = 0; c < 3; c++) p->dv[d][c] = calloc(p->ncell, sizeof(double));
  }
  p->ex = calloc(p->ncell, sizeof(double));
  p->ey = calloc(p->ncell, sizeof(double));
  p->ez = calloc(p->ncell, sizeof(double));
  p->cdt = calloc(p->ncell, sizeof(double));
  p->flag = calloc(p->ncell, 1);
  if (IS_CTU(cfg->stepping)) {
    for (d = 0; d < 3; d++)
      for (nv = 0; nv < NV; nv++) {
        p->up_s[d][nv] = calloc(p->ncell, sizeof(double));
        p->um_s[d][nv] = calloc(p->ncell, sizeof(double));
        p->rhs_s[d][nv] = calloc(p->ncell, sizeof(double));
      }
    for (nv = 0; nv < NV; nv++) p->uh[nv] = calloc(p->ncell, sizeof(double));
  }
  if (cfg->ct && (IS_CTU(cfg->stepping) || cfg->emf != OC_UCT_HLL)) {
    for (d = 0; d < 6; d++) p->eface[d] = calloc(p->ncell, sizeof(double));
    for (d = 0; d < 3; d++) {
      p->sv[d] = calloc(p->ncell, 1);
      p->ecc[d] = calloc(p->ncell, sizeof(double));
    }
  }
#ifdef _OPENMP
  if (cfg->nthreads > 0) omp_set_num_threads(cfg->nthreads);
#endif
  return p;
}

void oc_destroy(oc_problem *p) {
  int d, nv, c;
  if (!p) return;
  for (nv = 0; nv < NV; nv++) { free(p->vc[nv]); free(p->uc[nv]); free(p->u0[nv]); }
  for (d = 0; d < 3; d++)
    for (nv = 0; nv < NV; nv++) { free(p->up_s[d][nv]); free(p->um_s[d][nv]); free(p->rhs_s[d][nv]); }
  for (nv = 0; nv < NV; nv++) free(p->uh[nv]);
  for (d = 0; d < 6; d++) free(p->eface[d]);
  for (d = 0; d < 3; d++) { free(p->sv[d]); free(p->ecc[d]); }
  for (d = 0; d < 3; d++) {
    free(p->bs[d]); free(p->bs0[d]); free(p->sl[d]); free(p->sr[d]);
    for (c = 0; c < 3; c++) free(p->dv[d][c]);
  }
  free(p->ex); free(p->ey); free(p->ez); free(p->cdt); free(p->flag);
  free(p);
}

static void xfer(oc_problem *p, double *vc, double *bs[3], int to_problem) {
  int nx = p->c.nx[0], ny = p->c.nx[1], nz = p->c.nx[2];
  int nv, d, i, j, k;
  size_t q = 0;
  for (nv = 0; nv < NV; nv++)
    for (k = 0; k < nz; k++)
      for (j = 0; j < ny; j++)
        for (i = 0; i < nx; i++, q++) {
          size_t c = CI(p, k + p->beg[2], j + p->beg[1], i + p->beg[0]);
          if (to_problem) p->vc[nv][c] = vc[q];
          else vc[q] = p->vc[nv][c];
        }
  if (!p->c.ct) return;
  for (d = 0; d < p->c.dims; d++) {
    int fx = nx + (d == 0), fy = ny + (d == 1), fz = nz + (d == 2);
    q = 0;
    if (!bs[d]) continue;
    for (k = 0; k < fz; k++)
      for (j = 0; j < fy; j++)
        for (i = 0; i < fx; i++, q++) {
          /* dump face index 0 along d is reference index beg-1 */
          int ri = i + p->beg[0] - (d == 0), rj = j + p->beg[1] - (d == 1);
          int rk = k + p->beg[2] - (d == 2);
          size_t f = FI(p, d, rk, rj, ri);
          if (to_problem) p->bs[d][f] = bs[d][q];
          else bs[d][q] = p->bs[d][f];
        }
  }
}

void oc_set_userdef(oc_problem *p, oc_userdef_fn fn, void *user) {
  p->ud_fn = fn;
  p->ud_user = user;
}

void oc_set_internal(oc_problem *p, int on) { p->internal = on; }
unsigned char *oc_flags(oc_problem *p) { return p->flag; }

void oc_arrays(oc_problem *p, double **vc, double **bs) {
  int q;
  for (q = 0; q < NV; q++) vc[q] = p->vc[q];
  for (q = 0; q < 3; q++) bs[q] = p->bs[q];
}

void oc_set_state(oc_problem *p, const double *vc, const double *bs0,
                  const double *bs1, const double *bs2) {
  double *b[3] = {(double *)bs0, (double *)bs1, (double *)bs2};
  xfer(p, (double *)vc, b, 1);
}

void oc_get_state(const oc_problem *p, double *vc, double *bs0, double *bs1,
                  double *bs2) {
  double *b[3] = {bs0, bs1, bs2};
  xfer((oc_problem *)p, vc, b, 0);
}
