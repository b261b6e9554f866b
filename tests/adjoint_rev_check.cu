// Host check of the hand-derived reverse-mode point functions of the adjoint
// (pluto_gb300/csrc/pg_adjoint_pt.cuh) against forward-mode Dual<1>
// derivatives of the same point functions.  TEST INFRASTRUCTURE: compiled by
// tests/test_adjoint_rev.py with nvcc as a host program (no GPU needed).
//
// For seeded random interface states (families chosen to visit every HLLD
// region: L / R flux, single-star L / R, double-star L / R, the HLLC
// reversion) and random output adjoints lam, it forms J^T lam once by the
// reverse function and once column by column from 16 seeded Dual<1>
// evaluations of riemann_pt, likewise for the 40-input edge EMF, the PLM
// and PPM states and the prim/cons maps (floors included), and prints one line per check with the sample count, the branch
// counts and the largest relative difference.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>

#include "pg_adjoint_pt.cuh"

using namespace pg;
using D1 = Dual<1>;

static uint64_t s_rng = 0x9E3779B97F4A7C15ull;
static double urand() {  // xorshift64*, uniform in [0, 1)
  s_rng ^= s_rng >> 12;
  s_rng ^= s_rng << 25;
  s_rng ^= s_rng >> 27;
  return (double)((s_rng * 2685821657736338717ull) >> 11) * (1.0 / 9007199254740992.0);
}
static double urange(double a, double b) { return a + (b - a) * urand(); }

// HLLD region of the forward evaluation (the conditions of hlld_solver)
template <int DIR>
static int hlld_region(const double* vL, const double* vR, double gamma) {
  using R = Rot<DIR>;
  const RiemannBase<DIR> b(vL, vR, gamma);
  if (b.SL >= 0.0) return 0;
  if (b.SR <= 0.0) return 1;
  const double SL = b.SL, SR = b.SR;
  const double Bx = (SR * vR[R::bn] - SL * vL[R::bn]) * (1.0 / (SR - SL));
  const double duL = SL - vL[R::vn], duR = SR - vR[R::vn];
  const double SM = (duR * b.uR[R::vn] - duL * b.uL[R::vn] - b.ptR + b.ptL) *
                    (1.0 / (duR * b.uR[RHO] - duL * b.uL[RHO]));
  const double sqrL = ::sqrt(b.uL[RHO] * duL / (SL - SM)), sqrR = ::sqrt(b.uR[RHO] * duR / (SR - SM));
  double S1L = SM - ::fabs(Bx) / sqrL, S1R = SM + ::fabs(Bx) / sqrR;
  const bool rev = (S1L - SL) < 1.e-4 * (SM - SL) || (S1R - SR) > -1.e-4 * (SR - SM);
  if (rev) S1L = S1R = SM;
  if (S1L >= 0.0) return rev ? 6 : 2;
  if (S1R <= 0.0) return rev ? 7 : 3;
  return SM >= 0.0 ? 4 : 5;
}

static void draw_state(int family, double* vL, double* vR, int bn, int vn) {
  for (int nv = 0; nv < NV; nv++) {
    vL[nv] = urange(-2.0, 2.0);
    vR[nv] = urange(-2.0, 2.0);
  }
  vL[RHO] = urange(0.2, 5.0);
  vR[RHO] = urange(0.2, 5.0);
  vL[PRS] = urange(0.05, 5.0);
  vR[PRS] = urange(0.05, 5.0);
  switch (family) {
    case 1:  // nearby states
      for (int nv = 0; nv < NV; nv++) vR[nv] = vL[nv] * (1.0 + urange(-0.1, 0.1));
      break;
    case 2: {  // fast flow along the normal: the L or R flux
      const double u = urand() < 0.5 ? 15.0 : -15.0;
      vL[vn] += u;
      vR[vn] += u;
      break;
    }
    case 3:  // weak normal field: the HLLC reversion
      vL[bn] = vR[bn] = urange(-1e-3, 1e-3);
      break;
    case 4: {  // moderate drift: single-star regions
      const double u = urange(-3.0, 3.0);
      vL[vn] += u;
      vR[vn] += u;
      break;
    }
    case 5:  // the face-field override: equal normal field
      vR[bn] = vL[bn];
      break;
    case 6:  // strong normal field, weak tangential field and pressure: the
             // Alfven speed reaches the fast speed, the HLLC reversion
      for (int nv = BX1; nv < BX1 + 3; nv++)
        if (nv != bn) {
          vL[nv] *= 1e-3;
          vR[nv] *= 1e-3;
        }
      vL[bn] = vR[bn] = urange(1.0, 3.0) * (urand() < 0.5 ? 1.0 : -1.0);
      vL[PRS] *= 1e-3;
      vR[PRS] *= 1e-3;
      break;
    default:
      break;
  }
}

template <int DIR>
static double check_riemann(int solver, double gamma, int nsamp, long* regions) {
  using R = Rot<DIR>;
  double worst = 0.0;
  for (int t = 0; t < nsamp; t++) {
    double vL[NV], vR[NV], lam[kRiemannOut], gL[NV], gR[NV];
    draw_state(t % 7, vL, vR, R::bn, R::vn);
    for (int o = 0; o < kRiemannOut; o++) lam[o] = urange(-1.0, 1.0);
    if (solver == PG_HLLD) regions[hlld_region<DIR>(vL, vR, gamma)]++;
    riemann_rev<DIR>(solver, gamma, vL, vR, lam, gL, gR);
    double ref[2 * NV], scale = 0.0, diff = 0.0;
    for (int kk = 0; kk < 2 * NV; kk++) {
      D1 xL[NV], xR[NV], out[kRiemannOut];
      for (int nv = 0; nv < NV; nv++) {
        xL[nv] = D1(vL[nv]);
        xR[nv] = D1(vR[nv]);
      }
      if (kk < NV) xL[kk].d[0] = 1.0;
      else xR[kk - NV].d[0] = 1.0;
      riemann_pt<D1, DIR>(solver, gamma, true, xL, xR, out);
      double gk = 0.0;
      for (int o = 0; o < kRiemannOut; o++) gk += lam[o] * out[o].d[0];
      ref[kk] = gk;
      scale = fmax(scale, fabs(gk));
    }
    for (int kk = 0; kk < 2 * NV; kk++) {
      const double g = kk < NV ? gL[kk] : gR[kk - NV];
      diff = fmax(diff, fabs(g - ref[kk]));
    }
    const double rel = scale > 0.0 ? diff / scale : diff;
    if (!(rel <= worst)) worst = rel;  // NaN propagates as the worst
  }
  return worst;
}

static double check_emf(int nsamp, long* branches) {
  double worst = 0.0;
  for (int t = 0; t < nsamp; t++) {
    double in[kEdgeIn], g[kEdgeIn];
    for (int q = 0; q < 8; q++) in[q] = urange(0.1, 3.0);  // wave-speed magnitudes
    if (t % 3 == 0) in[1] = in[0];                        // ties of the MAX
    for (int q = 8; q < 16; q++) in[q] = urange(-1.0, 1.0);
    if (t % 4 == 1)  // monotone face fields: the MC slope branches
      for (int q = 8; q < 16; q++) in[q] = 0.1 * (q % 4) * (q % 4) + urange(0.0, 0.05);
    for (int q = 16; q < kEdgeIn; q++) in[q] = urange(-2.0, 2.0);
    const double lam = urange(-1.0, 1.0);
    emf_rev(in, lam, g);
    double diff = 0.0, scale = 0.0;
    for (int kk = 0; kk < kEdgeIn; kk++) {
      D1 x[kEdgeIn];
      for (int q = 0; q < kEdgeIn; q++) x[q] = D1(in[q]);
      x[kk].d[0] = 1.0;
      const double ref = lam * emf_pt(x).d[0];
      scale = fmax(scale, fabs(ref));
      diff = fmax(diff, fabs(g[kk] - ref));
    }
    const double dp = in[10] - in[9], dm = in[9] - in[8];
    branches[dp * dm < 0.0 ? 0 : (::fabs(0.5 * (dp + dm)) < ::fabs(2.0 * (::fabs(dp) < ::fabs(dm) ? dp : dm)) ? 1 : 2)]++;
    const double rel = scale > 0.0 ? diff / scale : diff;
    if (!(rel <= worst)) worst = rel;
  }
  return worst;
}

// PLM states (every limiter, the DEFAULT mix per variable) transposed
static double check_plm(int nsamp, long* branches) {
  double worst = 0.0;
  for (int t = 0; t < nsamp; t++) {
    double w[5];
    for (int q = 0; q < 5; q++) w[q] = urange(-1.0, 1.0);
    if (t % 3 == 0)  // monotone: the limiters' smooth branches
      for (int q = 0; q < 5; q++) w[q] = 0.3 * q * q * (t % 2 ? 1.0 : -1.0) + urange(0.0, 0.1);
    const int lim = t % 5, nv = (t / 5) % NV;
    const double lp = urange(-1.0, 1.0), lm = urange(-1.0, 1.0);
    double g[3];
    plm_rev(lim, nv, w[1], w[2], w[3], lp, lm, g);
    double diff = 0.0, scale = 0.0;
    for (int kk = 1; kk <= 3; kk++) {
      D1 x[5], vp, vm;
      for (int q = 0; q < 5; q++) x[q] = D1(w[q]);
      x[kk].d[0] = 1.0;
      recon_pt(PG_LINEAR, lim, nv, x, vp, vm);
      const double ref = lp * vp.d[0] + lm * vm.d[0];
      scale = fmax(scale, fabs(ref));
      diff = fmax(diff, fabs(g[kk - 1] - ref));
    }
    branches[(w[3] - w[2]) * (w[2] - w[1]) > 0.0 ? 1 : 0]++;
    const double rel = scale > 0.0 ? diff / scale : diff;
    if (!(rel <= worst)) worst = rel;
  }
  return worst;
}

// PPM states (interface values with the minmod clip, parabolic limiter)
// transposed; branches counted: limiter case (none / flat / vp clipped / vm
// clipped)
static double check_ppm(int nsamp, long* branches) {
  double worst = 0.0;
  for (int t = 0; t < nsamp; t++) {
    double w[5];
    for (int q = 0; q < 5; q++) w[q] = urange(-1.0, 1.0);
    if (t % 3 == 0)  // smooth profiles: the unclipped and one-sided branches
      for (int q = 0; q < 5; q++) w[q] = 0.2 * q + 0.05 * q * q * (t % 2 ? 1.0 : -1.0) + urange(0.0, 0.02);
    const double lp = urange(-1.0, 1.0), lm = urange(-1.0, 1.0);
    double g[5];
    ppm_rev(w, lp, lm, g);
    double diff = 0.0, scale = 0.0;
    for (int kk = 0; kk < 5; kk++) {
      D1 x[5], vp, vm;
      for (int q = 0; q < 5; q++) x[q] = D1(w[q]);
      x[kk].d[0] = 1.0;
      recon_pt(PG_PARABOLIC, 0, 0, x, vp, vm);
      const double ref = lp * vp.d[0] + lm * vm.d[0];
      scale = fmax(scale, fabs(ref));
      diff = fmax(diff, fabs(g[kk] - ref));
    }
    const double p = ppm_iface(w[1], w[2], w[3], w[4]) - w[2], m = ppm_iface(w[0], w[1], w[2], w[3]) - w[2];
    branches[p * m >= 0.0 ? 0 : (::fabs(p) >= 2.0 * ::fabs(m) ? 1 : (::fabs(m) >= 2.0 * ::fabs(p) ? 2 : 3))]++;
    const double rel = scale > 0.0 ? diff / scale : diff;
    if (!(rel <= worst)) worst = rel;
  }
  return worst;
}

// prim->cons and cons->prim (with the density, energy and pressure floors)
// transposed; branches counted: no floor / density / energy / pressure
static double check_maps(int nsamp, long* branches) {
  double worst = 0.0;
  const double gamma = 5.0 / 3.0, gmm1 = gamma - 1.0, small_rho = 1e-12, small_p = 1e-12;
  for (int t = 0; t < nsamp; t++) {
    double v[NV], u[NV], lam[NV], g[NV];
    for (int nv = 0; nv < NV; nv++) v[nv] = urange(-2.0, 2.0);
    v[RHO] = urange(0.2, 5.0);
    v[PRS] = urange(0.05, 5.0);
    for (int nv = 0; nv < NV; nv++) lam[nv] = urange(-1.0, 1.0);
    // prim -> cons
    for (int nv = 0; nv < NV; nv++) g[nv] = 0.0;
    p2c_rev(v, gmm1, lam, g);
    double diff = 0.0, scale = 0.0;
    for (int kk = 0; kk < NV; kk++) {
      D1 x[NV], y[NV];
      for (int q = 0; q < NV; q++) x[q] = D1(v[q]);
      x[kk].d[0] = 1.0;
      prim_to_cons(x, y, D1(gmm1));
      double ref = 0.0;
      for (int q = 0; q < NV; q++) ref += lam[q] * y[q].d[0];
      scale = fmax(scale, fabs(ref));
      diff = fmax(diff, fabs(g[kk] - ref));
    }
    // cons -> prim from a state that may need a floor
    prim_to_cons(v, u, gmm1);
    const int kind = t % 4;
    if (kind == 1) u[RHO] = -urange(0.01, 1.0);
    if (kind == 2) u[ENG] = -urange(0.01, 1.0);
    if (kind == 3) u[ENG] = 0.5 * (u[MX1] * u[MX1] + u[MX1 + 1] * u[MX1 + 1] + u[MX1 + 2] * u[MX1 + 2]) / u[RHO] +
                            0.5 * (u[BX1] * u[BX1] + u[BX2] * u[BX2] + u[BX3] * u[BX3]) - urange(0.01, 1.0);
    c2p_rev(u, gmm1, small_rho, lam, g);
    int fl_kind = 0;
    for (int kk = 0; kk < NV; kk++) {
      D1 x[NV], y[NV];
      for (int q = 0; q < NV; q++) x[q] = D1(u[q]);
      x[kk].d[0] = 1.0;
      unsigned char fl = 0;
      cons_to_prim(x, y, D1(gmm1), D1(small_rho), D1(small_p), &fl);
      double ref = 0.0;
      for (int q = 0; q < NV; q++) ref += lam[q] * y[q].d[0];
      scale = fmax(scale, fabs(ref));
      diff = fmax(diff, fabs(g[kk] - ref));
      if (fl) fl_kind = kind;
    }
    branches[fl_kind]++;
    const double rel = scale > 0.0 ? diff / scale : diff;
    if (!(rel <= worst)) worst = rel;
  }
  return worst;
}

int main(int argc, char** argv) {
  const int nsamp = argc > 1 ? atoi(argv[1]) : 20000;
  const double gamma = 5.0 / 3.0;
  for (int solver : {PG_HLLD, PG_HLL}) {
    for (int dir = 0; dir < 3; dir++) {
      long reg[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      const double w = dir == 0   ? check_riemann<0>(solver, gamma, nsamp, reg)
                       : dir == 1 ? check_riemann<1>(solver, gamma, nsamp, reg)
                                  : check_riemann<2>(solver, gamma, nsamp, reg);
      printf("riemann %s dir %d samples %d regions %ld %ld %ld %ld %ld %ld %ld %ld worst %.3e\n",
             solver == PG_HLLD ? "hlld" : "hll", dir, nsamp, reg[0], reg[1], reg[2], reg[3], reg[4], reg[5],
             reg[6], reg[7], w);
    }
  }
  long br[3] = {0, 0, 0};
  const double w = check_emf(nsamp, br);
  printf("emf samples %d branches %ld %ld %ld worst %.3e\n", nsamp, br[0], br[1], br[2], w);
  long bp[2] = {0, 0};
  const double wp = check_plm(nsamp, bp);
  printf("plm samples %d branches %ld %ld worst %.3e\n", nsamp, bp[0], bp[1], wp);
  long bq[4] = {0, 0, 0, 0};
  const double wq = check_ppm(nsamp, bq);
  printf("ppm samples %d branches %ld %ld %ld %ld worst %.3e\n", nsamp, bq[0], bq[1], bq[2], bq[3], wq);
  long bm[4] = {0, 0, 0, 0};
  const double wm = check_maps(nsamp, bm);
  printf("maps samples %d branches %ld %ld %ld %ld worst %.3e\n", nsamp, bm[0], bm[1], bm[2], bm[3], wm);
  return 0;
}
