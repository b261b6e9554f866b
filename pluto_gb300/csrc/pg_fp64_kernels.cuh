// FP64-path kernels templated on the value type T: T = double is the plain
// FP64 path (bit-compatible with the reference C code when compiled without
// FMA contraction); T = Dual<1> runs the same step as its tangent-linear
// model (pg_adjoint.cu).  See pg_fp64.cu for the reference map.
#pragma once
#include <cstdio>
#include <cstring>

#include "pg_internal.h"
#include "pg_physics.cuh"
#include "pg_dual.cuh"
#include "pg_bound_ct.cuh"
#include "pg_char.cuh"

namespace pg {

template <class T>
struct F64A {
  Geom g;
  T* V[8];
  T* U[8];
  T* U0[8];
  T* Bs[3];
  T* Bs0[3];
  T* VP[8];
  T* VM[8];
  T* F[8];
  T* P;
  T* CM;
  T* SL[3];
  T* SR[3];
  T* DV[3][3];
  T* E[3];
  T* Bm1[3];  // face -1 layers: Bm1[0][k][j], Bm1[1][k][i], Bm1[2][j][i]
  T* Upd[3][8];
  T* Umd[3][8];
  T* Rhd[3][8];
  T* Uh[8];
  T* EF[6];
  signed char* SV[3];
  T* CDT;
  unsigned char* flag;
  DevScalars* sc;
  double gamma, small_rho, small_p, cfl, cfl_max_var;
  int limiter, recon, ct, nbfield, ncomp;
  int device_dt;
  int bc[3];
  int ct_outflow;   // constrained transport with a non-periodic axis: per-axis boundary passes
  int intb;         // INTERNAL_BOUNDARY: flagged zones are not updated
  int div_dims;     // RK: invDt_hyp /= DIMENSIONS (update_stage.c:311); CTU: no
  int emf_avg, c3;
  int chtr;         // CTU predictor: characteristic tracing (else primitive Hancock)
  int cons_hancock; // CTU predictor: conservative Hancock step (PRIMITIVE_HANCOCK NO)
  int char_lim;     // CHAR_LIMITING YES: PLM limited in characteristic variables
};

// face-EMF slots of F64A::EF: ezi, ezj, eyi, eyk, exj, exk
enum : int { EF_ZI = 0, EF_ZJ, EF_YI, EF_YK, EF_XJ, EF_XK };

// CT_StoreUpwindEMF (Src/MHD/CT/ct_emf.c:104-190) for the ARITHMETIC, UCT0
// and UCT_CONTACT averages: the EMF components of the face flux and the sign
// of its mass flux (the UCT_CONTACT upwind direction, threshold 1e-6).
template <class T, int DIR>
__device__ __forceinline__ void store_face_emf(const F64A<T>& a, long long c, const T* f) {
  if (DIR == 0) {
    a.EF[EF_ZI][c] = -f[BX2];
    if (a.g.dims == 3) a.EF[EF_YI][c] = f[BX3];
  } else if (DIR == 1) {
    a.EF[EF_ZJ][c] = f[BX1];
    if (a.g.dims == 3) a.EF[EF_XJ][c] = -f[BX3];
  } else {
    a.EF[EF_YK][c] = -f[BX1];
    a.EF[EF_XK][c] = f[BX2];
  }
  const double fr = value_of(f[RHO]);
  a.SV[DIR][c] = fr > 1.e-6 ? 1 : (fr < -1.e-6 ? -1 : 0);
}

__device__ __forceinline__ void atomic_max_nonneg(unsigned long long* addr, double v) {
  // Non-negative doubles (and NaN) order like their bit patterns.
  atomicMax(addr, (unsigned long long)__double_as_longlong(v));
}

__device__ __forceinline__ double block_max(double v) {
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  // fmax drops NaN; keep NaN visible by a separate test below
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    v = (lane < (int)(blockDim.x >> 5)) ? red[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  }
  return v;
}

// ---------------------------------------------------------------------------
// Boundary: single pass over all ghost cells; the source index applies the
// per-axis map (periodic wrap or outflow clamp) on every axis, which equals
// the reference's side-by-side sequence (Src/boundary.c:137-300) because the
// maps are pure copies that compose axis by axis.  With faces stored on the
// +1/2 side of their cell, the periodic map of a staggered array is the same
// as the cell map (the face beg-1 receives face end, as in
// Src/boundary.c:482-522 applied to the X1FACE box).
// ---------------------------------------------------------------------------
__device__ __forceinline__ int bmap(int x, int beg, int end, int n, int type) {
  return bc_src(x, beg, end, n, type);
}

template <class T>
__global__ void k_bound(F64A<T> a, int bcx, int bcy, int bcz, GhostSlabs gs) {
  const Geom& g = a.g;
  long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  int i, j, k;
  if (!gs.coords(g, q, i, j, k)) return;
  int si = g.dims > 0 ? bmap(i, g.beg[0], g.end[0], g.nx[0], bcx) : i;
  int sj = g.dims > 1 ? bmap(j, g.beg[1], g.end[1], g.nx[1], bcy) : j;
  int sk = g.dims > 2 ? bmap(k, g.beg[2], g.end[2], g.nx[2], bcz) : k;
  long long dst = cidx(g, k, j, i), src = cidx(g, sk, sj, si);
  // reflective / equatorial-symmetric axes mirror with the FlipSign signs,
  // one factor per axis whose ghost region holds this zone
  const int bt[3] = {bcx, bcy, bcz};
  const int x[3] = {i, j, k};
  int flips = 0;  // bit nv set: variable nv changes sign
#pragma unroll
  for (int d = 0; d < 3; d++) {  // compile-time axis indices keep x, bt in registers
    if (d >= g.dims) break;
    if (x[d] < g.beg[d] || x[d] > g.end[d])
#pragma unroll
      for (int nv = 0; nv < NV; nv++)
        if (bc_flip(d, bc_side(bt[d], x[d] > g.end[d]), nv, a.ncomp) < 0) flips ^= 1 << nv;
  }
#pragma unroll
  for (int nv = 0; nv < NV; nv++) {
    const T v = a.V[nv][src];
    a.V[nv][dst] = ((flips >> nv) & 1) ? -v : v;
  }
  for (int d = 0; d < a.nbfield; d++) a.Bs[d][dst] = a.Bs[d][src];
}

// Stage-1 prologue: U = U0 = PrimToCons(V) over the domain (rk_step.c:93-96),
// Bs0 = Vs everywhere (:98-100), flags cleared (Src/main.c:329).
template <class T>
__global__ void k_begin_step(F64A<T> a, Box dom) {
  long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const Geom& g = a.g;
  if (q < g.ncell) {
    if (!a.intb) a.flag[q] = 0;  // with internal boundaries: cleared before the first fill
    for (int d = 0; d < a.nbfield; d++) a.Bs0[d][q] = a.Bs[d][q];
  }
  if (q == 0) {
    a.sc->inv_dt_bits = 0ull;
    a.sc->mach_bits = 0ull;
    a.sc->nfail = 0ull;
  }
  if (q >= dom.count()) return;
  int i, j, k;
  dom.coords(q, i, j, k);
  long long c = cidx(g, k, j, i);
  T v[NV], u[NV];
#pragma unroll
  for (int nv = 0; nv < NV; nv++) v[nv] = a.V[nv][c];
  prim_to_cons(v, u, T(a.gamma - 1.0));
#pragma unroll
  for (int nv = 0; nv < NV; nv++) {
    a.U[nv][c] = u[nv];
    a.U0[nv][c] = u[nv];
  }
}

// Reconstruction of one cell along DIR: left/right states and velocity slopes.
template <class T, int DIR>
__global__ void k_recon(F64A<T> a, Box box) {
  long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= box.count()) return;
  int i, j, k;
  box.coords(q, i, j, k);
  const Geom& g = a.g;
  const long long c = cidx(g, k, j, i), s = g.s[DIR];
  T vp[NV], vm[NV];
  bool done = false;
  if constexpr (std::is_same<T, double>::value) {
    if (a.char_lim && a.recon == PG_PARABOLIC) {  // CHAR_LIMITING YES, ppm_states.c:258-560
      double w2[NV], w1[NV], v0[NV], e1[NV], e2[NV];
#pragma unroll
      for (int nv = 0; nv < NV; nv++) {
        w2[nv] = a.V[nv][c - 2 * s];
        w1[nv] = a.V[nv][c - s];
        v0[nv] = a.V[nv][c];
        e1[nv] = a.V[nv][c + s];
        e2[nv] = a.V[nv][c + 2 * s];
      }
      ppm_char<DIR>(w2, w1, v0, e1, e2, a.gamma, a.c3 != 0, g.dims, vp, vm);
      done = true;
    } else if (a.char_lim) {  // CHAR_LIMITING YES, plm_states.c:446-705
      double vl[NV], v0[NV], vr[NV];
#pragma unroll
      for (int nv = 0; nv < NV; nv++) {
        vl[nv] = a.V[nv][c - s];
        v0[nv] = a.V[nv][c];
        vr[nv] = a.V[nv][c + s];
      }
      plm_char<DIR>(vl, v0, vr, a.gamma, a.limiter, a.c3 != 0, g.dims, vp, vm);
      done = true;
    }
  }
  if (done) {
  } else if (a.recon == PG_LINEAR) {
#pragma unroll
    for (int nv = 0; nv < NV; nv++) {
      const T* V = a.V[nv];
      T v0 = V[c];
      T dvp = V[c + s] - v0;
      T dvm = v0 - V[c - s];
      T dv = limit(a.limiter, nv, dvp, dvm);
      vp[nv] = v0 + dv * 0.5;
      vm[nv] = v0 - dv * 0.5;
    }
  } else {
#pragma unroll
    for (int nv = 0; nv < NV; nv++) {
      const T* V = a.V[nv];
      T w2 = V[c - 2 * s], w1 = V[c - s], v0 = V[c], e1 = V[c + s], e2 = V[c + 2 * s];
      T p = ppm_iface(w1, v0, e1, e2);  // interface c+1/2
      T m = ppm_iface(w2, w1, v0, e1);  // interface c-1/2
      ppm_limit(v0, p, m);
      vp[nv] = p;
      vm[nv] = m;
    }
  }
#pragma unroll
  for (int nv = 0; nv < NV; nv++) {
    a.VP[nv][c] = vp[nv];
    a.VM[nv][c] = vm[nv];
  }
  if (a.ct) {  // compile-time indices keep vp/vm in registers
#pragma unroll
    for (int comp = 0; comp < 3; comp++)
      if (comp < g.dims) a.DV[DIR][comp][c] = vp[VX1 + comp] - vm[VX1 + comp];
  }
}

// Riemann problem at interface c+1/2 along DIR.
template <class T, int DIR, int SOLVER, bool MACH>
__global__ void k_riemann(F64A<T> a, Box box, int want_invdt_1d) {
  long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  double invdt = 0.0, mach = 0.0;
  T machT = T(0.0);
  if (q < box.count()) {
    int i, j, k;
    box.coords(q, i, j, k);
    const Geom& g = a.g;
    const long long c = cidx(g, k, j, i), s = g.s[DIR];
    T vL[NV], vR[NV], uL[NV], uR[NV];
#pragma unroll
    for (int nv = 0; nv < NV; nv++) {
      vL[nv] = a.VP[nv][c];
      vR[nv] = a.VM[nv][c + s];
    }
    if (a.ct) {  // face-centred normal field, plm_states.c:271-275
      T bn = a.Bs[DIR][c];
      vL[Rot<DIR>::bn] = bn;
      vR[Rot<DIR>::bn] = bn;
    }
    const T gmm1 = T(a.gamma - 1.0);
    prim_to_cons(vL, uL, gmm1);
    prim_to_cons(vR, uR, gmm1);
    Iface<T> o;
    if (SOLVER == PG_HLL) {
      hll_solver<DIR, MACH>(vL, uL, vR, uR, T(a.gamma), o, machT);
    } else if (SOLVER == PG_ROE) {
      int bad = 0;
      roe_solver<DIR, MACH>(vL, uL, vR, uR, T(a.gamma), a.ncomp == 3, o, machT, bad);
      if (bad) atomicOr(&a.sc->status, 2);
    } else {
      hlld_solver<DIR, MACH>(vL, uL, vR, uR, T(a.gamma), o, machT);
    }
    mach = value_of(machT);
#pragma unroll
    for (int nv = 0; nv < NV; nv++) a.F[nv][c] = o.f[nv];
    a.P[c] = o.press;
    a.CM[c] = o.cmax;
    if (a.ct) {
      a.SL[DIR][c] = pmax(T(0.0), -o.SL);
      a.SR[DIR][c] = pmax(T(0.0), o.SR);
      if (a.emf_avg != PG_UCT_HLL) store_face_emf<T, DIR>(a, c, o.f);
    }
    if (want_invdt_1d) invdt = value_of(o.cmax) * g.inv_dx[DIR];  // update_stage.c:237-241
  }
  if (want_invdt_1d) {
    double m = block_max(invdt);
    if (threadIdx.x == 0) atomic_max_nonneg(&a.sc->inv_dt_bits, m);
  }
  if (MACH) {
    __syncthreads();
    double m = block_max(mach);
    if (threadIdx.x == 0) atomic_max_nonneg(&a.sc->mach_bits, m);
  }
}

// U += rhs along DIR; C_dt accumulation on stage 1.
template <class T, int DIR>
__global__ void k_update(F64A<T> a, Box box, int cdt_mode) {
  long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= box.count()) return;
  int i, j, k;
  box.coords(q, i, j, k);
  const Geom& g = a.g;
  const long long c = cidx(g, k, j, i), s = g.s[DIR];
  const double dt = a.sc->dt;
  const double scrh = dt / g.dx[DIR];
  // InternalBoundaryReset (Src/int_bound_reset.c:33-37): no update in
  // zones of an internal boundary
  const bool frozen = a.intb && (a.flag[c] & PG_FLAG_INTERNAL_BOUNDARY);
#pragma unroll
  for (int nv = 0; nv < NV; nv++) {
    T rhs = -scrh * (a.F[nv][c] - a.F[nv][c - s]);
    if (nv == Rot<DIR>::vn) rhs -= scrh * (a.P[c] - a.P[c - s]);
    if (frozen) rhs = 0.0;
    a.U[nv][c] += rhs;
  }
  if (cdt_mode) {
    T term = 0.5 * (a.CM[c - s] + a.CM[c]) * g.inv_dx[DIR];
    if (cdt_mode == 1) a.CDT[c] = term;  // first direction: C_dt was zeroed
    else a.CDT[c] += term;
  }
}

// Edge EMF along axis E (Ez at (i+1/2,j+1/2,k) etc.), UCT_HLL average.
template <class T, int E>
__device__ __forceinline__ T uct_edge(const F64A<T>& a, long long c) {
  constexpr int AX = E == 2 ? 0 : (E == 0 ? 1 : 2);
  constexpr int AY = E == 2 ? 1 : (E == 0 ? 2 : 0);
  const Geom& g = a.g;
  const long long sx = g.s[AX], sy = g.s[AY];
  const long long c00 = c, cx0 = c + sx, c0y = c + sy, cxy = c + sx + sy;
  T a_xp = pmax(a.SR[AX][c00], a.SR[AX][c0y]);
  T a_xm = pmax(a.SL[AX][c00], a.SL[AX][c0y]);
  T a_yp = pmax(a.SR[AY][c00], a.SR[AY][cx0]);
  T a_ym = pmax(a.SL[AY][c00], a.SL[AY][cx0]);
  const T* bxa = a.Bs[AX];
  const T* bya = a.Bs[AY];
  // CT_GetStagSlopes, ct_stag_slopes.c:51-89: slope of the x-face field along y
  // and of the y-face field along x.
  T sbS = mc_lim2(bxa[c00 + sy] - bxa[c00], bxa[c00] - bxa[c00 - sy]);
  T sbN = mc_lim2(bxa[c0y + sy] - bxa[c0y], bxa[c0y] - bxa[c0y - sy]);
  T sbW = mc_lim2(bya[c00 + sx] - bya[c00], bya[c00] - bya[c00 - sx]);
  T sbE = mc_lim2(bya[cx0 + sx] - bya[cx0], bya[cx0] - bya[cx0 - sx]);
  T bS = bxa[c00] + 0.5 * sbS;
  T bW = bya[c00] + 0.5 * sbW;
  T bN = bxa[c0y] - 0.5 * sbN;
  T bE = bya[cx0] - 0.5 * sbE;
  const T* vx = a.V[VX1 + AX];
  const T* vy = a.V[VX1 + AY];
  const T* dvx_dx = a.DV[AX][AX];
  const T* dvx_dy = a.DV[AY][AX];
  const T* dvy_dx = a.DV[AX][AY];
  const T* dvy_dy = a.DV[AY][AY];
  T eSW = (vy[c00] + 0.5 * (dvy_dx[c00] + dvy_dy[c00])) * bS - (vx[c00] + 0.5 * (dvx_dx[c00] + dvx_dy[c00])) * bW;
  T eSE = (vy[cx0] - 0.5 * (dvy_dx[cx0] - dvy_dy[cx0])) * bS - (vx[cx0] - 0.5 * (dvx_dx[cx0] - dvx_dy[cx0])) * bE;
  T eNE = (vy[cxy] - 0.5 * (dvy_dx[cxy] + dvy_dy[cxy])) * bN - (vx[cxy] - 0.5 * (dvx_dx[cxy] + dvx_dy[cxy])) * bE;
  T eNW = (vy[c0y] + 0.5 * (dvy_dx[c0y] - dvy_dy[c0y])) * bN - (vx[c0y] + 0.5 * (dvx_dx[c0y] - dvx_dy[c0y])) * bW;
  return uct_hll_combine(a_xp, a_xm, a_yp, a_ym, eSW, eSE, eNE, eNW, bS, bN, bW, bE);
}

template <class T>
__global__ void k_emf(F64A<T> a, Box box) {
  long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= box.count()) return;
  int i, j, k;
  box.coords(q, i, j, k);
  long long c = cidx(a.g, k, j, i);
  a.E[2][c] = uct_edge<T, 2>(a, c);
  if (a.g.dims == 3) {
    a.E[0][c] = uct_edge<T, 0>(a, c);
    a.E[1][c] = uct_edge<T, 1>(a, c);
  }
}

// CT_Update fused with the RK face combination of stages 2 and 3.
template <class T, int STAGE, int NSTAGE>
__global__ void k_ct_update(F64A<T> a, Box box) {
  long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= box.count()) return;
  int i, j, k;
  box.coords(q, i, j, k);
  const Geom& g = a.g;
  const long long c = cidx(g, k, j, i);
  const double dt = a.sc->dt;
  const double dx1 = g.dx[0], dx2 = g.dx[1], dx3 = g.dx[2];
  const T* Ex1 = a.E[0];
  const T* Ex2 = a.E[1];
  const T* Ex3 = a.E[2];
  const bool d3 = g.dims == 3;
  const int kb = d3 ? g.beg[2] : 0, ke = d3 ? g.end[2] : 0;
  for (int fd = 0; fd < g.dims; fd++) {
    // face ranges, ct_update.c:79-81, 132-134, 188-190
    bool in = true;
    for (int ax = 0; ax < g.dims; ax++) {
      int x = ax == 0 ? i : (ax == 1 ? j : k);
      int lo = g.beg[ax] - (ax == fd ? 1 : 0), hi = g.end[ax];
      in = in && x >= lo && x <= hi;
    }
    if (!d3) in = in && k == 0;
    (void)kb;
    (void)ke;
    if (!in) continue;
    T rhs;
    if (fd == 0) {
      if (!d3) rhs = 0.0 - dt / dx2 * (Ex3[c] - Ex3[c - g.s[1]]);
      else rhs = 0.0 - dt / dx2 * (Ex3[c] - Ex3[c - g.s[1]]) + dt / dx3 * (Ex2[c] - Ex2[c - g.s[2]]);
    } else if (fd == 1) {
      if (!d3) rhs = dt / dx1 * (Ex3[c] - Ex3[c - 1]);
      else rhs = dt / dx1 * (Ex3[c] - Ex3[c - 1]) - dt / dx3 * (Ex1[c] - Ex1[c - g.s[2]]);
    } else {
      rhs = -dt / dx1 * (Ex2[c] - Ex2[c - 1]) + dt / dx2 * (Ex1[c] - Ex1[c - g.s[1]]);
    }
    T b = a.Bs[fd][c] + rhs;
    if (STAGE == 2) {
      const double w0 = NSTAGE == 3 ? 0.75 : 0.5, wc = NSTAGE == 3 ? 0.25 : 0.5;
      b = w0 * a.Bs0[fd][c] + wc * b;
    } else if (STAGE == 3) {
      b = (a.Bs0[fd][c] + 2.0 * b) / 3.0;
    }
    a.Bs[fd][c] = b;
  }
}

// End of a stage: RK combination, face average, ConsToPrim, dt reduction.
template <class T, int STAGE, int NSTAGE>
__global__ void k_finalize(F64A<T> a, Box dom, int reduce_cdt) {
  long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  double cd = 0.0;
  unsigned long long fails = 0;
  bool bad = false;
  if (q < dom.count()) {
    int i, j, k;
    dom.coords(q, i, j, k);
    const Geom& g = a.g;
    const long long c = cidx(g, k, j, i);
    T u[NV], v[NV];
#pragma unroll
    for (int nv = 0; nv < NV; nv++) u[nv] = a.U[nv][c];
    if (STAGE == 2) {
      const double w0 = NSTAGE == 3 ? 0.75 : 0.5, wc = NSTAGE == 3 ? 0.25 : 0.5;
#pragma unroll
      for (int nv = 0; nv < NV; nv++) u[nv] = w0 * a.U0[nv][c] + wc * u[nv];
    } else if (STAGE == 3) {
      const double one_third = 1.0 / 3.0;
#pragma unroll
      for (int nv = 0; nv < NV; nv++) u[nv] = one_third * (a.U0[nv][c] + 2.0 * u[nv]);
    }
    if (a.ct) {
#pragma unroll
      for (int d = 0; d < 3; d++)
        if (d < g.dims) u[BX1 + d] = 0.5 * (a.Bs[d][c] + a.Bs[d][c - g.s[d]]);
    }
    unsigned char fl = a.flag[c];
    fails = cons_to_prim(u, v, T(a.gamma - 1.0), T(a.small_rho), T(a.small_p), &fl);
    if (fails) a.flag[c] |= fl;  // flag[i] |= FLAG_CONS2PRIM_FAIL (mappers.c)
#pragma unroll
    for (int nv = 0; nv < NV; nv++) {
      a.U[nv][c] = u[nv];
      a.V[nv][c] = v[nv];
      // CheckNaN equivalent (Src/tools.c:20): exponent all ones = Inf/NaN
      bad |= ((__double_as_longlong(value_of(v[nv])) >> 52) & 0x7ff) == 0x7ff;
    }
    if (reduce_cdt) cd = value_of(a.CDT[c]);
  }
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(&a.sc->status, 1);
  if (reduce_cdt) {
    double m = block_max(cd);
    if (threadIdx.x == 0) atomic_max_nonneg(&a.sc->inv_dt_bits, m);
  }
  unsigned ball = __ballot_sync(0xffffffffu, fails != 0);
  if ((threadIdx.x & 31) == 0 && ball) atomicAdd(&a.sc->nfail, (unsigned long long)__popc(ball));
}

// NextTimeStep (Src/main.c:459-532): next dt from the reduced invDt.
template <class T>
__global__ void k_end_step(F64A<T> a) {
  DevScalars* sc = a.sc;
  double inv = __longlong_as_double((long long)sc->inv_dt_bits);
  if (a.div_dims && a.g.dims > 1) inv /= (double)a.g.dims;  // update_stage.c:311
  sc->inv_dt_bits = (unsigned long long)__double_as_longlong(inv);
  if (!(inv == inv) || inv > 1e300) sc->status |= 1;  // NaN / inf guard
  if (a.device_dt) {
    double dt = sc->dt;
    sc->time += dt;
    double dt_hyp = 1.0 / inv;
    dt_hyp *= a.cfl;
    double dtnext = dt_hyp;
    dtnext = pmin(dtnext, a.cfl_max_var * dt);
    sc->dt_prev = dt;
    sc->dt = dtnext;
  }
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------

template <class T>
static F64A<T> make_args(Solver* S) {
  F64A<T> a;
  memset(&a, 0, sizeof a);
  a.g = S->g;
  for (int nv = 0; nv < 8; nv++) {
    a.V[nv] = (T*)S->V[nv];
    a.U[nv] = (T*)S->U[nv];
    a.U0[nv] = (T*)S->U0[nv];
    a.VP[nv] = (T*)S->VP[nv];
    a.VM[nv] = (T*)S->VM[nv];
    a.F[nv] = (T*)S->F[nv];
  }
  for (int d = 0; d < 3; d++) {
    a.Bs[d] = (T*)S->Bs[d];
    a.Bs0[d] = (T*)S->Bs0[d];
    a.SL[d] = (T*)S->SL[d];
    a.SR[d] = (T*)S->SR[d];
    a.E[d] = (T*)S->E[d];
    for (int c = 0; c < 3; c++) a.DV[d][c] = (T*)S->DV[d][c];
  }
  a.P = (T*)S->P;
  a.CM = (T*)S->CM;
  a.CDT = (T*)S->CDT;
  a.flag = S->flag;
  a.sc = S->sc;
  a.gamma = S->cfg.gamma;
  a.small_rho = S->cfg.small_density > 0 ? S->cfg.small_density : 1.e-12;
  a.small_p = S->cfg.small_pressure > 0 ? S->cfg.small_pressure : 1.e-12;
  a.cfl = S->cfl;
  a.cfl_max_var = S->cfl_max_var;
  a.limiter = S->cfg.limiter;
  a.recon = S->cfg.reconstruction;
  a.ct = S->cfg.divb == PG_CONSTRAINED_TRANSPORT;
  a.nbfield = a.ct ? S->g.dims : 0;
  a.ncomp = S->cfg.components;
  for (int d = 0; d < 3; d++) {
    a.Bm1[d] = (T*)S->Bm1[d];
    a.bc[d] = S->cfg.bc[d];
  }
  for (int d = 0; d < 3; d++)
    for (int nv = 0; nv < 8; nv++) {
      a.Upd[d][nv] = (T*)S->Upd[d][nv];
      a.Umd[d][nv] = (T*)S->Umd[d][nv];
      a.Rhd[d][nv] = (T*)S->Rhd[d][nv];
    }
  for (int nv = 0; nv < 8; nv++) a.Uh[nv] = (T*)S->Uh[nv];
  for (int q = 0; q < 6; q++) a.EF[q] = (T*)S->EF[q];
  for (int d = 0; d < 3; d++) a.SV[d] = S->SV[d];
  a.div_dims = !is_ctu(S->cfg.time_stepping);
  a.chtr = S->cfg.time_stepping == PG_CHAR_TRACING;
  a.cons_hancock = S->cfg.time_stepping == PG_HANCOCK_CONS;
  a.char_lim = S->cfg.char_limiting;
  a.emf_avg = S->cfg.emf_average;
  a.c3 = S->cfg.components == 3;
  a.intb = S->ud_internal ? 1 : 0;
  a.ct_outflow = 0;
  if (a.ct)
    for (int d = 0; d < S->g.dims; d++) a.ct_outflow |= S->cfg.bc[d] != PG_PERIODIC;

  a.device_dt = S->device_dt;
  return a;
}

static Box sweep_box(const Geom& g, int dir, int along_lo_off, int along_hi_off, bool ct) {
  Box b;
  for (int ax = 0; ax < 3; ax++) {
    if (ax >= g.dims) { b.lo[ax] = b.hi[ax] = 0; continue; }
    if (ax == dir) {
      b.lo[ax] = g.beg[ax] + along_lo_off;
      b.hi[ax] = g.end[ax] + along_hi_off;
    } else {
      int ext = ct ? 1 : 0;  // transverse extension, update_stage.c:144-148
      b.lo[ax] = g.beg[ax] - ext;
      b.hi[ax] = g.end[ax] + ext;
    }
  }
  return b.prepare();
}

template <class T, int DIR>
static void launch_sweep(Solver* S, const F64A<T>& a, int stage) {
  const Geom& g = S->g;
  const bool ct = a.ct;
  cudaStream_t st = S->stream;
  Box rb = sweep_box(g, DIR, -1, +1, ct);  // States on nbeg-1..nend+1
  PG_LAUNCH(S, "fp64_recon", (k_recon<T, DIR><<<grid_for(rb.count()), kThreads, 0, st>>>(a, rb)));
  Box ib = sweep_box(g, DIR, -1, 0, ct);   // Riemann on nbeg-1..nend
  int want1d = g.dims == 1;
  const bool mach = S->cfg.compute_mach != 0;
  unsigned gr = grid_for(ib.count(), 128);
  PG_LAUNCH(S, "fp64_riemann", {
    if (S->cfg.riemann == PG_HLL) {
      if (mach) k_riemann<T, DIR, PG_HLL, true><<<gr, 128, 0, st>>>(a, ib, want1d);
      else k_riemann<T, DIR, PG_HLL, false><<<gr, 128, 0, st>>>(a, ib, want1d);
    } else if (S->cfg.riemann == PG_ROE) {
      if (mach) k_riemann<T, DIR, PG_ROE, true><<<gr, 128, 0, st>>>(a, ib, want1d);
      else k_riemann<T, DIR, PG_ROE, false><<<gr, 128, 0, st>>>(a, ib, want1d);
    } else {
      if (mach) k_riemann<T, DIR, PG_HLLD, true><<<gr, 128, 0, st>>>(a, ib, want1d);
      else k_riemann<T, DIR, PG_HLLD, false><<<gr, 128, 0, st>>>(a, ib, want1d);
    }
  });
  Box ub = sweep_box(g, DIR, 0, 0, ct);    // RHS/update on nbeg..nend
  int cdt_mode = (g.dims > 1 && stage == 1) ? (DIR == 0 ? 1 : 2) : 0;
  PG_LAUNCH(S, "fp64_update", (k_update<T, DIR><<<grid_for(ub.count()), kThreads, 0, st>>>(a, ub, cdt_mode)));
}

// edge EMFs from the stored face EMFs (pg_ctu.cuh)
template <class T, int STAGE>
__global__ void k_ctu_emf(F64A<T> a, Box eb);

template <class T, int STAGE, int NSTAGE>
static void launch_stage_tail(Solver* S, const F64A<T>& a, const Box& dom) {
  const Geom& g = S->g;
  cudaStream_t st = S->stream;
  if (a.ct) {
    Box eb;
    for (int ax = 0; ax < 3; ax++) {
      if (ax < g.dims) { eb.lo[ax] = g.beg[ax] - 1; eb.hi[ax] = g.end[ax]; }
      else { eb.lo[ax] = eb.hi[ax] = 0; }
    }
    eb.prepare();
    if (a.emf_avg == PG_UCT_HLL)
      PG_LAUNCH(S, "fp64_emf", (k_emf<T><<<grid_for(eb.count(), 128), 128, 0, st>>>(a, eb)));
    else  // every RK stage integrates to the corner like the CTU corrector (no CTU guard)
      PG_LAUNCH(S, "fp64_emf", (k_ctu_emf<T, 2><<<grid_for(eb.count(), 128), 128, 0, st>>>(a, eb)));
    PG_LAUNCH(S, "fp64_ct_update", (k_ct_update<T, STAGE, NSTAGE><<<grid_for(eb.count()), kThreads, 0, st>>>(a, eb)));
  }
  int reduce = (STAGE == 1 && g.dims > 1);
  PG_LAUNCH(S, "fp64_finalize", (k_finalize<T, STAGE, NSTAGE><<<grid_for(dom.count()), kThreads, 0, st>>>(a, dom, reduce)));
}

template <class T>
static void launch_bound(Solver* S, const F64A<T>& a) {
  const Geom& g = S->g;
  if (S->ud_internal) launch_internal_boundary<T>(S, a.V, a.Bs, a.Bm1, a.nbfield, a.flag);
  if (a.ct_outflow || has_userdef(S)) {
    BoundCT<T> b;
    b.g = a.g;
    for (int nv = 0; nv < 8; nv++) b.V[nv] = a.V[nv];
    for (int d = 0; d < 3; d++) {
      b.Bs[d] = a.Bs[d];
      b.Bm1[d] = a.Bm1[d];
    }
    b.nbfield = a.nbfield;
    b.ncomp = a.ncomp;
    face_areas(g, b.area);
    launch_bound_ct<T, T>(S, b, "fp64_bound", "fp64_fill_normal");
  } else {
    const GhostSlabs gs(g);
    PG_LAUNCH(S, "fp64_bound", (k_bound<T><<<grid_for(gs.count()), kThreads, 0, S->stream>>>(
                                     a, S->cfg.bc[0], S->cfg.bc[1], S->cfg.bc[2], gs)));
  }
  S->ud_stage++;  // boundary fills so far in the step (the callbacks' stage index)
}

template <class T, int NSTAGE>
static void enqueue_rk(Solver* S, const F64A<T>& a) {
  const Geom& g = S->g;
  Box dom;
  for (int ax = 0; ax < 3; ax++) { dom.lo[ax] = g.beg[ax]; dom.hi[ax] = g.end[ax]; }
  dom.prepare();
  cudaStream_t st = S->stream;
  // stage 1
  launch_bound(S, a);
  PG_LAUNCH(S, "fp64_begin_step", (k_begin_step<T><<<grid_for(g.ncell), kThreads, 0, st>>>(a, dom)));
  launch_sweep<T, 0>(S, a, 1);
  if (g.dims > 1) launch_sweep<T, 1>(S, a, 1);
  if (g.dims > 2) launch_sweep<T, 2>(S, a, 1);
  launch_stage_tail<T, 1, NSTAGE>(S, a, dom);
  // stage 2 (EULER: the predictor alone, rk_step.c:145)
  if (NSTAGE >= 2) {
    launch_bound(S, a);
    launch_sweep<T, 0>(S, a, 2);
    if (g.dims > 1) launch_sweep<T, 1>(S, a, 2);
    if (g.dims > 2) launch_sweep<T, 2>(S, a, 2);
    launch_stage_tail<T, 2, NSTAGE>(S, a, dom);
  }
  if (NSTAGE == 3) {
    launch_bound(S, a);
    launch_sweep<T, 0>(S, a, 3);
    if (g.dims > 1) launch_sweep<T, 1>(S, a, 3);
    if (g.dims > 2) launch_sweep<T, 2>(S, a, 3);
    launch_stage_tail<T, 3, NSTAGE>(S, a, dom);
  }
  PG_LAUNCH(S, "fp64_end_step", (k_end_step<T><<<1, 1, 0, st>>>(a)));
}


}  // namespace pg

#include "pg_ctu.cuh"

namespace pg {

template <class T>
int fp64_enqueue_step_t(Solver* S) {
  F64A<T> a = make_args<T>(S);
  if (is_ctu(S->cfg.time_stepping)) enqueue_ctu<T>(S, a);
  else if (S->cfg.time_stepping == PG_RK3) enqueue_rk<T, 3>(S, a);
  else if (S->cfg.time_stepping == PG_EULER) enqueue_rk<T, 1>(S, a);
  else enqueue_rk<T, 2>(S, a);
  return cudaGetLastError() == cudaSuccess ? PG_OK : PG_ERR_CUDA;
}

}  // namespace pg
