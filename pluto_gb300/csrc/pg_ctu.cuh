// Corner Transport Upwind step (PLUTO's TIME_STEPPING HANCOCK and
// CHARACTERISTIC_TRACING, Src/Time_Stepping/ctu_step.c:140-727) on the FP64
// path, templated on the value type like the RK kernels.  Predictor: per
// direction, PLM states evolved by dt/2 with the primitive MUSCL-Hancock step
// (Src/States/hancock.c:36-172, PrimRHS Src/MHD/prim_eqn.c:29-112) or by
// characteristic tracing (Src/States/char_tracing.c:280-573, plain FP64
// only), CheckPrimStates (Src/check_states.c:18-70), Riemann problems, rhs with dt/2,
// CTU_CT_Source (ctu_step.c:731-816).  Half step: U^{n+1/2} = U^n + sum of
// the rhs, face field by dt/2, ConsToPrim on the domain plus one ghost layer.
// Corrector: corner-coupled states U+- + the other directions' rhs, face
// normal field at n+1/2, ConsToPrim, Riemann problems, U += rhs with dt; face
// field from Bs^n with dt.  EMF at edges by the ARITHMETIC or UCT_CONTACT
// averages of the flux EMFs (Src/MHD/CT/ct_emf.c:104-291,
// ct_emf_average.c:13-164).  invDt_hyp is the maximum of cmax/dx over both
// passes (ctu_step.c:425,639), not divided by DIMENSIONS.
#pragma once
#include <type_traits>

namespace pg {

// PrimRHS (ideal EOS, no 8-wave / GLM terms): A(v) . dv along DIR
template <int DIR, class T>
__device__ __forceinline__ void prim_rhs(const T* v, const T* dv, double gamma, bool c3, T* Adv) {
  using R = Rot<DIR>;
  constexpr int vn = R::vn, vt = R::vt, vb = R::vb, bn = R::bn, bt = R::bt, bb = R::bb;
  const T tau = T(1.0) / v[RHO];
#pragma unroll
  for (int nv = 0; nv < NV; nv++) Adv[nv] = T(0.0);
  Adv[RHO] = v[vn] * dv[RHO] + v[RHO] * dv[vn];
  const T scrh = c3 ? T(0.0) + v[bt] * dv[bt] + v[bb] * dv[bb] : T(0.0) + v[bt] * dv[bt];
  Adv[vn] = v[vn] * dv[vn] + tau * (dv[PRS] + scrh);
  Adv[vt] = v[vn] * dv[vt] - tau * v[bn] * dv[bt];
  if (c3) Adv[vb] = v[vn] * dv[vb] - tau * v[bn] * dv[bb];
  Adv[bn] = T(0.0);
  Adv[bt] = v[bt] * dv[vn] - v[bn] * dv[vt] + v[vn] * dv[bt];
  if (c3) Adv[bb] = v[bb] * dv[vn] - v[bn] * dv[vb] + v[vn] * dv[bb];
  Adv[PRS] = gamma * v[PRS] * dv[vn] + v[vn] * dv[PRS];
}

template <class T>
__global__ void k_ctu_begin(F64A<T> a) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const Geom& g = a.g;
  if (q == 0) {
    a.sc->inv_dt_bits = 0ull;
    a.sc->mach_bits = 0ull;
    a.sc->nfail = 0ull;
  }
  if (q >= g.ncell) return;
  a.flag[q] = 0;
  for (int d = 0; d < a.nbfield; d++) a.Bs0[d][q] = a.Bs[d][q];
  T v[NV], u[NV];  // PrimToCons3D over the whole grid (ctu_step.c:246-247)
#pragma unroll
  for (int nv = 0; nv < NV; nv++) v[nv] = a.V[nv][q];
  prim_to_cons(v, u, T(a.gamma - 1.0));
#pragma unroll
  for (int nv = 0; nv < NV; nv++) a.U[nv][q] = u[nv];
}

// Normal predictors of one zone along DIR.
template <class T, int DIR>
__global__ void k_ctu_states(F64A<T> a, Box box) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= box.count()) return;
  int i, j, k;
  box.coords(q, i, j, k);
  const Geom& g = a.g;
  using R = Rot<DIR>;
  const long long c = cidx(g, k, j, i), s = g.s[DIR];
  const double dt2 = 0.5 * a.sc->dt;
  const double inv_dl = g.inv_dx[DIR];
  T v0[NV], vp[NV], vm[NV];
  bool limited = false;
  if constexpr (std::is_same<T, double>::value) {
    if (a.char_lim && a.recon == PG_PARABOLIC) {  // CHAR_LIMITING YES, ppm_states.c:258-560
      double w2[NV], w1[NV], e1[NV], e2[NV];
#pragma unroll
      for (int nv = 0; nv < NV; nv++) {
        w2[nv] = a.V[nv][c - 2 * s];
        w1[nv] = a.V[nv][c - s];
        v0[nv] = a.V[nv][c];
        e1[nv] = a.V[nv][c + s];
        e2[nv] = a.V[nv][c + 2 * s];
      }
      ppm_char<DIR>(w2, w1, v0, e1, e2, a.gamma, a.c3 != 0, g.dims, vp, vm);
      limited = true;
    } else if (a.char_lim) {  // CHAR_LIMITING YES, plm_states.c:446-705
      double vl[NV], vr[NV];
#pragma unroll
      for (int nv = 0; nv < NV; nv++) {
        vl[nv] = a.V[nv][c - s];
        v0[nv] = a.V[nv][c];
        vr[nv] = a.V[nv][c + s];
      }
      plm_char<DIR>(vl, v0, vr, a.gamma, a.limiter, a.c3 != 0, g.dims, vp, vm);
      limited = true;
    }
  }
  if (!limited && a.recon == PG_PARABOLIC) {  // PPM states (ppm_states.c:68-253), then CharTracingStep
#pragma unroll
    for (int nv = 0; nv < NV; nv++) {
      const T* V = a.V[nv];
      const T w2 = V[c - 2 * s], w1 = V[c - s], e1 = V[c + s], e2 = V[c + 2 * s];
      v0[nv] = V[c];
      T p = ppm_iface(w1, v0[nv], e1, e2);  // interface c+1/2
      T m = ppm_iface(w2, w1, v0[nv], e1);  // interface c-1/2
      ppm_limit(v0[nv], p, m);
      vp[nv] = p;
      vm[nv] = m;
    }
  } else if (!limited) {
#pragma unroll
    for (int nv = 0; nv < NV; nv++) {
      const T* V = a.V[nv];
      v0[nv] = V[c];
      T dvp = V[c + s] - v0[nv];
      T dvm = v0[nv] - V[c - s];
      T dv = limit(a.limiter, nv, dvp, dvm);
      vp[nv] = v0[nv] + dv * 0.5;
      vm[nv] = v0[nv] - dv * 0.5;
    }
  }
  if (a.ct) {  // plm_states.c:271-275
    vp[R::bn] = a.Bs[DIR][c];
    vm[R::bn] = a.Bs[DIR][c - s];
  }
  bool traced = false;
  if constexpr (std::is_same<T, double>::value) {
    if (a.chtr) {  // characteristic tracing, then the face field again (char_tracing.c:536-540)
      if (a.recon == PG_PARABOLIC)
        char_tracing_ppm<DIR>(v0, vp, vm, a.gamma, a.sc->dt / g.dx[DIR], a.sc->dt, a.c3 != 0, g.dims,
                              a.char_lim ? 2 : 3);
      else
        char_tracing<DIR>(v0, vp, vm, a.gamma, a.sc->dt / g.dx[DIR], a.sc->dt, a.c3 != 0, g.dims);
      if (a.ct) {
        vp[R::bn] = a.Bs[DIR][c];
        vm[R::bn] = a.Bs[DIR][c - s];
      }
      traced = true;
    }
  }
  if (!traced && a.cons_hancock) {
    // conservative Hancock step (PRIMITIVE_HANCOCK NO, Src/States/hancock.c:159-434):
    // the zone's own interface states evolved by dt/2 with the difference of
    // their fluxes; where U^{n+1/2} fails ConsToPrim the zone falls back to
    // first order (its centre value on both sides)
    const T gm1 = T(a.gamma - 1.0);
    const double dtdx = dt2 / g.dx[DIR];
    T uc[NV], uL[NV], uR[NV], fp[NV], fm[NV], uh[NV], vh[NV], pp, pm;
    prim_to_cons(v0, uc, gm1);
    prim_to_cons(vp, uL, gm1);
    prim_to_cons(vm, uR, gm1);
    flux<DIR>(vp, uL, fp, pp);
    flux<DIR>(vm, uR, fm, pm);
#pragma unroll
    for (int nv = 0; nv < NV; nv++) {
      T rhs = -dtdx * (fp[nv] - fm[nv]);
      if (nv == R::vn) rhs = rhs - dtdx * (pp - pm);
      uh[nv] = uc[nv] + rhs;
    }
    unsigned char fl = 0;
    cons_to_prim(uh, vh, gm1, T(a.small_rho), T(a.small_p), &fl);
    if (fl) {
#pragma unroll
      for (int nv = 0; nv < NV; nv++) vh[nv] = vp[nv] = vm[nv] = v0[nv];
      if (a.ct) {
        vp[R::bn] = a.Bs[DIR][c];
        vm[R::bn] = a.Bs[DIR][c - s];
      }
    }
#pragma unroll
    for (int nv = 0; nv < NV; nv++) {
      const T P1 = vp[nv] - vm[nv];
      T dvp = vh[nv] - v0[nv];
      T dvm = dvp;
      dvp = dvp + 0.5 * P1;
      dvm = dvm - 0.5 * P1;
      vp[nv] = v0[nv] + dvp;
      vm[nv] = v0[nv] + dvm;
    }
    if (a.ct) {
      vp[R::bn] = a.Bs[DIR][c];
      vm[R::bn] = a.Bs[DIR][c - s];
    }
  } else if (!traced) {  // primitive Hancock step
    T dv[NV], Adv[NV];
#pragma unroll
    for (int nv = 0; nv < NV; nv++) dv[nv] = vp[nv] - vm[nv];
    prim_rhs<DIR>(v0, dv, a.gamma, a.c3 != 0, Adv);
#pragma unroll
    for (int nv = NV - 1; nv >= 0; nv--) {
      const T scrh = dt2 * (inv_dl * Adv[nv] - 0.0);
      vp[nv] -= scrh;
      vm[nv] -= scrh;
    }
  }
  if ((vp[PRS] < 0.0) || (vm[PRS] < 0.0) || (vp[RHO] < 0.0) || (vm[RHO] < 0.0)) {  // CheckPrimStates
    const T sp = vp[R::bn], sm = vm[R::bn];
#pragma unroll
    for (int nv = 0; nv < NV; nv++) vm[nv] = vp[nv] = v0[nv];
    if (a.ct) {
      vp[R::bn] = sp;
      vm[R::bn] = sm;
    }
  }
  T up[NV], um[NV];
  const T gmm1 = T(a.gamma - 1.0);
  prim_to_cons(vp, up, gmm1);
  prim_to_cons(vm, um, gmm1);
#pragma unroll
  for (int nv = 0; nv < NV; nv++) {
    a.VP[nv][c] = vp[nv];
    a.VM[nv][c] = vm[nv];
  }
  if (a.ct && !a.cons_hancock) {  // CTU_CT_Source (not with the conservative predictor, ctu_step.c:122-133)
    const bool c3 = a.c3 != 0;
    const T db = (dt2 / g.dx[DIR]) * (up[R::bn] - um[R::bn]);
    up[MX1] += v0[BX1] * db;
    um[MX1] += v0[BX1] * db;
    up[MX1 + 1] += v0[BX2] * db;
    um[MX1 + 1] += v0[BX2] * db;
    if (c3) {
      up[MX1 + 2] += v0[BX3] * db;
      um[MX1 + 2] += v0[BX3] * db;
    }
    up[R::bt] += v0[R::vt] * db;
    um[R::bt] += v0[R::vt] * db;
    if (c3) {
      up[R::bb] += v0[R::vb] * db;
      um[R::bb] += v0[R::vb] * db;
    }
    const T scrh = c3 ? v0[VX1] * v0[BX1] + v0[VX2] * v0[BX2] + v0[VX3] * v0[BX3]
                      : v0[VX1] * v0[BX1] + v0[VX2] * v0[BX2];
    up[ENG] += scrh * db;
    um[ENG] += scrh * db;
  }
#pragma unroll
  for (int nv = 0; nv < NV; nv++) {
    a.Upd[DIR][nv][c] = up[nv];
    a.Umd[DIR][nv][c] = um[nv];
  }
}

// Transverse rhs added to the corrector states (ctu_step.c:567-600)
template <class T, int DIR>
__device__ __forceinline__ T ctu_dU(const F64A<T>& a, int nv, long long c) {
  const int dims = a.g.dims;
  if (DIR == 0) {
    if (dims == 1) return T(0.0);
    if (dims == 2) return T(0.0) + a.Rhd[1][nv][c];
    return T(0.0) + a.Rhd[1][nv][c] + a.Rhd[2][nv][c];
  }
  if (DIR == 1) {
    if (dims == 2) return a.Rhd[0][nv][c] + 0.0;
    return a.Rhd[0][nv][c] + 0.0 + a.Rhd[2][nv][c];
  }
  return a.Rhd[0][nv][c] + a.Rhd[1][nv][c];
}

// Riemann problem at interface c+1/2: predictor (STAGE 1) or corrector (2).
template <class T, int DIR, int SOLVER, int STAGE>
__global__ void k_ctu_riemann(F64A<T> a, Box box, int nlo) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  double invdt = 0.0;
  if (q < box.count()) {
    int i, j, k;
    box.coords(q, i, j, k);
    const Geom& g = a.g;
    using R = Rot<DIR>;
    const long long c = cidx(g, k, j, i), s = g.s[DIR];
    const T gmm1 = T(a.gamma - 1.0);
    T vL[NV], vR[NV], uL[NV], uR[NV];
    if (STAGE == 1) {
#pragma unroll
      for (int nv = 0; nv < NV; nv++) {
        vL[nv] = a.VP[nv][c];
        vR[nv] = a.VM[nv][c + s];
      }
      prim_to_cons(vL, uL, gmm1);
      prim_to_cons(vR, uR, gmm1);
    } else {
#pragma unroll
      for (int nv = 0; nv < NV; nv++) {
        uL[nv] = a.Upd[DIR][nv][c] + ctu_dU<T, DIR>(a, nv, c);
        uR[nv] = a.Umd[DIR][nv][c + s] + ctu_dU<T, DIR>(a, nv, c + s);
      }
      if (a.ct) {
        uL[R::bn] = a.Bs[DIR][c];
        uR[R::bn] = a.Bs[DIR][c];
      }
      unsigned char fm = 0, fp = 0;
      cons_to_prim(uR, vR, gmm1, T(a.small_rho), T(a.small_p), &fm);
      cons_to_prim(uL, vL, gmm1, T(a.small_rho), T(a.small_p), &fp);
    }
    Iface<T> o;
    T mach = T(0.0);
    if (SOLVER == PG_HLL) {
      hll_solver<DIR, false>(vL, uL, vR, uR, T(a.gamma), o, mach);
    } else if (SOLVER == PG_ROE) {
      int bad = 0;
      roe_solver<DIR, false>(vL, uL, vR, uR, T(a.gamma), a.c3 != 0, o, mach, bad);
      if (bad) atomicOr(&a.sc->status, 2);
    } else {
      hlld_solver<DIR, false>(vL, uL, vR, uR, T(a.gamma), o, mach);
    }
#pragma unroll
    for (int nv = 0; nv < NV; nv++) a.F[nv][c] = o.f[nv];
    a.P[c] = o.press;
    if (a.ct) store_face_emf<T, DIR>(a, c, o.f);  // CT_StoreUpwindEMF
    const int x = DIR == 0 ? i : (DIR == 1 ? j : k);
    if (x >= nlo) invdt = value_of(o.cmax) * g.inv_dx[DIR];
  }
  const double m = block_max(invdt);
  if (threadIdx.x == 0) atomic_max_nonneg(&a.sc->inv_dt_bits, m);
}

// RightHandSide: predictor stores the rhs (dt/2), corrector updates U (dt).
template <class T, int DIR, int STAGE>
__global__ void k_ctu_rhs(F64A<T> a, Box box) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= box.count()) return;
  int i, j, k;
  box.coords(q, i, j, k);
  const Geom& g = a.g;
  const long long c = cidx(g, k, j, i), s = g.s[DIR];
  const double dt = a.sc->dt;
  const double scrh = (STAGE == 1 ? 0.5 * dt : dt) / g.dx[DIR];
#pragma unroll
  for (int nv = 0; nv < NV; nv++) {
    T rhs = -scrh * (a.F[nv][c] - a.F[nv][c - s]);
    if (nv == Rot<DIR>::vn) rhs -= scrh * (a.P[c] - a.P[c - s]);
    if (STAGE == 1) a.Rhd[DIR][nv][c] = rhs;
    else a.U[nv][c] += rhs;
  }
}

// U^{n+1/2} = U^n + sum_d rhs_d (ctu_step.c:456-468)
template <class T>
__global__ void k_ctu_half(F64A<T> a, Box box) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= box.count()) return;
  int i, j, k;
  box.coords(q, i, j, k);
  const long long c = cidx(a.g, k, j, i);
  const int dims = a.g.dims;
#pragma unroll
  for (int nv = 0; nv < NV; nv++) {
    T dU = a.Rhd[0][nv][c];
    if (dims > 1) dU = dU + a.Rhd[1][nv][c];
    if (dims > 2) dU = dU + a.Rhd[2][nv][c];
    a.Uh[nv][c] = a.U[nv][c] + dU;
  }
}

template <class T>
__device__ __forceinline__ T ctu_ef(const F64A<T>& a, int slot, int k, int j, int i) {
  return a.EF[slot][cidx(a.g, k, j, i)];
}
// cell-centred EMF component e (CT_ComputeCenterEMF, ct_emf.c:348-388)
template <class T>
__device__ __forceinline__ T ctu_ecc(const F64A<T>& a, int e, int k, int j, int i) {
  const long long c = cidx(a.g, k, j, i);
  const T vx1 = a.V[VX1][c], vx2 = a.V[VX2][c], vx3 = a.V[VX3][c];
  const T Bx1 = a.V[BX1][c], Bx2 = a.V[BX2][c], Bx3 = a.V[BX3][c];
  if (e == 0) return (vx3 * Bx2 - vx2 * Bx3);
  if (e == 1) return (vx1 * Bx3 - vx3 * Bx1);
  return (vx2 * Bx1 - vx1 * Bx2);
}
__device__ __forceinline__ int ctu_sv(const signed char* sv, const Geom& g, int k, int j, int i) {
  return sv[cidx(g, k, j, i)];
}

// Edge EMFs (CT_ComputeEMF, Src/MHD/CT/ct_emf.c:210-291): ARITHMETIC;
// UCT0 (each face EMF replaced by twice itself minus the mean of the
// centred EMFs of the two zones sharing the face, then the arithmetic
// average); or UCT_CONTACT (arithmetic sum, then the upwind corner
// integration of Gardiner & Stone, then x 1/4).  STAGE 1 is the CTU
// predictor, which skips the corner integration (ct_emf_average.c:89-91);
// the corrector and every RK stage pass 2.  Each edge adds its four
// corner-integration terms in the order the reference's loop applies them
// (ct_emf_average.c:82-156).
template <class T, int STAGE>
__global__ void k_ctu_emf(F64A<T> a, Box eb) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= eb.count()) return;
  int i, j, k;
  eb.coords(q, i, j, k);
  const Geom& g = a.g;
  const bool uct = a.emf_avg == PG_UCT_CONTACT, uct0 = a.emf_avg == PG_UCT0, d3 = g.dims == 3;
  const double w = uct ? 1.0 : 0.25;
  const long long c = cidx(g, k, j, i);
  // face EMF of a slot; under UCT0 2 e - (e_c + e_c')/2 (ct_emf.c:261-282)
  auto fe = [&](int slot, int kk, int jj, int ii) -> T {
    T f = ctu_ef(a, slot, kk, jj, ii);
    if (!uct0) return f;
    const int e = slot <= EF_ZJ ? 2 : (slot <= EF_YK ? 1 : 0);
    const int di = slot == EF_ZI || slot == EF_YI, dj = slot == EF_ZJ || slot == EF_XJ,
              dk = slot == EF_YK || slot == EF_XK;
    f = f * 2.0;
    return f - 0.5 * (ctu_ecc(a, e, kk, jj, ii) + ctu_ecc(a, e, kk + dk, jj + dj, ii + di));
  };
  T ez = w * (fe(EF_ZI, k, j, i) + fe(EF_ZI, k, j + 1, i) + fe(EF_ZJ, k, j, i) + fe(EF_ZJ, k, j, i + 1));
  T ex = T(0.0), ey = T(0.0);
  if (d3) {
    ex = w * (fe(EF_XK, k, j, i) + fe(EF_XK, k, j + 1, i) + fe(EF_XJ, k, j, i) + fe(EF_XJ, k + 1, j, i));
    ey = w * (fe(EF_YI, k, j, i) + fe(EF_YI, k + 1, j, i) + fe(EF_YK, k, j, i) + fe(EF_YK, k, j, i + 1));
  }
  if (uct && STAGE == 2) {
    // derivative terms (ct_emf_average.c:67-79)
    auto dez_dxp = [&](int kk, int jj, int ii) { return ctu_ef(a, EF_ZI, kk, jj, ii) - ctu_ecc(a, 2, kk, jj, ii); };
    auto dez_dyp = [&](int kk, int jj, int ii) { return ctu_ef(a, EF_ZJ, kk, jj, ii) - ctu_ecc(a, 2, kk, jj, ii); };
    auto dez_dxm = [&](int kk, int jj, int ii) { return ctu_ecc(a, 2, kk, jj, ii) - ctu_ef(a, EF_ZI, kk, jj, ii - 1); };
    auto dez_dym = [&](int kk, int jj, int ii) { return ctu_ecc(a, 2, kk, jj, ii) - ctu_ef(a, EF_ZJ, kk, jj - 1, ii); };
    const signed char* SX = a.SV[0];
    const signed char* SY = a.SV[1];
    {  // Ez
      int sx = ctu_sv(SX, g, k, j, i), sy = ctu_sv(SY, g, k, j, i);
      ez = ez + (sx == 0 ? 0.5 * (dez_dyp(k, j, i) + dez_dyp(k, j, i + 1)) : dez_dyp(k, j, sx > 0 ? i : i + 1));
      ez = ez + (sy == 0 ? 0.5 * (dez_dxp(k, j, i) + dez_dxp(k, j + 1, i)) : dez_dxp(k, sy > 0 ? j : j + 1, i));
      const int sy2 = ctu_sv(SY, g, k, j, i + 1);
      ez = ez - (sy2 == 0 ? 0.5 * (dez_dxm(k, j, i + 1) + dez_dxm(k, j + 1, i + 1))
                          : dez_dxm(k, sy2 > 0 ? j : j + 1, i + 1));
      const int sx2 = ctu_sv(SX, g, k, j + 1, i);
      ez = ez - (sx2 == 0 ? 0.5 * (dez_dym(k, j + 1, i) + dez_dym(k, j + 1, i + 1))
                          : dez_dym(k, j + 1, sx2 > 0 ? i : i + 1));
    }
    if (d3) {
      const signed char* SZ = a.SV[2];
      auto dex_dyp = [&](int kk, int jj, int ii) { return ctu_ef(a, EF_XJ, kk, jj, ii) - ctu_ecc(a, 0, kk, jj, ii); };
      auto dex_dzp = [&](int kk, int jj, int ii) { return ctu_ef(a, EF_XK, kk, jj, ii) - ctu_ecc(a, 0, kk, jj, ii); };
      auto dey_dxp = [&](int kk, int jj, int ii) { return ctu_ef(a, EF_YI, kk, jj, ii) - ctu_ecc(a, 1, kk, jj, ii); };
      auto dey_dzp = [&](int kk, int jj, int ii) { return ctu_ef(a, EF_YK, kk, jj, ii) - ctu_ecc(a, 1, kk, jj, ii); };
      auto dex_dym = [&](int kk, int jj, int ii) { return ctu_ecc(a, 0, kk, jj, ii) - ctu_ef(a, EF_XJ, kk, jj - 1, ii); };
      auto dex_dzm = [&](int kk, int jj, int ii) { return ctu_ecc(a, 0, kk, jj, ii) - ctu_ef(a, EF_XK, kk - 1, jj, ii); };
      auto dey_dxm = [&](int kk, int jj, int ii) { return ctu_ecc(a, 1, kk, jj, ii) - ctu_ef(a, EF_YI, kk, jj, ii - 1); };
      auto dey_dzm = [&](int kk, int jj, int ii) { return ctu_ecc(a, 1, kk, jj, ii) - ctu_ef(a, EF_YK, kk - 1, jj, ii); };
      {  // Ex: Y-span and Z-span of (k,j,i), Z-span of (k,j+1,i), Y-span of (k+1,j,i)
        int sy = ctu_sv(SY, g, k, j, i), sz = ctu_sv(SZ, g, k, j, i);
        ex = ex + (sy == 0 ? 0.5 * (dex_dzp(k, j, i) + dex_dzp(k, j + 1, i)) : dex_dzp(k, sy > 0 ? j : j + 1, i));
        ex = ex + (sz == 0 ? 0.5 * (dex_dyp(k, j, i) + dex_dyp(k + 1, j, i)) : dex_dyp(sz > 0 ? k : k + 1, j, i));
        const int sz2 = ctu_sv(SZ, g, k, j + 1, i);
        ex = ex - (sz2 == 0 ? 0.5 * (dex_dym(k, j + 1, i) + dex_dym(k + 1, j + 1, i))
                            : dex_dym(sz2 > 0 ? k : k + 1, j + 1, i));
        const int sy3 = ctu_sv(SY, g, k + 1, j, i);
        ex = ex - (sy3 == 0 ? 0.5 * (dex_dzm(k + 1, j, i) + dex_dzm(k + 1, j + 1, i))
                            : dex_dzm(k + 1, sy3 > 0 ? j : j + 1, i));
      }
      {  // Ey: X-span and Z-span of (k,j,i), Z-span of (k,j,i+1), X-span of (k+1,j,i)
        int sx = ctu_sv(SX, g, k, j, i), sz = ctu_sv(SZ, g, k, j, i);
        ey = ey + (sx == 0 ? 0.5 * (dey_dzp(k, j, i) + dey_dzp(k, j, i + 1)) : dey_dzp(k, j, sx > 0 ? i : i + 1));
        ey = ey + (sz == 0 ? 0.5 * (dey_dxp(k, j, i) + dey_dxp(k + 1, j, i)) : dey_dxp(sz > 0 ? k : k + 1, j, i));
        const int sz2 = ctu_sv(SZ, g, k, j, i + 1);
        ey = ey - (sz2 == 0 ? 0.5 * (dey_dxm(k, j, i + 1) + dey_dxm(k + 1, j, i + 1))
                            : dey_dxm(sz2 > 0 ? k : k + 1, j, i + 1));
        const int sx3 = ctu_sv(SX, g, k + 1, j, i);
        ey = ey - (sx3 == 0 ? 0.5 * (dey_dzm(k + 1, j, i) + dey_dzm(k + 1, j, i + 1))
                            : dey_dzm(k + 1, j, sx3 > 0 ? i : i + 1));
      }
    }
  }
  if (uct) {
    ez = ez * 0.25;
    if (d3) {
      ex = ex * 0.25;
      ey = ey * 0.25;
    }
  }
  a.E[2][c] = ez;
  if (d3) {
    a.E[0][c] = ex;
    a.E[1][c] = ey;
  }
}

// CT_Update over the emf box (ct_update.c:75-200): Bs = base + dt curl E.
template <class T>
__global__ void k_ctu_ct(F64A<T> a, Box eb, int from_base0, double dtfac) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= eb.count()) return;
  int i, j, k;
  eb.coords(q, i, j, k);
  const Geom& g = a.g;
  const long long c = cidx(g, k, j, i);
  const double dt = dtfac * a.sc->dt;
  const double dx1 = g.dx[0], dx2 = g.dx[1], dx3 = g.dx[2];
  const bool d3 = g.dims == 3;
  const int KO = d3 ? 1 : 0;
  const int ib = eb.lo[0], jb = eb.lo[1], kb = eb.lo[2];
  T* const* base = from_base0 ? a.Bs0 : a.Bs;
  const T* Ex1 = a.E[0];
  const T* Ex2 = a.E[1];
  const T* Ex3 = a.E[2];
  if (k >= kb + KO && j >= jb + 1) {
    T rhs_x;
    if (!d3) rhs_x = 0.0 - dt / dx2 * (Ex3[c] - Ex3[c - g.s[1]]);
    else rhs_x = 0.0 - dt / dx2 * (Ex3[c] - Ex3[c - g.s[1]]) + dt / dx3 * (Ex2[c] - Ex2[c - g.s[2]]);
    a.Bs[0][c] = base[0][c] + rhs_x;
  }
  if (k >= kb + KO && i >= ib + 1) {
    T rhs_y;
    if (!d3) rhs_y = dt / dx1 * (Ex3[c] - Ex3[c - 1]);
    else rhs_y = dt / dx1 * (Ex3[c] - Ex3[c - 1]) - dt / dx3 * (Ex1[c] - Ex1[c - g.s[2]]);
    a.Bs[1][c] = base[1][c] + rhs_y;
  }
  if (d3 && j >= jb + 1 && i >= ib + 1) {
    T rhs_z = -dt / dx1 * (Ex2[c] - Ex2[c - 1]) + dt / dx2 * (Ex1[c] - Ex1[c - g.s[1]]);
    a.Bs[2][c] = base[2][c] + rhs_z;
  }
}

// CT_AverageMagneticField into Uh (domain plus one ghost layer)
template <class T>
__global__ void k_ctu_avg_half(F64A<T> a, Box box) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= box.count()) return;
  int i, j, k;
  box.coords(q, i, j, k);
  const Geom& g = a.g;
  const long long c = cidx(g, k, j, i);
  for (int d = 0; d < g.dims; d++) a.Uh[BX1 + d][c] = 0.5 * (a.Bs[d][c] + a.Bs[d][c - g.s[d]]);
}

// ConsToPrim of U^{n+1/2} (ctu_step.c:505-516)
template <class T>
__global__ void k_ctu_c2p_half(F64A<T> a, Box box) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= box.count()) return;
  int i, j, k;
  box.coords(q, i, j, k);
  const long long c = cidx(a.g, k, j, i);
  T u[NV], v[NV];
#pragma unroll
  for (int nv = 0; nv < NV; nv++) u[nv] = a.Uh[nv][c];
  unsigned char fl = a.flag[c];
  if (cons_to_prim(u, v, T(a.gamma - 1.0), T(a.small_rho), T(a.small_p), &fl)) a.flag[c] |= fl;
#pragma unroll
  for (int nv = 0; nv < NV; nv++) {
    a.Uh[nv][c] = u[nv];
    a.V[nv][c] = v[nv];
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
// Box: along DIR [beg+nlo, end+nhi], transverse axes extended by ext
static Box ctu_box(const Geom& g, int dir, int nlo, int nhi, int ext) {
  Box b;
  for (int ax = 0; ax < 3; ax++) {
    if (ax >= g.dims) {
      b.lo[ax] = b.hi[ax] = 0;
    } else if (ax == dir) {
      b.lo[ax] = g.beg[ax] + nlo;
      b.hi[ax] = g.end[ax] + nhi;
    } else {
      b.lo[ax] = g.beg[ax] - ext;
      b.hi[ax] = g.end[ax] + ext;
    }
  }
  return b.prepare();
}
static Box ctu_cube(const Geom& g, int lo_off, int hi_off) {
  Box b;
  for (int ax = 0; ax < 3; ax++) {
    if (ax >= g.dims) b.lo[ax] = b.hi[ax] = 0;
    else {
      b.lo[ax] = g.beg[ax] + lo_off;
      b.hi[ax] = g.end[ax] + hi_off;
    }
  }
  return b.prepare();
}

template <class T, int DIR, int STAGE>
static void ctu_launch_riemann(Solver* S, const F64A<T>& a, const Box& ib, int nlo) {
  cudaStream_t st = S->stream;
  const unsigned gr = grid_for(ib.count(), 128);
  PG_LAUNCH(S, "ctu_riemann", {
    if (S->cfg.riemann == PG_HLL) k_ctu_riemann<T, DIR, PG_HLL, STAGE><<<gr, 128, 0, st>>>(a, ib, nlo);
    else if (S->cfg.riemann == PG_ROE) k_ctu_riemann<T, DIR, PG_ROE, STAGE><<<gr, 128, 0, st>>>(a, ib, nlo);
    else k_ctu_riemann<T, DIR, PG_HLLD, STAGE><<<gr, 128, 0, st>>>(a, ib, nlo);
  });
}

template <class T, int DIR>
static void ctu_predict(Solver* S, const F64A<T>& a) {
  const Geom& g = S->g;
  cudaStream_t st = S->stream;
  const int ct = a.ct ? 1 : 0, ext = 1 + ct;
  const Box sb = ctu_box(g, DIR, -1 - ct, 1 + ct, ext);  // states nbeg-1 .. nend+1
  const Box ib = ctu_box(g, DIR, -1 - ct, ct, ext);      // interfaces nbeg-1 .. nend
  const Box rb = ctu_box(g, DIR, -ct, ct, ext);          // zones nbeg .. nend
  PG_LAUNCH(S, "ctu_states", (k_ctu_states<T, DIR><<<grid_for(sb.count(), 128), 128, 0, st>>>(a, sb)));
  ctu_launch_riemann<T, DIR, 1>(S, a, ib, g.beg[DIR] - ct);
  PG_LAUNCH(S, "ctu_rhs", (k_ctu_rhs<T, DIR, 1><<<grid_for(rb.count()), kThreads, 0, st>>>(a, rb)));
}

template <class T, int DIR>
static void ctu_correct(Solver* S, const F64A<T>& a) {
  const Geom& g = S->g;
  cudaStream_t st = S->stream;
  const int ext = a.ct ? 1 : 0;
  const Box ib = ctu_box(g, DIR, -1, 0, ext);
  const Box rb = ctu_box(g, DIR, 0, 0, ext);
  ctu_launch_riemann<T, DIR, 2>(S, a, ib, g.beg[DIR]);
  PG_LAUNCH(S, "ctu_rhs", (k_ctu_rhs<T, DIR, 2><<<grid_for(rb.count()), kThreads, 0, st>>>(a, rb)));
}

template <class T>
static void enqueue_ctu(Solver* S, const F64A<T>& a) {
  const Geom& g = S->g;
  cudaStream_t st = S->stream;
  const int ct = a.ct ? 1 : 0;
  launch_bound(S, a);
  PG_LAUNCH(S, "ctu_begin", (k_ctu_begin<T><<<grid_for(g.ncell), kThreads, 0, st>>>(a)));
  ctu_predict<T, 0>(S, a);
  if (g.dims > 1) ctu_predict<T, 1>(S, a);
  if (g.dims > 2) ctu_predict<T, 2>(S, a);
  const Box hb = ctu_cube(g, -ct, ct);
  PG_LAUNCH(S, "ctu_half", (k_ctu_half<T><<<grid_for(hb.count()), kThreads, 0, st>>>(a, hb)));
  if (ct) {
    const Box eb = ctu_cube(g, -2, 1);  // emf box of the predictor sweeps
    PG_LAUNCH(S, "ctu_emf", (k_ctu_emf<T, 1><<<grid_for(eb.count(), 128), 128, 0, st>>>(a, eb)));
    PG_LAUNCH(S, "ctu_ct", (k_ctu_ct<T><<<grid_for(eb.count()), kThreads, 0, st>>>(a, eb, 0, 0.5)));
    PG_LAUNCH(S, "ctu_avg", (k_ctu_avg_half<T><<<grid_for(hb.count()), kThreads, 0, st>>>(a, hb)));
  }
  PG_LAUNCH(S, "ctu_c2p_half", (k_ctu_c2p_half<T><<<grid_for(hb.count()), kThreads, 0, st>>>(a, hb)));
  ctu_correct<T, 0>(S, a);
  if (g.dims > 1) ctu_correct<T, 1>(S, a);
  if (g.dims > 2) ctu_correct<T, 2>(S, a);
  if (ct) {
    const Box eb = ctu_cube(g, -1, 0);  // emf box of the corrector sweeps
    PG_LAUNCH(S, "ctu_emf", (k_ctu_emf<T, 2><<<grid_for(eb.count(), 128), 128, 0, st>>>(a, eb)));
    PG_LAUNCH(S, "ctu_ct", (k_ctu_ct<T><<<grid_for(eb.count()), kThreads, 0, st>>>(a, eb, 1, 1.0)));
  }
  const Box dom = ctu_cube(g, 0, 0);
  PG_LAUNCH(S, "ctu_finalize", (k_finalize<T, 1, 2><<<grid_for(dom.count()), kThreads, 0, st>>>(a, dom, 0)));
  PG_LAUNCH(S, "ctu_end_step", (k_end_step<T><<<1, 1, 0, st>>>(a)));
}

}  // namespace pg
