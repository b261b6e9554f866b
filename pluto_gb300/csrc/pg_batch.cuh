// Batched 1D ideal-MHD problems (independent "tubes" of uneven sizes) in
// one persistent launch.  Each CTA -- a team of warps -- pulls a tube from a
// work queue (largest first) and runs every step of it: per-tube dt
// (Src/main.c:389-575, the 1D rule of Src/Time_Stepping/update_stage.c:
// 237-241), ghost fill (Src/boundary.c), RK2/RK3 stages
// (Src/Time_Stepping/rk_step.c) with the same point physics as the other
// paths (pg_physics.cuh).
//
// Per stage the warps of the team share the tube's 30-zone chunks; inside a
// chunk neighbouring states and fluxes move between lanes by shuffles, so a
// stage needs one block barrier (before the next stage reads neighbours).
#pragma once
#include "pg_internal.h"
#include "pg_physics.cuh"
#include "pg_dw.cuh"

namespace pg {

// T: storage/flux type (double for the plain path, float for mixed);
// A: accumulator of the conserved update (double or dw; == T for FP64).
template <class T>
struct BatchArgs {
  int ntubes;
  const int* order;          // queue order (tube ids)
  const int* nx;             // interior zones per tube
  const long long* off;      // first (ghost) zone of each tube in the arrays
  const double* inv_dx;      // 1/dx per tube
  const double* dxv;         // dx per tube
  T* V[2][NV];               // stage ping-pong of primitives
  // Conserved state at the start of the step (U0) and the result of the
  // previous stage (U1), 8-byte elements: double on the FP64 path; on the
  // mixed path the accumulator type A (double or an FP32 pair).  The mixed
  // path keeps U0 resident across steps (written by the last stage); the
  // FP64 path rebuilds it from the primitives every step, as the reference.
  void* U0[NV];
  void* U1[NV];
  double* dt;                // per-tube dt (in: current, out: next)
  double* time;              // per-tube time
  unsigned long long* nfail; // per-tube floor events
  int* cur;                  // per-tube buffer holding the step-start state
  int* status;               // sticky error flags
  unsigned int* counter;     // work queue head
  double gamma, cfl, cfl_max_var, small_rho, small_p;
  int ng, bc, limiter, solver, ncomp;
};

// Reconstruction of one zone from V[c-2..c+2] (PLM uses c-1..c+1).
template <class T, int RS>
__device__ __forceinline__ void batch_recon(const T* V, long long c, int lim, int nv, T& vp, T& vm) {
  if (RS == 4) {  // PPM
    T w2 = V[c - 2], w1 = V[c - 1], v0 = V[c], e1 = V[c + 1], e2 = V[c + 2];
    T p = ppm_iface(w1, v0, e1, e2);
    T m = ppm_iface(w2, w1, v0, e1);
    ppm_limit(v0, p, m);
    vp = p;
    vm = m;
  } else {
    T w1 = V[c - 1], v0 = V[c], e1 = V[c + 1];
    const int L = RS == 0 ? LIM_MC : RS == 1 ? LIM_MINMOD : RS == 2 ? LIM_VANLEER : lim;
    T dv = limit(L, nv, e1 - v0, v0 - w1);
    vp = v0 + dv * T(0.5);
    vm = v0 - dv * T(0.5);
  }
}

// Stage update of one zone: U_stage = base + rhs, RK combination, ConsToPrim.
// FP64 instantiation follows the reference operation order exactly.
template <int STAGE, int NSTAGE>
__device__ __forceinline__ int batch_update_f64(const BatchArgs<double>& b, long long c, const double* rhs,
                                                const double* vin, double* vout) {
  double u[NV], v[NV];
  const double gmm1 = b.gamma - 1.0;
  if (STAGE == 1) {
    prim_to_cons(vin, u, gmm1);
#pragma unroll
    for (int nv = 0; nv < NV; nv++) {
      ((double*)b.U0[nv])[c] = u[nv];
      u[nv] += rhs[nv];
    }
  } else {
#pragma unroll
    for (int nv = 0; nv < NV; nv++) u[nv] = ((const double*)b.U1[nv])[c] + rhs[nv];
    if (STAGE == 2) {
      const double w0 = NSTAGE == 3 ? 0.75 : 0.5, wc = NSTAGE == 3 ? 0.25 : 0.5;
#pragma unroll
      for (int nv = 0; nv < NV; nv++) u[nv] = w0 * ((const double*)b.U0[nv])[c] + wc * u[nv];
    } else {
      const double one_third = 1.0 / 3.0;
#pragma unroll
      for (int nv = 0; nv < NV; nv++) u[nv] = one_third * (((const double*)b.U0[nv])[c] + 2.0 * u[nv]);
    }
  }
  unsigned char fl = 0;
  int fail = cons_to_prim(u, v, gmm1, b.small_rho, b.small_p, &fl);
  if (STAGE < NSTAGE) {
#pragma unroll
    for (int nv = 0; nv < NV; nv++) ((double*)b.U1[nv])[c] = u[nv];
  }
#pragma unroll
  for (int nv = 0; nv < NV; nv++) vout[nv] = v[nv];
  return fail;
}

// Mixed: FP32 primitives and fluxes; the conserved state stays resident in
// the accumulator type A across stages and steps (U0 at the start of the
// step, U1 the stage result), so the state is never re-rounded through FP32
// primitives between stages.  ConsToPrim (Src/MHD/mappers.c:88-254) with the
// pressure recovered in A and the reference's floors.
template <int STAGE, int NSTAGE, class A>
__device__ __forceinline__ int batch_update_mixed(const BatchArgs<float>& b, long long c, const float* rhs,
                                                  float* vout) {
  using O = Acc<A>;
  using TT = typename O::T;
  const double inv_gmm1_d = 1.0 / (b.gamma - 1.0);
  const TT inv_gmm1 = O::konst(inv_gmm1_d, (float)inv_gmm1_d, (float)(inv_gmm1_d - (double)(float)inv_gmm1_d));
  TT u[NV];
  if (STAGE == 1) {
#pragma unroll
    for (int nv = 0; nv < NV; nv++) u[nv] = O::addf(O::ld(b.U0[nv], c), rhs[nv]);
  } else if (STAGE == 2 && NSTAGE == 2) {  // (U0 + U1 + rhs) / 2
#pragma unroll
    for (int nv = 0; nv < NV; nv++) u[nv] = O::half_sum3(O::ld(b.U0[nv], c), O::ld(b.U1[nv], c), rhs[nv]);
  } else if (STAGE == 2) {
#pragma unroll
    for (int nv = 0; nv < NV; nv++)
      u[nv] = O::add(O::mulf(O::ld(b.U0[nv], c), 0.75f), O::mulf(O::addf(O::ld(b.U1[nv], c), rhs[nv]), 0.25f));
  } else {
    const TT third = O::konst(1.0 / 3.0, (float)(1.0 / 3.0), (float)(1.0 / 3.0 - (double)(float)(1.0 / 3.0)));
#pragma unroll
    for (int nv = 0; nv < NV; nv++)
      u[nv] = O::mul(O::add(O::ld(b.U0[nv], c), O::mulf(O::addf(O::ld(b.U1[nv], c), rhs[nv]), 2.0f)), third);
  }
  int fail = 0;
  if (O::neg(u[RHO])) {
    u[RHO] = O::from((float)b.small_rho);
    fail = 1;
  }
  const float rho_f = O::tof(u[RHO]);
  const float tau = 1.0f / rho_f;
  TT m2 = O::add(O::add(O::mul(u[VX1], u[VX1]), O::mul(u[VX2], u[VX2])), O::mul(u[VX3], u[VX3]));
  TT b2 = O::add(O::add(O::mul(u[BX1], u[BX1]), O::mul(u[BX2], u[BX2])), O::mul(u[BX3], u[BX3]));
  TT kinb2 = O::mulf(O::add(O::div(m2, u[RHO]), b2), 0.5f);
  if (O::neg(u[ENG])) {
    u[ENG] = O::add(O::mulf(inv_gmm1, (float)b.small_p), kinb2);
    fail = 1;
  }
  float p = O::tof(O::mulf(O::sub(u[ENG], kinb2), (float)(b.gamma - 1.0)));
  if (p < 0.f) {  // floor and recompute the energy (Src/MHD/mappers.c:190-200)
    p = (float)b.small_p;
    u[ENG] = O::add(O::mulf(inv_gmm1, p), kinb2);
    fail = 1;
  }
  void* const* Uout = STAGE == NSTAGE ? b.U0 : b.U1;
#pragma unroll
  for (int nv = 0; nv < NV; nv++) O::st(Uout[nv], c, u[nv]);
  vout[RHO] = rho_f;
#pragma unroll
  for (int q = 0; q < 3; q++) {
    vout[VX1 + q] = O::tof(u[VX1 + q]) * tau;
    vout[BX1 + q] = O::tof(u[BX1 + q]);
  }
  vout[PRS] = p;
  return fail;
}

template <class T, class A, int STAGE, int NSTAGE>
__device__ __forceinline__ int batch_update(const BatchArgs<T>& b, long long c, const T* rhs, const T* vin, T* vout) {
  if constexpr (sizeof(T) == 8) return batch_update_f64<STAGE, NSTAGE>(b, c, rhs, vin, vout);
  else return batch_update_mixed<STAGE, NSTAGE, A>(b, c, rhs, vout);
}

// One stage of one tube by the whole CTA.  The tube is cut into chunks of
// 30 zones; warp w takes chunks w, w + NW, ...  Within a chunk lane l
// reconstructs zone i = beg - 1 + 30 chunk + l, takes the right state of
// interface i+1/2 from lane l+1 and the flux of interface i-1/2 from lane
// l-1 (shuffles): 32 reconstructions, 31 interfaces, 30 updated zones, no
// block barrier.  Stage input and output are separate buffers, so chunks
// never see half-updated neighbours; the CTA synchronises once per stage.
// cm_max collects max(cmax/dx) over the tube's interfaces
// (Src/Time_Stepping/update_stage.c:237-241).
template <class T, class A, int RS, int SOLVER, int STAGE, int NSTAGE>
__device__ void batch_stage(const BatchArgs<T>& b, int tube, int in_buf, double dt, T& cm_max,
                            unsigned long long& fails) {
  T* const* Vin = b.V[in_buf];
  T* const* Vout = b.V[1 - in_buf];
  const int n = b.nx[tube], ng = b.ng;
  const long long base = b.off[tube];
  const int beg = ng, end = ng + n - 1;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5, nw = blockDim.x >> 5;
  const T inv_dx = (T)b.inv_dx[tube];
  const T dtdx = (T)(dt / b.dxv[tube]);
  // ghost fill of the stage input (outflow: copy edge zone; periodic: wrap;
  // reflective / equatorial-symmetric: mirror with the FlipSign signs)
  for (int q = tid; q < 2 * ng * NV; q += blockDim.x) {
    int nv = q / (2 * ng), gi = q % (2 * ng);
    int i = gi < ng ? gi : end + 1 + (gi - ng);
    int src = bc_src(i, beg, end, n, b.bc);
    const T v = Vin[nv][base + src];
    Vin[nv][base + i] = bc_flip(0, bc_side(b.bc, i > end), nv, b.ncomp) < 0 ? -v : v;
  }
  __syncthreads();
  const double gam = b.gamma;
  const T gmm1 = (T)(gam - 1.0);
  const int nch = (n + 29) / 30;
  for (int ch = w; ch < nch; ch += nw) {
    const int i = beg - 1 + 30 * ch + lane;
    const bool cell_ok = i <= end + 1;          // zones beg-1 .. end+1
    const bool face_ok = i <= end && lane < 31;  // interfaces beg-1+1/2 .. end+1/2
    const long long c = base + i;
    T vp[NV], vm[NV], v0[NV];
#pragma unroll
    for (int nv = 0; nv < NV; nv++) {
      vp[nv] = vm[nv] = v0[nv] = T(0);
      if (cell_ok) {
        batch_recon<T, RS>(Vin[nv], c, b.limiter, nv, vp[nv], vm[nv]);
        v0[nv] = Vin[nv][c];
      }
    }
    T vR[NV];
#pragma unroll
    for (int nv = 0; nv < NV; nv++) vR[nv] = __shfl_down_sync(0xffffffffu, vm[nv], 1);
    T fl[NV], pr = T(0);
#pragma unroll
    for (int nv = 0; nv < NV; nv++) fl[nv] = T(0);
    if (face_ok) {
      T uL[NV], uR[NV], mach;
      prim_to_cons(vp, uL, gmm1);
      prim_to_cons(vR, uR, gmm1);
      Iface<T> o;
      if (SOLVER == PG_HLL) {
        hll_solver<0, false>(vp, uL, vR, uR, (T)gam, o, mach);
      } else if (SOLVER == PG_ROE) {
        int bad = 0;
        roe_solver<0, false>(vp, uL, vR, uR, (T)gam, b.ncomp == 3, o, mach, bad);
        if (bad) atomicOr(b.status, 2);
      } else {
        hlld_solver<0, false>(vp, uL, vR, uR, (T)gam, o, mach);
      }
#pragma unroll
      for (int nv = 0; nv < NV; nv++) fl[nv] = o.f[nv];
      pr = o.press;
      T cmi = o.cmax * inv_dx;  // update_stage.c:239
      cm_max = (cmi > cm_max || cmi != cmi) ? cmi : cm_max;
    }
    T flm[NV];
#pragma unroll
    for (int nv = 0; nv < NV; nv++) flm[nv] = __shfl_up_sync(0xffffffffu, fl[nv], 1);
    const T prm = __shfl_up_sync(0xffffffffu, pr, 1);
    if (lane >= 1 && lane <= 30 && i <= end) {
      T rhs[NV], vout[NV];
#pragma unroll
      for (int nv = 0; nv < NV; nv++) rhs[nv] = -dtdx * (fl[nv] - flm[nv]);
      rhs[VX1] -= dtdx * (pr - prm);
      fails += batch_update<T, A, STAGE, NSTAGE>(b, c, rhs, v0, vout);
#pragma unroll
      for (int nv = 0; nv < NV; nv++) Vout[nv][c] = vout[nv];
    }
  }
  __syncthreads();  // the stage output is complete (the next stage reads neighbours)
}

template <class T>
__device__ __forceinline__ T block_max_T(T v, T* red) {
  for (int o = 16; o > 0; o >>= 1) {
    T w = __shfl_down_sync(0xffffffffu, v, o);
    v = (w > v || w != w) ? w : v;
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) red[w] = v;
  __syncthreads();
  T r = red[0];
  for (int q = 1; q < (int)(blockDim.x >> 5); q++) r = (red[q] > r || red[q] != red[q]) ? red[q] : r;
  __syncthreads();  // red is reused
  return r;
}

// Persistent kernel: each CTA (a team of NW warps) pulls a tube from the
// queue (largest first) and runs every step of it with its own dt
// (NextTimeStep, Src/main.c:459-532; 1D: no division by DIMENSIONS).
template <class T, class A, int RS, int SOLVER, int NSTAGE>
__global__ void __launch_bounds__(256) k_batch(BatchArgs<T> b, int nsteps) {
  __shared__ T red[8];
  __shared__ int s_t;
  for (;;) {
    if (threadIdx.x == 0) s_t = (int)atomicAdd(b.counter, 1u);
    __syncthreads();
    const int t = s_t;
    __syncthreads();
    if (t >= b.ntubes) break;
    const int tube = b.order[t];
    double dt = b.dt[tube], time = b.time[tube];
    int cur = b.cur[tube];
    unsigned long long fails = 0;
    for (int step = 0; step < nsteps; step++) {
      T cm = T(0);
      batch_stage<T, A, RS, SOLVER, 1, NSTAGE>(b, tube, cur, dt, cm, fails);
      batch_stage<T, A, RS, SOLVER, 2, NSTAGE>(b, tube, 1 - cur, dt, cm, fails);
      if (NSTAGE == 3) {
        batch_stage<T, A, RS, SOLVER, 3, NSTAGE>(b, tube, cur, dt, cm, fails);
        cur = 1 - cur;  // the result of stage 3 is in the other buffer
      }
      const double inv = (double)block_max_T<T>(cm, red);
      // cfl <= 0 keeps dt fixed
      time += dt;
      if (b.cfl > 0.0) {
        double dt_hyp = 1.0 / inv;
        dt_hyp *= b.cfl;
        dt = pmin(dt_hyp, b.cfl_max_var * dt);
      }
    }
    if (threadIdx.x == 0) {
      b.dt[tube] = dt;
      b.time[tube] = time;
      b.cur[tube] = cur;
      if (!(dt == dt) || !(dt > 0)) atomicOr(b.status, 1);
    }
    // per-tube floor count
    for (int o = 16; o > 0; o >>= 1) fails += __shfl_down_sync(0xffffffffu, fails, o);
    if ((threadIdx.x & 31) == 0 && fails) atomicAdd(&b.nfail[tube], fails);
    __syncthreads();
  }
}

// Mixed path: the resident conserved state U0 of every tube from its
// primitives (PrimToCons in A), after an upload or a restored snapshot.
// One CTA per tube.
template <class A>
__global__ void k_batch_cons_init(BatchArgs<float> b) {
  using O = Acc<A>;
  const int tube = blockIdx.x;
  if (tube >= b.ntubes) return;
  const int n = b.nx[tube], ng = b.ng;
  const long long base = b.off[tube];
  const int cur = b.cur[tube];
  const double inv_gmm1_d = 1.0 / (b.gamma - 1.0);
  const typename O::T inv_gmm1 =
      O::konst(inv_gmm1_d, (float)inv_gmm1_d, (float)(inv_gmm1_d - (double)(float)inv_gmm1_d));
  for (int i = ng + threadIdx.x; i < ng + n; i += blockDim.x) {
    const long long c = base + i;
    float v[NV];
#pragma unroll
    for (int nv = 0; nv < NV; nv++) v[nv] = b.V[cur][nv][c];
    typename O::T u[NV];
    u[RHO] = O::from(v[RHO]);
#pragma unroll
    for (int q = 0; q < 3; q++) {
      u[VX1 + q] = O::prod(v[RHO], v[VX1 + q]);
      u[BX1 + q] = O::from(v[BX1 + q]);
    }
    typename O::T kin = O::add(O::add(O::prod(v[VX1], v[VX1]), O::prod(v[VX2], v[VX2])), O::prod(v[VX3], v[VX3]));
    typename O::T b2 = O::add(O::add(O::prod(v[BX1], v[BX1]), O::prod(v[BX2], v[BX2])), O::prod(v[BX3], v[BX3]));
    u[ENG] = O::add(O::mulf(O::add(O::mulf(kin, v[RHO]), b2), 0.5f), O::mulf(inv_gmm1, v[PRS]));
#pragma unroll
    for (int nv = 0; nv < NV; nv++) O::st(b.U0[nv], c, u[nv]);
  }
}

}  // namespace pg
