// Batched 1D ideal-MHD problems (independent "tubes" of uneven sizes) in
// one persistent launch.  Each CTA pulls a tube from a work queue (largest
// first) and runs every step of it: per-tube dt (Src/main.c:389-575, the 1D
// rule of Src/Time_Stepping/update_stage.c:237-241), ghost fill
// (Src/boundary.c), RK2/RK3 stages (Src/Time_Stepping/rk_step.c) with the
// same point physics as the other paths (pg_physics.cuh).
//
// Per stage the tube is processed in chunks of blockDim zones: every zone of
// the chunk (plus one on each side) is reconstructed once into shared
// memory, every interface of the chunk is solved once, then the zones are
// updated.  Stage inputs and outputs live in separate buffers, so chunks
// never see half-updated neighbours.
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
  T* U0[NV];                 // conserved state at the start of the step
  T* U1[NV];                 // conserved result of the previous stage
  double* dt;                // per-tube dt (in: current, out: next)
  double* time;              // per-tube time
  unsigned long long* nfail; // per-tube floor events
  int* cur;                  // per-tube buffer holding the step-start state
  int* status;               // sticky error flags
  unsigned int* counter;     // work queue head
  double gamma, cfl, cfl_max_var, small_rho, small_p;
  int ng, bc, limiter, solver, ncomp;
};

template <class T> struct Batch;

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

template <class T>
__device__ __forceinline__ T block_max_T(T v, T* red) {
  for (int o = 16; o > 0; o >>= 1) {
    T w = __shfl_down_sync(0xffffffffu, v, o);
    v = (w > v || w != w) ? w : v;
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  T r = red[0];
  for (int q = 1; q < (int)(blockDim.x >> 5); q++) r = (red[q] > r || red[q] != red[q]) ? red[q] : r;
  return r;
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
      b.U0[nv][c] = u[nv];
      u[nv] += rhs[nv];
    }
  } else {
#pragma unroll
    for (int nv = 0; nv < NV; nv++) u[nv] = b.U1[nv][c] + rhs[nv];
    if (STAGE == 2) {
      const double w0 = NSTAGE == 3 ? 0.75 : 0.5, wc = NSTAGE == 3 ? 0.25 : 0.5;
#pragma unroll
      for (int nv = 0; nv < NV; nv++) u[nv] = w0 * b.U0[nv][c] + wc * u[nv];
    } else {
      const double one_third = 1.0 / 3.0;
#pragma unroll
      for (int nv = 0; nv < NV; nv++) u[nv] = one_third * (b.U0[nv][c] + 2.0 * u[nv]);
    }
  }
  unsigned char fl = 0;
  int fail = cons_to_prim(u, v, gmm1, b.small_rho, b.small_p, &fl);
  if (STAGE < NSTAGE) {
#pragma unroll
    for (int nv = 0; nv < NV; nv++) b.U1[nv][c] = u[nv];
  }
#pragma unroll
  for (int nv = 0; nv < NV; nv++) vout[nv] = v[nv];
  return fail;
}

// Mixed: FP32 primitives and fluxes, conserved accumulation in A.
template <int STAGE, int NSTAGE, class A>
__device__ __forceinline__ int batch_update_mixed(const BatchArgs<float>& b, long long c, const float* rhs,
                                                  const float* vin, float* vout) {
  using O = Acc<A>;
  using TT = typename O::T;
  const double inv_gmm1_d = 1.0 / (b.gamma - 1.0);
  const TT inv_gmm1 = O::konst(inv_gmm1_d, (float)inv_gmm1_d, (float)(inv_gmm1_d - (double)(float)inv_gmm1_d));
  TT u[NV];
  if (STAGE == 1) {
    u[RHO] = O::from(vin[RHO]);
#pragma unroll
    for (int q = 0; q < 3; q++) {
      u[VX1 + q] = O::prod(vin[RHO], vin[VX1 + q]);
      u[BX1 + q] = O::from(vin[BX1 + q]);
    }
    TT kin = O::add(O::add(O::prod(vin[VX1], vin[VX1]), O::prod(vin[VX2], vin[VX2])), O::prod(vin[VX3], vin[VX3]));
    TT b2 = O::add(O::add(O::prod(vin[BX1], vin[BX1]), O::prod(vin[BX2], vin[BX2])), O::prod(vin[BX3], vin[BX3]));
    u[ENG] = O::add(O::mulf(O::add(O::mulf(kin, vin[RHO]), b2), 0.5f), O::mulf(inv_gmm1, vin[PRS]));
    // U0 keeps the high part only when A is a double-word: store the value
    // rounded to FP32 (storage is FP32 in the mixed path).
#pragma unroll
    for (int nv = 0; nv < NV; nv++) {
      b.U0[nv][c] = O::tof(u[nv]);
      u[nv] = O::addf(u[nv], rhs[nv]);
    }
  } else {
#pragma unroll
    for (int nv = 0; nv < NV; nv++) u[nv] = O::addf(O::from(b.U1[nv][c]), rhs[nv]);
    if (STAGE == 2 && NSTAGE == 2) {
#pragma unroll
      for (int nv = 0; nv < NV; nv++) u[nv] = O::mulf(O::addf(u[nv], b.U0[nv][c]), 0.5f);
    } else if (STAGE == 2) {
#pragma unroll
      for (int nv = 0; nv < NV; nv++) u[nv] = O::add(O::mulf(O::from(b.U0[nv][c]), 0.75f), O::mulf(u[nv], 0.25f));
    } else {
      const TT third = O::konst(1.0 / 3.0, (float)(1.0 / 3.0), (float)(1.0 / 3.0 - (double)(float)(1.0 / 3.0)));
#pragma unroll
      for (int nv = 0; nv < NV; nv++) u[nv] = O::mul(O::add(O::from(b.U0[nv][c]), O::mulf(u[nv], 2.0f)), third);
    }
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
  if (p < 0.f) {
    p = (float)b.small_p;
    u[ENG] = O::add(O::mulf(inv_gmm1, p), kinb2);
    fail = 1;
  }
  if (STAGE < NSTAGE) {
#pragma unroll
    for (int nv = 0; nv < NV; nv++) b.U1[nv][c] = O::tof(u[nv]);
  }
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
  else return batch_update_mixed<STAGE, NSTAGE, A>(b, c, rhs, vin, vout);
}

// One stage of one tube.  Returns this stage's max(cmax/dx) contribution.
template <class T, class A, int RS, int SOLVER, int STAGE, int NSTAGE>
__device__ double batch_stage(const BatchArgs<T>& b, int tube, T* const* Vin, T* const* Vout, double dt, T* svp,
                              T* svm, T* sf, T* red, unsigned long long& fails) {
  const int n = b.nx[tube], ng = b.ng;
  const long long base = b.off[tube];
  const int beg = ng, end = ng + n - 1;
  const int B = blockDim.x, tid = threadIdx.x;
  const T inv_dx = (T)b.inv_dx[tube];
  const T dtdx = (T)(dt / b.dxv[tube]);
  // ghost fill of the stage input (outflow: copy edge zone; periodic: wrap;
  // reflective / equatorial-symmetric: mirror with the FlipSign signs)
  for (int q = tid; q < 2 * ng * NV; q += B) {
    int nv = q / (2 * ng), gi = q % (2 * ng);
    int i = gi < ng ? gi : end + 1 + (gi - ng);
    int src = bc_src(i, beg, end, n, b.bc);
    const T v = Vin[nv][base + src];
    Vin[nv][base + i] = bc_flip(0, bc_side(b.bc, i > end), nv, b.ncomp) < 0 ? -v : v;
  }
  __syncthreads();
  T cm_max = T(0);
  const double gam = b.gamma;
  for (int lo = beg; lo <= end; lo += B) {
    const int hi = min(lo + B - 1, end);
    // states of zones lo-1 .. hi+1
    for (int z = lo - 1 + tid; z <= hi + 1; z += B) {
      const int s = z - (lo - 1);
#pragma unroll
      for (int nv = 0; nv < NV; nv++) {
        T vp, vm;
        batch_recon<T, RS>(Vin[nv], base + z, b.limiter, nv, vp, vm);
        svp[nv * (B + 2) + s] = vp;
        svm[nv * (B + 2) + s] = vm;
      }
    }
    __syncthreads();
    // interfaces lo-1+1/2 .. hi+1/2
    for (int z = lo - 1 + tid; z <= hi; z += B) {
      const int s = z - (lo - 1);
      T vL[NV], vR[NV], uL[NV], uR[NV], mach;
#pragma unroll
      for (int nv = 0; nv < NV; nv++) {
        vL[nv] = svp[nv * (B + 2) + s];
        vR[nv] = svm[nv * (B + 2) + s + 1];
      }
      const T gmm1 = (T)(gam - 1.0);
      prim_to_cons(vL, uL, gmm1);
      prim_to_cons(vR, uR, gmm1);
      Iface<T> o;
      if (SOLVER == PG_HLL) {
        hll_solver<0, false>(vL, uL, vR, uR, (T)gam, o, mach);
      } else if (SOLVER == PG_ROE) {
        int bad = 0;
        roe_solver<0, false>(vL, uL, vR, uR, (T)gam, b.ncomp == 3, o, mach, bad);
        if (bad) atomicOr(b.status, 2);
      } else {
        hlld_solver<0, false>(vL, uL, vR, uR, (T)gam, o, mach);
      }
#pragma unroll
      for (int nv = 0; nv < NV; nv++) sf[nv * (B + 1) + s] = o.f[nv];
      sf[NV * (B + 1) + s] = o.press;
      T cmi = o.cmax * inv_dx;  // update_stage.c:239
      cm_max = (cmi > cm_max || cmi != cmi) ? cmi : cm_max;
    }
    __syncthreads();
    // zones lo .. hi
    for (int z = lo + tid; z <= hi; z += B) {
      const int s = z - (lo - 1);  // interface z+1/2 is slot s, z-1/2 is s-1
      T rhs[NV], vin[NV], vout[NV];
#pragma unroll
      for (int nv = 0; nv < NV; nv++) {
        rhs[nv] = -dtdx * (sf[nv * (B + 1) + s] - sf[nv * (B + 1) + s - 1]);
        vin[nv] = Vin[nv][base + z];
      }
      rhs[VX1] -= dtdx * (sf[NV * (B + 1) + s] - sf[NV * (B + 1) + s - 1]);
      fails += batch_update<T, A, STAGE, NSTAGE>(b, base + z, rhs, vin, vout);
#pragma unroll
      for (int nv = 0; nv < NV; nv++) Vout[nv][base + z] = vout[nv];
    }
    __syncthreads();
  }
  return (double)block_max_T<T>(cm_max, red);
}

template <class T, class A, int RS, int SOLVER, int NSTAGE>
__global__ void k_batch(BatchArgs<T> b, int nsteps) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int B = blockDim.x;
  T* svp = (T*)smem_raw;
  T* svm = svp + NV * (B + 2);
  T* sf = svm + NV * (B + 2);
  T* red = sf + (NV + 1) * (B + 1);
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
      T* A0[NV];
      T* A1[NV];
#pragma unroll
      for (int nv = 0; nv < NV; nv++) {
        A0[nv] = b.V[cur][nv];
        A1[nv] = b.V[1 - cur][nv];
      }
      double inv = 0.0, m;
      m = batch_stage<T, A, RS, SOLVER, 1, NSTAGE>(b, tube, A0, A1, dt, svp, svm, sf, red, fails);
      inv = m > inv ? m : inv;
      if (NSTAGE == 2) {
        m = batch_stage<T, A, RS, SOLVER, 2, NSTAGE>(b, tube, A1, A0, dt, svp, svm, sf, red, fails);
        inv = m > inv ? m : inv;
      } else {
        m = batch_stage<T, A, RS, SOLVER, 2, NSTAGE>(b, tube, A1, A0, dt, svp, svm, sf, red, fails);
        inv = m > inv ? m : inv;
        m = batch_stage<T, A, RS, SOLVER, 3, NSTAGE>(b, tube, A0, A1, dt, svp, svm, sf, red, fails);
        inv = m > inv ? m : inv;
        cur = 1 - cur;  // the result of stage 3 is in the other buffer
      }
      // NextTimeStep, Src/main.c:459-532 (1D: no division by DIMENSIONS);
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

template <class T>
inline size_t batch_smem_bytes(int B) {
  return sizeof(T) * ((size_t)2 * NV * (B + 2) + (size_t)(NV + 1) * (B + 1) + 32);
}

}  // namespace pg
