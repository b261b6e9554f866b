// Mixed-precision path: FP32 storage and FP32 reconstruction / Riemann /
// EMF arithmetic; the conserved-variable accumulation, the CT face-field
// update, the pressure recovery p = (g-1)(E - rho v^2/2 - B^2/2) and the
// global dt reduction in a wider accumulator: native FP64 (PG_MIXED) or an
// FP32 double-word pair (PG_MIXED_DW, 48-bit significand on the FP32 pipes,
// see pg_dw.cuh).
//
// One stage = seven launches:
//   k_mbound      ghost fill (Src/boundary.c:41-303)
//   k_msweep_x    reconstruct + Riemann + flux difference along x; one warp
//                 covers 31 cells of a row, the left interface flux comes
//                 from the neighbouring lane by shuffle
//   k_msweep_t    the same along y or z: blocks of 32 x-lanes by 8 rows, the
//                 left flux of a cell comes from the row below through
//                 shared memory (7 cells per 8 interfaces along the sweep)
//   k_memf        UCT_HLL edge EMFs (Src/MHD/CT/ct_emf_average.c:179-352)
//   k_mface       CT face update (Src/MHD/CT/ct_update.c) + RK face combination
//   k_mfinal      RK cell combination, face average, ConsToPrim
//                 (Src/MHD/mappers.c:88-254), dt reduction
// Stage outputs are written to a second state buffer (the stage input is
// still read by neighbours), so RK2/RK3 need two FP32 copies of the state.
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "pg_internal.h"
#include "pg_physics.cuh"
#include "pg_dw.cuh"
#include "pg_bound_ct.cuh"
#include "pg_xfer.cuh"
#include "pg_tma.cuh"

namespace pg {

struct MixBufs {
  float* V[2][8];
  float* Bs[2][3];
  float* dU[8];
  // RK2: the stage-2 increments, so that the stage-1 ones stay for the
  // corrector U0 + (dU0 + dU1)/2 (null for EULER and RK3)
  float* dU1[8];
  float* S[3][2];
  float* DV[3][3];
  float* E[3];
  float* CDT;
  unsigned char* flag;
  float* Bm1[3];  // face -1 layers (outflow sides under CT)
  // Resident conserved accumulators in the accumulator type (FP64, or FP32
  // pairs for PG_MIXED_DW), 8 arrays each: U[0] the state at the start of the
  // step, U[1] the stage result (PLUTO keeps the same pair, d->Uc and U0).
  void* U[2];
};

struct MixArgs {
  Geom g;
  const float* Vin[8];   // stage input (reconstruction, EMF velocities)
  const float* V0[8];    // state at the start of the step (RK combination)
  float* Vout[8];
  const float* Bin[3];
  const float* B0[3];
  float* Bout[3];
  float* dU[8];
  const float* dUp[8];  // RK2 stage 2: the stage-1 increments
  float* S[3][2];
  float* DV[3][3];
  float* E[3];
  float* CDT;
  unsigned char* flag;
  void* U0;  // conserved state at the start of the step (accumulator type)
  void* Us;  // conserved stage result
  DevScalars* sc;
  float gamma;
  float inv_dx_f[3];
  double gamma_d, small_rho, small_p, cfl, cfl_max_var;
  double inv_gmm1_d;     // 1/(gamma-1) as a double
  float inv_gmm1_hi, inv_gmm1_lo;  // the same as a double-word pair
  float third_hi, third_lo;        // 1/3 as a double-word pair
  int limiter, recon, ct, nbfield, accmask, device_dt, ncomp;
  int intb;  // INTERNAL_BOUNDARY: flagged zones are not updated
  // try limit of a TMA sweep's wait for its tile (the waits that drain copies
  // in flight after a timeout keep the default limit)
  int tile_tries;
};

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ float ldg(const float* p, long long i) { return __ldg(p + i); }

__device__ __forceinline__ void atomic_max_nonneg_d(unsigned long long* addr, double v) {
  atomicMax(addr, (unsigned long long)__double_as_longlong(v));
}

__device__ __forceinline__ double warp_max_d(double v) {
  for (int o = 16; o > 0; o >>= 1) {
    double w = __shfl_down_sync(0xffffffffu, v, o);
    v = (w > v || w != w) ? w : v;
  }
  return v;
}

// Reconstruction schemes known at compile time (the reference selects them
// with the RECONSTRUCTION / LIMITER macros of definitions.h).
enum : int { RS_PLM_MC = 0, RS_PLM_MINMOD = 1, RS_PLM_VANLEER = 2, RS_PLM_GENERIC = 3, RS_PPM = 4 };

__host__ __device__ constexpr int rs_ghost_reach(int rs) { return rs == RS_PPM ? 2 : 1; }

// States (vp, vm) of one cell from its stencil w2 w1 v0 e1 e2 (v[c-2..c+2]).
template <int RS>
__device__ __forceinline__ void recon(int lim, int nv, float w2, float w1, float v0, float e1, float e2, float& vp,
                                      float& vm) {
  if (RS == RS_PPM) {
    float p = ppm_iface(w1, v0, e1, e2);
    float m = ppm_iface(w2, w1, v0, e1);
    ppm_limit(v0, p, m);
    vp = p;
    vm = m;
  } else {
    const int L = RS == RS_PLM_MC ? LIM_MC : RS == RS_PLM_MINMOD ? LIM_MINMOD : RS == RS_PLM_VANLEER ? LIM_VANLEER : lim;
    float dv = limit(L, nv, e1 - v0, v0 - w1);
    vp = v0 + dv * 0.5f;
    vm = v0 - dv * 0.5f;
  }
}

template <int DIR, bool CT>
__device__ __forceinline__ void solve_iface(const MixArgs& a, int solver, float* vL, float* vR, float bn,
                                            Iface<float>& o) {
  if (CT) {
    vL[Rot<DIR>::bn] = bn;
    vR[Rot<DIR>::bn] = bn;
  }
  const float gmm1 = a.gamma - 1.0f;
  float uL[NV], uR[NV], mach;
  prim_to_cons(vL, uL, gmm1);
  prim_to_cons(vR, uR, gmm1);
  if (solver == PG_HLL) {
    hll_solver<DIR, false>(vL, uL, vR, uR, a.gamma, o, mach);
  } else if (solver == PG_ROE) {
    int bad = 0;
    roe_solver<DIR, false>(vL, uL, vR, uR, a.gamma, a.ncomp == 3, o, mach, bad);
    if (bad) atomicOr(&a.sc->status, 2);
  } else {
    hlld_solver<DIR, false>(vL, uL, vR, uR, a.gamma, o, mach);
  }
}

// ---------------------------------------------------------------------------
// boundary (same maps as the FP64 path)
// ---------------------------------------------------------------------------
__device__ __forceinline__ int mbmap(int x, int beg, int end, int n, int type) {
  return bc_src(x, beg, end, n, type);
}

struct BoundArrays {
  float* q[11];
  int n, ncomp;
};

__global__ void k_mbound(Geom g, BoundArrays arr, int bcx, int bcy, int bcz, GhostSlabs gs) {
  long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  int i, j, k;
  if (!gs.coords(g, q, i, j, k)) return;
  int si = mbmap(i, g.beg[0], g.end[0], g.nx[0], bcx);
  int sj = g.dims > 1 ? mbmap(j, g.beg[1], g.end[1], g.nx[1], bcy) : j;
  int sk = g.dims > 2 ? mbmap(k, g.beg[2], g.end[2], g.nx[2], bcz) : k;
  long long dst = cidx(g, k, j, i), src = cidx(g, sk, sj, si);
  // mirror signs (FlipSign) of the first NV arrays, the cell variables
  const int bt[3] = {bcx, bcy, bcz};
  const int x[3] = {i, j, k};
  int flips = 0;
#pragma unroll
  for (int d = 0; d < 3; d++) {  // compile-time axis indices keep x, bt in registers
    if (d >= g.dims) break;
    if (x[d] < g.beg[d] || x[d] > g.end[d])
#pragma unroll
      for (int nv = 0; nv < NV; nv++)
        if (bc_flip(d, bc_side(bt[d], x[d] > g.end[d]), nv, arr.ncomp) < 0) flips ^= 1 << nv;
  }
#pragma unroll
  for (int a = 0; a < 11; a++) {  // compile-time indices: the pointer table stays a parameter
    if (a >= arr.n) break;
    const float v = arr.q[a][src];
    arr.q[a][dst] = (a < NV && ((flips >> a) & 1)) ? -v : v;
  }
}

// ---------------------------------------------------------------------------
// x sweep: a warp covers 32 consecutive cells of one row; lane l reconstructs
// cell i = ibase + l once, gets the right state of interface i+1/2 from lane
// l+1 and the flux of interface i-1/2 from lane l-1 (shuffles).  Lanes 1..30
// update their cell: 30 cells per warp, 31 interfaces, 32 reconstructions.
// ---------------------------------------------------------------------------
template <int RS, bool CT>
__global__ void __launch_bounds__(128) k_msweep_x(MixArgs a, int solver, int t_lo, int t_n, int b_lo, int nrows,
                                                  int stage1, int oned, int nwx) {
  const Geom& g = a.g;
  const int lane = threadIdx.x & 31;
  const int wid = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int wx = wid % nwx;
  const int row = wid / nwx;
  if (row >= nrows) return;  // the whole warp leaves together
  const int j = t_lo + row % t_n;
  const int k = b_lo + row / t_n;
  const int i = g.beg[0] - 1 + 30 * wx + lane;
  const bool cell_ok = i <= g.end[0] + 1;          // cells beg-1 .. end+1
  const bool face_ok = i <= g.end[0] && lane < 31;  // interfaces beg-1+1/2 .. end+1/2
  const int c = (k * g.nt[1] + j) * (int)g.s[1] + i;
  // loaded up front so that their latency overlaps the reconstruction
  const float bn = (CT && face_ok) ? a.Bin[0][c] : 0.f;
  const float scrh = a.sc->dtdx[0];
  float vp[NV], vm[NV];
#pragma unroll
  for (int nv = 0; nv < NV; nv++) {
    vp[nv] = vm[nv] = 0.f;
    if (cell_ok) {
      const float* V = a.Vin[nv];
      float w2 = RS == RS_PPM ? __ldg(V + c - 2) : 0.f;
      float e2 = RS == RS_PPM ? __ldg(V + c + 2) : 0.f;
      recon<RS>(a.limiter, nv, w2, __ldg(V + c - 1), __ldg(V + c), __ldg(V + c + 1), e2, vp[nv], vm[nv]);
    }
  }
  if (CT && cell_ok) {  // compile-time indices keep vp/vm in registers
#pragma unroll
    for (int comp = 0; comp < 3; comp++)
      if (comp < g.dims) a.DV[0][comp][c] = vp[VX1 + comp] - vm[VX1 + comp];
  }
  float vR[NV];
#pragma unroll
  for (int nv = 0; nv < NV; nv++) vR[nv] = __shfl_down_sync(0xffffffffu, vm[nv], 1);
  float fl[NV], pr = 0.f, cm = 0.f;
#pragma unroll
  for (int nv = 0; nv < NV; nv++) fl[nv] = 0.f;
  if (face_ok) {
    Iface<float> o;
    solve_iface<0, CT>(a, solver, vp, vR, bn, o);
#pragma unroll
    for (int nv = 0; nv < NV; nv++) fl[nv] = o.f[nv];
    pr = o.press;
    cm = o.cmax;
    if (CT) {
      a.S[0][0][c] = pmax(0.f, -o.SL);
      a.S[0][1][c] = pmax(0.f, o.SR);
    }
  }
  float flm[NV];
#pragma unroll
  for (int nv = 0; nv < NV; nv++) flm[nv] = __shfl_up_sync(0xffffffffu, fl[nv], 1);
  const float prm = __shfl_up_sync(0xffffffffu, pr, 1);
  const float cmm = __shfl_up_sync(0xffffffffu, cm, 1);
  if (lane >= 1 && lane <= 30 && i >= g.beg[0] && i <= g.end[0]) {
#pragma unroll
    for (int nv = 0; nv < NV; nv++) {
      if (!((a.accmask >> nv) & 1)) continue;
      float rhs = -scrh * (fl[nv] - flm[nv]);
      if (nv == VX1) rhs -= scrh * (pr - prm);
      a.dU[nv][c] = rhs;
    }
    // 2D/3D: C_dt term of update_stage.c:233; 1D: the larger adjacent
    // cmax (the 1D reduction of update_stage.c:237-241 is a plain max).
    if (oned) a.CDT[c] = pmax(cmm, cm) * a.inv_dx_f[0];
    else if (stage1) a.CDT[c] = 0.5f * (cmm + cm) * a.inv_dx_f[0];
  }
}

// ---------------------------------------------------------------------------
// x sweep with TMA staging: tiles of kXR rows (consecutive j at one k) by
// kXC chunks of 30 cells; warp r walks row r chunk by chunk with the lane
// arithmetic of k_msweep_x (32 reconstructions, 31 interfaces, 30 updated
// cells per chunk).  The rows' stencil (8 variables, one 4D box kXW floats
// wide, starting on a 16-byte boundary) and normal face field of the next
// tile are loaded by TMA into the other half of a double buffer.
// ---------------------------------------------------------------------------
// kXW covers the chunks' cells, a PPM stencil reach of 2 each side and up to
// 3 floats of alignment: 30 (kXC - 1) + 32 + 4 + 3 = 99, rounded to 16 bytes.
// kXC = 3 keeps the double buffer at 58 KB, so 3 blocks fit on an SM.
constexpr int kXR = 8, kXC = 3, kXW = 100, kXBLK = 3;

struct XSweepMaps {
  CUtensorMap V, B;
};

constexpr int kXBUF = (8 + 1) * kXR * kXW;                  // floats per buffer
constexpr int kXSMEM = 2 * kXBUF * 4 + 16;

template <int RS, bool CT>
__global__ void __launch_bounds__(32 * kXR, kXBLK)
    k_msweep_x_tma(const __grid_constant__ XSweepMaps maps, MixArgs a, int solver, int t_lo, int t_n, int b_lo,
                   int nxt, int njt, int ntiles, int stage1) {
  constexpr int REACH = rs_ghost_reach(RS);
  extern __shared__ __align__(128) float smem[];
  uint64_t* bar = (uint64_t*)(smem + 2 * kXBUF);
  const Geom& g = a.g;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const bool leader = threadIdx.x == 0;
  const float scrh = a.sc->dtdx[0];
  const int pitch = (int)g.s[1];
  const uint32_t tx_bytes = (uint32_t)((8 + (CT ? 1 : 0)) * kXR * kXW * 4);
  if (leader) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
  auto tile_of = [&](int t, int& cs, int& xs, int& j0, int& k) {
    const int xt = t % nxt, rest = t / nxt;
    cs = g.beg[0] - 1 + 30 * kXC * xt;  // first cell of the tile
    xs = (cs - REACH) & ~3;
    j0 = t_lo + kXR * (rest % njt);
    k = b_lo + rest / njt;
  };
  auto issue = [&](int t, int b) {
    int cs, xs, j0, k;
    tile_of(t, cs, xs, j0, k);
    float* base = smem + b * kXBUF;
    mbar_arrive_expect_tx(&bar[b], tx_bytes);
    tma_load_4d(base, &maps.V, xs, j0, k, 0, &bar[b]);
    if (CT) tma_load_3d(base + 8 * kXR * kXW, &maps.B, xs, j0, k, &bar[b]);
  };
  int it = 0;
  if (leader && (int)blockIdx.x < ntiles) issue(blockIdx.x, 0);
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x, it++) {
    const int b = it & 1;
    const int tn = t + gridDim.x;
    if (leader && tn < ntiles) {
      fence_proxy_async_smem();
      issue(tn, b ^ 1);
    }
    const bool ok = mbar_wait_bounded(&bar[b], (uint32_t)((it >> 1) & 1), a.tile_tries);
    if (__syncthreads_or(!ok)) {
      if (leader) {
        atomicOr(&a.sc->status, 8);
        mbar_wait_bounded(&bar[b], (uint32_t)((it >> 1) & 1));
        if (tn < ntiles) mbar_wait_bounded(&bar[b ^ 1], (uint32_t)(((it + 1) >> 1) & 1));
      }
      __syncthreads();
      return;
    }
    int cs, xs, j0, k;
    tile_of(t, cs, xs, j0, k);
    const int j = j0 + w;
    const bool row_ok = j < t_lo + t_n;
    const float* sV = smem + b * kXBUF + w * kXW;   // row w of variable 0
    const float* sB = smem + b * kXBUF + 8 * kXR * kXW + w * kXW;
    for (int q = 0; q < kXC; q++) {
      const int i = cs + 30 * q + lane;
      const bool cell_ok = row_ok && i <= g.end[0] + 1;
      const bool face_ok = row_ok && i <= g.end[0] && lane < 31;
      const int c = (k * g.nt[1] + j) * pitch + i;
      const int x = i - xs;  // column in the staged rows
      float vp[NV], vm[NV];
#pragma unroll
      for (int nv = 0; nv < NV; nv++) {
        vp[nv] = vm[nv] = 0.f;
        if (cell_ok) {
          const float* p = sV + nv * kXR * kXW + x;
          const float w2 = RS == RS_PPM ? p[-2] : 0.f;
          const float e2 = RS == RS_PPM ? p[2] : 0.f;
          recon<RS>(a.limiter, nv, w2, p[-1], p[0], p[1], e2, vp[nv], vm[nv]);
        }
      }
      if (CT && cell_ok) {  // compile-time indices keep vp/vm in registers
#pragma unroll
        for (int comp = 0; comp < 3; comp++)
          if (comp < g.dims) a.DV[0][comp][c] = vp[VX1 + comp] - vm[VX1 + comp];
      }
      float vR[NV];
#pragma unroll
      for (int nv = 0; nv < NV; nv++) vR[nv] = __shfl_down_sync(0xffffffffu, vm[nv], 1);
      float fl[NV], pr = 0.f, cm = 0.f;
#pragma unroll
      for (int nv = 0; nv < NV; nv++) fl[nv] = 0.f;
      if (face_ok) {
        Iface<float> o;
        solve_iface<0, CT>(a, solver, vp, vR, CT ? sB[x] : 0.f, o);
#pragma unroll
        for (int nv = 0; nv < NV; nv++) fl[nv] = o.f[nv];
        pr = o.press;
        cm = o.cmax;
        if (CT) {
          a.S[0][0][c] = pmax(0.f, -o.SL);
          a.S[0][1][c] = pmax(0.f, o.SR);
        }
      }
      float flm[NV];
#pragma unroll
      for (int nv = 0; nv < NV; nv++) flm[nv] = __shfl_up_sync(0xffffffffu, fl[nv], 1);
      const float prm = __shfl_up_sync(0xffffffffu, pr, 1);
      const float cmm = __shfl_up_sync(0xffffffffu, cm, 1);
      if (row_ok && lane >= 1 && lane <= 30 && i >= g.beg[0] && i <= g.end[0]) {
#pragma unroll
        for (int nv = 0; nv < NV; nv++) {
          if (!((a.accmask >> nv) & 1)) continue;
          float rhs = -scrh * (fl[nv] - flm[nv]);
          if (nv == VX1) rhs -= scrh * (pr - prm);
          a.dU[nv][c] = rhs;
        }
        if (stage1) a.CDT[c] = 0.5f * (cmm + cm) * a.inv_dx_f[0];
      }
    }
    __syncthreads();  // the buffer is free again
  }
}

// ---------------------------------------------------------------------------
// y/z sweep: block = 32 lanes along x by kTY rows along DIR.  Row ty holds
// cell m = m0 - 1 + ty: every row reconstructs its cell once (left states of
// the row above go through shared memory), rows 0..kTY-2 solve interface
// m+1/2, rows 1..kTY-2 update their cell from the fluxes of rows ty-1, ty.
// ---------------------------------------------------------------------------
constexpr int kTY = 12;

template <int RS, int DIR, bool CT>
__global__ void __launch_bounds__(32 * kTY, 2) k_msweep_t(MixArgs a, int solver, int i_lo, int i_n, int o_lo,
                                                          int o_n, int stage1) {
  __shared__ float svm[NV][kTY][32];
  __shared__ float sf[NV + 2][kTY][32];
  const Geom& g = a.g;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int nbx = (i_n + 31) >> 5;
  const int bx = blockIdx.x % nbx;
  const int bo = blockIdx.x / nbx;
  const int ii = 32 * bx + tx;
  const int i = i_lo + ii;
  const int other = o_lo + bo;
  const int beg = g.beg[DIR], end = g.end[DIR];
  const int m = beg - 1 + (kTY - 2) * (int)blockIdx.y + ty;
  const bool col_ok = ii < i_n && bo < o_n;
  const bool cell_ok = col_ok && m <= end + 1;               // cells beg-1 .. end+1
  const bool face_ok = col_ok && m <= end && ty < kTY - 1;   // interfaces beg-1+1/2 .. end+1/2
  const int s = (int)g.s[DIR];
  const int c = (DIR == 1 ? other * (int)g.s[2] : other * (int)g.s[1]) + i + m * s;
  // the accumulated update of this zone, loaded now so that its latency
  // overlaps the reconstruction and the Riemann problem
  const bool upd = ty >= 1 && ty <= kTY - 2 && col_ok && m >= beg && m <= end;
  float du[NV], cdt = 0.f;
#pragma unroll
  for (int nv = 0; nv < NV; nv++) du[nv] = (upd && ((a.accmask >> nv) & 1)) ? a.dU[nv][c] : 0.f;
  if (upd && stage1) cdt = a.CDT[c];
  const float bn = (CT && face_ok) ? a.Bin[DIR][c] : 0.f;
  const float scrh = a.sc->dtdx[DIR];
  float vp[NV], vm[NV];
#pragma unroll
  for (int nv = 0; nv < NV; nv++) {
    vp[nv] = vm[nv] = 0.f;
    if (cell_ok) {
      const float* V = a.Vin[nv];
      float w2 = RS == RS_PPM ? __ldg(V + c - 2 * s) : 0.f;
      float e2 = RS == RS_PPM ? __ldg(V + c + 2 * s) : 0.f;
      recon<RS>(a.limiter, nv, w2, __ldg(V + c - s), __ldg(V + c), __ldg(V + c + s), e2, vp[nv], vm[nv]);
    }
    svm[nv][ty][tx] = vm[nv];
  }
  if (CT && cell_ok) {  // compile-time indices keep vp/vm in registers
#pragma unroll
    for (int comp = 0; comp < 3; comp++)
      if (comp < g.dims) a.DV[DIR][comp][c] = vp[VX1 + comp] - vm[VX1 + comp];
  }
  __syncthreads();
  float fl[NV], pr = 0.f, cm = 0.f;
#pragma unroll
  for (int nv = 0; nv < NV; nv++) fl[nv] = 0.f;
  if (face_ok) {
    float vR[NV];
#pragma unroll
    for (int nv = 0; nv < NV; nv++) vR[nv] = svm[nv][ty + 1][tx];
    Iface<float> o;
    solve_iface<DIR, CT>(a, solver, vp, vR, bn, o);
#pragma unroll
    for (int nv = 0; nv < NV; nv++) fl[nv] = o.f[nv];
    pr = o.press;
    cm = o.cmax;
    if (CT) {
      a.S[DIR][0][c] = pmax(0.f, -o.SL);
      a.S[DIR][1][c] = pmax(0.f, o.SR);
    }
  }
#pragma unroll
  for (int nv = 0; nv < NV; nv++) sf[nv][ty][tx] = fl[nv];
  sf[NV][ty][tx] = pr;
  sf[NV + 1][ty][tx] = cm;
  __syncthreads();
  if (upd) {
#pragma unroll
    for (int nv = 0; nv < NV; nv++) {
      if (!((a.accmask >> nv) & 1)) continue;
      float rhs = -scrh * (fl[nv] - sf[nv][ty - 1][tx]);
      if (nv == Rot<DIR>::vn) rhs -= scrh * (pr - sf[NV][ty - 1][tx]);
      a.dU[nv][c] = du[nv] + rhs;
    }
    if (stage1) a.CDT[c] = cdt + 0.5f * (sf[NV + 1][ty - 1][tx] + cm) * a.inv_dx_f[DIR];
  }
}


// ---------------------------------------------------------------------------
// y/z sweep with TMA staging (used when the row pitch is a multiple of 16
// bytes): the tile and arithmetic of k_msweep_t, run by persistent blocks
// over all tiles.  One thread issues the bulk tensor loads of the block's
// next tile -- the stencil rows of the 8 variables (one 4D box), the
// accumulated update and C_dt of the updated rows, the normal face field of
// the interface rows -- into the other half of a double buffer, completed on
// an mbarrier, so they land while the block solves the current tile.
// ---------------------------------------------------------------------------
struct SweepMaps {
  CUtensorMap V, dU, CDT, B;
  CUtensorMap dU1;  // the RK2 stage-2 increments (a copy of dU without them)
};

template <int RS>
struct SweepTile {
  static constexpr int REACH = rs_ghost_reach(RS);
  static constexpr int R = kTY + 2 * REACH;  // stencil rows
  static constexpr int NU = kTY - 2;         // updated rows
  static constexpr int NF = kTY - 1;         // interface rows
  static constexpr int BUF = (8 * R + 8 * NU + NU + NF) * 32;  // floats per buffer
  static constexpr int SMEM = (2 * BUF + (NV + NV + 2) * kTY * 32) * 4 + 16;
};

template <int RS, int DIR, bool CT>
__global__ void __launch_bounds__(32 * kTY, 2)
    k_msweep_tma(const __grid_constant__ SweepMaps maps, MixArgs a, int solver, int xa, int i_lo, int i_n, int o_lo,
                 int nbx, int ncols, int ntiles, int stage1, int dsel) {
  using TL = SweepTile<RS>;
  const CUtensorMap* du_map = dsel ? &maps.dU1 : &maps.dU;  // the array a.dU points to
  constexpr int REACH = TL::REACH, R = TL::R, NU = TL::NU, NF = TL::NF, BUF = TL::BUF;
  extern __shared__ __align__(128) float smem[];
  float* svm = smem + 2 * BUF;        // [NV][kTY][32]
  float* sf = svm + NV * kTY * 32;    // [NV + 2][kTY][32]
  uint64_t* bar = (uint64_t*)(sf + (NV + 2) * kTY * 32);
  const Geom& g = a.g;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const bool leader = tx == 0 && ty == 0;
  const int beg = g.beg[DIR], end = g.end[DIR];
  const int s = (int)g.s[DIR];
  const float scrh = a.sc->dtdx[DIR];
  const uint32_t tx_bytes = (uint32_t)((8 * R + 8 * NU + (stage1 ? NU : 0) + (CT ? NF : 0)) * 32 * 4);
  if (leader) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
  auto issue = [&](int t, int b) {
    const int col = t % ncols, rb = t / ncols;
    const int x0 = xa + 32 * (col % nbx), other = o_lo + col / nbx;
    const int m0 = beg + NU * rb;
    float* base = smem + b * BUF;
    mbar_arrive_expect_tx(&bar[b], tx_bytes);
    if (DIR == 1) {
      tma_load_4d(base, &maps.V, x0, m0 - 1 - REACH, other, 0, &bar[b]);
      tma_load_4d(base + 8 * R * 32, du_map, x0, m0, other, 0, &bar[b]);
      if (stage1) tma_load_3d(base + (8 * R + 8 * NU) * 32, &maps.CDT, x0, m0, other, &bar[b]);
      if (CT) tma_load_3d(base + (8 * R + 9 * NU) * 32, &maps.B, x0, m0 - 1, other, &bar[b]);
    } else {
      tma_load_4d(base, &maps.V, x0, other, m0 - 1 - REACH, 0, &bar[b]);
      tma_load_4d(base + 8 * R * 32, du_map, x0, other, m0, 0, &bar[b]);
      if (stage1) tma_load_3d(base + (8 * R + 8 * NU) * 32, &maps.CDT, x0, other, m0, &bar[b]);
      if (CT) tma_load_3d(base + (8 * R + 9 * NU) * 32, &maps.B, x0, other, m0 - 1, &bar[b]);
    }
  };
  int it = 0;
  if (leader && (int)blockIdx.x < ntiles) issue(blockIdx.x, 0);
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x, it++) {
    const int b = it & 1;
    const int tn = t + gridDim.x;
    if (leader && tn < ntiles) {
      fence_proxy_async_smem();  // buffer b^1 was read by the block in the previous iteration
      issue(tn, b ^ 1);
    }
    const bool ok = mbar_wait_bounded(&bar[b], (uint32_t)((it >> 1) & 1), a.tile_tries);
    if (__syncthreads_or(!ok)) {
      // a load did not complete in time: report, let the copies in flight
      // land (bounded), leave
      if (leader) {
        atomicOr(&a.sc->status, 8);
        mbar_wait_bounded(&bar[b], (uint32_t)((it >> 1) & 1));
        if (tn < ntiles) mbar_wait_bounded(&bar[b ^ 1], (uint32_t)(((it + 1) >> 1) & 1));
      }
      __syncthreads();
      return;
    }
    const int col = t % ncols, rb = t / ncols;
    const int i = xa + 32 * (col % nbx) + tx;
    const int other = o_lo + col / nbx;
    const int m = beg + NU * rb - 1 + ty;
    const bool col_ok = i >= i_lo && i < i_lo + i_n;
    const bool cell_ok = col_ok && m <= end + 1;
    const bool face_ok = col_ok && m <= end && ty < kTY - 1;
    const bool upd = ty >= 1 && ty <= kTY - 2 && col_ok && m >= beg && m <= end;
    const int c = (DIR == 1 ? other * (int)g.s[2] : other * (int)g.s[1]) + i + m * s;
    const float* sV = smem + b * BUF;
    const float* sDU = sV + 8 * R * 32;
    const float* sCDT = sDU + 8 * NU * 32;
    const float* sB = sCDT + NU * 32;
    float vp[NV], vm[NV];
#pragma unroll
    for (int nv = 0; nv < NV; nv++) {
      vp[nv] = vm[nv] = 0.f;
      if (cell_ok) {
        const float* q = sV + (nv * R + ty + REACH) * 32 + tx;
        const float w2 = RS == RS_PPM ? q[-64] : 0.f;
        const float e2 = RS == RS_PPM ? q[64] : 0.f;
        recon<RS>(a.limiter, nv, w2, q[-32], q[0], q[32], e2, vp[nv], vm[nv]);
      }
      svm[(nv * kTY + ty) * 32 + tx] = vm[nv];
    }
    if (CT && cell_ok) {  // compile-time indices keep vp/vm in registers
#pragma unroll
      for (int comp = 0; comp < 3; comp++)
        if (comp < g.dims) a.DV[DIR][comp][c] = vp[VX1 + comp] - vm[VX1 + comp];
    }
    __syncthreads();
    float fl[NV], pr = 0.f, cm = 0.f;
#pragma unroll
    for (int nv = 0; nv < NV; nv++) fl[nv] = 0.f;
    if (face_ok) {
      float vR[NV];
#pragma unroll
      for (int nv = 0; nv < NV; nv++) vR[nv] = svm[(nv * kTY + ty + 1) * 32 + tx];
      const float bn = CT ? sB[ty * 32 + tx] : 0.f;
      Iface<float> o;
      solve_iface<DIR, CT>(a, solver, vp, vR, bn, o);
#pragma unroll
      for (int nv = 0; nv < NV; nv++) fl[nv] = o.f[nv];
      pr = o.press;
      cm = o.cmax;
      if (CT) {
        a.S[DIR][0][c] = pmax(0.f, -o.SL);
        a.S[DIR][1][c] = pmax(0.f, o.SR);
      }
    }
#pragma unroll
    for (int nv = 0; nv < NV; nv++) sf[(nv * kTY + ty) * 32 + tx] = fl[nv];
    sf[(NV * kTY + ty) * 32 + tx] = pr;
    sf[((NV + 1) * kTY + ty) * 32 + tx] = cm;
    __syncthreads();
    if (upd) {
#pragma unroll
      for (int nv = 0; nv < NV; nv++) {
        if (!((a.accmask >> nv) & 1)) continue;
        float rhs = -scrh * (fl[nv] - sf[(nv * kTY + ty - 1) * 32 + tx]);
        if (nv == Rot<DIR>::vn) rhs -= scrh * (pr - sf[(NV * kTY + ty - 1) * 32 + tx]);
        a.dU[nv][c] = sDU[(nv * NU + ty - 1) * 32 + tx] + rhs;
      }
      if (stage1)
        a.CDT[c] = sCDT[(ty - 1) * 32 + tx] + 0.5f * (sf[((NV + 1) * kTY + ty - 1) * 32 + tx] + cm) * a.inv_dx_f[DIR];
    }
    __syncthreads();  // the buffer and the exchange arrays are free again
  }
}

// ---------------------------------------------------------------------------
// y/z sweep marching along DIR: a thread walks one column segment of `seg`
// cells, keeping the stencil planes, the left state of the interface above
// and the flux of the interface below in registers.  No halo rows: a
// segment reconstructs one extra cell and solves one extra Riemann problem
// at its start.  A warp covers 32 consecutive x, so every load and store is
// a whole 128-byte row.  What a cell needs from memory (the next stencil
// plane, its accumulated update, C_dt and normal face field) is copied
// asynchronously into a per-thread shared-memory slot one cell ahead, so no
// registers wait on it.  Same arithmetic, per cell, as k_msweep_t.
// ---------------------------------------------------------------------------
// resident blocks of k_msweep_m: PPM's five stencil planes need the
// registers of 3 blocks per SM (170 per thread), PLM fits 4 (128)
__host__ __device__ constexpr int march_min_blocks(int rs) { return rs == RS_PPM ? 3 : 4; }
constexpr int kMarchThreads = 128;

template <int RS, int DIR, bool CT>
__global__ void __launch_bounds__(kMarchThreads, march_min_blocks(RS))
    k_msweep_m(MixArgs a, int solver, int i_lo, int i_n, int o_lo, int o_n, int seg, int nseg, int stage1) {
  constexpr int REACH = rs_ghost_reach(RS);
  constexpr int NP = 2 * REACH + 1;  // stencil planes of one cell
  // staged per cell: the next plane (NV), dU (NV), C_dt, the face field
  constexpr int NS = 2 * NV + 2, S_PL = 0, S_DU = NV, S_CDT = 2 * NV, S_BN = 2 * NV + 1;
  __shared__ float sbuf[2][NS][kMarchThreads];
  const Geom& g = a.g;
  const int tid = threadIdx.x, lane = tid & 31;
  const long long wi = (blockIdx.x * (long long)blockDim.x + tid) >> 5;
  const int nbx = (i_n + 31) >> 5;
  const int bx = (int)(wi % nbx);
  const long long rest = wi / nbx;
  const int o = (int)(rest % o_n), sg = (int)(rest / o_n);
  const int i = i_lo + 32 * bx + lane;
  if (sg >= nseg || i >= i_lo + i_n) return;  // no block-wide synchronisation below
  const int other = o_lo + o;
  const int beg = g.beg[DIR], end = g.end[DIR];
  const int m0 = beg + sg * seg;
  const int m1 = m0 + seg - 1 < end ? m0 + seg - 1 : end;
  const long long s = g.s[DIR];
  const long long cb = (DIR == 1 ? (long long)other * g.s[2] : (long long)other * g.s[1]) + i;
  const float scrh = a.sc->dtdx[DIR];
  const float idx = a.inv_dx_f[DIR];
  constexpr int VN = Rot<DIR>::vn;
  // The interface two segments share (m0-1/2) is solved by the loop body in
  // both, the only inlined copy of the Riemann solver (two copies may
  // contract multiply-adds differently), from the same inputs: its flux is
  // bit-identical on either side and the update stays conservative.  The
  // left state there, cell m0-1's, is reconstructed before the loop under
  // PLM, whose only multiply-add (v0 +- dv/2) rounds the same contracted or
  // not; PPM's weighted sums may not, so under PPM the loop starts one cell
  // earlier: iteration m0-2 reconstructs cell m0-1 and its Riemann problem,
  // which has no left state, is discarded.
  constexpr bool kPre = RS != RS_PPM;
  const int mstart = kPre ? m0 - 1 : m0 - 2;
  // planes pl[t] = V at m - REACH + t for the cell m being reconstructed next
  float pl[NP][NV];
#pragma unroll
  for (int t = 0; t < NP; t++)
#pragma unroll
    for (int nv = 0; nv < NV; nv++) pl[t][nv] = ldg(a.Vin[nv], cb + (m0 - 1 - REACH + t) * s);
  // the copies iteration m reads: the plane of cell m+1's stencil top (not
  // in the discarded iteration, whose planes are already in place), dU and
  // C_dt of cell m when it is updated, the face field of interface m+1/2
  auto stage = [&](int b, int m) {
    const long long c = cb + m * s;
    const bool first = !kPre && m < m0 - 1, upd = m >= m0;
    if (!first) {
#pragma unroll
      for (int nv = 0; nv < NV; nv++) cp_async4(&sbuf[b][S_PL + nv][tid], a.Vin[nv] + c + (1 + REACH) * s);
      if (CT) cp_async4(&sbuf[b][S_BN][tid], a.Bin[DIR] + c);
    }
    if (upd) {
#pragma unroll
      for (int nv = 0; nv < NV; nv++)
        if ((a.accmask >> nv) & 1) cp_async4(&sbuf[b][S_DU + nv][tid], a.dU[nv] + c);
      if (stage1) cp_async4(&sbuf[b][S_CDT][tid], a.CDT + c);
    }
    cp_async_commit();
  };
  auto reconstruct = [&](float* vp, float* vm) {
#pragma unroll
    for (int nv = 0; nv < NV; nv++)
      recon<RS>(a.limiter, nv, RS == RS_PPM ? pl[0][nv] : 0.f, pl[REACH - 1][nv], pl[REACH][nv],
                pl[REACH + 1][nv], RS == RS_PPM ? pl[NP - 1][nv] : 0.f, vp[nv], vm[nv]);
  };
  auto store_dv = [&](long long c, const float* vp, const float* vm) {
#pragma unroll
    for (int comp = 0; comp < 3; comp++)
      if (comp < g.dims) a.DV[DIR][comp][c] = vp[VX1 + comp] - vm[VX1 + comp];
  };
  float vpC[NV], vmC[NV], fp[NV], pp = 0.f, cmp = 0.f;
#pragma unroll
  for (int nv = 0; nv < NV; nv++) vpC[nv] = vmC[nv] = fp[nv] = 0.f;
  if (kPre) {
    reconstruct(vpC, vmC);  // cell m0-1
  } else {
    vpC[RHO] = 1.f;  // a harmless left state for the discarded problem
    vpC[PRS] = 1.f;
  }
  stage(0, mstart);
  // cell m+1 reconstructed, interface m+1/2 solved, cell m updated
  // not unrolled: a second inlined copy of the solver could solve the
  // shared interface differently in the two segments
#pragma unroll 1
  for (int m = mstart, it = 0; m <= m1; m++, it++) {
    const int b = it & 1;
    if (m < m1) stage(b ^ 1, m + 1);  // buffer b^1 was read in the previous iteration
    else cp_async_commit();           // (an empty group keeps the count)
    cp_async_wait<1>();               // this iteration's copies have landed
    const long long c = cb + m * s;
    const bool upd = m >= m0;
    const bool first = !kPre && m < m0 - 1;          // the discarded problem
    const bool side = upd || (!first && m0 == beg);  // cell m0-1 and its interface: the first segment's
    const float bn = (CT && !first) ? sbuf[b][S_BN][tid] : 0.f;
    if (CT && side) store_dv(c, vpC, vmC);
    float vpN[NV], vmN[NV];
    if (!first) {  // the planes of cell m+1
#pragma unroll
      for (int t = 0; t + 1 < NP; t++)
#pragma unroll
        for (int nv = 0; nv < NV; nv++) pl[t][nv] = pl[t + 1][nv];
#pragma unroll
      for (int nv = 0; nv < NV; nv++) pl[NP - 1][nv] = sbuf[b][S_PL + nv][tid];
    }
    reconstruct(vpN, vmN);
    Iface<float> f;
    solve_iface<DIR, CT>(a, solver, vpC, vmN, bn, f);
    if (CT && side) {
      a.S[DIR][0][c] = pmax(0.f, -f.SL);
      a.S[DIR][1][c] = pmax(0.f, f.SR);
    }
    if (upd) {
#pragma unroll
      for (int nv = 0; nv < NV; nv++) {
        if (!((a.accmask >> nv) & 1)) continue;
        float rhs = -scrh * (f.f[nv] - fp[nv]);
        if (nv == VN) rhs -= scrh * (f.press - pp);
        a.dU[nv][c] = sbuf[b][S_DU + nv][tid] + rhs;
      }
      if (stage1) a.CDT[c] = sbuf[b][S_CDT][tid] + 0.5f * (cmp + f.cmax) * idx;
    }
#pragma unroll
    for (int nv = 0; nv < NV; nv++) {
      fp[nv] = f.f[nv];
      vpC[nv] = vpN[nv];
      vmC[nv] = vmN[nv];
    }
    pp = f.press;
    cmp = f.cmax;
  }
  cp_async_wait<0>();  // nothing left in flight when the thread exits
  if (CT && m1 == end) store_dv(cb + (end + 1) * s, vpC, vmC);
}

// ---------------------------------------------------------------------------
// edge EMFs (FP32)
// ---------------------------------------------------------------------------
template <int E>
__device__ __forceinline__ float muct_edge(const MixArgs& a, long long c) {
  constexpr int AX = E == 2 ? 0 : (E == 0 ? 1 : 2);
  constexpr int AY = E == 2 ? 1 : (E == 0 ? 2 : 0);
  const Geom& g = a.g;
  const long long sx = g.s[AX], sy = g.s[AY];
  const long long c00 = c, cx0 = c + sx, c0y = c + sy, cxy = c + sx + sy;
  float a_xp = pmax(ldg(a.S[AX][1], c00), ldg(a.S[AX][1], c0y));
  float a_xm = pmax(ldg(a.S[AX][0], c00), ldg(a.S[AX][0], c0y));
  float a_yp = pmax(ldg(a.S[AY][1], c00), ldg(a.S[AY][1], cx0));
  float a_ym = pmax(ldg(a.S[AY][0], c00), ldg(a.S[AY][0], cx0));
  const float* bxa = a.Bin[AX];
  const float* bya = a.Bin[AY];
  float sbS = mc_lim2(ldg(bxa, c00 + sy) - ldg(bxa, c00), ldg(bxa, c00) - ldg(bxa, c00 - sy));
  float sbN = mc_lim2(ldg(bxa, c0y + sy) - ldg(bxa, c0y), ldg(bxa, c0y) - ldg(bxa, c0y - sy));
  float sbW = mc_lim2(ldg(bya, c00 + sx) - ldg(bya, c00), ldg(bya, c00) - ldg(bya, c00 - sx));
  float sbE = mc_lim2(ldg(bya, cx0 + sx) - ldg(bya, cx0), ldg(bya, cx0) - ldg(bya, cx0 - sx));
  float bS = ldg(bxa, c00) + 0.5f * sbS;
  float bW = ldg(bya, c00) + 0.5f * sbW;
  float bN = ldg(bxa, c0y) - 0.5f * sbN;
  float bE = ldg(bya, cx0) - 0.5f * sbE;
  const float* vx = a.Vin[VX1 + AX];
  const float* vy = a.Vin[VX1 + AY];
  const float* dvx_dx = a.DV[AX][AX];
  const float* dvx_dy = a.DV[AY][AX];
  const float* dvy_dx = a.DV[AX][AY];
  const float* dvy_dy = a.DV[AY][AY];
  float eSW = (ldg(vy, c00) + 0.5f * (ldg(dvy_dx, c00) + ldg(dvy_dy, c00))) * bS -
              (ldg(vx, c00) + 0.5f * (ldg(dvx_dx, c00) + ldg(dvx_dy, c00))) * bW;
  float eSE = (ldg(vy, cx0) - 0.5f * (ldg(dvy_dx, cx0) - ldg(dvy_dy, cx0))) * bS -
              (ldg(vx, cx0) - 0.5f * (ldg(dvx_dx, cx0) - ldg(dvx_dy, cx0))) * bE;
  float eNE = (ldg(vy, cxy) - 0.5f * (ldg(dvy_dx, cxy) + ldg(dvy_dy, cxy))) * bN -
              (ldg(vx, cxy) - 0.5f * (ldg(dvx_dx, cxy) + ldg(dvx_dy, cxy))) * bE;
  float eNW = (ldg(vy, c0y) + 0.5f * (ldg(dvy_dx, c0y) - ldg(dvy_dy, c0y))) * bN -
              (ldg(vx, c0y) + 0.5f * (ldg(dvx_dx, c0y) - ldg(dvx_dy, c0y))) * bW;
  return uct_hll_combine(a_xp, a_xm, a_yp, a_ym, eSW, eSE, eNE, eNW, bS, bN, bW, bE);
}

__global__ void k_memf(MixArgs a, Box box) {
  long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= box.count()) return;
  int i, j, k;
  box.coords(q, i, j, k);
  long long c = cidx(a.g, k, j, i);
  // the three edges first, then the stores: with no store in between the
  // compiler shares the loads the edges have in common (S, velocities, slopes
  // and faces of the zone and of its +x/+y/+z neighbours)
  const float ez = muct_edge<2>(a, c);
  if (a.g.dims == 3) {
    const float ex = muct_edge<0>(a, c);
    const float ey = muct_edge<1>(a, c);
    a.E[0][c] = ex;
    a.E[1][c] = ey;
  }
  a.E[2][c] = ez;
}

// CT face update: EMF differences in FP32, accumulation into the face field
// and the RK face combination in the accumulator type A (double or dw).
template <int STAGE, int NSTAGE, class A>
__global__ void k_mface(MixArgs a, Box box) {
  using O = Acc<A>;
  long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= box.count()) return;
  int i, j, k;
  box.coords(q, i, j, k);
  const Geom& g = a.g;
  const long long c = cidx(g, k, j, i);
  const bool d3 = g.dims == 3;
  const float* E1 = a.E[0];
  const float* E2 = a.E[1];
  const float* E3 = a.E[2];
  const float f1 = a.sc->dtdx[0], f2 = a.sc->dtdx[1], f3 = a.sc->dtdx[2];
  // the box spans beg-1..end on every active axis; face fd needs x >= beg on
  // the other active axes
  const bool in0 = i >= g.beg[0], in1 = g.dims < 2 || j >= g.beg[1], in2 = g.dims < 3 || k >= g.beg[2];
#pragma unroll
  for (int fd = 0; fd < 3; fd++) {
    if (fd >= g.dims) break;
    const bool in = (fd == 0 || in0) && (fd == 1 || in1) && (fd == 2 || in2);
    if (!in) continue;
    float rhs;
    if (fd == 0) {
      rhs = -f2 * (E3[c] - E3[c - g.s[1]]);
      if (d3) rhs += f3 * (E2[c] - E2[c - g.s[2]]);
    } else if (fd == 1) {
      rhs = f1 * (E3[c] - E3[c - 1]);
      if (d3) rhs -= f3 * (E1[c] - E1[c - g.s[2]]);
    } else {
      rhs = -f1 * (E2[c] - E2[c - 1]) + f2 * (E1[c] - E1[c - g.s[1]]);
    }
    typename O::T bb;
    if (STAGE == 2 && NSTAGE == 2) {  // (B0 + B + rhs) / 2
      bb = O::half_sum3(O::from(a.B0[fd][c]), O::from(a.Bin[fd][c]), rhs);
    } else {
      bb = O::addf(O::from(a.Bin[fd][c]), rhs);
    }
    if (STAGE == 2) {
      if (NSTAGE == 3) bb = O::add(O::mulf(O::from(a.B0[fd][c]), 0.75f), O::mulf(bb, 0.25f));
    } else if (STAGE == 3) {
      typename O::T third = O::konst(1.0 / 3.0, a.third_hi, a.third_lo);
      bb = O::mul(O::add(O::from(a.B0[fd][c]), O::mulf(bb, 2.0f)), third);
    }
    a.Bout[fd][c] = O::tof(bb);
  }
}

// Conserved variables of an FP32 primitive state in the accumulator type.
template <class A>
struct ConsA {
  typename Acc<A>::T rho, m[3], E, b[3];
};

template <class A>
__device__ __forceinline__ ConsA<A> cons_of(const float* v, typename Acc<A>::T inv_gmm1) {
  using O = Acc<A>;
  ConsA<A> u;
  u.rho = O::from(v[RHO]);
#pragma unroll
  for (int q = 0; q < 3; q++) {
    u.m[q] = O::prod(v[RHO], v[VX1 + q]);
    u.b[q] = O::from(v[BX1 + q]);
  }
  typename O::T kin = O::add(O::add(O::prod(v[VX1], v[VX1]), O::prod(v[VX2], v[VX2])), O::prod(v[VX3], v[VX3]));
  typename O::T b2 = O::add(O::add(O::prod(v[BX1], v[BX1]), O::prod(v[BX2], v[BX2])), O::prod(v[BX3], v[BX3]));
  typename O::T kinb2 = O::mulf(O::add(O::mulf(kin, v[RHO]), b2), 0.5f);
  u.E = O::add(kinb2, O::mulf(inv_gmm1, v[PRS]));
  return u;
}

template <int STAGE, int NSTAGE, class A>
__global__ void k_mfinal(MixArgs a, Box dom, int reduce_cdt) {
  using O = Acc<A>;
  using T = typename O::T;
  long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  float cd = 0.f;
  bool fails = false, bad = false;
  if (q < dom.count()) {
    int i, j, k;
    dom.coords(q, i, j, k);
    const Geom& g = a.g;
    const long long c = cidx(g, k, j, i);
    const T inv_gmm1 = O::konst(a.inv_gmm1_d, a.inv_gmm1_hi, a.inv_gmm1_lo);
    const long long n = g.ncell;
    const int msk = a.accmask;
    // RK2 corrector (U0 + U1 + dU1)/2 with U1 = U0 + dU0: U0 + (dU0 + dU1)/2,
    // the FP32 increments summed before the one FP64 addition.  Where stage
    // 1 hit a floor, U1 is not U0 + dU0: that zone's U1 was stored and the
    // corrector takes it as written.
    const bool rk2c = STAGE == 2 && NSTAGE == 2;
    const bool floored1 = rk2c && (a.flag[c] & FLAG_CONS2PRIM_FAIL);
    // the resident accumulators: U of the previous stage (stage 1 and the
    // RK2 corrector: of the step start); the cell field under CT comes from
    // the faces below
    const void* Uin = (STAGE == 1 || (rk2c && !floored1)) ? a.U0 : a.Us;
    ConsA<A> u;
    u.rho = O::ld(Uin, RHO * n + c);
    u.E = O::ld(Uin, ENG * n + c);
#pragma unroll
    for (int d = 0; d < 3; d++) {
      u.m[d] = O::ld(Uin, (VX1 + d) * n + c);
      u.b[d] = (msk & (1 << (BX1 + d))) ? O::ld(Uin, (BX1 + d) * n + c) : O::from(0.f);
    }
    // U += dU (flux differences of all directions, FP32) in A; only the
    // accumulated variables (the cell field under CT comes from the faces)
    float du[NV];
#pragma unroll
    for (int nv = 0; nv < NV; nv++) du[nv] = (msk & (1 << nv)) ? a.dU[nv][c] : 0.f;
    const bool frozen = a.intb && (a.flag[c] & PG_FLAG_INTERNAL_BOUNDARY);  // Src/int_bound_reset.c:33-37
    if (frozen)
#pragma unroll
      for (int nv = 0; nv < NV; nv++) du[nv] = 0.f;
    if (rk2c && !floored1) {  // U0 + (dU0 + dU1)/2, the increments summed in A
      float dp[NV];
#pragma unroll
      for (int nv = 0; nv < NV; nv++) dp[nv] = ((msk & (1 << nv)) && !frozen) ? a.dUp[nv][c] : 0.f;
      if (msk & (1 << RHO)) u.rho = O::add_half_sum(u.rho, dp[RHO], du[RHO]);
#pragma unroll
      for (int d = 0; d < 3; d++) {
        if (msk & (1 << (VX1 + d))) u.m[d] = O::add_half_sum(u.m[d], dp[VX1 + d], du[VX1 + d]);
        if (msk & (1 << (BX1 + d))) u.b[d] = O::add_half_sum(u.b[d], dp[BX1 + d], du[BX1 + d]);
      }
      if (msk & (1 << ENG)) u.E = O::add_half_sum(u.E, dp[ENG], du[ENG]);
    } else if (rk2c) {  // (U0 + U1 + dU1) / 2 with the stored U1
      const T u0rho = O::ld(a.U0, RHO * n + c), u0E = O::ld(a.U0, ENG * n + c);
      u.rho = O::half_sum3(u0rho, u.rho, du[RHO]);
      u.E = O::half_sum3(u0E, u.E, du[ENG]);
#pragma unroll
      for (int d = 0; d < 3; d++) {
        u.m[d] = O::half_sum3(O::ld(a.U0, (VX1 + d) * n + c), u.m[d], du[VX1 + d]);
        if (msk & (1 << (BX1 + d))) u.b[d] = O::half_sum3(O::ld(a.U0, (BX1 + d) * n + c), u.b[d], du[BX1 + d]);
      }
    } else {
      if (msk & (1 << RHO)) u.rho = O::addf(u.rho, du[RHO]);
#pragma unroll
      for (int d = 0; d < 3; d++) {
        if (msk & (1 << (VX1 + d))) u.m[d] = O::addf(u.m[d], du[VX1 + d]);
        if (msk & (1 << (BX1 + d))) u.b[d] = O::addf(u.b[d], du[BX1 + d]);
      }
      if (msk & (1 << ENG)) u.E = O::addf(u.E, du[ENG]);
    }
    if (STAGE >= 2 && NSTAGE == 3) {
      ConsA<A> u0;
      u0.rho = O::ld(a.U0, RHO * n + c);
      u0.E = O::ld(a.U0, ENG * n + c);
#pragma unroll
      for (int d = 0; d < 3; d++) {
        u0.m[d] = O::ld(a.U0, (VX1 + d) * n + c);
        u0.b[d] = (msk & (1 << (BX1 + d))) ? O::ld(a.U0, (BX1 + d) * n + c) : O::from(0.f);
      }
      if (STAGE == 2) {
        u.rho = O::add(O::mulf(u0.rho, 0.75f), O::mulf(u.rho, 0.25f));
        u.E = O::add(O::mulf(u0.E, 0.75f), O::mulf(u.E, 0.25f));
#pragma unroll
        for (int d = 0; d < 3; d++) {
          u.m[d] = O::add(O::mulf(u0.m[d], 0.75f), O::mulf(u.m[d], 0.25f));
          u.b[d] = O::add(O::mulf(u0.b[d], 0.75f), O::mulf(u.b[d], 0.25f));
        }
      } else {
        const T third = O::konst(1.0 / 3.0, a.third_hi, a.third_lo);
        u.rho = O::mul(O::add(u0.rho, O::mulf(u.rho, 2.0f)), third);
        u.E = O::mul(O::add(u0.E, O::mulf(u.E, 2.0f)), third);
#pragma unroll
        for (int d = 0; d < 3; d++) {
          u.m[d] = O::mul(O::add(u0.m[d], O::mulf(u.m[d], 2.0f)), third);
          u.b[d] = O::mul(O::add(u0.b[d], O::mulf(u.b[d], 2.0f)), third);
        }
      }
    }
    // CT_AverageMagneticField: staggered components from the new faces
    if (a.ct) {  // compile-time indices keep the state in registers
#pragma unroll
      for (int d = 0; d < 3; d++)
        if (d < g.dims) u.b[d] = O::avg2(a.Bout[d][c], a.Bout[d][c - g.s[d]]);
    }
    // ConsToPrim (Src/MHD/mappers.c:88-254) with the pressure recovered in A
    unsigned char fl = 0;
    if (O::neg(u.rho)) {
      u.rho = O::from((float)a.small_rho);
      fl = FLAG_CONS2PRIM_FAIL;
    }
    const float rho_f = O::tof(u.rho);
    const float tau = 1.0f / rho_f;
    float vel[3];
#pragma unroll
    for (int d = 0; d < 3; d++) vel[d] = O::tof(u.m[d]) * tau;
    T m2 = O::add(O::add(O::mul(u.m[0], u.m[0]), O::mul(u.m[1], u.m[1])), O::mul(u.m[2], u.m[2]));
    T b2 = O::add(O::add(O::mul(u.b[0], u.b[0]), O::mul(u.b[1], u.b[1])), O::mul(u.b[2], u.b[2]));
    // twice the kinetic + magnetic energy density, m^2/rho + B^2, with the
    // reciprocal's last multiply fused into the sum; p = (E - kin2/2)(g-1)
    const T kin2 = O::fmadd(m2, O::rcp(u.rho), b2);
    if (O::neg(u.E)) {
      u.E = O::add(O::mulf(inv_gmm1, (float)a.small_p), O::mulf(kin2, 0.5f));
      fl = FLAG_CONS2PRIM_FAIL;
    }
    float p = O::tof(O::mulf(O::sub_half(u.E, kin2), a.gamma - 1.0f));
    if (p < 0.f) {  // floor and recompute the energy (Src/MHD/mappers.c:190-200)
      p = (float)a.small_p;
      u.E = O::add(O::mulf(inv_gmm1, (float)a.small_p), O::mulf(kin2, 0.5f));
      fl = FLAG_CONS2PRIM_FAIL;
    }
    // the accumulators of the next stage (the last stage: of the next step);
    // RK2's stage 1 stores its result only where a floor changed it (the
    // corrector rebuilds the others from U0 and the increments)
    void* Uout = STAGE == NSTAGE ? a.U0 : a.Us;
    if (!(NSTAGE == 2 && STAGE == 1) || fl) {
      O::st(Uout, RHO * n + c, u.rho);
      O::st(Uout, ENG * n + c, u.E);
#pragma unroll
      for (int d = 0; d < 3; d++) {
        O::st(Uout, (VX1 + d) * n + c, u.m[d]);
        if (msk & (1 << (BX1 + d))) O::st(Uout, (BX1 + d) * n + c, u.b[d]);
      }
    }
    float out[NV] = {rho_f, vel[0], vel[1], vel[2], O::tof(u.b[0]), O::tof(u.b[1]), O::tof(u.b[2]), p};
#pragma unroll
    for (int nv = 0; nv < NV; nv++) {
      a.Vout[nv][c] = out[nv];
      bad |= ((__float_as_uint(out[nv]) >> 23) & 0xff) == 0xff;
    }
    if (fl) {
      a.flag[c] |= fl;
      fails = true;
    }
    if (reduce_cdt) cd = a.CDT[c];
  }
  if (reduce_cdt) {  // the max is exact in FP32; the global reduction runs on FP64 bits
    for (int o = 16; o > 0; o >>= 1) {
      float w = __shfl_down_sync(0xffffffffu, cd, o);
      cd = (w > cd || w != w) ? w : cd;
    }
    if ((threadIdx.x & 31) == 0) atomic_max_nonneg_d(&a.sc->inv_dt_bits, (double)cd);
  }
  unsigned ball = __ballot_sync(0xffffffffu, fails);
  if ((threadIdx.x & 31) == 0 && ball) atomicAdd(&a.sc->nfail, (unsigned long long)__popc(ball));
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(&a.sc->status, 1);
}

// U0 from the primitive state (PrimToCons in the accumulator type), after
// the host set the state.
template <class A>
__global__ void k_mcons_init(MixArgs a, Box dom) {
  using O = Acc<A>;
  long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= dom.count()) return;
  int i, j, k;
  dom.coords(q, i, j, k);
  const Geom& g = a.g;
  const long long c = cidx(g, k, j, i), n = g.ncell;
  float v[NV];
#pragma unroll
  for (int nv = 0; nv < NV; nv++) v[nv] = a.Vin[nv][c];
  const ConsA<A> u = cons_of<A>(v, O::konst(a.inv_gmm1_d, a.inv_gmm1_hi, a.inv_gmm1_lo));
  O::st(a.U0, RHO * n + c, u.rho);
  O::st(a.U0, ENG * n + c, u.E);
#pragma unroll
  for (int d = 0; d < 3; d++) {
    O::st(a.U0, (VX1 + d) * n + c, u.m[d]);
    O::st(a.U0, (BX1 + d) * n + c, u.b[d]);
  }
}

// INTERNAL_BOUNDARY, stage 1: the reference builds U0 from the primitives
// after the callback (rk_step.c:93-96); here U0 is resident, so it is rebuilt
// in the zones whose primitives the callback changed (prev: the state before
// the callback; narrowing a widened float gives it back, so unchanged zones
// compare equal).
struct V8 {
  const float* p[8];
};
template <class A>
__global__ void k_mrefresh(MixArgs a, V8 prev, Box dom) {
  using O = Acc<A>;
  long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= dom.count()) return;
  int i, j, k;
  dom.coords(q, i, j, k);
  const Geom& g = a.g;
  const long long c = cidx(g, k, j, i), n = g.ncell;
  float v[NV];
  bool changed = false;
#pragma unroll
  for (int nv = 0; nv < NV; nv++) {
    v[nv] = a.Vin[nv][c];
    changed |= __float_as_uint(v[nv]) != __float_as_uint(prev.p[nv][c]);
  }
  if (!changed) return;
  const ConsA<A> u = cons_of<A>(v, O::konst(a.inv_gmm1_d, a.inv_gmm1_hi, a.inv_gmm1_lo));
  O::st(a.U0, RHO * n + c, u.rho);
  O::st(a.U0, ENG * n + c, u.E);
#pragma unroll
  for (int d = 0; d < 3; d++) {
    O::st(a.U0, (VX1 + d) * n + c, u.m[d]);
    O::st(a.U0, (BX1 + d) * n + c, u.b[d]);
  }
}

// 1D time step: max over interfaces of cmax/dx, every stage
// (Src/Time_Stepping/update_stage.c:237-241); cmax is not stored by the
// 1D sweep, so it is rebuilt from the per-cell C_dt sum: for 1D the sweep
// stores max(cmax(i-1/2), cmax(i+1/2)) in CDT instead.
__global__ void k_mbegin(MixArgs a, long long n) {
  long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q < n) a.flag[q] = 0;
  if (q == 0) {
    a.sc->inv_dt_bits = 0ull;
    a.sc->mach_bits = 0ull;
    a.sc->nfail = 0ull;
    for (int d = 0; d < 3; d++) a.sc->dtdx[d] = (float)(a.sc->dt * a.g.inv_dx[d]);
  }
}

__global__ void k_mend_step(MixArgs a) {
  DevScalars* sc = a.sc;
  double inv = __longlong_as_double((long long)sc->inv_dt_bits);
  if (a.g.dims > 1) inv /= (double)a.g.dims;
  sc->inv_dt_bits = (unsigned long long)__double_as_longlong(inv);
  if (!(inv == inv) || inv > 1e300) sc->status |= 1;
  if (a.device_dt) {
    double dt = sc->dt;
    sc->time += dt;
    double dt_hyp = 1.0 / inv;
    dt_hyp *= a.cfl;
    sc->dt_prev = dt;
    sc->dt = pmin(dt_hyp, a.cfl_max_var * dt);
  }
}

// 1D dt: reduce max(cmax)/dx over the row's interfaces (stored in CDT by the
// x sweep as the per-cell maximum of the two adjacent interfaces).
__global__ void k_m1d_dt(MixArgs a, Box dom) {
  long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  double v = 0.0;
  if (q < dom.count()) {
    int i, j, k;
    dom.coords(q, i, j, k);
    v = (double)a.CDT[cidx(a.g, k, j, i)];
  }
  double m = warp_max_d(v);
  if ((threadIdx.x & 31) == 0) atomic_max_nonneg_d(&a.sc->inv_dt_bits, m);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct MixedState {
  MixBufs b;
  int cur = 0;  // buffer holding the state at the start of the next step
  int tile_tries = 1 << 20;  // see MixArgs::tile_tries
  // TMA tensor maps of the y/z sweeps (tma: maps encoded, kernels configured)
  bool tma = false;
  // y/z sweeps by k_msweep_m (marching columns) instead of the TMA tiles,
  // with segments of march_seg cells (0: chosen per launch)
  bool march = false;
  int march_seg = 0;
  SweepMaps ymaps[2], zmaps[2];  // per state buffer (V, face field); dU, CDT shared
  XSweepMaps xmaps[2];
};

// Tensor maps and shared-memory opt-in of the TMA sweeps; false leaves the
// solver on k_msweep_t.  Needs a row pitch that is a multiple of 16 bytes,
// V and dU each one block of 8 arrays, and PLUTO_GB300_SWEEP_TMA not "0".
template <int RS, bool CT>
static bool mixed_prepare_tma_rs(Solver* S, MixedState* M) {
  const Geom& g = S->g;
  using TL = SweepTile<RS>;
  if (cudaFuncSetAttribute(k_msweep_tma<RS, 1, CT>, cudaFuncAttributeMaxDynamicSharedMemorySize, TL::SMEM) !=
          cudaSuccess ||
      (g.dims > 2 &&
       cudaFuncSetAttribute(k_msweep_tma<RS, 2, CT>, cudaFuncAttributeMaxDynamicSharedMemorySize, TL::SMEM) !=
           cudaSuccess)) {
    cudaGetLastError();
    return false;
  }
  if (cudaFuncSetAttribute(k_msweep_x_tma<RS, CT>, cudaFuncAttributeMaxDynamicSharedMemorySize, kXSMEM) !=
      cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  const uint64_t d4[4] = {(uint64_t)g.nt[0], (uint64_t)g.nt[1], (uint64_t)g.nt[2], 8};
  // global extents: the logical rows (loads past nt0 read the fill value);
  // strides: the padded row pitch
  const uint64_t s4[3] = {(uint64_t)g.s[1] * 4, (uint64_t)g.s[2] * 4, (uint64_t)g.ncell * 4};
  for (int sb = 0; sb < 2; sb++) {
    const uint32_t bv[4] = {kXW, kXR, 1, 8};
    const uint32_t bf[3] = {kXW, kXR, 1};
    if (!encode_f32_map(&M->xmaps[sb].V, M->b.V[sb][0], 4, d4, s4, bv)) return false;
    if (CT && !encode_f32_map(&M->xmaps[sb].B, M->b.Bs[sb][0], 3, d4, s4, bf)) return false;
    if (!CT) M->xmaps[sb].B = M->xmaps[sb].V;  // unused
  }
  for (int dir = 1; dir < g.dims; dir++) {
    auto box = [&](int rows, int r) {  // box of `rows` along dir
      return dir == 1 ? (r == 1 ? (uint32_t)rows : 1u) : (r == 2 ? (uint32_t)rows : 1u);
    };
    for (int sb = 0; sb < 2; sb++) {
      SweepMaps& m = dir == 1 ? M->ymaps[sb] : M->zmaps[sb];
      const uint32_t bv[4] = {32, box(TL::R, 1), box(TL::R, 2), 8};
      const uint32_t bu[4] = {32, box(TL::NU, 1), box(TL::NU, 2), 8};
      const uint32_t bc[3] = {32, box(TL::NU, 1), box(TL::NU, 2)};
      const uint32_t bf[3] = {32, box(TL::NF, 1), box(TL::NF, 2)};
      if (!encode_f32_map(&m.V, M->b.V[sb][0], 4, d4, s4, bv)) return false;
      if (!encode_f32_map(&m.dU, M->b.dU[0], 4, d4, s4, bu)) return false;
      if (M->b.dU1[0] ? !encode_f32_map(&m.dU1, M->b.dU1[0], 4, d4, s4, bu) : false) return false;
      if (!M->b.dU1[0]) m.dU1 = m.dU;
      if (!encode_f32_map(&m.CDT, M->b.CDT, 3, d4, s4, bc)) return false;
      if (CT && !encode_f32_map(&m.B, M->b.Bs[sb][dir], 3, d4, s4, bf)) return false;
      if (!CT) m.B = m.CDT;  // unused
    }
  }
  return true;
}

static bool mixed_prepare_tma(Solver* S, MixedState* M) {
  const char* env = getenv("PLUTO_GB300_SWEEP_TMA");
  if (env && env[0] == '0') return false;
  const Geom& g = S->g;
  if (g.dims < 2 || (g.s[1] % 4) != 0) return false;
  const bool ct = S->cfg.divb == PG_CONSTRAINED_TRANSPORT;
  int rs;
  if (S->cfg.reconstruction == PG_PARABOLIC) rs = RS_PPM;
  else if (S->cfg.limiter == PG_MC_LIM) rs = RS_PLM_MC;
  else if (S->cfg.limiter == PG_MINMOD_LIM) rs = RS_PLM_MINMOD;
  else if (S->cfg.limiter == PG_VANLEER_LIM) rs = RS_PLM_VANLEER;
  else rs = RS_PLM_GENERIC;
  switch (rs) {
    case RS_PLM_MC: return ct ? mixed_prepare_tma_rs<RS_PLM_MC, true>(S, M) : mixed_prepare_tma_rs<RS_PLM_MC, false>(S, M);
    case RS_PLM_MINMOD:
      return ct ? mixed_prepare_tma_rs<RS_PLM_MINMOD, true>(S, M) : mixed_prepare_tma_rs<RS_PLM_MINMOD, false>(S, M);
    case RS_PLM_VANLEER:
      return ct ? mixed_prepare_tma_rs<RS_PLM_VANLEER, true>(S, M) : mixed_prepare_tma_rs<RS_PLM_VANLEER, false>(S, M);
    case RS_PPM: return ct ? mixed_prepare_tma_rs<RS_PPM, true>(S, M) : mixed_prepare_tma_rs<RS_PPM, false>(S, M);
    default:
      return ct ? mixed_prepare_tma_rs<RS_PLM_GENERIC, true>(S, M) : mixed_prepare_tma_rs<RS_PLM_GENERIC, false>(S, M);
  }
}

int mixed_alloc(Solver* S) {
  MixedState* M = new MixedState();
  memset(&M->b, 0, sizeof M->b);
  S->mixed = M;
  const long long n = S->g.ncell;
  auto al = [&](float** p) -> int {
    if (cudaMalloc(p, n * sizeof(float)) != cudaSuccess) return PG_ERR_NOMEM;
    cudaMemset(*p, 0, n * sizeof(float));
    return PG_OK;
  };
  const bool ct = S->cfg.divb == PG_CONSTRAINED_TRANSPORT;
  // V of each state buffer and dU: one block of 8 arrays each (the TMA
  // sweeps read all 8 through one 4D tensor map)
  auto al8 = [&](float** p) -> int {
    float* base = nullptr;
    if (cudaMalloc(&base, 8 * n * sizeof(float)) != cudaSuccess) return PG_ERR_NOMEM;
    cudaMemset(base, 0, 8 * n * sizeof(float));
    for (int nv = 0; nv < 8; nv++) p[nv] = base + nv * n;
    return PG_OK;
  };
  for (int s = 0; s < 2; s++)
    if (al8(M->b.V[s])) return PG_ERR_NOMEM;
  if (al8(M->b.dU)) return PG_ERR_NOMEM;
  if (S->cfg.time_stepping == PG_RK2 && al8(M->b.dU1)) return PG_ERR_NOMEM;
  if (al(&M->b.CDT)) return PG_ERR_NOMEM;
  if (ct) {
    for (int d = 0; d < S->g.dims; d++) {
      for (int s = 0; s < 2; s++)
        if (al(&M->b.Bs[s][d])) return PG_ERR_NOMEM;
      if (al(&M->b.S[d][0]) || al(&M->b.S[d][1])) return PG_ERR_NOMEM;
      for (int c = 0; c < S->g.dims; c++)
        if (al(&M->b.DV[d][c])) return PG_ERR_NOMEM;
    }
    if (al(&M->b.E[2])) return PG_ERR_NOMEM;
    if (S->g.dims == 3 && (al(&M->b.E[0]) || al(&M->b.E[1]))) return PG_ERR_NOMEM;
    const Geom& g = S->g;
    const long long m[3] = {(long long)g.nt[1] * g.nt[2], (long long)g.nt[0] * g.nt[2],
                            (long long)g.nt[0] * g.nt[1]};
    for (int d = 0; d < g.dims; d++)
      if (S->cfg.bc[d] != PG_PERIODIC) {
        for (int e = 0; e < g.dims; e++) {
          if (cudaMalloc(&M->b.Bm1[e], m[e] * sizeof(float)) != cudaSuccess) return PG_ERR_NOMEM;
          cudaMemset(M->b.Bm1[e], 0, m[e] * sizeof(float));
        }
        break;
      }
  }
  if (cudaMalloc(&M->b.flag, n) != cudaSuccess) return PG_ERR_NOMEM;
  cudaMemset(M->b.flag, 0, n);
  for (int u = 0; u < 2; u++) {  // 8 bytes per element for double and for FP32 pairs
    if (cudaMalloc(&M->b.U[u], 8 * n * 8) != cudaSuccess) return PG_ERR_NOMEM;
    cudaMemset(M->b.U[u], 0, 8 * n * 8);
  }
  M->tma = mixed_prepare_tma(S, M);
  {
    // y/z sweeps: marching columns unless PLUTO_GB300_SWEEP=tile (the
    // TMA-staged tiles when the pitch allows them, else k_msweep_t)
    const char* e = getenv("PLUTO_GB300_SWEEP");
    M->march = S->g.dims > 1 && !(e && strcmp(e, "tile") == 0);
    const char* sg = getenv("PLUTO_GB300_MARCH_SEG");
    if (sg) M->march_seg = atoi(sg);
    if (M->march_seg < 0 || M->march_seg > 4096) M->march_seg = 0;
  }
  return PG_OK;
}

void mixed_free(Solver* S) {
  MixedState* M = (MixedState*)S->mixed;
  if (!M) return;
  auto f = [](void* p) {
    if (p) cudaFree(p);
  };
  for (int s = 0; s < 2; s++) f(M->b.V[s][0]);  // blocks of 8 arrays
  f(M->b.dU[0]);
  f(M->b.dU1[0]);
  f(M->b.CDT);
  f(M->b.flag);
  f(M->b.U[0]);
  f(M->b.U[1]);
  for (int d = 0; d < 3; d++) {
    for (int s = 0; s < 2; s++) f(M->b.Bs[s][d]);
    f(M->b.S[d][0]);
    f(M->b.S[d][1]);
    f(M->b.E[d]);
    f(M->b.Bm1[d]);
    for (int c = 0; c < 3; c++) f(M->b.DV[d][c]);
  }
  delete M;
  S->mixed = nullptr;
}

static MixArgs margs(Solver* S, int in_buf, int out_buf, int v0_buf) {
  MixedState* M = (MixedState*)S->mixed;
  MixArgs a;
  memset(&a, 0, sizeof a);
  a.g = S->g;
  for (int nv = 0; nv < 8; nv++) {
    a.Vin[nv] = M->b.V[in_buf][nv];
    a.V0[nv] = M->b.V[v0_buf][nv];
    a.Vout[nv] = M->b.V[out_buf][nv];
    a.dU[nv] = M->b.dU[nv];
  }
  for (int d = 0; d < 3; d++) {
    a.Bin[d] = M->b.Bs[in_buf][d];
    a.B0[d] = M->b.Bs[v0_buf][d];
    a.Bout[d] = M->b.Bs[out_buf][d];
    a.S[d][0] = M->b.S[d][0];
    a.S[d][1] = M->b.S[d][1];
    a.E[d] = M->b.E[d];
    for (int c = 0; c < 3; c++) a.DV[d][c] = M->b.DV[d][c];
  }
  a.CDT = M->b.CDT;
  a.flag = M->b.flag;
  a.U0 = M->b.U[0];
  a.Us = M->b.U[1];
  a.sc = S->sc;
  a.gamma = (float)S->cfg.gamma;
  a.gamma_d = S->cfg.gamma;
  for (int d = 0; d < 3; d++) a.inv_dx_f[d] = (float)S->g.inv_dx[d];
  a.inv_gmm1_d = 1.0 / (S->cfg.gamma - 1.0);
  a.inv_gmm1_hi = (float)a.inv_gmm1_d;
  a.inv_gmm1_lo = (float)(a.inv_gmm1_d - (double)a.inv_gmm1_hi);
  a.third_hi = (float)(1.0 / 3.0);
  a.third_lo = (float)(1.0 / 3.0 - (double)a.third_hi);
  a.small_rho = S->cfg.small_density > 0 ? S->cfg.small_density : 1e-12;
  a.small_p = S->cfg.small_pressure > 0 ? S->cfg.small_pressure : 1e-12;
  a.cfl = S->cfl;
  a.cfl_max_var = S->cfl_max_var;
  a.limiter = S->cfg.limiter;
  a.recon = S->cfg.reconstruction;
  a.ct = S->cfg.divb == PG_CONSTRAINED_TRANSPORT;
  a.nbfield = a.ct ? S->g.dims : 0;
  a.ncomp = S->cfg.components;
  // Variables whose flux difference is accumulated: all of them except the
  // cell-centred field components that CT rebuilds from the faces.
  a.accmask = 0xff;
  if (a.ct)
    for (int d = 0; d < S->g.dims; d++) a.accmask &= ~(1 << (BX1 + d));
  a.device_dt = S->device_dt;
  a.intb = S->ud_internal ? 1 : 0;
  a.tile_tries = M->tile_tries;
  return a;
}

static void mlaunch_bound(Solver* S, const MixArgs& a) {
  const Geom& g = S->g;
  MixedState* M = (MixedState*)S->mixed;
  if (S->ud_internal) {  // INTERNAL_BOUNDARY: the callback on the whole state first
    const bool first = S->ud_stage == 0;
    const int other = a.Vin[0] == M->b.V[0][0] ? 1 : 0;  // free during stage 1's fill
    if (first)
      cudaMemcpyAsync(M->b.V[other][0], a.Vin[0], 8 * (size_t)g.ncell * sizeof(float), cudaMemcpyDeviceToDevice,
                      S->stream);
    float* vin[8];
    float* bin[3];
    for (int nv = 0; nv < NV; nv++) vin[nv] = (float*)a.Vin[nv];
    for (int d = 0; d < 3; d++) bin[d] = (float*)a.Bin[d];
    launch_internal_boundary<float>(S, vin, bin, M->b.Bm1, a.nbfield, M->b.flag);
    if (first) {
      Box dom;
      for (int ax = 0; ax < 3; ax++) {
        dom.lo[ax] = g.beg[ax];
        dom.hi[ax] = g.end[ax];
      }
      dom.prepare();
      V8 prev;
      for (int nv = 0; nv < NV; nv++) prev.p[nv] = M->b.V[other][nv];
      if (S->cfg.precision == PG_MIXED_DW)
        k_mrefresh<dw><<<grid_for(dom.count()), kThreads, 0, S->stream>>>(a, prev, dom);
      else
        k_mrefresh<double><<<grid_for(dom.count()), kThreads, 0, S->stream>>>(a, prev, dom);
    }
  }
  if ((a.ct && M->b.Bm1[0]) || has_userdef(S)) {  // non-periodic axis under CT, or a user-defined side: per-axis passes
    BoundCT<float> b;
    b.g = g;
    for (int nv = 0; nv < NV; nv++) b.V[nv] = (float*)a.Vin[nv];
    for (int d = 0; d < 3; d++) {
      b.Bs[d] = (float*)a.Bin[d];
      b.Bm1[d] = M->b.Bm1[d];
    }
    b.nbfield = a.nbfield;
    b.ncomp = S->cfg.components;
    face_areas(g, b.area);
    launch_bound_ct<float, double>(S, b, "mixed_bound", "mixed_fill_normal");
    S->ud_stage++;
    return;
  }
  BoundArrays arr;
  arr.n = 0;
  arr.ncomp = S->cfg.components;
  for (int nv = 0; nv < NV; nv++) arr.q[arr.n++] = (float*)a.Vin[nv];
  for (int d = 0; d < a.nbfield; d++) arr.q[arr.n++] = (float*)a.Bin[d];
  const GhostSlabs gs(g);
  PG_LAUNCH(S, "mixed_bound", (k_mbound<<<grid_for(gs.count()), kThreads, 0, S->stream>>>(
                                    g, arr, S->cfg.bc[0], S->cfg.bc[1], S->cfg.bc[2], gs)));
  S->ud_stage++;
}


template <int RS, bool CT>
static void mlaunch_sweeps_rs(Solver* S, const MixArgs& a, int stage) {
  const Geom& g = S->g;
  cudaStream_t st = S->stream;
  const int solver = S->cfg.riemann;
  const int ext = CT ? 1 : 0;
  const int stage1 = (stage == 1) ? 1 : 0;
  MixedState* M = (MixedState*)S->mixed;
  if (M->tma) {  // x sweep, TMA-staged tiles of kXR rows by kXC chunks
    const int t_lo = g.beg[1] - ext, t_n = g.nx[1] + 2 * ext;
    const int b_lo = g.dims > 2 ? g.beg[2] - ext : 0, b_n = g.dims > 2 ? g.nx[2] + 2 * ext : 1;
    const int nxt = (g.nx[0] + 2 + 30 * kXC - 1) / (30 * kXC);  // chunks reach cell end+1
    const int njt = (t_n + kXR - 1) / kXR;
    const int ntiles = nxt * njt * b_n;
    int nsm = 152, dv = 0;
    if (cudaGetDevice(&dv) == cudaSuccess) cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dv);
    const int grid = ntiles < kXBLK * nsm ? ntiles : kXBLK * nsm;
    const int sb = a.Vin[0] == M->b.V[0][0] ? 0 : 1;
    PG_LAUNCH(S, "mixed_sweep_x_tma", (k_msweep_x_tma<RS, CT><<<grid, 32 * kXR, kXSMEM, st>>>(
                                          M->xmaps[sb], a, solver, t_lo, t_n, b_lo, nxt, njt, ntiles, stage1)));
  } else {  // x sweep over rows (j,k) of the transverse-extended box
    int t_lo = g.dims > 1 ? g.beg[1] - ext : 0, t_n = g.dims > 1 ? g.nx[1] + 2 * ext : 1;
    int b_lo = g.dims > 2 ? g.beg[2] - ext : 0, b_n = g.dims > 2 ? g.nx[2] + 2 * ext : 1;
    int nwx = (g.nx[0] + 2 + 29) / 30;  // lanes reach cell end+1
    int nrows = t_n * b_n;
    long long threads = (long long)nwx * nrows * 32;
    PG_LAUNCH(S, "mixed_sweep_x", (k_msweep_x<RS, CT><<<grid_for(threads, 128), 128, 0, st>>>(
                                      a, solver, t_lo, t_n, b_lo, nrows, stage1, g.dims == 1, nwx)));
  }
  for (int dir = 1; dir < g.dims; dir++) {
    int i_lo = g.beg[0] - ext, i_n = g.nx[0] + 2 * ext;
    int oax = dir == 1 ? 2 : 1;
    int o_lo = oax < g.dims ? g.beg[oax] - ext : 0, o_n = oax < g.dims ? g.nx[oax] + 2 * ext : 1;
    if (M->march) {
      // segment length: 64 cells, halved (down to 8) while the sweep has
      // fewer than four waves of resident warps (16 per SM)
      const long long wcols = (long long)((i_n + 31) / 32) * o_n;
      int seg = M->march_seg;
      if (seg <= 0) {
        int nsm = 152, dv = 0;
        if (cudaGetDevice(&dv) == cudaSuccess) cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dv);
        seg = 64;
        while (seg > 8 && wcols * ((g.nx[dir] + seg - 1) / seg) < 4LL * 16 * nsm) seg /= 2;
      }
      const int nseg = (g.nx[dir] + seg - 1) / seg;
      const long long threads = 32LL * wcols * nseg;
      if (dir == 1)
        PG_LAUNCH(S, "mixed_sweep_y_march", (k_msweep_m<RS, 1, CT><<<grid_for(threads, kMarchThreads), kMarchThreads, 0, st>>>(
                                                a, solver, i_lo, i_n, o_lo, o_n, seg, nseg, stage1)));
      else
        PG_LAUNCH(S, "mixed_sweep_z_march", (k_msweep_m<RS, 2, CT><<<grid_for(threads, kMarchThreads), kMarchThreads, 0, st>>>(
                                                a, solver, i_lo, i_n, o_lo, o_n, seg, nseg, stage1)));
      continue;
    }
    if (M->tma) {
      using TL = SweepTile<RS>;
      const int sb = a.Vin[0] == M->b.V[0][0] ? 0 : 1;
      const SweepMaps& maps = dir == 1 ? M->ymaps[sb] : M->zmaps[sb];
      const int xa = i_lo & ~3;  // tiles start on 16-byte boundaries
      const int nbt = (i_n + (i_lo - xa) + 31) / 32;
      const int nrb = (g.nx[dir] + 2 + TL::NU - 1) / TL::NU;  // rows reach cell end+1
      const int ncols = nbt * o_n, ntiles = ncols * nrb;
      int nsm = 152, dv = 0;
      if (cudaGetDevice(&dv) == cudaSuccess) cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dv);
      const int grid = ntiles < 2 * nsm ? ntiles : 2 * nsm;
      dim3 block(32, kTY);
      const int dsel = a.dU[0] == M->b.dU1[0] ? 1 : 0;
      if (dir == 1)
        PG_LAUNCH(S, "mixed_sweep_y_tma", (k_msweep_tma<RS, 1, CT><<<grid, block, TL::SMEM, st>>>(
                                          maps, a, solver, xa, i_lo, i_n, o_lo, nbt, ncols, ntiles, stage1, dsel)));
      else
        PG_LAUNCH(S, "mixed_sweep_z_tma", (k_msweep_tma<RS, 2, CT><<<grid, block, TL::SMEM, st>>>(
                                          maps, a, solver, xa, i_lo, i_n, o_lo, nbt, ncols, ntiles, stage1, dsel)));
      continue;
    }
    int nbx = (i_n + 31) / 32;
    int nblk = (g.nx[dir] + 2 + kTY - 3) / (kTY - 2);  // rows reach cell end+1
    dim3 grid((unsigned)(nbx * o_n), (unsigned)nblk), block(32, kTY);
    if (dir == 1)
      PG_LAUNCH(S, "mixed_sweep_y", (k_msweep_t<RS, 1, CT><<<grid, block, 0, st>>>(a, solver, i_lo, i_n, o_lo,
                                                                                     o_n, stage1)));
    else
      PG_LAUNCH(S, "mixed_sweep_z", (k_msweep_t<RS, 2, CT><<<grid, block, 0, st>>>(a, solver, i_lo, i_n, o_lo,
                                                                                     o_n, stage1)));
  }
}

template <bool CT>
static void mlaunch_sweeps(Solver* S, const MixArgs& a, int stage) {
  int rs;
  if (S->cfg.reconstruction == PG_PARABOLIC) rs = RS_PPM;
  else if (S->cfg.limiter == PG_MC_LIM) rs = RS_PLM_MC;
  else if (S->cfg.limiter == PG_MINMOD_LIM) rs = RS_PLM_MINMOD;
  else if (S->cfg.limiter == PG_VANLEER_LIM) rs = RS_PLM_VANLEER;
  else rs = RS_PLM_GENERIC;
  switch (rs) {
    case RS_PLM_MC: mlaunch_sweeps_rs<RS_PLM_MC, CT>(S, a, stage); break;
    case RS_PLM_MINMOD: mlaunch_sweeps_rs<RS_PLM_MINMOD, CT>(S, a, stage); break;
    case RS_PLM_VANLEER: mlaunch_sweeps_rs<RS_PLM_VANLEER, CT>(S, a, stage); break;
    case RS_PPM: mlaunch_sweeps_rs<RS_PPM, CT>(S, a, stage); break;
    default: mlaunch_sweeps_rs<RS_PLM_GENERIC, CT>(S, a, stage); break;
  }
}

template <int STAGE, int NSTAGE, class A>
static void mlaunch_tail(Solver* S, const MixArgs& a, const Box& dom) {
  const Geom& g = S->g;
  cudaStream_t st = S->stream;
  if (a.ct) {
    Box eb;
    for (int ax = 0; ax < 3; ax++) {
      if (ax < g.dims) { eb.lo[ax] = g.beg[ax] - 1; eb.hi[ax] = g.end[ax]; }
      else { eb.lo[ax] = eb.hi[ax] = 0; }
    }
    eb.prepare();
    PG_LAUNCH(S, "mixed_emf", (k_memf<<<grid_for(eb.count()), kThreads, 0, st>>>(a, eb)));
    PG_LAUNCH(S, "mixed_face", (k_mface<STAGE, NSTAGE, A><<<grid_for(eb.count()), kThreads, 0, st>>>(a, eb)));
  }
  if (g.dims == 1) PG_LAUNCH(S, "mixed_dt1d", (k_m1d_dt<<<grid_for(dom.count()), kThreads, 0, st>>>(a, dom)));
  int reduce = (STAGE == 1 && g.dims > 1);
  PG_LAUNCH(S, "mixed_final", (k_mfinal<STAGE, NSTAGE, A><<<grid_for(dom.count()), kThreads, 0, st>>>(a, dom, reduce)));
}

template <int NSTAGE, class A>
static void menqueue(Solver* S) {
  MixedState* M = (MixedState*)S->mixed;
  const Geom& g = S->g;
  Box dom;
  for (int ax = 0; ax < 3; ax++) { dom.lo[ax] = g.beg[ax]; dom.hi[ax] = g.end[ax]; }
  dom.prepare();
  const int bA = M->cur, bB = 1 - M->cur;
  const bool ct = S->cfg.divb == PG_CONSTRAINED_TRANSPORT;
  // stage 1: A -> B (EULER: in place, A -> A; the final kernel reads no
  // primitive state)
  MixArgs a1 = NSTAGE == 1 ? margs(S, bA, bA, bA) : margs(S, bA, bB, bA);
  PG_LAUNCH(S, "mixed_begin", (k_mbegin<<<grid_for(g.ncell), kThreads, 0, S->stream>>>(a1, g.ncell)));
  mlaunch_bound(S, a1);
  if (ct) mlaunch_sweeps<true>(S, a1, 1); else mlaunch_sweeps<false>(S, a1, 1);
  mlaunch_tail<1, NSTAGE, A>(S, a1, dom);
  if (NSTAGE == 1) {
    PG_LAUNCH(S, "mixed_end_step", (k_mend_step<<<1, 1, 0, S->stream>>>(a1)));
  } else if (NSTAGE == 2) {
    // stage 2: B (+A) -> A; its increments go to the second buffer, the
    // corrector reads both
    MixArgs a2 = margs(S, bB, bA, bA);
    for (int nv = 0; nv < 8; nv++) {
      a2.dUp[nv] = M->b.dU[nv];
      a2.dU[nv] = M->b.dU1[nv];
    }
    mlaunch_bound(S, a2);
    if (ct) mlaunch_sweeps<true>(S, a2, 2); else mlaunch_sweeps<false>(S, a2, 2);
    mlaunch_tail<2, NSTAGE, A>(S, a2, dom);
    PG_LAUNCH(S, "mixed_end_step", (k_mend_step<<<1, 1, 0, S->stream>>>(a2)));
  } else {
    MixArgs a2 = margs(S, bB, bB, bA);  // in place: the final kernel reads its own cell only
    mlaunch_bound(S, a2);
    if (ct) mlaunch_sweeps<true>(S, a2, 2); else mlaunch_sweeps<false>(S, a2, 2);
    mlaunch_tail<2, NSTAGE, A>(S, a2, dom);
    MixArgs a3 = margs(S, bB, bA, bA);
    mlaunch_bound(S, a3);
    if (ct) mlaunch_sweeps<true>(S, a3, 3); else mlaunch_sweeps<false>(S, a3, 3);
    mlaunch_tail<3, NSTAGE, A>(S, a3, dom);
    PG_LAUNCH(S, "mixed_end_step", (k_mend_step<<<1, 1, 0, S->stream>>>(a3)));
  }
}

int mixed_enqueue_step(Solver* S) {
  const bool dwacc = S->cfg.precision == PG_MIXED_DW;
  // PLUTO_GB300_TILE_WAIT_TRIES: the try limit of the sweeps' tile waits, read
  // whenever a step is enqueued (a captured graph keeps the value it was
  // captured with).  A fault-injection knob for tests: with 0 every tile wait
  // times out at once, the step reports PG_ERR_TIMEOUT and its results are
  // invalid; unset, the limit is 2^20 tries.
  MixedState* M = (MixedState*)S->mixed;
  const char* tries = getenv("PLUTO_GB300_TILE_WAIT_TRIES");
  M->tile_tries = (tries && tries[0]) ? atoi(tries) : (1 << 20);
  if (M->tile_tries < 0) M->tile_tries = 0;
  if (S->cfg.time_stepping == PG_RK3) {
    if (dwacc) menqueue<3, dw>(S);
    else menqueue<3, double>(S);
  } else if (S->cfg.time_stepping == PG_EULER) {
    if (dwacc) menqueue<1, dw>(S);
    else menqueue<1, double>(S);
  } else {
    if (dwacc) menqueue<2, dw>(S);
    else menqueue<2, double>(S);
  }
  return cudaGetLastError() == cudaSuccess ? PG_OK : PG_ERR_CUDA;
}

}  // namespace pg

using namespace pg;

// Host transfers for the mixed path: FP64 host arrays <-> FP32 device state.
static int mixed_xfer(Solver* S, const double* const vars[8], double* const outv[8], const double* const faces[3],
                      double* const outf[3], int layout, bool to_dev) {
  MixedState* M = (MixedState*)S->mixed;
  const Geom& g = S->g;
  // pinned staging, only for host memory the device cannot reach: one array
  // in the host layout (the device arrays may have padded rows)
  double* pin = nullptr;
  size_t pin_n = 0;
  int rc = PG_OK;
  const int cur = M->cur;
  auto one = [&](float* dev, const double* hin, double* hout, int fd) -> int {
    if (double* alias = host_alias(to_dev ? hin : hout)) {
      launch_host_xfer<float>(S->stream, alias, dev, g, fd, layout, to_dev);
      return cudaGetLastError() == cudaSuccess ? PG_OK : PG_ERR_CUDA;
    }
    const HostBox hb = host_box(g, fd, layout);
    const size_t n = (size_t)hb.hn[0] * hb.hn[1] * hb.hn[2];
    if (n > pin_n) {
      if (pin) cudaFreeHost(pin);
      pin = nullptr;
      pin_n = 0;
      if (cudaHostAlloc((void**)&pin, n * sizeof(double), cudaHostAllocMapped) != cudaSuccess) return PG_ERR_NOMEM;
      pin_n = n;
    }
    double* alias = host_alias(pin);
    if (!alias) return PG_ERR_CUDA;
    if (to_dev) memcpy(pin, hin, n * sizeof(double));
    launch_host_xfer<float>(S->stream, alias, dev, g, fd, layout, to_dev);
    if (cudaStreamSynchronize(S->stream) != cudaSuccess) return PG_ERR_CUDA;  // the staging array is reused
    if (!to_dev) memcpy(hout, pin, n * sizeof(double));
    return PG_OK;
  };
  for (int nv = 0; nv < 8 && !rc; nv++) {
    if (to_dev) {
      if (vars[nv]) rc = one(M->b.V[cur][nv], vars[nv], nullptr, -1);
      else cudaMemsetAsync(M->b.V[cur][nv], 0, g.ncell * sizeof(float), S->stream);
    } else if (outv[nv]) {
      rc = one(M->b.V[cur][nv], nullptr, outv[nv], -1);
    }
  }
  if (S->cfg.divb == PG_CONSTRAINED_TRANSPORT)
    for (int d = 0; d < g.dims && !rc; d++) {
      if (to_dev && faces && faces[d]) rc = one(M->b.Bs[cur][d], faces[d], nullptr, d);
      if (!to_dev && outf && outf[d]) rc = one(M->b.Bs[cur][d], nullptr, outf[d], d);
    }
  if (cudaStreamSynchronize(S->stream) != cudaSuccess && !rc) rc = PG_ERR_CUDA;
  if (pin) cudaFreeHost(pin);
  return rc;
}

int mixed_upload_host(Solver* S, const double* const vars[8], const double* const faces[3], int layout) {
  int rc = mixed_xfer(S, vars, nullptr, faces, nullptr, layout, true);
  if (rc) return rc;
  MixedState* M = (MixedState*)S->mixed;
  const MixArgs a = margs(S, M->cur, M->cur, M->cur);
  Box dom;
  for (int ax = 0; ax < 3; ax++) {
    dom.lo[ax] = S->g.beg[ax];
    dom.hi[ax] = S->g.end[ax];
  }
  dom.prepare();
  if (S->cfg.precision == PG_MIXED_DW)
    k_mcons_init<dw><<<grid_for(dom.count()), kThreads, 0, S->stream>>>(a, dom);
  else
    k_mcons_init<double><<<grid_for(dom.count()), kThreads, 0, S->stream>>>(a, dom);
  if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(S->stream) != cudaSuccess) return PG_ERR_CUDA;
  return PG_OK;
}
int mixed_download(Solver* S, double* const vars[8], double* const faces[3], int layout) {
  return mixed_xfer(S, nullptr, vars, nullptr, faces, layout, false);
}
// the current FP32 state arrays (what mixed_download widens), for the output packer
float* mixed_cell_array(Solver* S, int nv) {
  MixedState* M = (MixedState*)S->mixed;
  return M ? M->b.V[M->cur][nv] : nullptr;
}
float* mixed_face_array(Solver* S, int d) {
  MixedState* M = (MixedState*)S->mixed;
  return (M && S->cfg.divb == PG_CONSTRAINED_TRANSPORT && d < S->g.dims) ? M->b.Bs[M->cur][d] : nullptr;
}

namespace pg {

__device__ __forceinline__ bool same_bits_d(double a, double b) {
  return __double_as_longlong(a) == __double_as_longlong(b) || (a != a && b != b);
}
__device__ __forceinline__ bool same_bits_f(float a, float b) {
  return __float_as_uint(a) == __float_as_uint(b) || (a != a && b != b);
}

// IEEE conversions without flush-to-zero (this unit is compiled with
// --use_fast_math, under which the compiler's own conversions flush
// subnormals): the reference the integer forms are checked against.
__device__ __forceinline__ double cvt_f64_f32(float f) {
  double d;
  asm("cvt.f64.f32 %0, %1;" : "=d"(d) : "f"(f));
  return d;
}
__device__ __forceinline__ float cvt_rn_f32_f64(double d) {
  float f;
  asm("cvt.rn.f32.f64 %0, %1;" : "=f"(f) : "d"(d));
  return f;
}

// widen over every float bit pattern; narrow over doubles built from each
// float pattern with five choices of the 29 bits below float precision
// (zero, exactly half, half - 1, half + 1, a hash) and over doubles with the
// exponent taken from a hash (underflow, overflow, subnormal results).
__global__ void k_selftest_conv(unsigned long long* bad) {
  unsigned long long nw = 0, nn = 0;
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long q = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; q < (1ull << 32);
       q += stride) {
    const unsigned u = (unsigned)q;
    const float f = __uint_as_float(u);
    const double h = cvt_f64_f32(f);
    nw += same_bits_d(widen(f), h) ? 0 : 1;
    const unsigned hash = (u * 2654435761u) ^ (u >> 13);
    const unsigned long long top = (unsigned long long)__double_as_longlong(h) & ~0x1fffffffull;
    const unsigned pats[5] = {0u, 0x10000000u, 0x0fffffffu, 0x10000001u, hash & 0x1fffffffu};
#pragma unroll
    for (int p = 0; p < 5; p++) {
      const double d = __longlong_as_double((long long)(top | pats[p]));
      nn += same_bits_f(narrow(d), cvt_rn_f32_f64(d)) ? 0 : 1;
    }
    const unsigned long long e2 = (unsigned long long)((hash >> 7) & 0x7ffu);
    const unsigned long long wide = (top & 0x800fffffffffffffull) | (e2 << 52) | (hash & 0x1fffffffu);
    const double d2 = __longlong_as_double((long long)wide);
    nn += same_bits_f(narrow(d2), cvt_rn_f32_f64(d2)) ? 0 : 1;
  }
  if (nw) atomicAdd(&bad[0], nw);
  if (nn) atomicAdd(&bad[1], nn);
}

int mixed_selftest_conversions(unsigned long long counts[2]) {
  unsigned long long* d = nullptr;
  if (cudaMalloc(&d, 2 * sizeof(unsigned long long)) != cudaSuccess) {
    set_last_error("pg_selftest_conversions: cudaMalloc failed");
    return PG_ERR_NOMEM;
  }
  cudaError_t e = cudaMemset(d, 0, 2 * sizeof(unsigned long long));
  int nsm = 152;
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) {
    k_selftest_conv<<<nsm * 8, 256>>>(d);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(counts, d, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) {
    set_last_error((std::string("pg_selftest_conversions: ") + cudaGetErrorString(e)).c_str());
    return PG_ERR_CUDA;
  }
  return PG_OK;
}

}  // namespace pg
