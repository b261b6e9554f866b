// Mixed-precision path: FP32 storage and FP32 reconstruction / Riemann /
// EMF arithmetic; FP64 for the conserved-variable accumulation, the CT
// face-field update, the pressure recovery p = (g-1)(E - rho v^2/2 - B^2/2)
// and the global dt reduction.
//
// One stage = seven launches:
//   k_mbound      ghost fill (Src/boundary.c:41-303)
//   k_msweep_x    reconstruct + Riemann + flux difference along x; one warp
//                 covers 31 cells of a row, the left interface flux comes
//                 from the neighbouring lane by shuffle
//   k_msweep_yz   the same along y or z; each thread marches along the
//                 direction with a three-cell register window, so every
//                 cell is reconstructed once and every interface solved once
//   k_memf        UCT_HLL edge EMFs (Src/MHD/CT/ct_emf_average.c:179-352)
//   k_mface       CT face update (Src/MHD/CT/ct_update.c) + RK face combination
//   k_mfinal      RK cell combination, face average, ConsToPrim
//                 (Src/MHD/mappers.c:88-254), dt reduction
// Stage outputs are written to a second state buffer (the stage input is
// still read by neighbours), so RK2/RK3 need two FP32 copies of the state.
#include <cstdio>
#include <cstring>

#include "pg_internal.h"
#include "pg_physics.cuh"

namespace pg {

struct MixBufs {
  float* V[2][8];
  float* Bs[2][3];
  float* dU[8];
  float* S[3][2];
  float* DV[3][3];
  float* E[3];
  float* CDT;
  unsigned char* flag;
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
  float* S[3][2];
  float* DV[3][3];
  float* E[3];
  float* CDT;
  unsigned char* flag;
  DevScalars* sc;
  float gamma;
  double gamma_d, small_rho, small_p, cfl, cfl_max_var;
  int limiter, recon, ct, nbfield, accmask, device_dt;
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

// PLM or PPM states of one cell from its stencil (w2, w1, v0, e1, e2).
__device__ __forceinline__ void recon_cell(int recon, int lim, int nv, float w2, float w1, float v0, float e1,
                                           float e2, float& vp, float& vm) {
  if (recon == PG_LINEAR) {
    float dv = limit(lim, nv, e1 - v0, v0 - w1);
    vp = v0 + dv * 0.5f;
    vm = v0 - dv * 0.5f;
  } else {
    float p = ppm_iface(w1, v0, e1, e2);
    float m = ppm_iface(w2, w1, v0, e1);
    ppm_limit(v0, p, m);
    vp = p;
    vm = m;
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
  if (solver == PG_HLL) hll_solver<DIR, false>(vL, uL, vR, uR, a.gamma, o, mach);
  else hlld_solver<DIR, false>(vL, uL, vR, uR, a.gamma, o, mach);
}

// ---------------------------------------------------------------------------
// boundary (same maps as the FP64 path)
// ---------------------------------------------------------------------------
__device__ __forceinline__ int mbmap(int x, int beg, int end, int n, int type) {
  if (x < beg) return type == PG_PERIODIC ? x + n : beg;
  if (x > end) return type == PG_PERIODIC ? x - n : end;
  return x;
}

struct BoundArrays {
  float* q[11];
  int n;
};

__global__ void k_mbound(Geom g, BoundArrays arr, int bcx, int bcy, int bcz, long long n0, long long n1,
                         long long n2) {
  long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  int i, j, k;
  int gx = g.beg[0], gy = g.beg[1], gz = g.beg[2];
  if (q < n0) {
    int ng2 = 2 * gx;
    int ii = (int)(q % ng2);
    long long r = q / ng2;
    j = (int)(r % g.nt[1]);
    k = (int)(r / g.nt[1]);
    i = ii < gx ? ii : g.end[0] + 1 + (ii - gx);
  } else if (q < n0 + n1) {
    q -= n0;
    int ng2 = 2 * gy;
    i = g.beg[0] + (int)(q % g.nx[0]);
    long long r = q / g.nx[0];
    int jj = (int)(r % ng2);
    k = (int)(r / ng2);
    j = jj < gy ? jj : g.end[1] + 1 + (jj - gy);
  } else if (q < n0 + n1 + n2) {
    q -= n0 + n1;
    i = g.beg[0] + (int)(q % g.nx[0]);
    long long r = q / g.nx[0];
    j = g.beg[1] + (int)(r % g.nx[1]);
    int kk = (int)(r / g.nx[1]);
    k = kk < gz ? kk : g.end[2] + 1 + (kk - gz);
  } else {
    return;
  }
  int si = mbmap(i, g.beg[0], g.end[0], g.nx[0], bcx);
  int sj = g.dims > 1 ? mbmap(j, g.beg[1], g.end[1], g.nx[1], bcy) : j;
  int sk = g.dims > 2 ? mbmap(k, g.beg[2], g.end[2], g.nx[2], bcz) : k;
  long long dst = cidx(g, k, j, i), src = cidx(g, sk, sj, si);
  for (int a = 0; a < arr.n; a++) arr.q[a][dst] = arr.q[a][src];
}

// ---------------------------------------------------------------------------
// x sweep: warp = 32 consecutive cells of one row, 31 of them updated
// ---------------------------------------------------------------------------
template <bool CT>
__global__ void __launch_bounds__(128) k_msweep_x(MixArgs a, int solver, int t_lo, int t_n, int b_lo,
                                                  long long nrows, int stage1, int oned, int nwx) {
  const Geom& g = a.g;
  const int lane = threadIdx.x & 31;
  long long wid = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const int wx = (int)(wid % nwx);
  const long long row = wid / nwx;
  if (row >= nrows) return;  // whole warp leaves together
  const int j = t_lo + (int)(row % t_n);
  const int k = b_lo + (int)(row / t_n);
  const int i = g.beg[0] - 1 + 31 * wx + lane;
  const bool cell_ok = i <= g.end[0] + 1;    // slopes of cells beg-1..end+1
  const bool face_ok = i <= g.end[0];        // interfaces beg-1+1/2 .. end+1/2
  const long long c = cidx(g, k, j, i);
  float vL[NV], vR[NV], slope[3] = {0.f, 0.f, 0.f};
  // Stencil reads: cell i needs i-1..i+1 (PLM) or i-2..i+2 (PPM); the right
  // state of interface i+1/2 (cell i+1, only when face_ok) needs one more.
  // With ng = 2 (PLM) / 3 (PPM) ghosts every read stays inside the row.
  const bool ppm = a.recon == PG_PARABOLIC;
  if (cell_ok) {
#pragma unroll
    for (int nv = 0; nv < NV; nv++) {
      const float* V = a.Vin[nv];
      float w2 = ppm ? ldg(V, c - 2) : 0.f;
      float w1 = ldg(V, c - 1), v0 = ldg(V, c), e1 = ldg(V, c + 1);
      float e2 = (ppm || face_ok) ? ldg(V, c + 2) : 0.f;
      float e3 = (ppm && face_ok) ? ldg(V, c + 3) : 0.f;
      float vp, vm, vp1 = 0.f, vm1 = 0.f;
      recon_cell(a.recon, a.limiter, nv, w2, w1, v0, e1, e2, vp, vm);      // cell i
      if (face_ok) recon_cell(a.recon, a.limiter, nv, w1, v0, e1, e2, e3, vp1, vm1);  // cell i+1
      vL[nv] = vp;
      vR[nv] = vm1;
      if (nv >= VX1 && nv <= VX3) slope[nv - VX1] = vp - vm;
    }
  }
  Iface<float> o;
  float fl[NV], pr = 0.f, cm = 0.f;
  if (face_ok) {
    float bn = CT ? a.Bin[0][c] : 0.f;
    solve_iface<0, CT>(a, solver, vL, vR, bn, o);
#pragma unroll
    for (int nv = 0; nv < NV; nv++) fl[nv] = o.f[nv];
    pr = o.press;
    cm = o.cmax;
    if (CT) {
      a.S[0][0][c] = pmax(0.f, -o.SL);
      a.S[0][1][c] = pmax(0.f, o.SR);
    }
  } else {
#pragma unroll
    for (int nv = 0; nv < NV; nv++) fl[nv] = 0.f;
  }
  if (CT && cell_ok)
    for (int comp = 0; comp < g.dims; comp++) a.DV[0][comp][c] = slope[comp];
  // left interface (i-1/2) from the previous lane
  float flm[NV];
#pragma unroll
  for (int nv = 0; nv < NV; nv++) flm[nv] = __shfl_up_sync(0xffffffffu, fl[nv], 1);
  float prm = __shfl_up_sync(0xffffffffu, pr, 1);
  float cmm = __shfl_up_sync(0xffffffffu, cm, 1);
  if (lane >= 1 && i >= g.beg[0] && i <= g.end[0]) {
    const float scrh = (float)(a.sc->dt * g.inv_dx[0]);
#pragma unroll
    for (int nv = 0; nv < NV; nv++) {
      if (!((a.accmask >> nv) & 1)) continue;
      float rhs = -scrh * (fl[nv] - flm[nv]);
      if (nv == VX1) rhs -= scrh * (pr - prm);
      a.dU[nv][c] = rhs;
    }
    // 2D/3D: C_dt term of update_stage.c:233; 1D: the larger adjacent
    // cmax (the 1D reduction of update_stage.c:237-241 is a plain max).
    if (oned) a.CDT[c] = pmax(cmm, cm) * (float)g.inv_dx[0];
    else if (stage1) a.CDT[c] = 0.5f * (cmm + cm) * (float)g.inv_dx[0];
  }
}

// ---------------------------------------------------------------------------
// y/z sweep: lanes along x, each thread marches along DIR over a segment
// ---------------------------------------------------------------------------
template <int DIR, bool CT>
__global__ void __launch_bounds__(128) k_msweep_yz(MixArgs a, int solver, int i_lo, int i_n, int o_lo, int o_n,
                                                   int seg_len, int nseg, int stage1, int first_dir) {
  const Geom& g = a.g;
  long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int ii = (int)(tid % i_n);
  long long r = tid / i_n;
  const int oo = (int)(r % o_n);
  const int sg = (int)(r / o_n);
  if (sg >= nseg) return;
  const int i = i_lo + ii;
  // the other transverse axis: z for DIR=y, y for DIR=z
  const int other = o_lo + oo;
  const long long s = g.s[DIR];
  const int beg = g.beg[DIR], end = g.end[DIR];
  const int d0 = beg + sg * seg_len;
  const int d1 = min(d0 + seg_len - 1, end);  // cells updated: d0..d1
  long long base = DIR == 1 ? cidx(g, other, 0, i) : cidx(g, 0, other, i);
  const bool ppm = a.recon == PG_PARABOLIC;
  const float scrh = (float)(a.sc->dt * g.inv_dx[DIR]);
  const float invdx = (float)g.inv_dx[DIR];
  // window: w[0]=v[m-1], w[1]=v[m], w[2]=v[m+1], w[3]=v[m+2] (PPM also w[-1])
  float wm2[NV], w0[NV], w1[NV], w2[NV], w3[NV];
  float vprev[NV];           // vp of cell m
  float fprev[NV], pprev = 0.f, cprev = 0.f;
  int m = d0 - 1;
#pragma unroll
  for (int nv = 0; nv < NV; nv++) {
    const float* V = a.Vin[nv];
    wm2[nv] = ppm ? ldg(V, base + (m - 2) * s) : 0.f;
    w0[nv] = ldg(V, base + (m - 1) * s);
    w1[nv] = ldg(V, base + m * s);
    w2[nv] = ldg(V, base + (m + 1) * s);
    w3[nv] = ppm ? ldg(V, base + (m + 2) * s) : 0.f;
    float vp, vm;
    recon_cell(a.recon, a.limiter, nv, wm2[nv], w0[nv], w1[nv], w2[nv], w3[nv], vp, vm);
    vprev[nv] = vp;
    if (CT && nv >= VX1 && nv < VX1 + g.dims && m >= beg - 1) a.DV[DIR][nv - VX1][base + m * s] = vp - vm;
    fprev[nv] = 0.f;
  }
  for (; m <= d1; m++) {
    // shift window so that w0=v[m], w1=v[m+1], w2=v[m+2], w3=v[m+3]
    float vL[NV], vR[NV];
#pragma unroll
    for (int nv = 0; nv < NV; nv++) {
      const float* V = a.Vin[nv];
      float nw = ldg(V, base + (m + (ppm ? 3 : 2)) * s);
      wm2[nv] = w0[nv];
      w0[nv] = w1[nv];
      w1[nv] = w2[nv];
      if (ppm) {
        w2[nv] = w3[nv];
        w3[nv] = nw;
      } else {
        w2[nv] = nw;
      }
      float vp, vm;  // states of cell m+1
      recon_cell(a.recon, a.limiter, nv, wm2[nv], w0[nv], w1[nv], w2[nv], w3[nv], vp, vm);
      vL[nv] = vprev[nv];
      vR[nv] = vm;
      vprev[nv] = vp;
      if (CT && nv >= VX1 && nv < VX1 + g.dims && m + 1 <= end + 1)
        a.DV[DIR][nv - VX1][base + (m + 1) * s] = vp - vm;
    }
    const long long c = base + m * s;  // interface m+1/2 is stored at cell m
    Iface<float> o;
    float bn = CT ? a.Bin[DIR][c] : 0.f;
    solve_iface<DIR, CT>(a, solver, vL, vR, bn, o);
    if (CT) {
      a.S[DIR][0][c] = pmax(0.f, -o.SL);
      a.S[DIR][1][c] = pmax(0.f, o.SR);
    }
    if (m >= d0) {  // update cell m from interfaces m-1/2 (prev) and m+1/2
#pragma unroll
      for (int nv = 0; nv < NV; nv++) {
        if (!((a.accmask >> nv) & 1)) continue;
        float rhs = -scrh * (o.f[nv] - fprev[nv]);
        if (nv == Rot<DIR>::vn) rhs -= scrh * (o.press - pprev);
        if (first_dir) a.dU[nv][c] = rhs;
        else a.dU[nv][c] += rhs;
      }
      if (stage1) {
        float term = 0.5f * (cprev + o.cmax) * invdx;
        if (first_dir) a.CDT[c] = term;
        else a.CDT[c] += term;
      }
    }
#pragma unroll
    for (int nv = 0; nv < NV; nv++) fprev[nv] = o.f[nv];
    pprev = o.press;
    cprev = o.cmax;
  }
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
  a.E[2][c] = muct_edge<2>(a, c);
  if (a.g.dims == 3) {
    a.E[0][c] = muct_edge<0>(a, c);
    a.E[1][c] = muct_edge<1>(a, c);
  }
}

// CT face update: EMF differences in FP32, accumulation into the face field
// in FP64, RK face combination in FP64.
template <int STAGE, int NSTAGE>
__global__ void k_mface(MixArgs a, Box box) {
  long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= box.count()) return;
  int i, j, k;
  box.coords(q, i, j, k);
  const Geom& g = a.g;
  const long long c = cidx(g, k, j, i);
  const double dt = a.sc->dt;
  const bool d3 = g.dims == 3;
  const float* E1 = a.E[0];
  const float* E2 = a.E[1];
  const float* E3 = a.E[2];
  const float f1 = (float)(dt * g.inv_dx[0]), f2 = (float)(dt * g.inv_dx[1]), f3 = (float)(dt * g.inv_dx[2]);
  for (int fd = 0; fd < g.dims; fd++) {
    bool in = true;
    for (int ax = 0; ax < g.dims; ax++) {
      int x = ax == 0 ? i : (ax == 1 ? j : k);
      int lo = g.beg[ax] - (ax == fd ? 1 : 0), hi = g.end[ax];
      in = in && x >= lo && x <= hi;
    }
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
    double bb = (double)a.Bin[fd][c] + (double)rhs;
    if (STAGE == 2) {
      const double w0 = NSTAGE == 3 ? 0.75 : 0.5, wc = NSTAGE == 3 ? 0.25 : 0.5;
      bb = w0 * (double)a.B0[fd][c] + wc * bb;
    } else if (STAGE == 3) {
      bb = ((double)a.B0[fd][c] + 2.0 * bb) * (1.0 / 3.0);
    }
    a.Bout[fd][c] = (float)bb;
  }
}

// Conservative variables in FP64 from FP32 primitives (Src/MHD/mappers.c:25-86).
__device__ __forceinline__ void prim_to_cons_d(const float* vf, double* u, double inv_gmm1) {
  double rho = vf[RHO];
  double vx = vf[VX1], vy = vf[VX2], vz = vf[VX3];
  double bx = vf[BX1], by = vf[BX2], bz = vf[BX3];
  u[RHO] = rho;
  u[MX1] = rho * vx;
  u[MX1 + 1] = rho * vy;
  u[MX1 + 2] = rho * vz;
  u[BX1] = bx;
  u[BX2] = by;
  u[BX3] = bz;
  double kin = vx * vx + vy * vy + vz * vz;
  double kinb2 = 0.5 * (rho * kin + (bx * bx + by * by + bz * bz));
  u[ENG] = kinb2 + (double)vf[PRS] * inv_gmm1;
}

template <int STAGE, int NSTAGE>
__global__ void k_mfinal(MixArgs a, Box dom, int reduce_cdt) {
  long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  double cd = 0.0;
  bool fails = false, bad = false;
  if (q < dom.count()) {
    int i, j, k;
    dom.coords(q, i, j, k);
    const Geom& g = a.g;
    const long long c = cidx(g, k, j, i);
    const double gmm1 = a.gamma_d - 1.0, inv_gmm1 = 1.0 / gmm1;
    float vin[NV];
#pragma unroll
    for (int nv = 0; nv < NV; nv++) vin[nv] = a.Vin[nv][c];
    double u[NV];
    prim_to_cons_d(vin, u, inv_gmm1);
#pragma unroll
    for (int nv = 0; nv < NV; nv++)
      if ((a.accmask >> nv) & 1) u[nv] += (double)a.dU[nv][c];
    if (STAGE >= 2) {
      float v0[NV];
#pragma unroll
      for (int nv = 0; nv < NV; nv++) v0[nv] = a.V0[nv][c];
      double u0[NV];
      prim_to_cons_d(v0, u0, inv_gmm1);
      if (STAGE == 2) {
        const double w0 = NSTAGE == 3 ? 0.75 : 0.5, wc = NSTAGE == 3 ? 0.25 : 0.5;
#pragma unroll
        for (int nv = 0; nv < NV; nv++) u[nv] = w0 * u0[nv] + wc * u[nv];
      } else {
#pragma unroll
        for (int nv = 0; nv < NV; nv++) u[nv] = (u0[nv] + 2.0 * u[nv]) * (1.0 / 3.0);
      }
    }
    if (a.ct)
      for (int d = 0; d < g.dims; d++)
        u[BX1 + d] = 0.5 * ((double)a.Bout[d][c] + (double)a.Bout[d][c - g.s[d]]);
    // ConsToPrim with FP64 pressure recovery; velocities in FP32.
    unsigned char fl = 0;
    if (u[RHO] < 0.0) {
      u[RHO] = a.small_rho;
      fl = FLAG_CONS2PRIM_FAIL;
    }
    float rho_f = (float)u[RHO];
    float tau = 1.0f / rho_f;
    float vx = (float)u[MX1] * tau, vy = (float)u[MX1 + 1] * tau, vz = (float)u[MX1 + 2] * tau;
    double ke = 0.5 * (u[MX1] * (double)vx + u[MX1 + 1] * (double)vy + u[MX1 + 2] * (double)vz);
    double kinb2 = ke + 0.5 * (u[BX1] * u[BX1] + u[BX2] * u[BX2] + u[BX3] * u[BX3]);
    if (u[ENG] < 0.0) {
      u[ENG] = a.small_p * inv_gmm1 + kinb2;
      fl = FLAG_CONS2PRIM_FAIL;
    }
    double p = gmm1 * (u[ENG] - kinb2);
    if (p < 0.0) {
      p = a.small_p;
      fl = FLAG_CONS2PRIM_FAIL;
    }
    float out[NV] = {rho_f, vx, vy, vz, (float)u[BX1], (float)u[BX2], (float)u[BX3], (float)p};
#pragma unroll
    for (int nv = 0; nv < NV; nv++) {
      a.Vout[nv][c] = out[nv];
      bad |= ((__float_as_uint(out[nv]) >> 23) & 0xff) == 0xff;
    }
    if (fl) {
      a.flag[c] = fl;
      fails = true;
    }
    if (reduce_cdt) cd = (double)a.CDT[c];
  }
  if (reduce_cdt) {
    double m = warp_max_d(cd);
    if ((threadIdx.x & 31) == 0) atomic_max_nonneg_d(&a.sc->inv_dt_bits, m);
  }
  unsigned ball = __ballot_sync(0xffffffffu, fails);
  if ((threadIdx.x & 31) == 0 && ball) atomicAdd(&a.sc->nfail, (unsigned long long)__popc(ball));
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(&a.sc->status, 1);
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
};

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
  for (int s = 0; s < 2; s++)
    for (int nv = 0; nv < 8; nv++)
      if (al(&M->b.V[s][nv])) return PG_ERR_NOMEM;
  for (int nv = 0; nv < 8; nv++)
    if (al(&M->b.dU[nv])) return PG_ERR_NOMEM;
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
  }
  if (cudaMalloc(&M->b.flag, n) != cudaSuccess) return PG_ERR_NOMEM;
  cudaMemset(M->b.flag, 0, n);
  return PG_OK;
}

void mixed_free(Solver* S) {
  MixedState* M = (MixedState*)S->mixed;
  if (!M) return;
  auto f = [](void* p) {
    if (p) cudaFree(p);
  };
  for (int s = 0; s < 2; s++)
    for (int nv = 0; nv < 8; nv++) f(M->b.V[s][nv]);
  for (int nv = 0; nv < 8; nv++) f(M->b.dU[nv]);
  f(M->b.CDT);
  f(M->b.flag);
  for (int d = 0; d < 3; d++) {
    for (int s = 0; s < 2; s++) f(M->b.Bs[s][d]);
    f(M->b.S[d][0]);
    f(M->b.S[d][1]);
    f(M->b.E[d]);
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
  a.sc = S->sc;
  a.gamma = (float)S->cfg.gamma;
  a.gamma_d = S->cfg.gamma;
  a.small_rho = S->cfg.small_density > 0 ? S->cfg.small_density : 1e-12;
  a.small_p = S->cfg.small_pressure > 0 ? S->cfg.small_pressure : 1e-12;
  a.cfl = S->cfl;
  a.cfl_max_var = S->cfl_max_var;
  a.limiter = S->cfg.limiter;
  a.recon = S->cfg.reconstruction;
  a.ct = S->cfg.divb == PG_CONSTRAINED_TRANSPORT;
  a.nbfield = a.ct ? S->g.dims : 0;
  // Variables whose flux difference is accumulated: all of them except the
  // cell-centred field components that CT rebuilds from the faces.
  a.accmask = 0xff;
  if (a.ct)
    for (int d = 0; d < S->g.dims; d++) a.accmask &= ~(1 << (BX1 + d));
  a.device_dt = S->device_dt;
  return a;
}

static void mlaunch_bound(Solver* S, const MixArgs& a) {
  const Geom& g = S->g;
  BoundArrays arr;
  arr.n = 0;
  for (int nv = 0; nv < NV; nv++) arr.q[arr.n++] = (float*)a.Vin[nv];
  for (int d = 0; d < a.nbfield; d++) arr.q[arr.n++] = (float*)a.Bin[d];
  long long n0 = 2LL * g.beg[0] * g.nt[1] * g.nt[2];
  long long n1 = g.dims > 1 ? 2LL * g.beg[1] * g.nx[0] * g.nt[2] : 0;
  long long n2 = g.dims > 2 ? 2LL * g.beg[2] * g.nx[0] * g.nx[1] : 0;
  PG_LAUNCH(S, "mixed_bound", (k_mbound<<<grid_for(n0 + n1 + n2), kThreads, 0, S->stream>>>(
                                    g, arr, S->cfg.bc[0], S->cfg.bc[1], S->cfg.bc[2], n0, n1, n2)));
}

static const int kSeg = 32;

template <bool CT>
static void mlaunch_sweeps(Solver* S, const MixArgs& a, int stage) {
  const Geom& g = S->g;
  cudaStream_t st = S->stream;
  const int solver = S->cfg.riemann;
  const int ext = CT ? 1 : 0;
  const int stage1 = (stage == 1) ? 1 : 0;
  // x sweep over rows (j,k) in the transverse-extended box
  {
    int t_lo = g.dims > 1 ? g.beg[1] - ext : 0, t_n = g.dims > 1 ? g.nx[1] + 2 * ext : 1;
    int b_lo = g.dims > 2 ? g.beg[2] - ext : 0, b_n = g.dims > 2 ? g.nx[2] + 2 * ext : 1;
    int nwx = (g.nx[0] + 2 + 30) / 31;
    long long nrows = (long long)t_n * b_n;
    long long threads = (long long)nwx * nrows * 32;
    PG_LAUNCH(S, "mixed_sweep_x", (k_msweep_x<CT><<<grid_for(threads, 128), 128, 0, st>>>(
                                      a, solver, t_lo, t_n, b_lo, nrows, stage1, g.dims == 1, nwx)));
  }
  for (int dir = 1; dir < g.dims; dir++) {
    int i_lo = g.beg[0] - ext, i_n = g.nx[0] + 2 * ext;
    int oax = dir == 1 ? 2 : 1;
    int o_lo = oax < g.dims ? g.beg[oax] - ext : 0, o_n = oax < g.dims ? g.nx[oax] + 2 * ext : 1;
    int nseg = (g.nx[dir] + kSeg - 1) / kSeg;
    long long threads = (long long)i_n * o_n * nseg;
    if (dir == 1)
      PG_LAUNCH(S, "mixed_sweep_y", (k_msweep_yz<1, CT><<<grid_for(threads, 128), 128, 0, st>>>(
                                        a, solver, i_lo, i_n, o_lo, o_n, kSeg, nseg, stage1, 0)));
    else
      PG_LAUNCH(S, "mixed_sweep_z", (k_msweep_yz<2, CT><<<grid_for(threads, 128), 128, 0, st>>>(
                                        a, solver, i_lo, i_n, o_lo, o_n, kSeg, nseg, stage1, 0)));
  }
}

template <int STAGE, int NSTAGE>
static void mlaunch_tail(Solver* S, const MixArgs& a, const Box& dom) {
  const Geom& g = S->g;
  cudaStream_t st = S->stream;
  if (a.ct) {
    Box eb;
    for (int ax = 0; ax < 3; ax++) {
      if (ax < g.dims) { eb.lo[ax] = g.beg[ax] - 1; eb.hi[ax] = g.end[ax]; }
      else { eb.lo[ax] = eb.hi[ax] = 0; }
    }
    PG_LAUNCH(S, "mixed_emf", (k_memf<<<grid_for(eb.count()), kThreads, 0, st>>>(a, eb)));
    PG_LAUNCH(S, "mixed_face", (k_mface<STAGE, NSTAGE><<<grid_for(eb.count()), kThreads, 0, st>>>(a, eb)));
  }
  if (g.dims == 1) PG_LAUNCH(S, "mixed_dt1d", (k_m1d_dt<<<grid_for(dom.count()), kThreads, 0, st>>>(a, dom)));
  int reduce = (STAGE == 1 && g.dims > 1);
  PG_LAUNCH(S, "mixed_final", (k_mfinal<STAGE, NSTAGE><<<grid_for(dom.count()), kThreads, 0, st>>>(a, dom, reduce)));
}

template <int NSTAGE>
static void menqueue(Solver* S) {
  MixedState* M = (MixedState*)S->mixed;
  const Geom& g = S->g;
  Box dom;
  for (int ax = 0; ax < 3; ax++) { dom.lo[ax] = g.beg[ax]; dom.hi[ax] = g.end[ax]; }
  const int A = M->cur, B = 1 - M->cur;
  const bool ct = S->cfg.divb == PG_CONSTRAINED_TRANSPORT;
  // stage 1: A -> B
  MixArgs a1 = margs(S, A, B, A);
  PG_LAUNCH(S, "mixed_begin", (k_mbegin<<<grid_for(g.ncell), kThreads, 0, S->stream>>>(a1, g.ncell)));
  mlaunch_bound(S, a1);
  if (ct) mlaunch_sweeps<true>(S, a1, 1); else mlaunch_sweeps<false>(S, a1, 1);
  mlaunch_tail<1, NSTAGE>(S, a1, dom);
  if (NSTAGE == 2) {
    // stage 2: B (+A) -> A
    MixArgs a2 = margs(S, B, A, A);
    mlaunch_bound(S, a2);
    if (ct) mlaunch_sweeps<true>(S, a2, 2); else mlaunch_sweeps<false>(S, a2, 2);
    mlaunch_tail<2, NSTAGE>(S, a2, dom);
    PG_LAUNCH(S, "mixed_end_step", (k_mend_step<<<1, 1, 0, S->stream>>>(a2)));
  } else {
    MixArgs a2 = margs(S, B, B, A);  // in place: the final kernel reads its own cell only
    mlaunch_bound(S, a2);
    if (ct) mlaunch_sweeps<true>(S, a2, 2); else mlaunch_sweeps<false>(S, a2, 2);
    mlaunch_tail<2, NSTAGE>(S, a2, dom);
    MixArgs a3 = margs(S, B, A, A);
    mlaunch_bound(S, a3);
    if (ct) mlaunch_sweeps<true>(S, a3, 3); else mlaunch_sweeps<false>(S, a3, 3);
    mlaunch_tail<3, NSTAGE>(S, a3, dom);
    PG_LAUNCH(S, "mixed_end_step", (k_mend_step<<<1, 1, 0, S->stream>>>(a3)));
  }
}

int mixed_enqueue_step(Solver* S) {
  if (S->cfg.time_stepping == PG_RK3) menqueue<3>(S);
  else menqueue<2>(S);
  return cudaGetLastError() == cudaSuccess ? PG_OK : PG_ERR_CUDA;
}

}  // namespace pg

using namespace pg;

// Host transfers for the mixed path: FP64 host arrays <-> FP32 device state.
__global__ void k_f64_to_f32(const double* src, float* dst, long long n) {
  long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q < n) dst[q] = (float)src[q];
}
__global__ void k_f32_to_f64(const float* src, double* dst, long long n) {
  long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q < n) dst[q] = (double)src[q];
}

static int mixed_xfer(Solver* S, const double* const vars[8], double* const outv[8], const double* const faces[3],
                      double* const outf[3], int layout, bool to_dev) {
  MixedState* M = (MixedState*)S->mixed;
  const Geom& g = S->g;
  const long long n = g.ncell;
  double* tmp = nullptr;
  if (cudaMalloc(&tmp, n * sizeof(double)) != cudaSuccess) return PG_ERR_NOMEM;
  int rc = PG_OK;
  const int cur = M->cur;
  auto one = [&](float* dev, const double* hin, double* hout, int fd) -> int {
    if (to_dev) {
      cudaMemsetAsync(tmp, 0, n * sizeof(double), S->stream);
      int r = xfer_f64(S, tmp, (double*)hin, fd, layout, true);
      if (r) return r;
      k_f64_to_f32<<<grid_for(n), kThreads, 0, S->stream>>>(tmp, dev, n);
      return PG_OK;
    }
    k_f32_to_f64<<<grid_for(n), kThreads, 0, S->stream>>>(dev, tmp, n);
    return xfer_f64(S, tmp, hout, fd, layout, false);
  };
  for (int nv = 0; nv < 8 && !rc; nv++) {
    if (to_dev) {
      if (vars[nv]) rc = one(M->b.V[cur][nv], vars[nv], nullptr, -1);
      else cudaMemsetAsync(M->b.V[cur][nv], 0, n * sizeof(float), S->stream);
    } else if (outv[nv]) {
      rc = one(M->b.V[cur][nv], nullptr, outv[nv], -1);
    }
    cudaStreamSynchronize(S->stream);
  }
  if (S->cfg.divb == PG_CONSTRAINED_TRANSPORT)
    for (int d = 0; d < g.dims && !rc; d++) {
      if (to_dev && faces && faces[d]) rc = one(M->b.Bs[cur][d], faces[d], nullptr, d);
      if (!to_dev && outf && outf[d]) rc = one(M->b.Bs[cur][d], nullptr, outf[d], d);
      cudaStreamSynchronize(S->stream);
    }
  if (cudaStreamSynchronize(S->stream) != cudaSuccess && !rc) rc = PG_ERR_CUDA;
  cudaFree(tmp);
  return rc;
}

int mixed_upload_host(Solver* S, const double* const vars[8], const double* const faces[3], int layout) {
  return mixed_xfer(S, vars, nullptr, faces, nullptr, layout, true);
}
int mixed_download(Solver* S, double* const vars[8], double* const faces[3], int layout) {
  return mixed_xfer(S, nullptr, vars, nullptr, faces, layout, false);
}
