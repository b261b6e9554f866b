// Differentiated FP64 path: tangent-linear model, adjoint of one EULER /
// RK2 / RK3 step, device-resident checkpoints.
//
// Tangent-linear: the FP64 step kernels of pg_fp64_kernels.cuh instantiated
// with T = Dual<1>; value parts are the plain FP64 step, derivative parts its
// directional derivative through the branches taken (precision
// PG_FP64_TANGENT).
//
// Adjoint: pg_adjoint_step maps lambda(n+1) -> lambda(n) for one step of
// a given (frozen) dt.  The step is recomputed from the solver's state, then
// each forward operation is undone in reverse order by a hand-written kernel:
//   k_adj_c2p      ConsToPrim                  (Src/MHD/mappers.c:88-254)
//   k_adj_avg      CT_AverageMagneticField     (Src/MHD/CT/ct_field_average.c:13)
//   k_adj_rk_*     RK combinations             (Src/Time_Stepping/rk_step.c:93-233)
//   k_adj_ct       CT_Update                   (Src/MHD/CT/ct_update.c:29-220)
//   k_adj_emf      CT_EMF_HLL_Solver           (Src/MHD/CT/ct_emf_average.c:179-352)
//   k_adj_flux     RightHandSide, U += rhs     (Src/MHD/rhs.c:193-201)
//   k_adj_riemann  HLL / HLLD / Roe flux with the face-field override
//                  (Src/MHD/hll.c, hlld.c, roe.c, Src/States/plm_states.c:271)
//   k_adj_recon    States (PLM / PPM) and CT_StoreVelSlopes
//   k_adj_bound    Boundary (periodic / outflow copies), transposed
//   k_adj_p2c      PrimToCons3D                (Src/mappers3D.c:74)
// The local derivatives inside those kernels belong to exactly the branch
// the forward evaluation takes, floors included.  The HLL / HLLD Riemann
// outputs, the edge EMF, the PLM / PPM states and the prim<->cons maps are
// transposed by hand-derived reverse-mode point functions
// (pg_adjoint_pt.cuh), all inputs in one evaluation; the Roe solver
// evaluates the same templated point function as the forward kernels with
// Dual<1> inputs, one seeded input at a time.
#include <cstddef>
#include <cstring>
#include <initializer_list>
#include <string>
#include <utility>
#include <vector>

#include "pg_adjoint_pt.cuh"
#include "pg_fp64_kernels.cuh"

namespace pg {

using D1 = Dual<1>;

int tl_enqueue_step(Solver* S) { return fp64_enqueue_step_t<D1>(S); }

// ---------------------------------------------------------------------------
// tangent-solver transfers: FP64 staging array <-> value / tangent parts
// ---------------------------------------------------------------------------
__global__ void k_tl_put(D1* dst, const double* src, long long n, int part) {
  long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= n) return;
  if (part == 0) {
    dst[q].v = src[q];
    dst[q].d[0] = 0.0;
  } else {
    dst[q].d[0] = src[q];
  }
}
__global__ void k_tl_get(double* dst, const D1* src, long long n, int part) {
  long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q < n) dst[q] = part == 0 ? src[q].v : src[q].d[0];
}

static int ensure_stage(Solver* S) {
  if (S->stage) return PG_OK;
  if (cudaMalloc(&S->stage, S->g.ncell * sizeof(double)) != cudaSuccess) {
    S->stage = nullptr;
    set_last_error("staging allocation failed");
    return PG_ERR_NOMEM;
  }
  return PG_OK;
}

int tl_xfer(Solver* S, double* const vars[8], double* const faces[3], int layout, bool to_dev, int part) {
  if (layout != PG_LAYOUT_INTERIOR && layout != PG_LAYOUT_PLUTO) {
    set_last_error("bad layout");
    return PG_ERR_INVALID;
  }
  int rc = ensure_stage(S);
  if (rc) return rc;
  const Geom& g = S->g;
  const long long n = g.ncell;
  cudaStream_t st = S->stream;
  const bool ct = S->cfg.divb == PG_CONSTRAINED_TRANSPORT;
  if (to_dev && ct && !faces) {
    set_last_error("constrained transport needs staggered fields");
    return PG_ERR_INVALID;
  }
  auto one = [&](double* dev_arr, double* host, int fd) -> int {
    D1* arr = (D1*)dev_arr;
    if (to_dev) {
      cudaMemsetAsync(S->stage, 0, n * sizeof(double), st);
      if (host) {
        int r = xfer_f64(S, S->stage, host, fd, layout, true);
        if (r) return r;
      }
      k_tl_put<<<grid_for(n), kThreads, 0, st>>>(arr, S->stage, n, part);
    } else if (host) {
      k_tl_get<<<grid_for(n), kThreads, 0, st>>>(S->stage, arr, n, part);
      int r = xfer_f64(S, S->stage, host, fd, layout, false);
      if (r) return r;
    }
    return PG_OK;
  };
  for (int nv = 0; nv < 8; nv++)
    if ((rc = one(S->V[nv], vars ? vars[nv] : nullptr, -1))) return rc;
  if (ct && faces)
    for (int d = 0; d < g.dims; d++) {
      if (to_dev && !faces[d]) {
        set_last_error("missing staggered component");
        return PG_ERR_INVALID;
      }
      if ((rc = one(S->Bs[d], faces[d], d))) return rc;
    }
  cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    set_last_error(cudaGetErrorString(e));
    return PG_ERR_CUDA;
  }
  return PG_OK;
}

// ---------------------------------------------------------------------------
// adjoint buffers
// ---------------------------------------------------------------------------
struct AdjBufs {
  // adjoint variables (full ghosted arrays)
  double* lV[8];    // on the primitive state after the part being undone
  double* lB[3];    // on the face field likewise
  double* lVin[8];  // on the stage-input primitives
  double* lBin[3];  // on the stage-input faces
  double* lU[8];    // on the conserved variables inside a stage
  double* lU0[8];   // on U0 = PrimToCons(V^n)
  double* lUx[8];   // on U1 through the base of stage 2
  double* lB0[3];   // on B^n through the RK2 face combination
  double* lVP[8];
  double* lVM[8];
  double* lF[8];
  double* lP;
  double* lS[3][2];  // on max(0,-SL) and max(0,SR) per direction
  double* lDV[3][3];
  double* lE[3];
  double* lBm1[3];  // on the face field's -1 layers (non-periodic axes under CT)
  // forward states saved by the recomputation
  double* Vn[8];
  double* Bn[3];
  double* Vst[2][8];  // stage inputs V1, V2 (the results of stages 1, 2)
  double* Bst[2][3];  // and their faces
  double* Ust[3][8];  // conserved result of each stage
  // what the forward recomputation produced in each stage s: the
  // reconstructed states of each direction d, the wave speeds and the
  // velocity slopes (under CT).  The stage reversals read them instead of
  // reconstructing and solving every direction again.
  double* sVP[3][3][8];
  double* sVM[3][3][8];
  double* sSL[3][3];
  double* sSR[3][3];
  double* sDV[3][3][3];
};

struct AdjArgs {
  F64A<double> f;  // forward arrays (the solver's own)
  AdjBufs b;
  double dt;
  CellMap cm;
};

struct Tab8 {
  double* p[8];
};

__device__ __forceinline__ bool in_dom(const Geom& g, int i, int j, int k) {
  return i >= g.beg[0] && i <= g.end[0] && j >= g.beg[1] && j <= g.end[1] && k >= g.beg[2] && k <= g.end[2];
}
// faces written by CT_Update for component fd (ct_update.c:79-81,132-134,188-190)
__device__ __forceinline__ bool ct_face(const Geom& g, int fd, int i, int j, int k) {
  const int x[3] = {i, j, k};
  for (int ax = 0; ax < g.dims; ax++) {
    const int lo = g.beg[ax] - (ax == fd ? 1 : 0), hi = g.end[ax];
    if (x[ax] < lo || x[ax] > hi) return false;
  }
  return g.dims == 3 || k == 0;
}

#define ADJ_CELL_PROLOGUE                                         \
  long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; \
  const Geom& g = A.f.g;                                          \
  if (c >= g.ncell) return;                                       \
  int i, j, k;                                                    \
  A.cm.ijk(c, i, j, k);

// lU = J_C(U)^T lambda_V (+ lUx), zero off the domain.  One thread per zone.
__global__ void k_adj_c2p(AdjArgs A, Tab8 Ust, Tab8 L, int add_ux) {
  ADJ_CELL_PROLOGUE
  if (!in_dom(g, i, j, k)) {
#pragma unroll
    for (int nv = 0; nv < NV; nv++) A.b.lU[nv][c] = 0.0;
    return;
  }
  double u[NV], lv[NV], lu[NV];
#pragma unroll
  for (int nv = 0; nv < NV; nv++) {
    u[nv] = Ust.p[nv][c];
    lv[nv] = L.p[nv][c];
  }
  c2p_rev(u, A.f.gamma - 1.0, A.f.small_rho, lv, lu);
#pragma unroll
  for (int nv = 0; nv < NV; nv++) A.b.lU[nv][c] = lu[nv] + (add_ux ? A.b.lUx[nv][c] : 0.0);
}

// lVin[dom] += J_P(V^n)^T lU0.  One thread per zone.
__global__ void k_adj_p2c(AdjArgs A) {
  ADJ_CELL_PROLOGUE
  if (!in_dom(g, i, j, k)) return;
  double v[NV], au[NV], av[NV];
#pragma unroll
  for (int nv = 0; nv < NV; nv++) {
    v[nv] = A.b.Vn[nv][c];
    au[nv] = A.b.lU0[nv][c];
    av[nv] = 0.0;
  }
  p2c_rev(v, A.f.gamma - 1.0, au, av);
#pragma unroll
  for (int nv = 0; nv < NV; nv++) A.b.lVin[nv][c] += av[nv];
}

// Face average U[BX] = (B[f] + B[f-s]) / 2 on the domain, transposed.
__global__ void k_adj_avg(AdjArgs A, Tab8 lBdst) {
  ADJ_CELL_PROLOGUE
  for (int d = 0; d < g.dims; d++) {
    int o[3] = {0, 0, 0};
    o[d] = 1;
    double s = 0.0;
    if (in_dom(g, i, j, k)) s += 0.5 * A.b.lU[BX1 + d][c];
    if (in_dom(g, i + o[0], j + o[1], k + o[2])) s += 0.5 * A.b.lU[BX1 + d][c + g.s[d]];
    if (s != 0.0) lBdst.p[d][c] += s;
  }
}
// The averaged components replaced the conserved ones: clear their adjoint.
__global__ void k_adj_zero_bx(AdjArgs A) {
  long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (c >= A.f.g.ncell) return;
  for (int d = 0; d < A.f.g.dims; d++) A.b.lU[BX1 + d][c] = 0.0;
}

// RK combination of stage s >= 2 transposed, cell part:
// U_s = w0 U0 + wc U  =>  lU0 += w0 lU, lU <- wc lU, lUx = lU (adjoint on
// U_{s-1}, the base of U).
__global__ void k_adj_rk_cells(AdjArgs A, double w0, double wc) {
  long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (c >= A.f.g.ncell) return;
#pragma unroll
  for (int nv = 0; nv < NV; nv++) {
    const double l = A.b.lU[nv][c];
    A.b.lU0[nv][c] += w0 * l;
    A.b.lU[nv][c] = wc * l;
    A.b.lUx[nv][c] = wc * l;
  }
}
// Face part on the CT faces: B_s = w0 B0 + wc (B + dt curl E)
// => lB0 += w0 lB, lB <- wc lB (the curl part is then taken from the scaled lB).
__global__ void k_adj_rk_faces(AdjArgs A, double w0, double wc) {
  ADJ_CELL_PROLOGUE
  for (int d = 0; d < g.dims; d++) {
    const double l = A.b.lB[d][c];
    const bool on = ct_face(g, d, i, j, k);
    if (on) A.b.lB0[d][c] += w0 * l;
    A.b.lB[d][c] = on ? wc * l : l;
  }
}
// Stage-1: U before the sweeps equals U0 (both PrimToCons(V^n)).
__global__ void k_adj_add_u0(AdjArgs A) {
  long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (c >= A.f.g.ncell) return;
#pragma unroll
  for (int nv = 0; nv < NV; nv++) A.b.lU0[nv][c] += A.b.lU[nv][c];
}
__global__ void k_add(double* y, const double* x, long long n) {
  long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q < n) y[q] += x[q];
}

// CT_Update transposed: lBin += lB on the CT faces (identity part) and
// lE = curl^T lB.
__global__ void k_adj_ct(AdjArgs A, Tab8 lBc) {
  ADJ_CELL_PROLOGUE
  auto lb = [&](int fd, int ii, int jj, int kk) -> double {
    if (ii >= g.nt[0] || jj >= g.nt[1] || kk >= g.nt[2]) return 0.0;
    if (!ct_face(g, fd, ii, jj, kk)) return 0.0;
    return lBc.p[fd][cidx(g, kk, jj, ii)];
  };
  for (int fd = 0; fd < g.dims; fd++)
    if (ct_face(g, fd, i, j, k)) A.b.lBin[fd][c] += lBc.p[fd][c];
  const double dt = A.dt;
  const double c1 = dt / g.dx[0], c2 = dt / g.dx[1], c3 = g.dims == 3 ? dt / g.dx[2] : 0.0;
  // Bx[f] += -c2 (Ez[f] - Ez[f-sy]) + c3 (Ey[f] - Ey[f-sz])
  // By[f] +=  c1 (Ez[f] - Ez[f-sx]) - c3 (Ex[f] - Ex[f-sz])
  // Bz[f] += -c1 (Ey[f] - Ey[f-sx]) + c2 (Ex[f] - Ex[f-sy])
  A.b.lE[2][c] = -c2 * (lb(0, i, j, k) - lb(0, i, j + 1, k)) + c1 * (lb(1, i, j, k) - lb(1, i + 1, j, k));
  if (g.dims == 3) {
    A.b.lE[1][c] = c3 * (lb(0, i, j, k) - lb(0, i, j, k + 1)) - c1 * (lb(2, i, j, k) - lb(2, i + 1, j, k));
    A.b.lE[0][c] = -c3 * (lb(1, i, j, k) - lb(1, i, j, k + 1)) + c2 * (lb(2, i, j, k) - lb(2, i, j + 1, k));
  }
}

// One edge EMF component transposed: gathers the 40 inputs, forms
// lam * d(edge value)/d(input) for all of them in one reverse evaluation and
// scatters the non-zero ones.
template <int E>
__device__ __forceinline__ void adj_edge(const AdjArgs& A, long long c, double lam) {
  if (lam == 0.0) return;
  constexpr int AX = E == 2 ? 0 : (E == 0 ? 1 : 2);
  constexpr int AY = E == 2 ? 1 : (E == 0 ? 2 : 0);
  const Geom& g = A.f.g;
  const F64A<double>& f = A.f;
  const AdjBufs& b = A.b;
  const long long sx = g.s[AX], sy = g.s[AY];
  const long long c00 = c, cx0 = c + sx, c0y = c + sy, cxy = c + sx + sy;
  const long long cells[4] = {c00, cx0, c0y, cxy};
  double in[kEdgeIn];
  double* dst[kEdgeIn];
  in[0] = f.SR[AX][c00]; dst[0] = &b.lS[AX][1][c00];
  in[1] = f.SR[AX][c0y]; dst[1] = &b.lS[AX][1][c0y];
  in[2] = f.SL[AX][c00]; dst[2] = &b.lS[AX][0][c00];
  in[3] = f.SL[AX][c0y]; dst[3] = &b.lS[AX][0][c0y];
  in[4] = f.SR[AY][c00]; dst[4] = &b.lS[AY][1][c00];
  in[5] = f.SR[AY][cx0]; dst[5] = &b.lS[AY][1][cx0];
  in[6] = f.SL[AY][c00]; dst[6] = &b.lS[AY][0][c00];
  in[7] = f.SL[AY][cx0]; dst[7] = &b.lS[AY][0][cx0];
  const long long bxi[4] = {c00 - sy, c00, c0y, c0y + sy};
  const long long byi[4] = {c00 - sx, c00, cx0, cx0 + sx};
#pragma unroll
  for (int t = 0; t < 4; t++) {
    in[8 + t] = f.Bs[AX][bxi[t]];
    dst[8 + t] = &b.lBin[AX][bxi[t]];
    in[12 + t] = f.Bs[AY][byi[t]];
    dst[12 + t] = &b.lBin[AY][byi[t]];
  }
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const long long cc = cells[q];
    double** d6 = dst + 16 + 6 * q;
    double* i6 = in + 16 + 6 * q;
    i6[0] = f.V[VX1 + AY][cc]; d6[0] = &b.lVin[VX1 + AY][cc];
    i6[1] = f.V[VX1 + AX][cc]; d6[1] = &b.lVin[VX1 + AX][cc];
    i6[2] = f.DV[AX][AY][cc];  d6[2] = &b.lDV[AX][AY][cc];
    i6[3] = f.DV[AY][AY][cc];  d6[3] = &b.lDV[AY][AY][cc];
    i6[4] = f.DV[AX][AX][cc];  d6[4] = &b.lDV[AX][AX][cc];
    i6[5] = f.DV[AY][AX][cc];  d6[5] = &b.lDV[AY][AX][cc];
  }
  double gk[kEdgeIn];
  emf_rev(in, lam, gk);
#pragma unroll
  for (int q = 0; q < kEdgeIn; q++)
    if (gk[q] != 0.0) atomicAdd(dst[q], gk[q]);
}

__global__ void k_adj_emf(AdjArgs A, Box box) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int ncomp = A.f.g.dims == 3 ? 3 : 1;
  if (q >= box.count() * ncomp) return;
  const int e = (int)(q % ncomp);
  int i, j, k;
  box.coords(q / ncomp, i, j, k);
  const long long c = cidx(A.f.g, k, j, i);
  if (ncomp == 1 || e == 2) adj_edge<2>(A, c, A.b.lE[2][c]);
  else if (e == 0) adj_edge<0>(A, c, A.b.lE[0][c]);
  else adj_edge<1>(A, c, A.b.lE[1][c]);
}

// U[c] += -dt/dx (F[c] - F[c-s]) (and the pressure term on the normal
// momentum) transposed: adjoint on the interface fluxes at c+1/2.
template <int DIR>
__global__ void k_adj_flux(AdjArgs A, Box box) {
  long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= box.count()) return;
  int i, j, k;
  box.coords(q, i, j, k);
  const Geom& g = A.f.g;
  const long long c = cidx(g, k, j, i), s = g.s[DIR];
  const double scrh = A.dt / g.dx[DIR];
#pragma unroll
  for (int nv = 0; nv < NV; nv++) A.b.lF[nv][c] = -scrh * (A.b.lU[nv][c] - A.b.lU[nv][c + s]);
  A.b.lP[c] = -scrh * (A.b.lU[Rot<DIR>::vn][c] - A.b.lU[Rot<DIR>::vn][c + s]);
}

// Riemann problem at interface c+1/2 transposed: adjoint on VP[c], VM[c+s]
// (and on the face field that replaces their normal component under CT).
// HLL / HLLD: one thread per interface, all 16 inputs in one reverse
// evaluation.  Roe: one thread per (interface, seeded input of the 16
// states).  lVP / lVM are zero on entry.
template <int DIR>
__device__ __forceinline__ bool adj_riemann_load(const AdjArgs& A, long long c, long long s, double* lam,
                                                 double* vL, double* vR) {
  const bool ct = A.f.ct;
#pragma unroll
  for (int nv = 0; nv < NV; nv++) lam[nv] = A.b.lF[nv][c];
  lam[NV] = A.b.lP[c];
  lam[NV + 1] = ct ? A.b.lS[DIR][0][c] : 0.0;
  lam[NV + 2] = ct ? A.b.lS[DIR][1][c] : 0.0;
  bool any = false;
#pragma unroll
  for (int o = 0; o < kRiemannOut; o++) any |= lam[o] != 0.0;
  if (!any) return false;
#pragma unroll
  for (int nv = 0; nv < NV; nv++) {
    vL[nv] = A.f.VP[nv][c];
    vR[nv] = A.f.VM[nv][c + s];
  }
  if (ct) {
    const double bn = A.f.Bs[DIR][c];
    vL[Rot<DIR>::bn] = bn;
    vR[Rot<DIR>::bn] = bn;
  }
  return true;
}

template <int DIR, int SOLVER>
__global__ void k_adj_riemann(AdjArgs A, Box box) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= box.count()) return;
  int i, j, k;
  box.coords(q, i, j, k);
  const Geom& g = A.f.g;
  const long long c = cidx(g, k, j, i), s = g.s[DIR];
  double lam[kRiemannOut], vL[NV], vR[NV], gL[NV], gR[NV];
  if (!adj_riemann_load<DIR>(A, c, s, lam, vL, vR)) return;
  if (SOLVER == PG_HLL) hll_rev<DIR>(vL, vR, A.f.gamma, lam, gL, gR);
  else hlld_rev<DIR>(vL, vR, A.f.gamma, lam, gL, gR);
  constexpr int BN = Rot<DIR>::bn;
#pragma unroll
  for (int nv = 0; nv < NV; nv++) {
    if (A.f.ct && nv == BN) continue;
    A.b.lVP[nv][c] = gL[nv];
    A.b.lVM[nv][c + s] = gR[nv];
  }
  if (A.f.ct) {
    const double gb = gL[BN] + gR[BN];
    if (gb != 0.0) atomicAdd(&A.b.lBin[DIR][c], gb);
  }
}

template <int DIR>
__global__ void k_adj_riemann_dual(AdjArgs A, Box box, int solver) {
  const long long qq = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (qq >= box.count() * 2 * NV) return;
  const int kk = (int)(qq % (2 * NV));
  int i, j, k;
  box.coords(qq / (2 * NV), i, j, k);
  const Geom& g = A.f.g;
  const long long c = cidx(g, k, j, i), s = g.s[DIR];
  const bool ct = A.f.ct;
  double lam[kRiemannOut], vL[NV], vR[NV];
  if (!adj_riemann_load<DIR>(A, c, s, lam, vL, vR)) return;
  constexpr int BN = Rot<DIR>::bn;
  D1 xL[NV], xR[NV], out[kRiemannOut];
#pragma unroll
  for (int nv = 0; nv < NV; nv++) {
    xL[nv] = D1(vL[nv]);
    xR[nv] = D1(vR[nv]);
  }
  if (kk < NV) xL[kk].d[0] = 1.0;
  else xR[kk - NV].d[0] = 1.0;
  riemann_pt<D1, DIR>(solver, A.f.gamma, A.f.ncomp == 3, xL, xR, out);
  double gk = 0.0;
#pragma unroll
  for (int o = 0; o < kRiemannOut; o++) gk += lam[o] * out[o].d[0];
  const int nv = kk < NV ? kk : kk - NV;
  if (ct && nv == BN) {
    if (gk != 0.0) atomicAdd(&A.b.lBin[DIR][c], gk);
  } else if (kk < NV) {
    A.b.lVP[nv][c] = gk;
  } else {
    A.b.lVM[nv][c + s] = gk;
  }
}

// States of zone c (and its velocity slopes DV = vp - vm) transposed:
// scatter into the adjoint on the stage-input primitives of its stencil.
template <int DIR>
__global__ void k_adj_recon(AdjArgs A, Box box) {
  const long long qq = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (qq >= box.count() * NV) return;
  int i, j, k;
  box.coords(qq / NV, i, j, k);
  const Geom& g = A.f.g;
  const long long c = cidx(g, k, j, i), s = g.s[DIR];
  const int recon = A.f.recon;
  {
    const int nv = (int)(qq % NV);
    double lp = A.b.lVP[nv][c], lm = A.b.lVM[nv][c];
    if (A.f.ct && nv >= VX1 && nv < VX1 + g.dims) {
      const double ld = A.b.lDV[DIR][nv - VX1][c];
      lp += ld;
      lm -= ld;
    }
    if (lp == 0.0 && lm == 0.0) return;
    if (recon == PG_LINEAR) {
      double gw[3];
      plm_rev(A.f.limiter, nv, A.f.V[nv][c - s], A.f.V[nv][c], A.f.V[nv][c + s], lp, lm, gw);
#pragma unroll
      for (int t = 0; t < 3; t++)
        if (gw[t] != 0.0) atomicAdd(&A.b.lVin[nv][c + (t - 1) * s], gw[t]);
      return;
    }
    double w[5], gw[5];
#pragma unroll
    for (int t = 0; t < 5; t++) w[t] = A.f.V[nv][c + (t - 2) * s];
    ppm_rev(w, lp, lm, gw);
#pragma unroll
    for (int t = 0; t < 5; t++)
      if (gw[t] != 0.0) atomicAdd(&A.b.lVin[nv][c + (t - 2) * s], gw[t]);
  }
}

// Boundary transposed: the adjoint on every ghost zone goes to the zone it
// was copied from (the single-pass map of k_bound), and the ghost is cleared.
struct BoundTab {
  double* p[12];
};
__global__ void k_adj_bound(Geom g, CellMap cm, BoundTab t, int narr, int bcx, int bcy, int bcz, int ncomp) {
  long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (c >= g.ncell) return;
  int i, j, k;
  cm.ijk(c, i, j, k);
  if (in_dom(g, i, j, k)) return;
  const int si = bmap(i, g.beg[0], g.end[0], g.nx[0], bcx);
  const int sj = g.dims > 1 ? bmap(j, g.beg[1], g.end[1], g.nx[1], bcy) : j;
  const int sk = g.dims > 2 ? bmap(k, g.beg[2], g.end[2], g.nx[2], bcz) : k;
  const long long src = cidx(g, sk, sj, si);
  const int bt[3] = {bcx, bcy, bcz};
  const int x[3] = {i, j, k};
  int flips = 0;  // mirror signs of the cell variables (the first NV arrays)
  for (int d = 0; d < g.dims; d++)
    if (x[d] < g.beg[d] || x[d] > g.end[d])
      for (int nv = 0; nv < NV; nv++)
        if (bc_flip(d, bc_side(bt[d], x[d] > g.end[d]), nv, ncomp) < 0) flips ^= 1 << nv;
  for (int a = 0; a < narr; a++) {
    const double v = t.p[a][c];
    if (v != 0.0) {
      atomicAdd(&t.p[a][src], (a < NV && ((flips >> a) & 1)) ? -v : v);
      t.p[a][c] = 0.0;
    }
  }
}

// ---------------------------------------------------------------------------
// Boundary fill under CT with a non-periodic axis, transposed.  The forward
// (launch_bound_ct, pg_bound_ct.cuh) goes axis by axis: ghost copies
// (k_bound_axis), then on a non-periodic axis the normal face component
// marched away from the boundary from div B = 0 and, on outflow sides, its
// cell averages (k_fill_normal).  Undone in reverse order; every value the
// forward overwrote gets the adjoint zero once its share has been passed on.
// la: the adjoint arrays in the forward's layout (cells, faces, -1 layers).
// ---------------------------------------------------------------------------
template <int AX>
__global__ void k_adj_bound_axis(BoundCT<double> la, int type, AxisGhosts ag) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= ag.n) return;
  const Geom& g = la.g;
  constexpr int B1 = AX == 0 ? 1 : 0, B2 = AX == 2 ? 1 : 2;
  const int ng = g.beg[AX], n = g.nx[AX];
  int l, c[3], s[3];
  ag.coords(q, l, c[B1], c[B2]);
  const bool lo = l < ng;
  c[AX] = lo ? l : g.end[AX] + 1 + (l - ng);
  s[B1] = c[B1];
  s[B2] = c[B2];
  s[AX] = bc_src(c[AX], g.beg[AX], g.end[AX], n, type);
  const int side = bc_side(type, !lo);
  if (side == PG_USERDEF) return;  // no adjoint of user-defined sides
  const long long dst = cidx(g, c[2], c[1], c[0]), src = cidx(g, s[2], s[1], s[0]);
  auto pass = [](double* d, double* from, bool neg) {  // d += +-from, from = 0
    const double w = *from;
    *from = 0.0;
    if (w != 0.0) atomicAdd(d, neg ? -w : w);
  };
#pragma unroll
  for (int nv = 0; nv < NV; nv++) pass(&la.V[nv][src], &la.V[nv][dst], bc_flip(AX, side, nv, la.ncomp) < 0);
  for (int fd = 0; fd < la.nbfield; fd++) {
    if (fd != AX) {
      const bool neg = bc_flip(AX, side, BX1 + fd, la.ncomp) < 0;
      pass(&la.Bs[fd][src], &la.Bs[fd][dst], neg);
      if (c[fd] == 0) {
        int cm[3] = {c[0], c[1], c[2]}, sm[3] = {s[0], s[1], s[2]};
        cm[fd] = -1;
        sm[fd] = -1;
        pass(bct_face(la, fd, sm[2], sm[1], sm[0]), bct_face(la, fd, cm[2], cm[1], cm[0]), neg);
      }
    } else if (type == PG_PERIODIC) {
      if (lo || c[AX] != g.end[AX]) pass(&la.Bs[fd][src], &la.Bs[fd][dst], false);
      if (lo && c[AX] == 0) {
        int cm[3] = {c[0], c[1], c[2]}, sm[3] = {s[0], s[1], s[2]};
        cm[AX] = -1;
        sm[AX] = n - 1;
        pass(bct_face(la, fd, sm[2], sm[1], sm[0]), bct_face(la, fd, cm[2], cm[1], cm[0]), false);
      }
    }
  }
}

// k_fill_normal transposed: one thread per transverse line and side; its
// normal-face and cell-average adjoints are its own, the transverse faces
// the march read are shared with the neighbouring lines (atomic).
template <int AX>
__global__ void k_adj_fill_normal(BoundCT<double> la, long long ntrans, int type, AxisGhosts ag) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= 2 * ntrans) return;
  const Geom& g = la.g;
  constexpr int B1 = AX == 0 ? 1 : 0, B2 = AX == 2 ? 1 : 2;
  const bool lo = (q & 1) == 0;
  const int st = bc_side(type, !lo);
  if (st == PG_PERIODIC) return;
  const bool average = st == PG_OUTFLOW || st == PG_USERDEF;
  const long long t = q >> 1;
  int c[3];
  ag.transverse(t, c[B1], c[B2]);
  const bool d3 = g.dims == 3;
  const double An = la.area[AX];
  auto lface = [&](int fd, const int* x) { return bct_face(la, fd, x[2], x[1], x[0]); };
  // w * d(A_fd b_fd(+) - A_fd b_fd(-))/d(faces) for the transverse
  // components the march read at cell c (x, y, z order; no z in 2D)
  auto scatter_others = [&](double w) {
    for (int fd = 0; fd < 3; fd++) {
      if (fd == AX || (fd == 2 && !d3)) continue;
      int m[3] = {c[0], c[1], c[2]};
      m[fd] -= 1;
      atomicAdd(lface(fd, c), w * la.area[fd]);
      atomicAdd(lface(fd, m), -w * la.area[fd]);
    }
  };
  // cell averages 0.5 (b(x) + b(x-1)) of the normal component, transposed
  auto average_rev = [&](int x) {
    c[AX] = x;
    int m[3] = {c[0], c[1], c[2]};
    m[AX] = x - 1;
    double* pv = &la.V[BX1 + AX][cidx(g, c[2], c[1], c[0])];
    const double a = *pv;
    *pv = 0.0;
    *lface(AX, c) += 0.5 * a;
    *lface(AX, m) += 0.5 * a;
  };
  if (lo) {
    if (average)
      for (int x = 0; x < g.beg[AX]; x++) average_rev(x);
    // forward, x = beg-1 .. 0: b(x-1) = (An b(x) + others(x)) / An
    for (int x = 0; x <= g.beg[AX] - 1; x++) {
      c[AX] = x;
      int m[3] = {c[0], c[1], c[2]};
      m[AX] = x - 1;
      double* pr = lface(AX, m);
      const double a = *pr;
      *pr = 0.0;
      *lface(AX, c) += a;
      scatter_others(a / An);
    }
  } else {
    if (average)
      for (int x = g.end[AX] + 1; x < g.nt[AX]; x++) average_rev(x);
    // forward, x = end+1 .. nt-1: b(x) = (An b(x-1) - others(x)) / An
    for (int x = g.nt[AX] - 1; x >= g.end[AX] + 1; x--) {
      c[AX] = x;
      int m[3] = {c[0], c[1], c[2]};
      m[AX] = x - 1;
      double* pr = lface(AX, c);
      const double a = *pr;
      *pr = 0.0;
      *lface(AX, m) += a;
      scatter_others(-a / An);
    }
  }
}

// Adjoint input: the cell adjoint on ghosts and the face adjoint off the
// faces the step writes are cleared (those values are refilled, not evolved).
__global__ void k_adj_clean(AdjArgs A, int ct) {
  ADJ_CELL_PROLOGUE
  if (!in_dom(g, i, j, k))
    for (int nv = 0; nv < NV; nv++) A.b.lV[nv][c] = 0.0;
  if (ct)
    for (int d = 0; d < g.dims; d++)
      if (!ct_face(g, d, i, j, k)) A.b.lB[d][c] = 0.0;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct Checkpoints {
  std::vector<std::vector<void*>> slots;  // per slot: 8 cell arrays + the face arrays
};

// The adjoint buffers and the one device block their arrays live in, back
// to back in the order of AdjBufs (S->adj points here; AdjBufs first).
struct AdjState {
  AdjBufs b;
  double* block = nullptr;
  // the block's own pointers of the saved forward states (AdjBufs from Vn
  // to the end; null where the scheme does not use the array), and the
  // per-step copies of them allocated by pg_adjoint_slots
  std::vector<double*> home;
  std::vector<double*> slots;
};

// index of AdjBufs::Vn among the struct's pointers: the saved forward
// states are the members from there to the end
static size_t saved_first() { return offsetof(AdjBufs, Vn) / sizeof(double*); }

// point the saved-state members of A->b at slot's copies (slot < 0: at the
// block's own arrays)
static void bind_slot(AdjState* A, long long n, int slot) {
  double** p = (double**)&A->b;
  const size_t f0 = saved_first();
  size_t k = 0;
  for (size_t h = 0; h < A->home.size(); h++) {
    if (!A->home[h]) continue;
    p[f0 + h] = slot < 0 ? A->home[h] : A->slots[slot] + (k++) * n;
  }
}

static int adjoint_alloc(Solver* S, AdjBufs** out) {
  if (S->adj) {
    *out = (AdjBufs*)S->adj;
    return PG_OK;
  }
  AdjState* A = new AdjState();
  AdjBufs* B = &A->b;
  memset(B, 0, sizeof *B);
  S->adj = A;
  *out = B;
  const long long n = S->g.ncell;
  double** p = (double**)B;
  const size_t np = sizeof(AdjBufs) / sizeof(double*);
  // the per-stage arrays of directions >= dims (and, without CT, the wave
  // speeds and slopes) are not needed
  const bool ct = S->cfg.divb == PG_CONSTRAINED_TRANSPORT;
  std::vector<char> used(np, 1);
  for (size_t q = 0; q < np; q++) {
    bool unused = false;
    const int ns = S->cfg.time_stepping == PG_RK3 ? 3 : (S->cfg.time_stepping == PG_EULER ? 1 : 2);
    for (int k = 0; k < 3; k++) {  // the saved states of stages the scheme does not have
      for (int nv = 0; nv < NV; nv++) {
        unused |= k >= ns - 1 && k < 2 && &p[q] == &B->Vst[k][nv];
        unused |= k >= ns && &p[q] == &B->Ust[k][nv];
      }
      for (int d = 0; d < 3; d++) unused |= k < 2 && (k >= ns - 1 || !ct || d >= S->g.dims) && &p[q] == &B->Bst[k][d];
    }
    for (int st = 0; st < 3; st++)
      for (int d = 0; d < 3; d++) {
        const bool stage_off = st >= ns;
        const bool dir_off = d >= S->g.dims || stage_off;
        for (int nv = 0; nv < NV; nv++)
          unused |= dir_off && (&p[q] == &B->sVP[st][d][nv] || &p[q] == &B->sVM[st][d][nv]);
        unused |= (dir_off || !ct) && (&p[q] == &B->sSL[st][d] || &p[q] == &B->sSR[st][d]);
        for (int c = 0; c < 3; c++) unused |= (dir_off || c >= S->g.dims || !ct) && &p[q] == &B->sDV[st][d][c];
      }
    bool ct_outflow = false;
    for (int d = 0; d < S->g.dims; d++) ct_outflow |= ct && S->cfg.bc[d] != PG_PERIODIC;
    for (int d = 0; d < 3; d++) unused |= !ct_outflow && &p[q] == &B->lBm1[d];
    used[q] = !unused;
  }
  size_t count = 0;
  for (size_t q = 0; q < np; q++) count += used[q];
  const size_t bytes = sizeof(double) * (size_t)n * count;
  // on failure nothing stays behind: the next call allocates again instead
  // of handing out null arrays
  auto drop = [&](int rc) {
    if (A->block) cudaFree(A->block);
    delete A;
    S->adj = nullptr;
    *out = nullptr;
    return rc;
  };
  if (cudaMalloc(&A->block, bytes) != cudaSuccess) {
    A->block = nullptr;
    cudaGetLastError();
    return drop(PG_ERR_NOMEM);
  }
  if (cudaMemset(A->block, 0, bytes) != cudaSuccess) return drop(PG_ERR_CUDA);
  size_t k = 0;
  for (size_t q = 0; q < np; q++)
    if (used[q]) p[q] = A->block + (k++) * n;
  A->home.assign(p + saved_first(), p + np);
  return PG_OK;
}

static void free_slots(AdjState* A) {
  for (double* q : A->slots) cudaFree(q);
  A->slots.clear();
}

// Zeroes p[0..count) with one cudaMemsetAsync per run of arrays that lie
// back to back in the block (the adjoint's groups are contiguous, also after
// the lV/lVin swaps, which exchange whole groups).
static void zero_arrays(std::initializer_list<double* const*> groups, const int* counts, long long n,
                        cudaStream_t st) {
  std::vector<double*> p;
  int g = 0;
  for (double* const* grp : groups) {
    for (int i = 0; i < counts[g]; i++)
      if (grp[i]) p.push_back(grp[i]);  // arrays a scheme does not use are not allocated
    g++;
  }
  size_t i = 0;
  while (i < p.size()) {
    size_t j = i + 1;
    while (j < p.size() && p[j] == p[j - 1] + n) j++;
    cudaMemsetAsync(p[i], 0, (j - i) * (size_t)n * sizeof(double), st);
    i = j;
  }
}

void adjoint_free(Solver* S) {
  if (S->adj) {
    AdjState* A = (AdjState*)S->adj;
    free_slots(A);
    if (A->block) cudaFree(A->block);
    delete A;
    S->adj = nullptr;
  }
  if (S->ckpt) {
    Checkpoints* C = (Checkpoints*)S->ckpt;
    for (auto& sl : C->slots)
      for (void* q : sl)
        if (q) cudaFree(q);
    delete C;
    S->ckpt = nullptr;
  }
  if (S->stage) {
    cudaFree(S->stage);
    S->stage = nullptr;
  }
}

}  // namespace pg

using namespace pg;

namespace {

constexpr int kT = kThreads;

// Up to 16 device arrays of n doubles copied in one launch (blockIdx.y:
// the array).
struct CopyTab {
  double* dst[16];
  const double* src[16];
};
__global__ void k_copy_arrays(CopyTab t, long long n) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) t.dst[blockIdx.y][i] = t.src[blockIdx.y][i];
}

// dstV[0..nv) = srcV[..], dstB[0..nb) = srcB[..] (cell arrays, then faces)
void copy_state(double* const* dstV, const double* const* srcV, int nv, double* const* dstB,
                const double* const* srcB, int nb, long long n, cudaStream_t st) {
  CopyTab t;
  int k = 0;
  for (int q = 0; q < nv; q++, k++) {
    t.dst[k] = dstV[q];
    t.src[k] = srcV[q];
  }
  for (int q = 0; q < nb; q++, k++) {
    t.dst[k] = dstB[q];
    t.src[k] = srcB[q];
  }
  if (k == 0) return;
  k_copy_arrays<<<dim3(grid_for(n), (unsigned)k), kT, 0, st>>>(t, n);
}

Box dir_box(const Geom& g, int dir, int lo_off, int hi_off, bool ct) {
  Box b;
  for (int ax = 0; ax < 3; ax++) {
    if (ax >= g.dims) {
      b.lo[ax] = b.hi[ax] = 0;
    } else if (ax == dir) {
      b.lo[ax] = g.beg[ax] + lo_off;
      b.hi[ax] = g.end[ax] + hi_off;
    } else {
      const int e = ct ? 1 : 0;
      b.lo[ax] = g.beg[ax] - e;
      b.hi[ax] = g.end[ax] + e;
    }
  }
  return b.prepare();
}

// The forward arrays with stage s's saved outputs: the states of direction
// d, the wave speeds and slopes of every direction (see AdjBufs::sVP).
F64A<double> stage_args(const F64A<double>& f, const AdjBufs& b, int s, int d) {
  F64A<double> r = f;
  for (int nv = 0; nv < NV; nv++) {
    r.VP[nv] = b.sVP[s][d][nv];
    r.VM[nv] = b.sVM[s][d][nv];
  }
  if (f.ct)
    for (int e = 0; e < f.g.dims; e++) {
      r.SL[e] = b.sSL[s][e];
      r.SR[e] = b.sSR[s][e];
      for (int c = 0; c < f.g.dims; c++) r.DV[e][c] = b.sDV[s][e][c];
    }
  return r;
}
AdjArgs stage_adj(const AdjArgs& A, int s, int d) {
  AdjArgs r = A;
  r.f = stage_args(A.f, A.b, s, d);
  return r;
}

// Direction DIR reversed; A carries the stage's saved states of DIR.
template <int DIR>
void rev_dir(Solver* S, const AdjArgs& A) {
  const Geom& g = S->g;
  cudaStream_t st = S->stream;
  const long long n = g.ncell;
  Box rb = dir_box(g, DIR, -1, 1, A.f.ct), ib = dir_box(g, DIR, -1, 0, A.f.ct);
  {
    const int cnt[2] = {NV, NV};
    zero_arrays({A.b.lVP, A.b.lVM}, cnt, n, st);
  }
  k_adj_flux<DIR><<<grid_for(ib.count()), kT, 0, st>>>(A, ib);
  if (S->cfg.riemann == PG_HLLD)
    k_adj_riemann<DIR, PG_HLLD><<<grid_for(ib.count(), 64), 64, 0, st>>>(A, ib);
  else if (S->cfg.riemann == PG_HLL)
    k_adj_riemann<DIR, PG_HLL><<<grid_for(ib.count(), 64), 64, 0, st>>>(A, ib);
  else
    k_adj_riemann_dual<DIR><<<grid_for(ib.count() * 2 * NV, 64), 64, 0, st>>>(A, ib, S->cfg.riemann);
  k_adj_recon<DIR><<<grid_for(rb.count() * NV, 128), 128, 0, st>>>(A, rb);
}

BoundCT<double> bound_args(const Geom& g, double* const* V, double* const* Bs, double* const* Bm1, int nbfield,
                           int ncomp) {
  BoundCT<double> b;
  b.g = g;
  for (int nv = 0; nv < 8; nv++) b.V[nv] = V[nv];
  for (int d = 0; d < 3; d++) {
    b.Bs[d] = Bs[d];
    b.Bm1[d] = Bm1[d];
  }
  b.nbfield = nbfield;
  b.ncomp = ncomp;
  face_areas(g, b.area);
  return b;
}

void fwd_bound(Solver* S, const F64A<double>& f) {
  const Geom& g = S->g;
  if (f.ct_outflow) {  // the axis-by-axis sequence with FillMagneticField
    launch_bound_ct<double, double>(S, bound_args(g, f.V, f.Bs, f.Bm1, f.nbfield, f.ncomp), "fp64_bound",
                                    "fp64_fill_normal");
    return;
  }
  const GhostSlabs gs(g);
  k_bound<double><<<grid_for(gs.count()), kT, 0, S->stream>>>(f, S->cfg.bc[0], S->cfg.bc[1], S->cfg.bc[2], gs);
}

Tab8 tab(double* const* p, int n) {
  Tab8 t;
  for (int q = 0; q < 8; q++) t.p[q] = q < n ? p[q] : nullptr;
  return t;
}

// Axis AX of the CT boundary fill reversed: the normal-face march and cell
// averages first, then the ghost copies (the forward's order reversed).
template <int AX>
void rev_bound_axis(Solver* S, const BoundCT<double>& la) {
  const Geom& g = la.g;
  constexpr int B1 = AX == 0 ? 1 : 0, B2 = AX == 2 ? 1 : 2;
  const long long ntrans = (long long)g.nt[B1] * g.nt[B2];
  const AxisGhosts ag(g, AX);
  if (S->cfg.bc[AX] != PG_PERIODIC && la.nbfield > 0)
    k_adj_fill_normal<AX><<<grid_for(2 * ntrans, 128), 128, 0, S->stream>>>(la, ntrans, S->cfg.bc[AX], ag);
  k_adj_bound_axis<AX><<<grid_for(ag.n), kT, 0, S->stream>>>(la, S->cfg.bc[AX], ag);
}

// One stage reversed.  On entry lU holds the adjoint on the stage's
// conserved result (after the face-average part was undone) and lB the
// adjoint on the faces after CT_Update; the solver's V/Bs hold the stage
// input.  On exit lVin/lBin hold the adjoint on the stage input before its
// boundary fill.  add_b0: stage 1 of RK2, where Bs0 copies Bs after the fill.
// stage: 0 or 1, whose saved states, wave speeds and slopes are read.
void rev_stage(Solver* S, const AdjArgs& A, bool add_b0, int stage) {
  const Geom& g = S->g;
  cudaStream_t st = S->stream;
  const long long n = g.ncell;
  const bool ct = A.f.ct;
  const AdjBufs& b = A.b;
  {
    const int cnt[6] = {NV, 3, 6, 9, 3, 3};
    if (A.f.ct_outflow) zero_arrays({b.lVin, b.lBin, &b.lS[0][0], &b.lDV[0][0], b.lE, b.lBm1}, cnt, n, st);
    else if (ct) zero_arrays({b.lVin, b.lBin, &b.lS[0][0], &b.lDV[0][0], b.lE}, cnt, n, st);
    else zero_arrays({b.lVin, b.lBin}, cnt, n, st);
  }
  fwd_bound(S, A.f);  // the stage input's ghosts, read by the reversed reconstruction
  const AdjArgs A0 = stage_adj(A, stage, 0);
  if (ct) {
    k_adj_ct<<<grid_for(n), kT, 0, st>>>(A0, tab(b.lB, 3));
    Box eb;
    for (int ax = 0; ax < 3; ax++) {
      if (ax < g.dims) {
        eb.lo[ax] = g.beg[ax] - 1;
        eb.hi[ax] = g.end[ax];
      } else {
        eb.lo[ax] = eb.hi[ax] = 0;
      }
    }
    eb.prepare();
    k_adj_emf<<<grid_for(eb.count() * (g.dims == 3 ? 3 : 1), 64), 64, 0, st>>>(A0, eb);
  }
  if (g.dims > 2) rev_dir<2>(S, stage_adj(A, stage, 2));
  if (g.dims > 1) rev_dir<1>(S, stage_adj(A, stage, 1));
  rev_dir<0>(S, A0);
  if (add_b0)
    for (int d = 0; d < g.dims; d++) k_add<<<grid_for(n), kT, 0, st>>>(b.lBin[d], b.lB0[d], n);
  if (A.f.ct_outflow) {  // the axis-by-axis fill with FillMagneticField, reversed
    const BoundCT<double> la = bound_args(g, b.lVin, b.lBin, b.lBm1, A.f.nbfield, A.f.ncomp);
    if (g.dims > 2) rev_bound_axis<2>(S, la);
    if (g.dims > 1) rev_bound_axis<1>(S, la);
    rev_bound_axis<0>(S, la);
    return;
  }
  BoundTab t;
  int na = 0;
  for (int nv = 0; nv < NV; nv++) t.p[na++] = b.lVin[nv];
  if (ct)
    for (int d = 0; d < g.dims; d++) t.p[na++] = b.lBin[d];
  k_adj_bound<<<grid_for(n), kT, 0, st>>>(g, CellMap(g), t, na, S->cfg.bc[0], S->cfg.bc[1], S->cfg.bc[2],
                                          S->cfg.components);
}

int check_fp64(pg_solver* h, const char* who, bool tangent_ok) {
  if (!h) {
    set_last_error("null solver");
    return PG_ERR_INVALID;
  }
  const int p = h->S.cfg.precision;
  if (p == PG_FP64 || (tangent_ok && p == PG_FP64_TANGENT)) return PG_OK;
  std::string m = std::string(who) + ": needs a PG_FP64" + (tangent_ok ? " or PG_FP64_TANGENT" : "") + " solver";
  set_last_error(m.c_str());
  return PG_ERR_INVALID;
}

int sync_status(Solver* S) {
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(S->stream);
  if (e != cudaSuccess) {
    set_last_error(cudaGetErrorString(e));
    return PG_ERR_CUDA;
  }
  return PG_OK;
}

}  // namespace

extern "C" int pg_tangent_upload(pg_solver* h, const double* const vars[8], const double* const faces[3],
                                 int layout) {
  if (!h || !vars) {
    set_last_error("null argument");
    return PG_ERR_INVALID;
  }
  if (h->S.cfg.precision != PG_FP64_TANGENT && h->S.cfg.precision != PG_FP64_DD) {
    set_last_error("pg_tangent_upload: needs a PG_FP64_TANGENT or PG_FP64_DD solver");
    return PG_ERR_INVALID;
  }
  return tl_xfer(&h->S, (double* const*)vars, (double* const*)faces, layout, true, 1);
}

extern "C" int pg_tangent_download(pg_solver* h, double* const vars[8], double* const faces[3], int layout) {
  if (!h || !vars) {
    set_last_error("null argument");
    return PG_ERR_INVALID;
  }
  if (h->S.cfg.precision != PG_FP64_TANGENT && h->S.cfg.precision != PG_FP64_DD) {
    set_last_error("pg_tangent_download: needs a PG_FP64_TANGENT or PG_FP64_DD solver");
    return PG_ERR_INVALID;
  }
  return tl_xfer(&h->S, vars, faces, layout, false, 1);
}

extern "C" int pg_tangent_kink(pg_solver* h, int enable, double* margin) {
  if (!h) {
    set_last_error("null argument");
    return PG_ERR_INVALID;
  }
  Solver* S = &h->S;
  if (S->cfg.precision != PG_FP64_TANGENT) {
    set_last_error("pg_tangent_kink: needs a PG_FP64_TANGENT solver");
    return PG_ERR_INVALID;
  }
  const double inf = __builtin_inf();
  unsigned long long bits = 0;
  memcpy(&bits, &inf, sizeof bits);
  const int on = enable ? 1 : 0;
  cudaError_t e = cudaStreamSynchronize(S->stream);
  if (e == cudaSuccess && !enable && margin) {
    e = cudaMemcpyFromSymbol(&bits, g_pg_kink_bits, sizeof bits);
    memcpy(margin, &bits, sizeof bits);
  }
  if (e == cudaSuccess && enable) e = cudaMemcpyToSymbol(g_pg_kink_bits, &bits, sizeof bits);
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_pg_kink_on, &on, sizeof on);
  if (e != cudaSuccess) {
    set_last_error(cudaGetErrorString(e));
    return PG_ERR_CUDA;
  }
  return PG_OK;
}

extern "C" int pg_adjoint_set(pg_solver* h, const double* const vars[8], const double* const faces[3], int layout) {
  int rc = check_fp64(h, "pg_adjoint_set", false);
  if (rc) return rc;
  Solver* S = &h->S;
  if (!vars) {
    set_last_error("pg_adjoint_set: null vars");
    return PG_ERR_INVALID;
  }
  if (layout != PG_LAYOUT_INTERIOR && layout != PG_LAYOUT_PLUTO) {
    set_last_error("bad layout");
    return PG_ERR_INVALID;
  }
  if (S->cfg.time_stepping != PG_RK2 && S->cfg.time_stepping != PG_RK3 && S->cfg.time_stepping != PG_EULER) {
    set_last_error("pg_adjoint_set: the adjoint covers EULER, RK2 and RK3 time stepping");
    return PG_ERR_INVALID;
  }
  if (S->cfg.char_limiting) {
    set_last_error("pg_adjoint_set: no adjoint of the characteristic-limited states");
    return PG_ERR_INVALID;
  }
  if (S->cfg.divb == PG_CONSTRAINED_TRANSPORT && S->cfg.emf_average != PG_UCT_HLL) {
    set_last_error("pg_adjoint_set: the adjoint covers the UCT_HLL emf average");
    return PG_ERR_INVALID;
  }
  for (int d = 0; d < S->g.dims; d++)
    if (bc_side(S->cfg.bc[d], false) == PG_USERDEF || bc_side(S->cfg.bc[d], true) == PG_USERDEF) {
      set_last_error("pg_adjoint_set: user-defined boundaries have no adjoint");
      return PG_ERR_INVALID;
    }
  AdjBufs* B = nullptr;
  if ((rc = adjoint_alloc(S, &B))) {
    adjoint_free(S);
    set_last_error("pg_adjoint_set: allocation failed");
    return rc;
  }
  const long long n = S->g.ncell;
  cudaStream_t st = S->stream;
  const bool ct = S->cfg.divb == PG_CONSTRAINED_TRANSPORT;
  for (int nv = 0; nv < NV; nv++) {
    cudaMemsetAsync(B->lV[nv], 0, n * sizeof(double), st);
    if (vars[nv] && (rc = xfer_f64(S, B->lV[nv], (double*)vars[nv], -1, layout, true))) return rc;
  }
  for (int d = 0; d < 3; d++) cudaMemsetAsync(B->lB[d], 0, n * sizeof(double), st);
  if (ct && faces)
    for (int d = 0; d < S->g.dims; d++)
      if (faces[d] && (rc = xfer_f64(S, B->lB[d], (double*)faces[d], d, layout, true))) return rc;
  AdjArgs A{};  // zero-initialized
  A.f = make_args<double>(S);
  A.b = *B;
  A.cm = CellMap(S->g);
  k_adj_clean<<<grid_for(n), kT, 0, st>>>(A, ct);
  return sync_status(S);
}

extern "C" int pg_adjoint_get(pg_solver* h, double* const vars[8], double* const faces[3], int layout) {
  int rc = check_fp64(h, "pg_adjoint_get", false);
  if (rc) return rc;
  Solver* S = &h->S;
  if (!S->adj || !vars) {
    set_last_error("pg_adjoint_get: no adjoint set, or null vars");
    return PG_ERR_INVALID;
  }
  if (layout != PG_LAYOUT_INTERIOR && layout != PG_LAYOUT_PLUTO) {
    set_last_error("bad layout");
    return PG_ERR_INVALID;
  }
  AdjBufs* B = (AdjBufs*)S->adj;
  for (int nv = 0; nv < NV; nv++)
    if (vars[nv] && (rc = xfer_f64(S, B->lV[nv], vars[nv], -1, layout, false))) return rc;
  if (S->cfg.divb == PG_CONSTRAINED_TRANSPORT && faces)
    for (int d = 0; d < S->g.dims; d++)
      if (faces[d] && (rc = xfer_f64(S, B->lB[d], faces[d], d, layout, false))) return rc;
  return sync_status(S);
}

// The checks every adjoint step entry makes; on success S and B are set.
static int adj_step_checks(pg_solver* h, const char* name, double dt, Solver** Sout, AdjBufs** Bout) {
  int rc = check_fp64(h, name, false);
  if (rc) return rc;
  Solver* S = &h->S;
  if (!S->adj) {
    set_last_error((std::string(name) + ": call pg_adjoint_set first").c_str());
    return PG_ERR_INVALID;
  }
  if (!(dt > 0)) {
    set_last_error((std::string(name) + ": dt must be positive").c_str());
    return PG_ERR_INVALID;
  }
  *Sout = S;
  *Bout = (AdjBufs*)S->adj;
  return PG_OK;
}

// Forward recomputation of one step from the solver's state: the saved
// states (start state, stage inputs and results, each stage's reconstructed
// states, wave speeds and slopes) go to B's saved-state arrays; the solver
// is left at the step's end.
static void adj_forward(Solver* S, AdjBufs* B, double dt) {
  const Geom& g = S->g;
  const long long n = g.ncell;
  const bool ct = S->cfg.divb == PG_CONSTRAINED_TRANSPORT;
  const int nb = ct ? g.dims : 0;
  cudaStream_t st = S->stream;
  if (S->device_dt) {
    S->device_dt = false;
    S->graph_dirty = true;
  }
  S->sc_host->dt = dt;
  cudaMemcpyAsync(&S->sc->dt, &S->sc_host->dt, sizeof(double), cudaMemcpyHostToDevice, st);
  copy_state(B->Vn, S->V, NV, B->Bn, S->Bs, nb, n, st);
  Box dom;
  for (int ax = 0; ax < 3; ax++) {
    dom.lo[ax] = g.beg[ax];
    dom.hi[ax] = g.end[ax];
  }
  dom.prepare();
  // each stage's sweeps write their states, wave speeds and slopes into
  // that stage's own arrays (stage_args), which the reversal reads
  const F64A<double> f = make_args<double>(S);
  const int ns = S->cfg.time_stepping == PG_RK3 ? 3 : (S->cfg.time_stepping == PG_EULER ? 1 : 2);
  launch_bound<double>(S, f);
  k_begin_step<double><<<grid_for(n), kT, 0, st>>>(f, dom);
  for (int s = 1; s <= ns; s++) {
    if (s > 1) launch_bound<double>(S, f);
    launch_sweep<double, 0>(S, stage_args(f, *B, s - 1, 0), s);
    if (g.dims > 1) launch_sweep<double, 1>(S, stage_args(f, *B, s - 1, 1), s);
    if (g.dims > 2) launch_sweep<double, 2>(S, stage_args(f, *B, s - 1, 2), s);
    const F64A<double> fs = stage_args(f, *B, s - 1, 0);
    if (ns == 1) launch_stage_tail<double, 1, 1>(S, fs, dom);
    else if (ns == 2 && s == 1) launch_stage_tail<double, 1, 2>(S, fs, dom);
    else if (ns == 2) launch_stage_tail<double, 2, 2>(S, fs, dom);
    else if (s == 1) launch_stage_tail<double, 1, 3>(S, fs, dom);
    else if (s == 2) launch_stage_tail<double, 2, 3>(S, fs, dom);
    else launch_stage_tail<double, 3, 3>(S, fs, dom);
    if (s < ns) copy_state(B->Vst[s - 1], S->V, NV, B->Bst[s - 1], S->Bs, nb, n, st);
    copy_state(B->Ust[s - 1], S->U, NV, nullptr, nullptr, 0, n, st);
  }
}

// The step reversed from B's saved states: the adjoint on the step's end
// becomes the adjoint on its start, and the solver is left at the step's
// start.
static void adj_reverse(Solver* S, AdjBufs* B, double dt) {
  const Geom& g = S->g;
  const long long n = g.ncell;
  const bool ct = S->cfg.divb == PG_CONSTRAINED_TRANSPORT;
  const int nb = ct ? g.dims : 0;
  cudaStream_t st = S->stream;
  const F64A<double> f = make_args<double>(S);
  const int ns = S->cfg.time_stepping == PG_RK3 ? 3 : (S->cfg.time_stepping == PG_EULER ? 1 : 2);
  AdjArgs A{};  // zero-initialized
  A.f = f;
  A.dt = dt;
  A.cm = CellMap(f.g);
  {
    const int cnt[2] = {NV, 3};
    zero_arrays({B->lU0, B->lB0}, cnt, n, st);  // accumulated over the stages
  }
  // the weights of U_s = w0 U0 + wc (U_{s-1} + dt L) (rk_step.c:18-24)
  auto weights = [&](int s, double& w0, double& wc) {
    if (ns == 2) w0 = wc = 0.5;
    else if (s == 2) { w0 = 0.75; wc = 0.25; }
    else { w0 = 1.0 / 3.0; wc = 2.0 / 3.0; }
  };
  for (int s = ns; s >= 1; s--) {
    A.b = *B;
    // lU: adjoint on U_s from that on V_s (and on U_s as the next stage's base)
    k_adj_c2p<<<grid_for(n), kT, 0, st>>>(A, tab(B->Ust[s - 1], 8), tab(B->lV, 8), s < ns ? 1 : 0);
    if (ct) {
      k_adj_avg<<<grid_for(n), kT, 0, st>>>(A, tab(B->lB, 3));
      k_adj_zero_bx<<<grid_for(n), kT, 0, st>>>(A);
    }
    if (s >= 2) {
      double w0, wc;
      weights(s, w0, wc);
      if (ct) k_adj_rk_faces<<<grid_for(n), kT, 0, st>>>(A, w0, wc);
      k_adj_rk_cells<<<grid_for(n), kT, 0, st>>>(A, w0, wc);
      copy_state(S->V, B->Vst[s - 2], NV, S->Bs, B->Bst[s - 2], nb, n, st);
    } else {
      k_adj_add_u0<<<grid_for(n), kT, 0, st>>>(A);  // stage 1's base is U0
      copy_state(S->V, B->Vn, NV, S->Bs, B->Bn, nb, n, st);
    }
    rev_stage(S, A, s == 1 && ct, s - 1);
    if (s == 1) k_adj_p2c<<<grid_for(n), kT, 0, st>>>(A);
    // lVin / lBin hold the adjoint on the stage input: they become lV / lB
    for (int nv = 0; nv < NV; nv++) std::swap(B->lV[nv], B->lVin[nv]);
    for (int d = 0; d < 3; d++) std::swap(B->lB[d], B->lBin[d]);
  }
  // the solver's state is the step's start again
  copy_state(S->V, B->Vn, NV, S->Bs, B->Bn, nb, n, st);
}

extern "C" int pg_adjoint_step(pg_solver* h, double dt) {
  Solver* S;
  AdjBufs* B;
  int rc = adj_step_checks(h, "pg_adjoint_step", dt, &S, &B);
  if (rc) return rc;
  bind_slot((AdjState*)S->adj, S->g.ncell, -1);
  adj_forward(S, B, dt);
  adj_reverse(S, B, dt);
  return sync_status(S);
}

extern "C" int pg_adjoint_slots(pg_solver* h, int nslots) {
  int rc = check_fp64(h, "pg_adjoint_slots", false);
  if (rc) return rc;
  Solver* S = &h->S;
  if (!S->adj) {
    set_last_error("pg_adjoint_slots: call pg_adjoint_set first");
    return PG_ERR_INVALID;
  }
  if (nslots < 0 || nslots > PG_MAX_CHECKPOINTS) {
    set_last_error("pg_adjoint_slots: nslots outside 0..PG_MAX_CHECKPOINTS");
    return PG_ERR_INVALID;
  }
  AdjState* A = (AdjState*)S->adj;
  bind_slot(A, S->g.ncell, -1);
  if ((int)A->slots.size() == nslots) return PG_OK;
  free_slots(A);
  if (nslots == 0) return PG_OK;
  size_t count = 0;
  for (double* q : A->home) count += q != nullptr;
  const size_t bytes = sizeof(double) * (size_t)S->g.ncell * count;
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess || bytes * (size_t)nslots > free_b / 2) {
    cudaGetLastError();
    set_last_error("pg_adjoint_slots: the slots would take more than half of the free device memory");
    return PG_ERR_NOMEM;
  }
  for (int k = 0; k < nslots; k++) {
    double* q = nullptr;
    if (cudaMalloc(&q, bytes) != cudaSuccess) {
      cudaGetLastError();
      free_slots(A);
      set_last_error("pg_adjoint_slots: allocation failed");
      return PG_ERR_NOMEM;
    }
    A->slots.push_back(q);
  }
  return PG_OK;
}

static int slot_checks(pg_solver* h, const char* name, double dt, int slot, Solver** S, AdjBufs** B) {
  int rc = adj_step_checks(h, name, dt, S, B);
  if (rc) return rc;
  AdjState* A = (AdjState*)(*S)->adj;
  if (slot < 0 || slot >= (int)A->slots.size()) {
    set_last_error((std::string(name) + ": slot outside the slots allocated by pg_adjoint_slots").c_str());
    return PG_ERR_INVALID;
  }
  return PG_OK;
}

extern "C" int pg_adjoint_forward(pg_solver* h, double dt, int slot) {
  Solver* S;
  AdjBufs* B;
  int rc = slot_checks(h, "pg_adjoint_forward", dt, slot, &S, &B);
  if (rc) return rc;
  AdjState* A = (AdjState*)S->adj;
  bind_slot(A, S->g.ncell, slot);
  adj_forward(S, B, dt);
  bind_slot(A, S->g.ncell, -1);
  return sync_status(S);
}

extern "C" int pg_adjoint_reverse(pg_solver* h, double dt, int slot) {
  Solver* S;
  AdjBufs* B;
  int rc = slot_checks(h, "pg_adjoint_reverse", dt, slot, &S, &B);
  if (rc) return rc;
  AdjState* A = (AdjState*)S->adj;
  bind_slot(A, S->g.ncell, slot);
  adj_reverse(S, B, dt);
  bind_slot(A, S->g.ncell, -1);
  return sync_status(S);
}

static int ckpt_xfer(pg_solver* h, int slot, bool save) {
  int rc = check_fp64(h, save ? "pg_checkpoint_save" : "pg_checkpoint_load", true);
  if (rc) return rc;
  Solver* S = &h->S;
  if (slot < 0 || slot >= PG_MAX_CHECKPOINTS) {
    set_last_error("checkpoint slot out of range");
    return PG_ERR_INVALID;
  }
  if (!S->ckpt) S->ckpt = new Checkpoints();
  Checkpoints* C = (Checkpoints*)S->ckpt;
  if ((int)C->slots.size() <= slot) C->slots.resize(slot + 1);
  std::vector<void*>& sl = C->slots[slot];
  const size_t bytes = S->elem_bytes * S->g.ncell;
  const int nb = S->cfg.divb == PG_CONSTRAINED_TRANSPORT ? S->g.dims : 0;
  if (sl.empty()) {
    if (!save) {
      set_last_error("pg_checkpoint_load: empty slot");
      return PG_ERR_INVALID;
    }
    sl.assign(NV + nb, nullptr);
    for (auto& q : sl)
      if (cudaMalloc(&q, bytes) != cudaSuccess) {
        for (auto& r : sl)
          if (r) cudaFree(r);
        sl.clear();
        set_last_error("checkpoint allocation failed");
        return PG_ERR_NOMEM;
      }
  }
  for (int a = 0; a < NV + nb; a++) {
    void* arr = a < NV ? (void*)S->V[a] : (void*)S->Bs[a - NV];
    if (save) cudaMemcpyAsync(sl[a], arr, bytes, cudaMemcpyDeviceToDevice, S->stream);
    else cudaMemcpyAsync(arr, sl[a], bytes, cudaMemcpyDeviceToDevice, S->stream);
  }
  return sync_status(S);
}

extern "C" int pg_checkpoint_save(pg_solver* h, int slot) { return ckpt_xfer(h, slot, true); }
extern "C" int pg_checkpoint_load(pg_solver* h, int slot) { return ckpt_xfer(h, slot, false); }
