// FP64 path: one kernel per reference sub-step, double precision throughout,
// compiled without multiply-add contraction (--fmad=false) so that every
// result rounds exactly as PLUTO 4.3's C code compiled with
// -ffp-contract=off.  The plain FP64 path is bound by the GB300's FP64
// issue rate, not by HBM, so it stores intermediate sweep data in HBM
// (states, fluxes) and computes each interface exactly once.
//
// Kernel <-> reference map (files inside the PLUTO source tree):
//   k_bound        Boundary(), Src/boundary.c:41-303 (periodic/outflow/reflective/eqtsymmetric)
//   k_begin_step   PrimToCons3D + U0/Bs0 save, Src/Time_Stepping/rk_step.c:93-100
//   k_recon<D>     States(), Src/States/plm_states.c:80-312, ppm_states.c:68-253,
//                  plus CT_StoreVelSlopes, Src/MHD/CT/ct_stag_slopes.c:5-49
//   k_riemann<D>   HLL_Solver / HLLD_Solver (Src/MHD/hll.c:30, hlld.c:44) and
//                  CT_StoreUpwindEMF (Src/MHD/CT/ct_emf.c:104-207)
//   k_update<D>    RightHandSide (Src/MHD/rhs.c:193-201), U += rhs and the
//                  C_dt bookkeeping (Src/Time_Stepping/update_stage.c:214-241)
//   k_emf          CT_ComputeEMF -> CT_EMF_HLL_Solver (ct_emf_average.c:179-352)
//   k_ct_update<S> CT_Update (Src/MHD/CT/ct_update.c:29-220) fused with the
//                  RK face combination (rk_step.c:172-174, 231-233)
//   k_finalize<S>  RK cell combination (rk_step.c:168-170, 227-229),
//                  CT_AverageMagneticField (ct_field_average.c:13-132),
//                  ConsToPrim3D (Src/mappers3D.c:16-72), dt reduction
//                  (update_stage.c:308-312)
//   k_end_step     NextTimeStep (Src/main.c:459-532)
#include <cstdio>
#include <cstring>
#include <mutex>

#include "pg_fp64_kernels.cuh"

namespace pg {

int fp64_alloc(Solver* S) {
  const long long n = S->g.ncell;
  const size_t es = S->elem_bytes;  // 8 (double) or 16 (Dual<1>, tangent-linear)
  auto alloc = [&](double** p) -> int {
    if (cudaMalloc(p, n * es) != cudaSuccess) return PG_ERR_NOMEM;
    cudaMemset(*p, 0, n * es);
    return PG_OK;
  };
  const bool ct = S->cfg.divb == PG_CONSTRAINED_TRANSPORT;
  for (int nv = 0; nv < 8; nv++) {
    if (alloc(&S->V[nv]) || alloc(&S->U[nv]) || alloc(&S->U0[nv]) || alloc(&S->VP[nv]) ||
        alloc(&S->VM[nv]) || alloc(&S->F[nv]))
      return PG_ERR_NOMEM;
  }
  if (alloc(&S->P) || alloc(&S->CM) || alloc(&S->CDT)) return PG_ERR_NOMEM;
  if (ct) {
    for (int d = 0; d < S->g.dims; d++) {
      if (alloc(&S->Bs[d]) || alloc(&S->Bs0[d]) || alloc(&S->SL[d]) || alloc(&S->SR[d])) return PG_ERR_NOMEM;
      for (int c = 0; c < S->g.dims; c++)
        if (alloc(&S->DV[d][c])) return PG_ERR_NOMEM;
    }
    if (alloc(&S->E[2])) return PG_ERR_NOMEM;
    if (S->g.dims == 3 && (alloc(&S->E[0]) || alloc(&S->E[1]))) return PG_ERR_NOMEM;
    bool outflow = false;
    for (int d = 0; d < S->g.dims; d++) outflow |= S->cfg.bc[d] != PG_PERIODIC;
    if (outflow) {
      const Geom& g = S->g;
      const long long m[3] = {(long long)g.nt[1] * g.nt[2], (long long)g.nt[0] * g.nt[2],
                              (long long)g.nt[0] * g.nt[1]};
      for (int d = 0; d < g.dims; d++) {
        if (cudaMalloc(&S->Bm1[d], m[d] * es) != cudaSuccess) return PG_ERR_NOMEM;
        cudaMemset(S->Bm1[d], 0, m[d] * es);
      }
    }
  }
  if (is_ctu(S->cfg.time_stepping)) {
    for (int d = 0; d < S->g.dims; d++)
      for (int nv = 0; nv < 8; nv++)
        if (alloc(&S->Upd[d][nv]) || alloc(&S->Umd[d][nv]) || alloc(&S->Rhd[d][nv])) return PG_ERR_NOMEM;
    for (int nv = 0; nv < 8; nv++)
      if (alloc(&S->Uh[nv])) return PG_ERR_NOMEM;
  }
  // face EMFs and mass-flux signs: CTU, and RK with the ARITHMETIC/UCT0/UCT_CONTACT averages
  if (ct && (is_ctu(S->cfg.time_stepping) || S->cfg.emf_average != PG_UCT_HLL)) {
    for (int q = 0; q < 6; q++)
      if (alloc(&S->EF[q])) return PG_ERR_NOMEM;
    for (int d = 0; d < S->g.dims; d++) {
      if (cudaMalloc(&S->SV[d], n) != cudaSuccess) return PG_ERR_NOMEM;
      cudaMemset(S->SV[d], 0, n);
    }
  }
  if (cudaMalloc(&S->flag, n) != cudaSuccess) return PG_ERR_NOMEM;
  cudaMemset(S->flag, 0, n);
  return PG_OK;
}

void fp64_free(Solver* S) {
  auto f = [](void* p) {
    if (p) cudaFree(p);
  };
  for (int nv = 0; nv < 8; nv++) {
    f(S->V[nv]); f(S->U[nv]); f(S->U0[nv]); f(S->VP[nv]); f(S->VM[nv]); f(S->F[nv]);
    S->V[nv] = S->U[nv] = S->U0[nv] = S->VP[nv] = S->VM[nv] = S->F[nv] = nullptr;
  }
  f(S->P); f(S->CM); f(S->CDT); f(S->flag);
  S->P = S->CM = S->CDT = nullptr;
  S->flag = nullptr;
  for (int d = 0; d < 3; d++) {
    f(S->Bs[d]); f(S->Bs0[d]); f(S->SL[d]); f(S->SR[d]); f(S->E[d]); f(S->Bm1[d]);
    S->Bs[d] = S->Bs0[d] = S->SL[d] = S->SR[d] = S->E[d] = S->Bm1[d] = nullptr;
    for (int c = 0; c < 3; c++) { f(S->DV[d][c]); S->DV[d][c] = nullptr; }
    for (int nv = 0; nv < 8; nv++) {
      f(S->Upd[d][nv]); f(S->Umd[d][nv]); f(S->Rhd[d][nv]);
      S->Upd[d][nv] = S->Umd[d][nv] = S->Rhd[d][nv] = nullptr;
    }
    f(S->SV[d]);
    S->SV[d] = nullptr;
  }
  for (int nv = 0; nv < 8; nv++) { f(S->Uh[nv]); S->Uh[nv] = nullptr; }
  for (int q = 0; q < 6; q++) { f(S->EF[q]); S->EF[q] = nullptr; }
}

int fp64_enqueue_step(Solver* S) { return fp64_enqueue_step_t<double>(S); }

}  // namespace pg

// ===========================================================================
// Allocation-free entry point: pg_tube_step_static
//
// For callers that cannot call cudaMalloc while they run: a host application
// that has handed all device memory to its own pool allocator, or a real-time
// loop that must not hit the implicit device synchronisation of
// cudaMalloc/cudaFree.  One plain-FP64 AdvanceStep of a 1D problem without
// constrained transport (the Riemann-tube family: HLL/HLLD/Roe, PLM/PPM,
// EULER/RK2/RK3, periodic, outflow, reflective or equatorial-symmetric sides)
// runs with every work array carved out of the file-scope device array
// below, the same kernels as pg_advance.  CTU time stepping (its predictor
// needs three more sets of arrays) and user-defined sides (they call back
// into a host function registered on a solver) are rejected before anything
// is launched.
//
// The array is sized for PG_STATIC_MAX_ZONES interior zones (plus ghosts):
// 51 double arrays + flags + scalars, about 13.4 MB, held by every GPU that
// loads this library until the process exits.  Larger problems are
// rejected with PG_ERR_TOO_LARGE.  All calls share the array and it keeps
// the last call's contents; everything a step reads is written earlier in
// the same step, and the scalars are cleared on entry.  Calls that overlap
// on the GPU (two streams, two host threads) race on the array: serialise
// them.  The first call on a device looks up the array's device address
// (cudaGetSymbolAddress) with that device current and caches it for the
// process; cudaDeviceReset invalidates the cache, so do not reset a device
// between calls.
// ===========================================================================
namespace pg {

constexpr long long kStaticZones = PG_STATIC_MAX_ZONES + 6;  // + up to 3 ghosts per side
constexpr int kStaticArrays = 6 * 8 + 3;                     // V U U0 VP VM F, P CM CDT
constexpr size_t kStaticDoubles = (size_t)kStaticArrays * kStaticZones;
constexpr size_t kStaticBytes =
    kStaticDoubles * sizeof(double) + ((kStaticZones + 255) / 256) * 256 + sizeof(DevScalars);

static __device__ __align__(256) unsigned char g_pg_static_scratch[kStaticBytes];

static void* s_static_base[64];  // device address of the array, per device
static std::mutex s_static_mutex;  // guards the lookup of s_static_base

__global__ void k_static_setup(DevScalars* sc, double dt) {
  sc->dt = dt;
  sc->dt_prev = 0.0;
  sc->time = 0.0;
  sc->inv_dt_bits = 0ull;
  sc->mach_bits = 0ull;
  sc->nfail = 0ull;
  sc->status = 0;
}

// The pointer table travels by value as a kernel argument.
struct StaticVTab {
  double* V[8];
};

// Caller's [8][nx] interior state <-> the ghosted arrays of the step.
__global__ void k_static_copy(StaticVTab t, const double* src, double* dst, int nx, int beg, int to_state) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= NV * nx) return;
  int nv = q / nx, i = q - nv * nx;
  if (to_state) t.V[nv][beg + i] = src[q];
  else dst[q] = t.V[nv][beg + i];
}

}  // namespace pg

extern "C" int pg_tube_step_static(const pg_config* cfg, const double* v_in, double* v_out, double dt,
                                   void* cuda_stream, pg_step_info* info) {
  using namespace pg;
  if (!cfg || !v_in || !v_out) {
    set_last_error("pg_tube_step_static: null argument");
    return PG_ERR_INVALID;
  }
  int rc = validate_config(cfg);
  if (rc) return rc;
  if (cfg->dims != 1 || cfg->divb != PG_DIVB_NONE || cfg->precision != PG_FP64) {
    set_last_error("pg_tube_step_static: only 1D FP64 problems without constrained transport");
    return PG_ERR_INVALID;
  }
  if (is_ctu(cfg->time_stepping)) {  // the CTU predictor's arrays are not in the static array
    set_last_error("pg_tube_step_static: CTU time stepping is not supported (EULER, RK2 or RK3)");
    return PG_ERR_INVALID;
  }
  if (cfg->bc[0] == PG_USERDEF || (cfg->bc_sides && cfg->bc_hi[0] == PG_USERDEF)) {
    set_last_error("pg_tube_step_static: user-defined sides need a solver (pg_set_userdef)");
    return PG_ERR_INVALID;
  }
  if (cfg->nx[0] > PG_STATIC_MAX_ZONES) {
    set_last_error("pg_tube_step_static: nx exceeds PG_STATIC_MAX_ZONES (32768 zones)");
    return PG_ERR_TOO_LARGE;
  }
  if (!(dt > 0)) {
    set_last_error("pg_tube_step_static: dt must be positive");
    return PG_ERR_INVALID;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    set_last_error("pg_tube_step_static: no current CUDA device");
    return PG_ERR_CUDA;
  }
  void* base = nullptr;
  {
    std::lock_guard<std::mutex> lock(s_static_mutex);
    if (!s_static_base[dev]) {  // once per device, with that device current
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_pg_static_scratch);
      if (e != cudaSuccess || !p) {
        set_last_error("pg_tube_step_static: cudaGetSymbolAddress failed");
        return PG_ERR_CUDA;
      }
      s_static_base[dev] = p;
    }
    base = s_static_base[dev];
  }
  // A solver description on the host stack; every device pointer is a slice
  // of the static array.
  Solver S;
  S.cfg = *cfg;
  pack_bc(&S.cfg);
  init_geom(&S);
  S.stream = (cudaStream_t)cuda_stream;
  S.device_dt = false;
  const long long n = S.g.ncell;  // <= kStaticZones
  double* d = (double*)base;
  int a = 0;
  for (int nv = 0; nv < 8; nv++) {
    S.V[nv] = d + (size_t)(a++) * kStaticZones;
    S.U[nv] = d + (size_t)(a++) * kStaticZones;
    S.U0[nv] = d + (size_t)(a++) * kStaticZones;
    S.VP[nv] = d + (size_t)(a++) * kStaticZones;
    S.VM[nv] = d + (size_t)(a++) * kStaticZones;
    S.F[nv] = d + (size_t)(a++) * kStaticZones;
  }
  S.P = d + (size_t)(a++) * kStaticZones;
  S.CM = d + (size_t)(a++) * kStaticZones;
  S.CDT = d + (size_t)(a++) * kStaticZones;
  unsigned char* tail = (unsigned char*)(d + kStaticDoubles);
  S.flag = tail;
  S.sc = (DevScalars*)(tail + ((kStaticZones + 255) / 256) * 256);
  (void)n;
  StaticVTab vt;
  for (int nv = 0; nv < 8; nv++) vt.V[nv] = S.V[nv];
  k_static_setup<<<1, 1, 0, S.stream>>>(S.sc, dt);
  const int nx = S.g.nx[0], beg = S.g.beg[0];
  k_static_copy<<<(8 * nx + 255) / 256, 256, 0, S.stream>>>(vt, v_in, nullptr, nx, beg, 1);
  rc = fp64_enqueue_step(&S);
  if (rc) {
    cudaStreamSynchronize(S.stream);  // nothing queued may outlive this call
    set_last_error("pg_tube_step_static: kernel launch failed");
    return PG_ERR_CUDA;
  }
  k_static_copy<<<(8 * nx + 255) / 256, 256, 0, S.stream>>>(vt, nullptr, v_out, nx, beg, 0);
  DevScalars hs;
  if (cudaMemcpyAsync(&hs, S.sc, sizeof hs, cudaMemcpyDeviceToHost, S.stream) != cudaSuccess ||
      cudaStreamSynchronize(S.stream) != cudaSuccess) {
    set_last_error("pg_tube_step_static: CUDA error during the step");
    return PG_ERR_CUDA;
  }
  if (info) {
    double inv, mach;
    memcpy(&inv, &hs.inv_dt_bits, sizeof inv);
    memcpy(&mach, &hs.mach_bits, sizeof mach);
    info->inv_dt_hyp = inv;
    info->max_mach = mach;
    info->nfail = (int64_t)hs.nfail;
  }
  if (hs.status) {
    set_last_error("pg_tube_step_static: non-finite state");
    return PG_ERR_NAN;
  }
  return PG_OK;
}
