// C ABI of libpluto_gb300: solver lifetime, host<->device transfers, the
// AdvanceStep-equivalent and the device-resident step loop.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "pg_internal.h"
#include "pg_userdef.cuh"
#include "pg_xfer.cuh"

using namespace pg;

static thread_local std::string g_last_error = "";

static int fail(int code, const char* msg) {
  g_last_error = msg;
  return code;
}
static int cuda_fail(cudaError_t e, const char* where) {
  g_last_error = std::string(where) + ": " + cudaGetErrorString(e);
  return PG_ERR_CUDA;
}
#define CK(call)                                          \
  do {                                                    \
    cudaError_t _e = (call);                              \
    if (_e != cudaSuccess) return cuda_fail(_e, #call);   \
  } while (0)

extern "C" const char* pg_last_error(void) { return g_last_error.c_str(); }
extern "C" int pg_abi_version(void) { return PG_ABI_VERSION; }
extern "C" int pg_selftest_conversions(unsigned long long counts[2]) {
  if (!counts) return fail(PG_ERR_INVALID, "pg_selftest_conversions: null counts");
  return pg::mixed_selftest_conversions(counts);
}

namespace pg {
// The library's private copy of a validated config keeps both sides' types
// in bc[d] = beginning | end << 4 (as bc_pack in pg_physics.cuh); PERIODIC on
// both sides stays 0.
void pack_bc(pg_config* c) {
  for (int d = 0; d < 3; d++) c->bc[d] = c->bc[d] | ((c->bc_sides ? c->bc_hi[d] : c->bc[d]) << 4);
}

int validate_config(const pg_config* c) {
  if (!c) return fail(PG_ERR_INVALID, "null config");
  if (c->dims < 1 || c->dims > 3) return fail(PG_ERR_INVALID, "dims must be 1..3");
  if (c->components != 2 && c->components != 3) return fail(PG_ERR_INVALID, "components must be 2 or 3");
  if (c->components < c->dims) return fail(PG_ERR_INVALID, "components < dims");
  for (int d = 0; d < c->dims; d++) {
    if (c->nx[d] < 4) return fail(PG_ERR_INVALID, "nx must be >= 4 on active axes");
    if (!(c->dx[d] > 0)) return fail(PG_ERR_INVALID, "dx must be positive");
    if (c->bc[d] < PG_PERIODIC || c->bc[d] > PG_USERDEF) return fail(PG_ERR_INVALID, "unsupported boundary");
    if (c->bc_sides != 0 && c->bc_sides != 1) return fail(PG_ERR_INVALID, "bc_sides must be 0 or 1");
    if (c->bc_sides) {
      if (c->bc_hi[d] < PG_PERIODIC || c->bc_hi[d] > PG_USERDEF)
        return fail(PG_ERR_INVALID, "unsupported boundary (end side)");
      if ((c->bc[d] == PG_PERIODIC) != (c->bc_hi[d] == PG_PERIODIC))
        return fail(PG_ERR_INVALID, "a periodic axis is periodic on both sides");
    }
  }
  if (!(c->gamma > 1.0)) return fail(PG_ERR_INVALID, "gamma must be > 1");
  if (c->reconstruction != PG_LINEAR && c->reconstruction != PG_PARABOLIC)
    return fail(PG_ERR_INVALID, "unsupported reconstruction");
  if (c->limiter < PG_FLAT_LIM || c->limiter > PG_DEFAULT_LIM) return fail(PG_ERR_INVALID, "unsupported limiter");
  if (c->riemann != PG_HLL && c->riemann != PG_HLLD && c->riemann != PG_ROE)
    return fail(PG_ERR_INVALID, "unsupported Riemann solver");
  if (c->time_stepping != PG_EULER && c->time_stepping != PG_RK2 && c->time_stepping != PG_RK3 &&
      !is_ctu(c->time_stepping))
    return fail(PG_ERR_INVALID, "unsupported time stepping");
  if (is_ctu(c->time_stepping)) {
    // Src/States/hancock.c:64-67: the Hancock predictor takes linear states;
    // characteristic tracing takes linear or parabolic ones
    if (c->reconstruction != PG_LINEAR && c->time_stepping != PG_CHAR_TRACING)
      return fail(PG_ERR_INVALID, "the MUSCL-Hancock predictor needs linear reconstruction");
    if (c->precision != PG_FP64 && c->precision != PG_FP64_TANGENT)
      return fail(PG_ERR_INVALID, "CTU runs on the FP64 path");
    if (c->time_stepping == PG_CHAR_TRACING && c->precision != PG_FP64)
      return fail(PG_ERR_INVALID, "characteristic tracing runs on the plain FP64 path (no tangent-linear model)");
  }
  if (c->divb == PG_CONSTRAINED_TRANSPORT) {
    if (c->dims < 2) return fail(PG_ERR_INVALID, "constrained transport needs dims >= 2");
    if (c->emf_average < PG_ARITHMETIC || c->emf_average > PG_UCT_HLL)
      return fail(PG_ERR_INVALID, "unsupported emf average");
    if (is_ctu(c->time_stepping) && c->emf_average == PG_UCT_HLL)  // Src/MHD/CT/ct_emf.c:196-200
      return fail(PG_ERR_INVALID, "CTU takes the ARITHMETIC, UCT0 or UCT_CONTACT emf average");
    // the mixed sweeps fuse the UCT_HLL edge data into the sweep kernels
    if (c->emf_average != PG_UCT_HLL && c->precision != PG_FP64 && c->precision != PG_FP64_TANGENT)
      return fail(PG_ERR_INVALID, "the ARITHMETIC, UCT0 and UCT_CONTACT averages run on the FP64 path");

  } else if (c->divb != PG_DIVB_NONE) {
    return fail(PG_ERR_INVALID, "unsupported divergence control");
  }
  if (c->precision != PG_FP64 && c->precision != PG_MIXED && c->precision != PG_MIXED_DW &&
      c->precision != PG_FP64_TANGENT && c->precision != PG_FP64_DD)
    return fail(PG_ERR_INVALID, "unsupported precision");
  if (c->precision == PG_FP64_DD) {
    if (is_ctu(c->time_stepping)) return fail(PG_ERR_INVALID, "PG_FP64_DD takes EULER, RK2 or RK3 time stepping");
    if (c->char_limiting) return fail(PG_ERR_INVALID, "PG_FP64_DD has no CHAR_LIMITING");
    for (int d = 0; d < c->dims; d++)
      if (c->bc[d] == PG_USERDEF || (c->bc_sides && c->bc_hi[d] == PG_USERDEF))
        return fail(PG_ERR_INVALID, "PG_FP64_DD has no user-defined boundaries");
  }
  if (c->char_limiting != 0 && c->char_limiting != 1) return fail(PG_ERR_INVALID, "char_limiting is 0 or 1");
  if (c->char_limiting) {
    if (c->precision != PG_FP64)
      return fail(PG_ERR_INVALID, "CHAR_LIMITING runs on the plain FP64 path (no mixed or tangent-linear form)");
  }
  if (c->precision == PG_FP64_TANGENT)
    for (int d = 0; d < c->dims; d++)
      if (c->bc[d] == PG_USERDEF || (c->bc_sides && c->bc_hi[d] == PG_USERDEF))
        return fail(PG_ERR_INVALID, "user-defined boundaries have no tangent-linear model");
  return PG_OK;
}

void init_geom(Solver* S) {
  const pg_config* cfg = &S->cfg;
  S->ng = cfg->reconstruction == PG_PARABOLIC ? 3 : 2;  // Src/get_nghost.c:28-104
  // CTU with constrained transport keeps one more ghost layer (get_nghost.c:84-90)
  if (is_ctu(cfg->time_stepping) && cfg->divb == PG_CONSTRAINED_TRANSPORT) S->ng++;
  Geom& g = S->g;
  g.dims = cfg->dims;
  for (int d = 0; d < 3; d++) {
    bool act = d < cfg->dims;
    g.nx[d] = act ? cfg->nx[d] : 1;
    g.nt[d] = act ? cfg->nx[d] + 2 * S->ng : 1;
    g.beg[d] = act ? S->ng : 0;
    g.end[d] = act ? S->ng + cfg->nx[d] - 1 : 0;
    g.dx[d] = act ? cfg->dx[d] : 1.0;
    g.inv_dx[d] = 1.0 / g.dx[d];  // Src/set_geometry.c:244
  }
  // Row pitch: the mixed paths pad rows to a multiple of 4 floats so that the
  // TMA-staged sweeps (16-byte global strides) run at every grid size, e.g.
  // 768^3 with PPM's 3 ghosts (774-zone rows -> pitch 776).
  long long pitch = g.nt[0];
  const bool mixed = cfg->precision == PG_MIXED || cfg->precision == PG_MIXED_DW;
  const char* tma = getenv("PLUTO_GB300_SWEEP_TMA");
  if (mixed && g.dims >= 2 && !(tma && tma[0] == '0')) pitch = (pitch + 3) & ~3LL;
  g.s[0] = 1;
  g.s[1] = pitch;
  g.s[2] = pitch * g.nt[1];
  g.ncell = pitch * g.nt[1] * g.nt[2];
}

void set_last_error(const char* msg) { g_last_error = msg; }
}  // namespace pg

static void free_all(Solver* S) {
  output_free(S);
  if (S->graph) cudaGraphExecDestroy(S->graph);
  S->graph = nullptr;
  if (S->stream) cudaStreamSynchronize(S->stream);
  for (int q = 0; q < 11; q++)
    if (S->ud_pinned[q]) {
      cudaHostUnregister(S->ud_pinned[q]);
      S->ud_pinned[q] = nullptr;
    }
  if (S->ud_pinned_flag) {
    cudaHostUnregister(S->ud_pinned_flag);
    S->ud_pinned_flag = nullptr;
  }
  adjoint_free(S);
  fp64_free(S);
  mixed_free(S);
  if (S->sc) cudaFree(S->sc);
  if (S->sc_host) cudaFreeHost(S->sc_host);
  if (S->stream) cudaStreamDestroy(S->stream);
  S->sc = nullptr;
  S->sc_host = nullptr;
  S->stream = nullptr;
}

extern "C" int pg_create(const pg_config* cfg, pg_solver** out) {
  if (!out) return fail(PG_ERR_INVALID, "null output pointer");
  *out = nullptr;
  int rc = validate_config(cfg);
  if (rc) return rc;
  pg_solver* h = new pg_solver();
  Solver* S = &h->S;
  S->cfg = *cfg;
  pack_bc(&S->cfg);
  init_geom(S);
  cudaError_t e = cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete h;
    return cuda_fail(e, "cudaStreamCreate");
  }
  if (cudaMalloc(&S->sc, sizeof(DevScalars)) != cudaSuccess ||
      cudaMallocHost(&S->sc_host, sizeof(DevScalars)) != cudaSuccess) {
    free_all(S);
    delete h;
    return fail(PG_ERR_NOMEM, "scalar allocation failed");
  }
  cudaMemset(S->sc, 0, sizeof(DevScalars));
  memset(S->sc_host, 0, sizeof(DevScalars));
  const bool f64 = cfg->precision == PG_FP64 || cfg->precision == PG_FP64_TANGENT || cfg->precision == PG_FP64_DD;
  if (cfg->precision == PG_FP64_TANGENT || cfg->precision == PG_FP64_DD)
    S->elem_bytes = 2 * sizeof(double);  // value + tangent, or high + low part
  rc = f64 ? fp64_alloc(S) : mixed_alloc(S);
  if (rc) {
    free_all(S);
    delete h;
    return fail(rc, "device allocation failed");
  }
  CK(cudaDeviceSynchronize());
  *out = h;
  return PG_OK;
}

extern "C" int pg_set_userdef(pg_solver* h, pg_userdef_fn fn, void* user, double* const vars[8],
                              double* const faces[3]) {
  if (!h || !fn || !vars) return fail(PG_ERR_INVALID, "pg_set_userdef: null argument");
  Solver* S = &h->S;
  const Geom& g = S->g;
  const bool ct = S->cfg.divb == PG_CONSTRAINED_TRANSPORT;
  if (ct && !faces) return fail(PG_ERR_INVALID, "pg_set_userdef: constrained transport needs the face arrays");
  CK(cudaStreamSynchronize(S->stream));
  for (int q = 0; q < 11; q++)
    if (S->ud_pinned[q]) {
      cudaHostUnregister(S->ud_pinned[q]);
      S->ud_pinned[q] = nullptr;
    }
  auto reach = [&](double* p, size_t n, int q) -> double* {
    if (!p) return nullptr;
    if (double* a = host_alias(p)) return a;
    if (cudaHostRegister(p, n * sizeof(double), cudaHostRegisterMapped) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    S->ud_pinned[q] = p;
    void* d = nullptr;
    if (cudaHostGetDevicePointer(&d, p, 0) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    return (double*)d;
  };
  for (int nv = 0; nv < 8; nv++) {
    S->ud_dev_v[nv] = reach(vars[nv], (size_t)host_cells(g), nv);
    if (vars[nv] && !S->ud_dev_v[nv]) return fail(PG_ERR_CUDA, "pg_set_userdef: host array not reachable");
  }
  for (int d = 0; d < 3; d++) {
    S->ud_dev_f[d] = nullptr;
    if (!ct || d >= g.dims) continue;
    const size_t n = (size_t)(g.nt[0] + (d == 0)) * (g.nt[1] + (d == 1)) * (g.nt[2] + (d == 2));
    S->ud_dev_f[d] = reach(faces[d], n, 8 + d);
    if (faces[d] && !S->ud_dev_f[d]) return fail(PG_ERR_CUDA, "pg_set_userdef: host face array not reachable");
  }
  S->ud_fn = fn;
  S->ud_user = user;
  S->graph_dirty = true;
  return PG_OK;
}

extern "C" int pg_set_internal_boundary(pg_solver* h, unsigned char* flags) {
  if (!h || !flags) return fail(PG_ERR_INVALID, "pg_set_internal_boundary: null argument");
  Solver* S = &h->S;
  if (!S->ud_fn) return fail(PG_ERR_INVALID, "pg_set_internal_boundary: call pg_set_userdef first");
  if (S->cfg.precision == PG_FP64_TANGENT || S->cfg.precision == PG_FP64_DD || is_ctu(S->cfg.time_stepping))
    return fail(PG_ERR_INVALID, "pg_set_internal_boundary: EULER/RK2/RK3 time stepping, FP64 or mixed");
  CK(cudaStreamSynchronize(S->stream));
  if (S->ud_pinned_flag) {
    cudaHostUnregister(S->ud_pinned_flag);
    S->ud_pinned_flag = nullptr;
  }
  unsigned char* d = nullptr;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, flags) == cudaSuccess && at.type == cudaMemoryTypeHost && at.devicePointer) {
    d = (unsigned char*)at.devicePointer;
  } else {
    cudaGetLastError();
    int dev = 0, ats = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&ats, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) == cudaSuccess &&
        ats == 1) {
      d = flags;
    } else {
      cudaGetLastError();
      if (cudaHostRegister(flags, (size_t)host_cells(S->g), cudaHostRegisterMapped) != cudaSuccess ||
          cudaHostGetDevicePointer((void**)&d, flags, 0) != cudaSuccess) {
        cudaGetLastError();
        return fail(PG_ERR_CUDA, "pg_set_internal_boundary: flag array not reachable");
      }
      S->ud_pinned_flag = flags;
    }
  }
  S->ud_dev_flag = d;
  S->ud_internal = true;
  S->graph_dirty = true;
  return PG_OK;
}

extern "C" int pg_destroy(pg_solver* h) {
  if (!h) return PG_OK;
  free_all(&h->S);
  delete h;
  return PG_OK;
}

// -------------------------------------------------------------------------
// transfers
// -------------------------------------------------------------------------

// Copy between a host array and a device cell/face array.
//   layout INTERIOR: host holds the interior box (faces one longer along fd)
//   layout PLUTO   : host holds the whole ghosted array (faces with the -1 layer)
namespace pg {
int xfer_f64(Solver* S, double* dev, double* host, int fd, int layout, bool to_dev) {
  const Geom& g = S->g;
  cudaStream_t st = S->stream;
  if (double* alias = host_alias(host)) {
    launch_host_xfer<double>(st, alias, dev, g, fd, layout, to_dev);
    CK(cudaGetLastError());
    return PG_OK;
  }
  const size_t e = sizeof(double);
  cudaMemcpyKind kind = to_dev ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost;
  // the FP64 arrays have unpadded rows (only the mixed paths pad them)
  if (g.s[1] != g.nt[0]) return fail(PG_ERR_INVALID, "xfer_f64: padded rows");
  if (layout == PG_LAYOUT_PLUTO) {
    if (fd < 0) {
      size_t n = (size_t)g.ncell;
      CK(to_dev ? cudaMemcpyAsync(dev, host, n * e, kind, st) : cudaMemcpyAsync(host, dev, n * e, kind, st));
      return PG_OK;
    }
    // host array has one more element along fd; skip its first (-1) layer
    size_t nx = g.nt[0], ny = g.nt[1], nz = g.nt[2];
    if (fd == 0) {
      double* h = host + 1;
      if (to_dev) CK(cudaMemcpy2DAsync(dev, nx * e, h, (nx + 1) * e, nx * e, ny * nz, kind, st));
      else CK(cudaMemcpy2DAsync(h, (nx + 1) * e, dev, nx * e, nx * e, ny * nz, kind, st));
    } else if (fd == 1) {
      double* h = host + nx;
      if (to_dev) CK(cudaMemcpy2DAsync(dev, nx * ny * e, h, nx * (ny + 1) * e, nx * ny * e, nz, kind, st));
      else CK(cudaMemcpy2DAsync(h, nx * (ny + 1) * e, dev, nx * ny * e, nx * ny * e, nz, kind, st));
    } else {
      double* h = host + nx * ny;
      size_t n = nx * ny * nz;
      CK(to_dev ? cudaMemcpyAsync(dev, h, n * e, kind, st) : cudaMemcpyAsync(h, dev, n * e, kind, st));
    }
    return PG_OK;
  }
  // interior layout: a 3D box copy; the face box starts one layer earlier
  int lo[3], n[3];
  for (int ax = 0; ax < 3; ax++) {
    lo[ax] = g.beg[ax] - ((ax == fd && ax < g.dims) ? 1 : 0);
    n[ax] = g.nx[ax] + ((ax == fd && ax < g.dims) ? 1 : 0);
  }
  cudaMemcpy3DParms p;
  memset(&p, 0, sizeof p);
  cudaPitchedPtr dp = make_cudaPitchedPtr(dev, g.nt[0] * e, g.nt[0], g.nt[1]);
  cudaPitchedPtr hp = make_cudaPitchedPtr(host, n[0] * e, n[0], n[1]);
  if (to_dev) {
    p.srcPtr = hp;
    p.dstPtr = dp;
    p.dstPos = make_cudaPos(lo[0] * e, lo[1], lo[2]);
  } else {
    p.srcPtr = dp;
    p.srcPos = make_cudaPos(lo[0] * e, lo[1], lo[2]);
    p.dstPtr = hp;
  }
  p.extent = make_cudaExtent(n[0] * e, n[1], n[2]);
  p.kind = kind;
  CK(cudaMemcpy3DAsync(&p, st));
  return PG_OK;
}
}  // namespace pg

int mixed_download(Solver* S, double* const vars[8], double* const faces[3], int layout);
int mixed_upload_host(Solver* S, const double* const vars[8], const double* const faces[3], int layout);

extern "C" int pg_upload(pg_solver* h, const double* const vars[8], const double* const faces[3], int layout) {
  if (!h || !vars) return fail(PG_ERR_INVALID, "null argument");
  if (layout != PG_LAYOUT_INTERIOR && layout != PG_LAYOUT_PLUTO) return fail(PG_ERR_INVALID, "bad layout");
  Solver* S = &h->S;
  const bool ct = S->cfg.divb == PG_CONSTRAINED_TRANSPORT;
  if (ct && !faces) return fail(PG_ERR_INVALID, "constrained transport needs staggered fields");
  // a new state: the sticky error flags of earlier steps (NaN, timeout) no
  // longer apply
  CK(cudaMemsetAsync(&S->sc->status, 0, sizeof(int), S->stream));
  if (S->cfg.precision == PG_FP64_TANGENT) return tl_xfer(S, (double* const*)vars, (double* const*)faces, layout, true, 0);
  if (S->cfg.precision == PG_FP64_DD) {  // high parts; the low parts start at zero
    for (int nv = 0; nv < 8; nv++) CK(cudaMemsetAsync(S->V[nv], 0, S->g.ncell * S->elem_bytes, S->stream));
    if (ct)
      for (int d = 0; d < S->g.dims; d++) CK(cudaMemsetAsync(S->Bs[d], 0, S->g.ncell * S->elem_bytes, S->stream));
    return tl_xfer(S, (double* const*)vars, (double* const*)faces, layout, true, 0);
  }
  if (S->cfg.precision != PG_FP64) return mixed_upload_host(S, vars, faces, layout);
  for (int nv = 0; nv < 8; nv++) {
    if (vars[nv]) {
      int rc = xfer_f64(S, S->V[nv], (double*)vars[nv], -1, layout, true);
      if (rc) return rc;
    } else {
      CK(cudaMemsetAsync(S->V[nv], 0, S->g.ncell * sizeof(double), S->stream));
    }
  }
  if (ct)
    for (int d = 0; d < S->g.dims; d++) {
      if (!faces[d]) return fail(PG_ERR_INVALID, "missing staggered component");
      int rc = xfer_f64(S, S->Bs[d], (double*)faces[d], d, layout, true);
      if (rc) return rc;
    }
  CK(cudaStreamSynchronize(S->stream));
  return PG_OK;
}

extern "C" int pg_download(pg_solver* h, double* const vars[8], double* const faces[3], int layout) {
  if (!h || !vars) return fail(PG_ERR_INVALID, "null argument");
  if (layout != PG_LAYOUT_INTERIOR && layout != PG_LAYOUT_PLUTO) return fail(PG_ERR_INVALID, "bad layout");
  Solver* S = &h->S;
  const bool ct = S->cfg.divb == PG_CONSTRAINED_TRANSPORT;
  if (S->cfg.precision == PG_FP64_TANGENT || S->cfg.precision == PG_FP64_DD)
    return tl_xfer(S, vars, faces, layout, false, 0);
  if (S->cfg.precision != PG_FP64) return mixed_download(S, vars, faces, layout);
  for (int nv = 0; nv < 8; nv++)
    if (vars[nv]) {
      int rc = xfer_f64(S, S->V[nv], vars[nv], -1, layout, false);
      if (rc) return rc;
    }
  if (ct && faces)
    for (int d = 0; d < S->g.dims; d++)
      if (faces[d]) {
        int rc = xfer_f64(S, S->Bs[d], faces[d], d, layout, false);
        if (rc) return rc;
      }
  CK(cudaStreamSynchronize(S->stream));
  return PG_OK;
}

// -------------------------------------------------------------------------
// stepping
// -------------------------------------------------------------------------

static int enqueue_step(Solver* S) {
  if (has_userdef(S) && !S->ud_fn)
    return fail(PG_ERR_INVALID, "a user-defined boundary side needs pg_set_userdef before the first step");
  S->ud_stage = 0;
  if (S->cfg.precision == PG_FP64) return fp64_enqueue_step(S);
  if (S->cfg.precision == PG_FP64_TANGENT) return tl_enqueue_step(S);
  if (S->cfg.precision == PG_FP64_DD) return dd_enqueue_step(S);
  return mixed_enqueue_step(S);
}

static int read_scalars(Solver* S) {
  CK(cudaMemcpyAsync(S->sc_host, S->sc, sizeof(DevScalars), cudaMemcpyDeviceToHost, S->stream));
  CK(cudaStreamSynchronize(S->stream));
  if (S->sc_host->status & 8)
    return fail(PG_ERR_TIMEOUT, "a sweep's wait for its TMA-staged tile ran out (the step's results are invalid)");
  if (S->sc_host->status & 2)
    return fail(PG_ERR_NAN, "Roe solver: negative sound speed squared (Src/MHD/roe.c stops the run here)");
  if (S->sc_host->status) return fail(PG_ERR_NAN, "non-finite inverse time step (NaN or Inf in the state)");
  return PG_OK;
}

static void fill_info(Solver* S, pg_step_info* info) {
  if (!info) return;
  DevScalars* h = S->sc_host;
  double inv, mach;
  memcpy(&inv, &h->inv_dt_bits, sizeof inv);
  memcpy(&mach, &h->mach_bits, sizeof mach);
  info->inv_dt_hyp = inv;
  info->max_mach = mach;
  info->nfail = (int64_t)h->nfail;
}

extern "C" int pg_advance(pg_solver* h, double dt, pg_step_info* info) {
  if (!h) return fail(PG_ERR_INVALID, "null solver");
  if (!(dt > 0)) return fail(PG_ERR_INVALID, "dt must be positive");
  Solver* S = &h->S;
  if (S->device_dt) {
    S->device_dt = false;
    S->graph_dirty = true;
  }
  S->sc_host->dt = dt;
  CK(cudaMemcpyAsync(&S->sc->dt, &S->sc_host->dt, sizeof(double), cudaMemcpyHostToDevice, S->stream));
  int rc = enqueue_step(S);
  if (rc) return rc == PG_ERR_CUDA ? cuda_fail(cudaGetLastError(), "kernel launch") : rc;
  rc = read_scalars(S);
  fill_info(S, info);
  S->steps_done++;
  return rc;
}

static int ensure_graph(Solver* S) {
  if (S->graph && !S->graph_dirty) return PG_OK;
  if (S->graph) {
    cudaGraphExecDestroy(S->graph);
    S->graph = nullptr;
  }
  cudaGraph_t graph;
  CK(cudaStreamBeginCapture(S->stream, cudaStreamCaptureModeThreadLocal));
  int rc = enqueue_step(S);
  cudaError_t e = cudaStreamEndCapture(S->stream, &graph);
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(&S->graph, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
  S->graph_dirty = false;
  return PG_OK;
}

extern "C" int pg_run_async(pg_solver* h, int nsteps, double first_dt, double cfl, double cfl_max_var) {
  if (!h) return fail(PG_ERR_INVALID, "null solver");
  if (nsteps < 0) return fail(PG_ERR_INVALID, "nsteps < 0");
  if (!(cfl > 0) || !(cfl_max_var > 0)) return fail(PG_ERR_INVALID, "cfl must be positive");
  Solver* S = &h->S;
  if (!S->device_dt || S->cfl != cfl || S->cfl_max_var != cfl_max_var) {
    S->device_dt = true;
    S->cfl = cfl;
    S->cfl_max_var = cfl_max_var;
    S->graph_dirty = true;
  }
  if (first_dt > 0) {
    S->sc_host->dt = first_dt;
    CK(cudaMemcpyAsync(&S->sc->dt, &S->sc_host->dt, sizeof(double), cudaMemcpyHostToDevice, S->stream));
  }
  int rc = ensure_graph(S);
  if (rc) return rc;
  for (int s = 0; s < nsteps; s++) CK(cudaGraphLaunch(S->graph, S->stream));
  S->steps_done += nsteps;
  return PG_OK;
}

extern "C" int pg_sync(pg_solver* h) {
  if (!h) return fail(PG_ERR_INVALID, "null solver");
  return read_scalars(&h->S);
}

extern "C" int pg_run(pg_solver* h, int nsteps, double first_dt, double cfl, double cfl_max_var, double* t_out,
                      double* next_dt_out) {
  int rc = pg_run_async(h, nsteps, first_dt, cfl, cfl_max_var);
  if (rc) return rc;
  rc = pg_sync(h);
  Solver* S = &h->S;
  if (t_out) *t_out = S->sc_host->time;
  if (next_dt_out) *next_dt_out = S->sc_host->dt;
  return rc;
}

extern "C" int pg_get_stream(pg_solver* h, void** st) {
  if (!h || !st) return fail(PG_ERR_INVALID, "null argument");
  *st = (void*)h->S.stream;
  return PG_OK;
}

extern "C" int pg_get_info(pg_solver* h, pg_step_info* info, double* time, double* dt) {
  if (!h) return fail(PG_ERR_INVALID, "null solver");
  int rc = read_scalars(&h->S);
  fill_info(&h->S, info);
  if (time) *time = h->S.sc_host->time;
  if (dt) *dt = h->S.sc_host->dt;
  return rc;
}

extern "C" int pg_kernel_launches_per_step(pg_solver* h) {
  if (!h) return -1;
  Solver* S = &h->S;
  cudaGraph_t gr;
  // count kernel nodes of a freshly captured step
  cudaStreamBeginCapture(S->stream, cudaStreamCaptureModeThreadLocal);
  enqueue_step(S);
  if (cudaStreamEndCapture(S->stream, &gr) != cudaSuccess) return -1;
  size_t n = 0;
  cudaGraphGetNodes(gr, nullptr, &n);
  int kernels = 0;
  if (n) {
    cudaGraphNode_t* nodes = new cudaGraphNode_t[n];
    cudaGraphGetNodes(gr, nodes, &n);
    for (size_t q = 0; q < n; q++) {
      cudaGraphNodeType t;
      cudaGraphNodeGetType(nodes[q], &t);
      if (t == cudaGraphNodeTypeKernel) kernels++;
    }
    delete[] nodes;
  }
  cudaGraphDestroy(gr);
  return kernels;
}

// -------------------------------------------------------------------------
// timing and per-kernel profile (CUDA events on the solver's stream)
// -------------------------------------------------------------------------
namespace pg {
void prof_mark(Solver* S, const char* name, bool begin) {
  Prof* P = S->prof;
  if (begin) P->names.push_back(name);
  if (P->used >= P->ev.size()) {
    cudaEvent_t e;
    cudaEventCreate(&e);
    P->ev.push_back(e);
  }
  cudaEventRecord(P->ev[P->used++], S->stream);
}
}  // namespace pg

extern "C" int pg_run_timed(pg_solver* h, int nsteps, double first_dt, double cfl, double cfl_max_var,
                            double* elapsed_ms) {
  if (!h || !elapsed_ms) return fail(PG_ERR_INVALID, "null argument");
  Solver* S = &h->S;
  // build the graph outside the timed region
  if (!S->device_dt || S->cfl != cfl || S->cfl_max_var != cfl_max_var || S->graph_dirty) {
    int rc = pg_run_async(h, 0, first_dt, cfl, cfl_max_var);
    if (rc) return rc;
    first_dt = 0;
  }
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  CK(cudaEventRecord(e0, S->stream));
  int rc = pg_run_async(h, nsteps, first_dt, cfl, cfl_max_var);
  CK(cudaEventRecord(e1, S->stream));
  CK(cudaEventSynchronize(e1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *elapsed_ms = ms;
  if (rc) return rc;
  return read_scalars(S);
}

extern "C" int pg_profile_kernels(pg_solver* h, int nsteps, double first_dt, double cfl, double cfl_max_var,
                                  char* names, int name_stride, double* total_ms, int* launches, int max_kernels,
                                  int* n_kernels) {
  if (!h || !names || !total_ms || !launches || !n_kernels || name_stride < 8)
    return fail(PG_ERR_INVALID, "null argument");
  Solver* S = &h->S;
  S->device_dt = true;
  S->cfl = cfl;
  S->cfl_max_var = cfl_max_var;
  S->graph_dirty = true;
  if (first_dt > 0) {
    S->sc_host->dt = first_dt;
    CK(cudaMemcpyAsync(&S->sc->dt, &S->sc_host->dt, sizeof(double), cudaMemcpyHostToDevice, S->stream));
  }
  Prof P;
  S->prof = &P;
  int rc = PG_OK;
  for (int s = 0; s < nsteps && !rc; s++) rc = enqueue_step(S);
  S->prof = nullptr;
  CK(cudaStreamSynchronize(S->stream));
  std::vector<std::string> uniq;
  std::vector<double> tot;
  std::vector<int> cnt;
  for (size_t q = 0; q < P.names.size(); q++) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, P.ev[2 * q], P.ev[2 * q + 1]);
    size_t u = 0;
    while (u < uniq.size() && uniq[u] != P.names[q]) u++;
    if (u == uniq.size()) {
      uniq.push_back(P.names[q]);
      tot.push_back(0.0);
      cnt.push_back(0);
    }
    tot[u] += ms;
    cnt[u] += 1;
  }
  for (cudaEvent_t e : P.ev) cudaEventDestroy(e);
  int n = (int)uniq.size() < max_kernels ? (int)uniq.size() : max_kernels;
  for (int u = 0; u < n; u++) {
    strncpy(names + (size_t)u * name_stride, uniq[u].c_str(), name_stride - 1);
    names[(size_t)u * name_stride + name_stride - 1] = 0;
    total_ms[u] = tot[u];
    launches[u] = cnt[u];
  }
  *n_kernels = n;
  S->steps_done += nsteps;
  if (rc) return rc;
  return read_scalars(S);
}
