// USERDEF sides: the user's boundary code (PLUTO's UserDefBoundary, through
// the callback set by pg_set_userdef) runs on the host, in stream order
// inside the step, so a captured step graph replays it too.  Per side, in the
// reference's order (Src/boundary.c:258-288):
//   1. one kernel per array writes the side's slab -- the ghost layers and as
//      many interior layers, over the whole transverse extent -- into the
//      caller's host arrays (PLUTO layout; face arrays with their -1 layer);
//   2. a host function calls the callback for the cell box, then for each
//      staggered component's box (UserDefBoundary with center_box, then
//      x1face_box, x2face_box, x3face_box);
//   3. one kernel per array reads those boxes back.
// Under CT, FillMagneticField, CT_AverageNormalMagField and
// CT_AverageTransverseMagField then run on the device (pg_bound_ct.cuh).  The host arrays are reached through their device
// alias (pinned memory) or directly (page-table access); pg_set_userdef pins
// arrays the device cannot reach.
#pragma once
#include "pg_internal.h"
#include "pg_dw.cuh"
#include "pg_physics.cuh"

namespace pg {

// inclusive index box in PLUTO's index space (faces: -1 allowed along their axis)
struct IBox {
  int lo[3], hi[3];
  __host__ __device__ long long count() const {
    return (long long)(hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1) * (hi[2] - lo[2] + 1);
  }
};

__device__ __forceinline__ void ud_to_dev(double v, float* d) { *d = narrow(v); }
__device__ __forceinline__ void ud_to_dev(double v, double* d) { *d = v; }
__device__ __forceinline__ double ud_to_host(float v) { return widen(v); }
__device__ __forceinline__ double ud_to_host(double v) { return v; }
// dual and double-double numbers (their solvers reject USERDEF sides and
// internal boundaries; instantiated only)
template <class D>
__device__ __forceinline__ void ud_to_dev(double v, D* d) { *d = D(v); }
template <class D>
__device__ __forceinline__ double ud_to_host(const D& v) { return value_of(v); }

// host: PLUTO-layout array (cells: nt0 x nt1 x nt2; face fd: one more along
// fd with the -1 layer first); dev: the device cell/face array; bm1: the
// device -1 plane of face fd (Bm1[fd]) or null.
template <class T>
__global__ void k_box_xfer(double* host, T* dev, T* bm1, Geom g, int fd, IBox b, int to_dev) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= b.count()) return;
  const int nx = b.hi[0] - b.lo[0] + 1, ny = b.hi[1] - b.lo[1] + 1;
  const int i = b.lo[0] + (int)(q % nx);
  const long long r = q / nx;
  const int j = b.lo[1] + (int)(r % ny), k = b.lo[2] + (int)(r / ny);
  long long h;
  T* d;
  if (fd < 0) {
    h = ((long long)k * g.nt[1] + j) * g.nt[0] + i;
    d = dev + cidx(g, k, j, i);
  } else {
    const int sx = g.nt[0] + (fd == 0), sy = g.nt[1] + (fd == 1);
    h = ((long long)(k + (fd == 2)) * sy + (j + (fd == 1))) * sx + (i + (fd == 0));
    const int x = fd == 0 ? i : (fd == 1 ? j : k);
    if (x < 0) {
      if (!bm1) return;
      d = bm1 + (fd == 0 ? (long long)k * g.nt[1] + j : (fd == 1 ? (long long)k * g.nt[0] + i
                                                                   : (long long)j * g.nt[0] + i));
    } else {
      d = dev + cidx(g, k, j, i);
    }
  }
  if (to_dev) ud_to_dev(host[h], d);
  else host[h] = ud_to_host(*d);
}

inline bool has_userdef(const Solver* S) {
  for (int d = 0; d < S->g.dims; d++)
    if (bc_side(S->cfg.bc[d], false) == PG_USERDEF || bc_side(S->cfg.bc[d], true) == PG_USERDEF) return true;
  return false;
}

// the slab a callback may read (down) and PLUTO's boxes it writes (up) for
// side `end` of axis ax; fd = -1 for cells, else the face component
inline IBox ud_box(const Geom& g, int ax, bool end, int fd, bool up) {
  IBox b;
  const int ng = g.beg[ax];
  for (int d = 0; d < 3; d++) {
    const bool act = d < g.dims;
    b.lo[d] = 0;
    b.hi[d] = act ? g.nt[d] - 1 : 0;
    if (d == fd && d != ax) b.lo[d] = -1;  // transverse face component: its -1 layer
  }
  if (up) {  // RBoxDefine of Src/boundary.c:144-164
    if (!end) {
      b.lo[ax] = fd == ax ? -1 : 0;
      b.hi[ax] = ng - 1;
    } else {
      b.lo[ax] = fd == ax ? g.end[ax] : g.end[ax] + 1;
      b.hi[ax] = g.nt[ax] - 1;
    }
  } else {  // the ghosts and as many interior layers
    if (!end) {
      b.lo[ax] = fd == ax ? -1 : 0;
      b.hi[ax] = 2 * ng - 1;
    } else {
      b.lo[ax] = g.nt[ax] - 2 * ng;
      b.hi[ax] = g.nt[ax] - 1;
    }
  }
  return b;
}

inline void CUDART_CB ud_host_call(void* p) {
  const UdCall* c = (const UdCall*)p;
  const Solver* S = c->S;
  S->ud_fn(S->ud_user, c->side, 0, c->stage);  // cells (CENTER)
  for (int fd = 0; fd < c->nbfield; fd++) S->ud_fn(S->ud_user, c->side, 1 + fd, c->stage);  // X*FACE
}

// zone flags: host array in PLUTO's layout, device array with the row pitch
static __global__ void k_flag_xfer(unsigned char* host, unsigned char* dev, Geom g, int to_dev) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= (long long)g.nt[0] * g.nt[1] * g.nt[2]) return;
  const int i = (int)(q % g.nt[0]);
  const long long r = q / g.nt[0];
  const long long c = cidx(g, (int)(r / g.nt[1]), (int)(r % g.nt[1]), i);
  if (to_dev) dev[c] = host[q];
  else host[q] = dev[c];
}

// INTERNAL_BOUNDARY (Src/boundary.c:90-92): before the fill, the callback
// with side PG_SIDE_INTERNAL on the whole state and the zone flags; the flags
// are cleared before the step's first fill (Src/main.c:329).
template <class T>
inline void launch_internal_boundary(Solver* S, T* const V[8], T* const Bs[3], T* const Bm1[3], int nbfield,
                                     unsigned char* dflag) {
  const Geom& g = S->g;
  cudaStream_t st = S->stream;
  const int stage = S->ud_stage < kUdStages ? S->ud_stage : kUdStages - 1;
  if (S->ud_stage == 0) cudaMemsetAsync(dflag, 0, (size_t)g.ncell, st);
  IBox cb;
  for (int d = 0; d < 3; d++) {
    cb.lo[d] = 0;
    cb.hi[d] = g.nt[d] - 1;
  }
  for (int dir = 0; dir < 2; dir++) {
    const int up = dir;
    if (up) {
      UdCall* c = &S->ud_calls[stage][PG_SIDE_INTERNAL];
      c->S = S;
      c->side = PG_SIDE_INTERNAL;
      c->stage = S->ud_stage + 1;
      c->nbfield = 0;  // one call, UserDefBoundary (d, NULL, 0, grid)
      cudaLaunchHostFunc(st, ud_host_call, c);
    }
    for (int nv = 0; nv < NV; nv++)
      if (S->ud_dev_v[nv])
        k_box_xfer<T><<<grid_for(cb.count()), kThreads, 0, st>>>(S->ud_dev_v[nv], V[nv], (T*)nullptr, g, -1, cb, up);
    for (int fd = 0; fd < nbfield; fd++) {
      if (!S->ud_dev_f[fd]) continue;
      IBox fb = cb;
      fb.lo[fd] = -1;
      k_box_xfer<T><<<grid_for(fb.count()), kThreads, 0, st>>>(S->ud_dev_f[fd], Bs[fd], Bm1[fd], g, fd, fb, up);
    }
    k_flag_xfer<<<grid_for(host_cells(g)), kThreads, 0, st>>>(S->ud_dev_flag, dflag, g, up);
  }
}

// the USERDEF sides of axis ax, after the other sides of the axis were filled
template <class T>
inline void launch_userdef_axis(Solver* S, T* const V[8], T* const Bs[3], T* const Bm1[3], int nbfield, int ax) {
  const Geom& g = S->g;
  cudaStream_t st = S->stream;
  const int stage = S->ud_stage < kUdStages ? S->ud_stage : kUdStages - 1;
  for (int end = 0; end < 2; end++) {
    if (bc_side(S->cfg.bc[ax], end != 0) != PG_USERDEF) continue;
    const int side = 2 * ax + end;
    for (int dir = 0; dir < 2; dir++) {
      const bool up = dir == 1;
      if (up) {
        UdCall* c = &S->ud_calls[stage][side];
        c->S = S;
        c->side = side;
        c->stage = S->ud_stage + 1;
        c->nbfield = nbfield;
        cudaLaunchHostFunc(st, ud_host_call, c);
      }
      const IBox cb = ud_box(g, ax, end != 0, -1, up);
      for (int nv = 0; nv < NV; nv++)
        if (S->ud_dev_v[nv])
          k_box_xfer<T><<<grid_for(cb.count()), kThreads, 0, st>>>(S->ud_dev_v[nv], V[nv], (T*)nullptr, g, -1, cb,
                                                                   up ? 1 : 0);
      for (int fd = 0; fd < nbfield; fd++) {
        if (!S->ud_dev_f[fd]) continue;
        const IBox fb = ud_box(g, ax, end != 0, fd, up);
        k_box_xfer<T><<<grid_for(fb.count()), kThreads, 0, st>>>(S->ud_dev_f[fd], Bs[fd], Bm1[fd], g, fd, fb,
                                                                 up ? 1 : 0);
      }
    }
  }
}

}  // namespace pg
