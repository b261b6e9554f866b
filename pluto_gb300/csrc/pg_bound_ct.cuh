// Boundary fill under constrained transport when an axis is not periodic,
// and whenever a side is user-defined (then also without CT, nbfield 0):
// the reference's side-by-side sequence (Src/boundary.c:137-300), one axis
// after the other.  Per axis, k_bound_axis copies the cells and the
// transverse face components (zero gradient, periodic image, or mirror image
// with the FlipSign signs; the normal component too on a periodic axis),
// including the faces' -1 layers (index -1 along their own axis,
// Src/initialize.c:448-453), which live in Bm1 because the face arrays do not
// store them; then, on a non-periodic axis, k_fill_normal recovers the normal
// face component in the ghost faces from div B = 0 (FillMagneticField,
// Src/MHD/CT/ct_fill_mag_field.c:38-180) and, on outflow and user-defined
// sides, averages it to the cell centres (CT_AverageNormalMagField,
// Src/MHD/CT/ct_field_average.c:134-275).  T is the storage type, C the
// arithmetic type (double for the FP32-storage mixed path).
#pragma once
#include "pg_internal.h"
#include "pg_physics.cuh"
#include "pg_userdef.cuh"

namespace pg {

template <class T>
struct BoundCT {
  Geom g;
  T* V[8];
  T* Bs[3];
  T* Bm1[3];  // -1 layers: Bm1[0][k][j], Bm1[1][k][i], Bm1[2][j][i]
  int nbfield, ncomp;
  double area[3];
};

// Cartesian face areas, Src/set_geometry.c:139-210 (D_EXPAND over DIMENSIONS).
inline void face_areas(const Geom& g, double A[3]) {
  const double* dx = g.dx;
  if (g.dims == 2) {
    A[0] = 1.0 * dx[1];
    A[1] = dx[0] * 1.0;
    A[2] = 0.0;
  } else {
    A[0] = 1.0 * dx[1] * dx[2];
    A[1] = dx[0] * 1.0 * dx[2];
    A[2] = dx[0] * dx[1] * 1.0;
  }
}

template <class T>
__device__ __forceinline__ T* bct_face(const BoundCT<T>& a, int fd, int k, int j, int i) {
  const Geom& g = a.g;
  const int x = fd == 0 ? i : (fd == 1 ? j : k);
  if (x < 0) {
    if (fd == 0) return a.Bm1[0] + (long long)k * g.nt[1] + j;
    if (fd == 1) return a.Bm1[1] + (long long)k * g.nt[0] + i;
    return a.Bm1[2] + (long long)j * g.nt[0] + i;
  }
  return a.Bs[fd] + cidx(g, k, j, i);
}

// Ghost layers of axis AX over the full extent of the other axes (the
// reference's CENTER / X*FACE boxes).  Sources are interior along AX, so the
// threads are independent.
template <class T, int AX>
__global__ void k_bound_axis(BoundCT<T> a, int type, AxisGhosts ag) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= ag.n) return;
  const Geom& g = a.g;
  constexpr int B1 = AX == 0 ? 1 : 0, B2 = AX == 2 ? 1 : 2;
  const int ng = g.beg[AX], n = g.nx[AX];
  int l, c[3], s[3];
  ag.coords(q, l, c[B1], c[B2]);
  const bool lo = l < ng;
  c[AX] = lo ? l : g.end[AX] + 1 + (l - ng);
  s[B1] = c[B1];
  s[B2] = c[B2];
  s[AX] = bc_src(c[AX], g.beg[AX], g.end[AX], n, type);
  const int side = bc_side(type, !lo);  // this ghost's side of the axis
  if (side == PG_USERDEF) return;       // the host callback fills it
  const long long dst = cidx(g, c[2], c[1], c[0]), src = cidx(g, s[2], s[1], s[0]);
#pragma unroll
  for (int nv = 0; nv < NV; nv++) {
    const T v = a.V[nv][src];
    a.V[nv][dst] = bc_flip(AX, side, nv, a.ncomp) < 0 ? -v : v;
  }
#pragma unroll
  for (int fd = 0; fd < 3; fd++) {  // compile-time fd keeps c, s, cm, sm in registers
    if (fd >= a.nbfield) break;
    if (fd != AX) {
      const bool neg = bc_flip(AX, side, BX1 + fd, a.ncomp) < 0;
      const T v = a.Bs[fd][src];
      a.Bs[fd][dst] = neg ? -v : v;
      if (c[fd] == 0) {  // the -1 layer of this transverse component
        int cm[3] = {c[0], c[1], c[2]}, sm[3] = {s[0], s[1], s[2]};
        cm[fd] = -1;
        sm[fd] = -1;
        const T w = *bct_face(a, fd, sm[2], sm[1], sm[0]);
        *bct_face(a, fd, cm[2], cm[1], cm[0]) = neg ? -w : w;
      }
    } else if (type == PG_PERIODIC) {
      // normal component: faces beg-1 .. -1 from their images; on the end
      // side the face at end keeps its value (its image beg-1 is set equal
      // to it by the begin side)
      if (lo || c[AX] != g.end[AX]) a.Bs[fd][dst] = a.Bs[fd][src];
      if (lo && c[AX] == 0) {
        int cm[3] = {c[0], c[1], c[2]}, sm[3] = {s[0], s[1], s[2]};
        cm[AX] = -1;
        sm[AX] = n - 1;
        *bct_face(a, fd, cm[2], cm[1], cm[0]) = *bct_face(a, fd, sm[2], sm[1], sm[0]);
      }
    }
  }
}

// One thread per transverse position and side: the normal component marched
// away from the boundary face, then (outflow sides) its cell average.  type:
// the axis's packed side types.
template <class T, class C, int AX>
__global__ void k_fill_normal(BoundCT<T> a, long long ntrans, int type, AxisGhosts ag) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= 2 * ntrans) return;
  const Geom& g = a.g;
  constexpr int B1 = AX == 0 ? 1 : 0, B2 = AX == 2 ? 1 : 2;
  const bool lo = (q & 1) == 0;
  const int st = bc_side(type, !lo);
  const bool average = st == PG_OUTFLOW || st == PG_USERDEF;
  const long long t = q >> 1;
  int c[3];
  ag.transverse(t, c[B1], c[B2]);
  const bool d3 = g.dims == 3;
  auto face = [&](int fd, int k, int j, int i) -> C { return C(*bct_face(a, fd, k, j, i)); };
  // A_d b_d(+) - A_d b_d(-) of component fd at cell c
  auto dB = [&](int fd) -> C {
    int m[3] = {c[0], c[1], c[2]};
    m[fd] -= 1;
    return a.area[fd] * face(fd, c[2], c[1], c[0]) - a.area[fd] * face(fd, m[2], m[1], m[0]);
  };
  // the other two terms in x, y, z order (zero for z in 2D)
  auto others = [&]() -> C {
    if (AX == 0) return dB(1) + (d3 ? dB(2) : C(0.0));
    if (AX == 1) return dB(0) + (d3 ? dB(2) : C(0.0));
    return dB(0) + dB(1);
  };
  const double An = a.area[AX];
  auto cell_average = [&](int x) {
    c[AX] = x;
    int m[3] = {c[0], c[1], c[2]};
    m[AX] = x - 1;
    const C avg = 0.5 * (face(AX, c[2], c[1], c[0]) + face(AX, m[2], m[1], m[0]));
    a.V[BX1 + AX][cidx(g, c[2], c[1], c[0])] = T(avg);
  };
  if (lo) {
    for (int x = g.beg[AX] - 1; x >= 0; x--) {
      c[AX] = x;
      const C bp = face(AX, c[2], c[1], c[0]);
      C r;
      if (AX == 0) r = (An * bp + dB(1) + (d3 ? dB(2) : C(0.0))) / An;
      else if (AX == 1) r = (An * bp + dB(0) + (d3 ? dB(2) : C(0.0))) / An;
      else r = (An * bp + dB(0) + dB(1)) / An;
      int m[3] = {c[0], c[1], c[2]};
      m[AX] = x - 1;
      *bct_face(a, AX, m[2], m[1], m[0]) = T(r);
    }
    if (average)
      for (int x = 0; x < g.beg[AX]; x++) cell_average(x);
  } else {
    for (int x = g.end[AX] + 1; x < g.nt[AX]; x++) {
      c[AX] = x;
      int m[3] = {c[0], c[1], c[2]};
      m[AX] = x - 1;
      const C bm = face(AX, m[2], m[1], m[0]);
      *bct_face(a, AX, c[2], c[1], c[0]) = T((An * bm - others()) / An);
    }
    if (average)
      for (int x = g.end[AX] + 1; x < g.nt[AX]; x++) cell_average(x);
  }
}

// CT_AverageTransverseMagField (Src/MHD/CT/ct_field_average.c:275-440,
// Cartesian) on the user-defined sides of axis AX: the transverse
// cell-centred components in the ghost zones from the staggered field
// (0.5 (b + b(-1)) along the component's axis, its -1 layer from Bm1).  The
// same thread layout as k_bound_axis.
template <class T, class C, int AX>
__global__ void k_avg_transverse(BoundCT<T> a, int type, AxisGhosts ag) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= ag.n) return;
  const Geom& g = a.g;
  constexpr int B1 = AX == 0 ? 1 : 0, B2 = AX == 2 ? 1 : 2;
  const int ng = g.beg[AX];
  int l, c[3];
  ag.coords(q, l, c[B1], c[B2]);
  const bool lo = l < ng;
  if (bc_side(type, !lo) != PG_USERDEF) return;
  c[AX] = lo ? l : g.end[AX] + 1 + (l - ng);
  for (int fd = 0; fd < a.nbfield; fd++) {
    if (fd == AX) continue;
    int m[3] = {c[0], c[1], c[2]};
    m[fd] -= 1;
    const C avg = 0.5 * (C(*bct_face(a, fd, c[2], c[1], c[0])) + C(*bct_face(a, fd, m[2], m[1], m[0])));
    a.V[BX1 + fd][cidx(g, c[2], c[1], c[0])] = T(avg);
  }
}

template <class T, class C, int AX>
static void launch_bound_ct_axis(Solver* S, const BoundCT<T>& b, const char* copy_name, const char* fill_name) {
  const Geom& g = b.g;
  constexpr int B1 = AX == 0 ? 1 : 0, B2 = AX == 2 ? 1 : 2;
  const long long ntrans = (long long)g.nt[B1] * g.nt[B2];
  const AxisGhosts ag(g, AX);
  const long long nghost = ag.n;
  PG_LAUNCH(S, copy_name, (k_bound_axis<T, AX><<<grid_for(nghost), kThreads, 0, S->stream>>>(
                              b, S->cfg.bc[AX], ag)));
  if (bc_side(S->cfg.bc[AX], false) == PG_USERDEF || bc_side(S->cfg.bc[AX], true) == PG_USERDEF)
    launch_userdef_axis<T>(S, b.V, b.Bs, b.Bm1, b.nbfield, AX);
  // per side, outflow and user-defined: FillMagneticField +
  // CT_AverageNormalMagField; reflective and equatorial-symmetric:
  // FillMagneticField only (Src/boundary.c:188-206, 285-288)
  if (S->cfg.bc[AX] != PG_PERIODIC && b.nbfield > 0)
    PG_LAUNCH(S, fill_name, (k_fill_normal<T, C, AX><<<grid_for(2 * ntrans, 128), 128, 0, S->stream>>>(
                                b, ntrans, S->cfg.bc[AX], ag)));
  // user-defined sides under CT: CT_AverageTransverseMagField too
  // (Src/boundary.c:287-289)
  if (b.nbfield > 0 &&
      (bc_side(S->cfg.bc[AX], false) == PG_USERDEF || bc_side(S->cfg.bc[AX], true) == PG_USERDEF))
    PG_LAUNCH(S, fill_name, (k_avg_transverse<T, C, AX><<<grid_for(nghost), kThreads, 0, S->stream>>>(
                                b, S->cfg.bc[AX], ag)));
}

template <class T, class C>
static void launch_bound_ct(Solver* S, const BoundCT<T>& b, const char* copy_name, const char* fill_name) {
  launch_bound_ct_axis<T, C, 0>(S, b, copy_name, fill_name);
  if (b.g.dims > 1) launch_bound_ct_axis<T, C, 1>(S, b, copy_name, fill_name);
  if (b.g.dims > 2) launch_bound_ct_axis<T, C, 2>(S, b, copy_name, fill_name);
}

}  // namespace pg
