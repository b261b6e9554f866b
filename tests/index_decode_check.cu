// Host check of the index decoding the kernels use (pg_internal.h): the
// multiply-and-shift division Div32 / Box::fdiv against exact division, and
// the thread-index -> zone maps of the boundary fills (GhostSlabs,
// AxisGhosts), of the per-zone kernels (CellMap) and of the domain boxes
// (Box::coords) against the plain 64-bit div/mod formulas they replaced --
// both the 32-bit branch and the 64-bit branch kept for 2^32 zones or more
// (forced here on small grids).  Compiled by nvcc as a host program
// (tests/test_index_decode.py); prints one line per check and exits 1 on the
// first mismatch.
#include <cstdio>
#include <cstdlib>
#include <random>

#include "pg_internal.h"

using pg::AxisGhosts;
using pg::Box;
using pg::CellMap;
using pg::Div32;
using pg::Geom;
using pg::GhostSlabs;

static int fails = 0;
#define CHECK(cond, ...)              \
  do {                                \
    if (!(cond)) {                    \
      printf("FAIL " __VA_ARGS__);    \
      printf("\n");                   \
      if (++fails > 10) exit(1);      \
    }                                 \
  } while (0)

static Geom make_geom(int dims, int nx0, int nx1, int nx2, int ng) {
  Geom g{};
  g.dims = dims;
  const int nx[3] = {nx0, nx1, nx2};
  for (int a = 0; a < 3; a++) {
    const bool act = a < dims;
    g.nx[a] = act ? nx[a] : 1;
    g.beg[a] = act ? ng : 0;
    g.end[a] = g.beg[a] + g.nx[a] - 1;
    g.nt[a] = act ? nx[a] + 2 * ng : 1;
  }
  g.s[0] = 1;
  g.s[1] = g.nt[0];
  g.s[2] = (long long)g.nt[0] * g.nt[1];
  g.ncell = g.s[2] * g.nt[2];
  return g;
}

// the formulas of the single-pass ghost fill before the magic divisions
static void ghost_ref(const Geom& g, long long q, long long n0, long long n1, int& i, int& j, int& k) {
  const int gx = g.beg[0], gy = g.beg[1], gz = g.beg[2];
  if (q < n0) {
    const int ng2 = 2 * gx;
    const int ii = (int)(q % ng2);
    const long long r = q / ng2;
    j = (int)(r % g.nt[1]);
    k = (int)(r / g.nt[1]);
    i = ii < gx ? ii : g.end[0] + 1 + (ii - gx);
  } else if (q < n0 + n1) {
    q -= n0;
    const int ng2 = 2 * gy;
    i = g.beg[0] + (int)(q % g.nx[0]);
    const long long r = q / g.nx[0];
    const int jj = (int)(r % ng2);
    k = (int)(r / ng2);
    j = jj < gy ? jj : g.end[1] + 1 + (jj - gy);
  } else {
    q -= n0 + n1;
    i = g.beg[0] + (int)(q % g.nx[0]);
    const long long r = q / g.nx[0];
    j = g.beg[1] + (int)(r % g.nx[1]);
    const int kk = (int)(r / g.nx[1]);
    k = kk < gz ? kk : g.end[2] + 1 + (kk - gz);
  }
}

int main() {
  // Div32 against exact division
  std::mt19937_64 rng(7);
  long long ndiv = 0;
  for (unsigned d = 1; d <= 5000; d++) {
    const Div32 dv(d);
    const unsigned ns[] = {0u, 1u, d - 1, d, d + 1, 2 * d, 0xffffffffu, 0xfffffffeu, 0x80000000u};
    for (unsigned n : ns) {
      CHECK(dv.div(n) == n / d, "div32 n=%u d=%u", n, d);
      ndiv++;
    }
    for (int r = 0; r < 40; r++) {
      const unsigned n = (unsigned)rng();
      CHECK(dv.div(n) == n / d, "div32 n=%u d=%u", n, d);
      ndiv++;
    }
  }
  for (int r = 0; r < 20000; r++) {
    const unsigned d = 1 + (unsigned)(rng() % 0x7fffffffu), n = (unsigned)rng();
    CHECK(Div32(d).div(n) == n / d, "div32 n=%u d=%u", n, d);
    ndiv++;
  }
  printf("div32 %lld divisions ok\n", ndiv);

  struct G {
    int dims, nx0, nx1, nx2, ng;
  };
  const G geoms[] = {{1, 37, 1, 1, 2}, {1, 5, 1, 1, 4}, {2, 13, 9, 1, 2}, {2, 5, 11, 1, 4}, {2, 1, 7, 1, 3},
                     {3, 7, 5, 6, 3}, {3, 8, 8, 8, 2}, {3, 1, 9, 4, 2}, {3, 11, 3, 2, 4}};
  long long nslab = 0, naxis = 0, ncell = 0, nbox = 0;
  for (const G& gg : geoms) {
    const Geom g = make_geom(gg.dims, gg.nx0, gg.nx1, gg.nx2, gg.ng);
    // ghost slabs, 32-bit and 64-bit branches
    for (int wide = 0; wide < 2; wide++) {
      GhostSlabs gs(g);
      gs.wide = wide;
      for (long long q = 0; q < gs.count(); q++) {
        int i, j, k, ri, rj, rk;
        const bool in = gs.coords(g, q, i, j, k);
        ghost_ref(g, q, gs.n0, gs.n1, ri, rj, rk);
        CHECK(in && i == ri && j == rj && k == rk, "ghost dims=%d wide=%d q=%lld: (%d,%d,%d) vs (%d,%d,%d)", g.dims,
              wide, q, i, j, k, ri, rj, rk);
        nslab++;
      }
      int i, j, k;
      CHECK(!gs.coords(g, gs.count(), i, j, k), "ghost dims=%d: index past the end accepted", g.dims);
    }
    // per-axis ghost layers and transverse lines
    for (int ax = 0; ax < g.dims; ax++) {
      const int b1 = ax == 0 ? 1 : 0;
      for (int wide = 0; wide < 2; wide++) {
        AxisGhosts ag(g, ax);
        ag.wide = wide;
        const int ng2 = 2 * g.beg[ax];
        for (long long q = 0; q < ag.n; q++) {
          int l, c1, c2;
          ag.coords(q, l, c1, c2);
          const long long t = q / ng2;
          CHECK(l == (int)(q % ng2) && c1 == (int)(t % g.nt[b1]) && c2 == (int)(t / g.nt[b1]),
                "axis %d wide=%d q=%lld", ax, wide, q);
          ag.transverse(t, c1, c2);
          CHECK(c1 == (int)(t % g.nt[b1]) && c2 == (int)(t / g.nt[b1]), "transverse %d wide=%d t=%lld", ax, wide, t);
          naxis++;
        }
      }
    }
    // zone index -> (i, j, k)
    for (int wide = 0; wide < 2; wide++) {
      CellMap cm(g);
      cm.wide = wide;
      for (long long c = 0; c < g.ncell; c++) {
        int i, j, k;
        cm.ijk(c, i, j, k);
        CHECK(i == (int)(c % g.nt[0]) && j == (int)((c / g.nt[0]) % g.nt[1]) &&
                  k == (int)(c / ((long long)g.nt[0] * g.nt[1])),
              "cellmap wide=%d c=%lld", wide, c);
        ncell++;
      }
    }
    // boxes: prepared (magic numbers) against unprepared (64-bit div/mod)
    Box b;
    for (int a = 0; a < 3; a++) {
      b.lo[a] = a < g.dims ? g.beg[a] - 1 : 0;
      b.hi[a] = a < g.dims ? g.end[a] : 0;
    }
    Box plain = b;
    b.prepare();
    for (long long q = 0; q < b.count(); q++) {
      int i, j, k, pi, pj, pk;
      b.coords(q, i, j, k);
      plain.coords(q, pi, pj, pk);
      CHECK(i == pi && j == pj && k == pk, "box q=%lld", q);
      nbox++;
    }
  }
  printf("ghost slabs %lld, axis layers %lld, zone maps %lld, box coords %lld ok\n", nslab, naxis, ncell, nbox);
  if (fails) return 1;
  printf("all ok\n");
  return 0;
}
