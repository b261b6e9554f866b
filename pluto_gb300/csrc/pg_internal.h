// Internal solver state shared by the translation units of libpluto_gb300.
#pragma once
#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/pluto_gb300.h"

namespace pg {

// Grid geometry as seen by the kernels: every cell array, and every face
// array, has the same [nt2][nt1][nt0] shape.  Face array d stores the face on
// the +1/2 side of cell (k,j,i) along d at (k,j,i), i.e. the reference index
// of d->Vs[d][k][j][i] (Src/initialize.c:448-453) without its -1 layer.
struct Geom {
  int dims;
  int nt[3];       // total cells per axis (1 on inactive axes)
  int beg[3];      // first interior index (0 on inactive axes)
  int end[3];      // last interior index
  int nx[3];       // interior cells
  // strides in elements: 1, the row pitch P, P*nt1.  P = nt0, except on the
  // mixed path where rows are padded to a multiple of 4 floats (16 bytes, the
  // TMA stride rule); the padding zones are never read or written.
  long long s[3];
  long long ncell;  // elements of one device array: P*nt1*nt2 (host arrays: nt0*nt1*nt2)
  double dx[3], inv_dx[3];
};

__host__ __device__ inline long long cidx(const Geom& g, int k, int j, int i) {
  return (long long)k * g.s[2] + (long long)j * g.s[1] + i;
}

// zones of one host array in PLUTO's ghosted layout (no row padding)
inline long long host_cells(const Geom& g) { return (long long)g.nt[0] * g.nt[1] * g.nt[2]; }

// Inclusive index box.  coords() decodes a linear thread index into (i,j,k);
// after prepare() it divides by the box extents with the multiply-and-shift
// method of Granlund and Montgomery ("Division by invariant integers using
// multiplication", PLDI 1994, sec. 4) on 32-bit indices, so no integer
// division runs on the device (64-bit division is a long instruction
// sequence, and the conversions of the 32-bit one issue on the FP64 pipe).
struct Box {
  int lo[3], hi[3];
  unsigned mi = 0, mj = 0;                  // magic multipliers (0: not prepared)
  unsigned char si1 = 0, si2 = 0, sj1 = 0, sj2 = 0;
  __host__ __device__ long long count() const {
    return (long long)(hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1) * (hi[2] - lo[2] + 1);
  }
  // magic numbers for an unsigned 32-bit division by d >= 1:
  // l = ceil(log2 d), m = floor(2^32 (2^l - d) / d) + 1, n / d =
  // (t + ((n - t) >> min(l, 1))) >> max(l - 1, 0) with t = umulhi(n, m)
  static void magic(unsigned d, unsigned& m, unsigned char& s1, unsigned char& s2) {
    int l = 0;
    while ((1ull << l) < d) l++;
    m = (unsigned)((((1ull << l) - d) << 32) / d + 1);
    s1 = (unsigned char)(l < 1 ? l : 1);
    s2 = (unsigned char)(l > 1 ? l - 1 : 0);
  }
  __host__ Box& prepare() {
    mi = mj = 0;
    if (count() < (1ll << 32)) {
      magic((unsigned)(hi[0] - lo[0] + 1), mi, si1, si2);
      magic((unsigned)(hi[1] - lo[1] + 1), mj, sj1, sj2);
    }
    return *this;
  }
  __host__ __device__ static unsigned fdiv(unsigned n, unsigned m, unsigned s1, unsigned s2) {
#ifdef __CUDA_ARCH__
    const unsigned t = __umulhi(n, m);
#else  // the same on the host (tests/index_decode_check.cu)
    const unsigned t = (unsigned)(((unsigned long long)n * m) >> 32);
#endif
    return (t + ((n - t) >> s1)) >> s2;
  }
  __host__ __device__ void coords(long long q, int& i, int& j, int& k) const {
    int ni = hi[0] - lo[0] + 1, nj = hi[1] - lo[1] + 1;
    if (mi) {  // prepared: 32-bit multiply-and-shift division
      const unsigned u = (unsigned)q;
      const unsigned r = fdiv(u, mi, si1, si2);
      const unsigned p = fdiv(r, mj, sj1, sj2);
      i = lo[0] + (int)(u - r * (unsigned)ni);
      j = lo[1] + (int)(r - p * (unsigned)nj);
      k = lo[2] + (int)p;
      return;
    }
    i = lo[0] + (int)(q % ni);
    q /= ni;
    j = lo[1] + (int)(q % nj);
    k = lo[2] + (int)(q / nj);
  }
};

// Unsigned 32-bit division by a divisor fixed at launch, as multiply-and-shift
// with Box::magic's numbers (no division instruction sequence in the kernel).
struct Div32 {
  unsigned d = 1, m = 1;
  unsigned char s1 = 0, s2 = 0;
  Div32() = default;
  __host__ explicit Div32(unsigned dd) : d(dd) { Box::magic(dd, m, s1, s2); }
  __host__ __device__ unsigned div(unsigned n) const { return Box::fdiv(n, m, s1, s2); }
};

// Thread index -> ghost zone of the single-pass boundary fill: first the x
// ghost columns (2 beg0 per row, every j and k), then the y ghost rows
// (interior i, 2 beg1 per column, every k), then the z ghost planes
// (interior i and j).  32-bit divisions while the count is below 2^32.
struct GhostSlabs {
  long long n0 = 0, n1 = 0, n2 = 0;
  Div32 x_ng2, x_nt1, y_nx0, y_ng2, z_nx0, z_nx1;
  bool wide = false;
  __host__ explicit GhostSlabs(const Geom& g) {
    n0 = g.dims > 0 ? 2LL * g.beg[0] * g.nt[1] * g.nt[2] : 0;
    n1 = g.dims > 1 ? 2LL * g.beg[1] * g.nx[0] * g.nt[2] : 0;
    n2 = g.dims > 2 ? 2LL * g.beg[2] * g.nx[0] * g.nx[1] : 0;
    wide = count() >= (1LL << 32);
    if (g.dims > 0) { x_ng2 = Div32(2u * g.beg[0]); x_nt1 = Div32(g.nt[1]); }
    if (g.dims > 1) { y_nx0 = Div32(g.nx[0]); y_ng2 = Div32(2u * g.beg[1]); }
    if (g.dims > 2) { z_nx0 = Div32(g.nx[0]); z_nx1 = Div32(g.nx[1]); }
  }
  __host__ __device__ long long count() const { return n0 + n1 + n2; }
  // false: q is past the last ghost zone
  __host__ __device__ bool coords(const Geom& g, long long q, int& i, int& j, int& k) const {
    int a, b, c;
    int slab;
    if (q < n0) slab = 0;
    else if (q < n0 + n1) { q -= n0; slab = 1; }
    else if (q < count()) { q -= n0 + n1; slab = 2; }
    else return false;
    // divisors selected by value (a pointer to a parameter would force a
    // local copy of the struct)
    const Div32 da = slab == 0 ? x_ng2 : (slab == 1 ? y_nx0 : z_nx0);
    const Div32 db = slab == 0 ? x_nt1 : (slab == 1 ? y_ng2 : z_nx1);
    if (!wide) {
      const unsigned u = (unsigned)q, r = da.div(u), p = db.div(r);
      a = (int)(u - r * da.d);
      b = (int)(r - p * db.d);
      c = (int)p;
    } else {
      a = (int)(q % da.d);
      const long long r = q / da.d;
      b = (int)(r % db.d);
      c = (int)(r / db.d);
    }
    if (slab == 0) {  // a: ghost column, b = j, c = k
      const int gx = g.beg[0];
      i = a < gx ? a : g.end[0] + 1 + (a - gx);
      j = b;
      k = c;
    } else if (slab == 1) {  // a: interior i, b: ghost row, c = k
      const int gy = g.beg[1];
      i = g.beg[0] + a;
      j = b < gy ? b : g.end[1] + 1 + (b - gy);
      k = c;
    } else {  // a, b: interior i, j, c: ghost plane
      const int gz = g.beg[2];
      i = g.beg[0] + a;
      j = g.beg[1] + b;
      k = c < gz ? c : g.end[2] + 1 + (c - gz);
    }
    return true;
  }
};

// Thread index -> ghost zone of axis AX's layers over the full extent of the
// other axes B1 (faster) and B2: l in [0, 2 beg[AX]) (lower layers first),
// then c1 = the B1 index, c2 = the B2 index.
struct AxisGhosts {
  long long n = 0;  // 2 beg[AX] nt[B1] nt[B2]
  Div32 ng2, nt1;
  bool wide = false;
  __host__ AxisGhosts(const Geom& g, int ax) {
    const int b1 = ax == 0 ? 1 : 0, b2 = ax == 2 ? 1 : 2;
    n = 2LL * g.beg[ax] * g.nt[b1] * g.nt[b2];
    wide = 2 * n >= (1LL << 32);  // k_fill_normal indexes 2 nt[B1] nt[B2] threads
    ng2 = Div32(2u * (g.beg[ax] > 0 ? g.beg[ax] : 1));
    nt1 = Div32(g.nt[b1]);
  }
  __host__ __device__ void coords(long long q, int& l, int& c1, int& c2) const {
    if (!wide) {
      const unsigned u = (unsigned)q, t = ng2.div(u), p = nt1.div(t);
      l = (int)(u - t * ng2.d);
      c1 = (int)(t - p * nt1.d);
      c2 = (int)p;
    } else {
      l = (int)(q % ng2.d);
      const long long t = q / ng2.d;
      c1 = (int)(t % nt1.d);
      c2 = (int)(t / nt1.d);
    }
  }
  // the transverse zone t in [0, nt[B1] nt[B2])
  __host__ __device__ void transverse(long long t, int& c1, int& c2) const {
    if (!wide) {
      const unsigned u = (unsigned)t, p = nt1.div(u);
      c1 = (int)(u - p * nt1.d);
      c2 = (int)p;
    } else {
      c1 = (int)(t % nt1.d);
      c2 = (int)(t / nt1.d);
    }
  }
};

// linear zone index -> (i, j, k) of arrays whose row pitch is nt0 (the FP64
// paths), with the row and plane divisors prepared on the host (32-bit
// divisions while the arrays have fewer than 2^32 zones)
struct CellMap {
  Div32 nt0, nt1;
  bool wide = false;
  CellMap() = default;
  __host__ explicit CellMap(const Geom& g) : nt0(g.nt[0]), nt1(g.nt[1]), wide(g.ncell >= (1LL << 32)) {}
  __host__ __device__ void ijk(long long c, int& i, int& j, int& k) const {
    if (!wide) {
      const unsigned u = (unsigned)c, r = nt0.div(u), p = nt1.div(r);
      i = (int)(u - r * nt0.d);
      j = (int)(r - p * nt1.d);
      k = (int)p;
    } else {
      i = (int)(c % nt0.d);
      j = (int)((c / nt0.d) % nt1.d);
      k = (int)(c / ((long long)nt0.d * nt1.d));
    }
  }
};

// Device scalars of one solver (one allocation).
struct DevScalars {
  double dt;             // time step used by the kernels of the current step
  double dt_prev;        // previous step's dt (for the cfl_max_var cap)
  double time;           // simulated time
  unsigned long long inv_dt_bits;  // running max of invDt (non-negative double bits)
  unsigned long long mach_bits;    // running max of the Mach estimate
  unsigned long long nfail;        // floor events
  int status;                      // sticky device error flags
  int pad;
  float dtdx[3];                   // FP32 dt/dx per axis for the mixed sweeps
  float pad2;
};

// Optional per-launch timing with CUDA events on the solver's stream.
struct Prof {
  std::vector<std::string> names;
  std::vector<cudaEvent_t> ev;  // two events per launch
  size_t used = 0;
};

struct Solver;
void prof_mark(Solver* S, const char* name, bool begin);
#define PG_LAUNCH(S, name, ...)                   \
  do {                                            \
    if ((S)->prof) prof_mark((S), (name), true);  \
    __VA_ARGS__;                                  \
    if ((S)->prof) prof_mark((S), (name), false); \
  } while (0)

int fp64_alloc(Solver* S);
void fp64_free(Solver* S);
int fp64_enqueue_step(Solver* S);  // all stages of one step on S->stream

int tl_enqueue_step(Solver* S);  // PG_FP64_TANGENT: state and tangent
int dd_enqueue_step(Solver* S);  // PG_FP64_DD: the step in double-double
int tl_xfer(Solver* S, double* const vars[8], double* const faces[3], int layout, bool to_dev, int part);
void adjoint_free(Solver* S);      // adjoint buffers, checkpoints, staging

int mixed_alloc(Solver* S);
void mixed_free(Solver* S);
int mixed_enqueue_step(Solver* S);
int mixed_selftest_conversions(unsigned long long counts[2]);
int validate_config(const pg_config* c);
void pack_bc(pg_config* c);
void init_geom(Solver* S);
void set_last_error(const char* msg);
// host <-> device copy of one FP64 array in the interior or PLUTO layout
int xfer_f64(Solver* S, double* dev, double* host, int fd, int layout, bool to_dev);

// arguments of one USERDEF host call (captured into the step graph)
struct UdCall {
  const Solver* S;
  int side, stage, nbfield;
};
constexpr int kUdStages = 4;  // boundary fills per step: RK3 has 3, CTU 1

struct Solver {
  pg_config cfg;
  Geom g;
  int ng;
  cudaStream_t stream = nullptr;
  DevScalars* sc = nullptr;        // device
  DevScalars* sc_host = nullptr;   // pinned mirror
  // FP64 path arrays (NV cell arrays each)
  double* V[8] = {};
  double* U[8] = {};
  double* U0[8] = {};
  double* Bs[3] = {};
  double* Bs0[3] = {};
  double* VP[8] = {};   // reconstructed +1/2 states (per sweep)
  double* VM[8] = {};   // reconstructed -1/2 states
  double* F[8] = {};    // interface fluxes
  double* P = nullptr;  // interface total pressure
  double* CM = nullptr; // interface cmax
  double* SL[3] = {};   // max(0,-SL) per direction
  double* SR[3] = {};   // max(0, SR)
  double* DV[3][3] = {};// velocity slopes DV[dir][comp]
  double* E[3] = {};    // edge EMFs
  double* Bm1[3] = {};  // face -1 layers (boundary scratch for outflow sides under CT)
  // CTU work arrays (TIME_STEPPING HANCOCK)
  double* Upd[3][8] = {};  // predicted conservative +/- states per direction
  double* Umd[3][8] = {};
  double* Rhd[3][8] = {};  // predictor right-hand sides per direction (dt/2)
  double* Uh[8] = {};      // conservative state at the half step
  double* EF[6] = {};      // face EMFs from the fluxes: ezi, ezj, eyi, eyk, exj, exk
  signed char* SV[3] = {}; // sign of the mass flux per face (UCT_CONTACT)
  double* CDT = nullptr;
  unsigned char* flag = nullptr;
  // mixed path
  void* mixed = nullptr;
  // graph of one step
  cudaGraphExec_t graph = nullptr;
  bool graph_dirty = true;
  Prof* prof = nullptr;
  size_t elem_bytes = sizeof(double);  // FP64-path array element size (16 with tangents)
  void* adj = nullptr;     // adjoint buffers (pg_adjoint.cu)
  void* ckpt = nullptr;    // checkpoint slots
  double* stage = nullptr; // FP64 staging array for tangent-solver transfers
  double cfl = 0.4, cfl_max_var = 1.1;
  bool device_dt = false;  // kernels end each step by computing the next dt
  int steps_done = 0;
  // USERDEF sides (pg_set_userdef)
  pg_userdef_fn ud_fn = nullptr;
  void* ud_user = nullptr;
  double* ud_dev_v[8] = {};   // device-usable addresses of the caller's host arrays
  double* ud_dev_f[3] = {};
  void* ud_pinned[11] = {};   // host arrays this library pinned (unpinned by pg_destroy)
  int ud_stage = 0;           // boundary fills enqueued so far in the step
  UdCall ud_calls[kUdStages][7] = {};  // sides 0..5, PG_SIDE_INTERNAL
  bool ud_internal = false;   // INTERNAL_BOUNDARY: a callback with the whole state per fill
  unsigned char* ud_dev_flag = nullptr;  // device-usable address of the caller's flag array
  void* ud_pinned_flag = nullptr;
  void* out = nullptr;        // output staging, copy stream and writer thread (pg_output.cu)
};

void output_free(Solver* S);  // waits for pending outputs, then releases their resources

constexpr int kThreads = 256;
// TIME_STEPPING of the CTU family (ctu_step.c): HANCOCK or CHARACTERISTIC_TRACING
inline bool is_ctu(int time_stepping) {
  return time_stepping == PG_HANCOCK || time_stepping == PG_CHAR_TRACING || time_stepping == PG_HANCOCK_CONS;
}

inline unsigned grid_for(long long n, int threads = kThreads) {
  long long b = (n + threads - 1) / threads;
  return (unsigned)(b < 1 ? 1 : b);
}

}  // namespace pg

// The opaque handle of the C ABI.
struct pg_solver {
  pg::Solver S;
};
