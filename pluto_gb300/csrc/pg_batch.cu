// Batched 1D problems: host API, CUDA-graph capture of the persistent
// launch, and the schedule autotuner.  FP64 kernel instantiations live here
// (compiled without FMA contraction, bit-compatible with the reference C
// path tube by tube); the mixed ones in pg_batch_mixed.cu.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "pg_batch.cuh"

namespace pg {

// Schemes compiled for the batch: reconstruction x solver x RK stages.
template <class T, class A>
static cudaError_t launch_batch_t(const BatchArgs<T>& b, int rs, int solver, int nstage, int nsteps, int grid,
                                  int threads, cudaStream_t st) {
#define PG_BATCH_CASE(RS_, SOLV_, NST_)                                                                  \
  if (rs == RS_ && solver == SOLV_ && nstage == NST_) {                                                  \
    k_batch<T, A, RS_, SOLV_, NST_><<<grid, threads, 0, st>>>(b, nsteps);                                \
    return cudaGetLastError();                                                                           \
  }
  PG_BATCH_CASE(1, PG_HLLD, 2)
  PG_BATCH_CASE(1, PG_HLLD, 3)
  PG_BATCH_CASE(1, PG_HLL, 2)
  PG_BATCH_CASE(1, PG_HLL, 3)
  PG_BATCH_CASE(0, PG_HLLD, 2)
  PG_BATCH_CASE(0, PG_HLLD, 3)
  PG_BATCH_CASE(0, PG_HLL, 2)
  PG_BATCH_CASE(0, PG_HLL, 3)
  PG_BATCH_CASE(4, PG_HLLD, 2)
  PG_BATCH_CASE(4, PG_HLLD, 3)
  PG_BATCH_CASE(4, PG_HLL, 2)
  PG_BATCH_CASE(4, PG_HLL, 3)
  PG_BATCH_CASE(1, PG_ROE, 2)
  PG_BATCH_CASE(1, PG_ROE, 3)
  PG_BATCH_CASE(0, PG_ROE, 2)
  PG_BATCH_CASE(0, PG_ROE, 3)
  PG_BATCH_CASE(4, PG_ROE, 2)
  PG_BATCH_CASE(4, PG_ROE, 3)
#undef PG_BATCH_CASE
  return cudaErrorInvalidValue;
}

cudaError_t launch_batch_f64(const BatchArgs<double>& b, int rs, int solver, int nstage, int nsteps, int grid,
                             int threads, cudaStream_t st) {
  return launch_batch_t<double, double>(b, rs, solver, nstage, nsteps, grid, threads, st);
}
cudaError_t launch_batch_mixed(const BatchArgs<float>& b, bool dw, int rs, int solver, int nstage, int nsteps,
                               int grid, int threads, cudaStream_t st);
cudaError_t launch_batch_cons_init(const BatchArgs<float>& b, bool dw, cudaStream_t st);

}  // namespace pg

using namespace pg;

struct pg_batch {
  pg_config cfg;
  int ntubes = 0, ng = 2, rs = 1;
  long long total = 0;  // zones including ghosts
  std::vector<int> nx;
  std::vector<long long> off;
  std::vector<double> dx;
  bool f64 = true;
  cudaStream_t stream = nullptr;
  // device
  int *d_order = nullptr, *d_nx = nullptr, *d_cur = nullptr, *d_status = nullptr;
  long long* d_off = nullptr;
  double *d_inv_dx = nullptr, *d_dx = nullptr, *d_dt = nullptr, *d_time = nullptr;
  unsigned long long* d_nfail = nullptr;
  unsigned int* d_counter = nullptr;
  void* V[2][8] = {};
  void* U0[8] = {};  // 8-byte elements (double, or FP32 pairs for PG_MIXED_DW)
  void* U1[8] = {};
  // schedule
  int threads = 128, blocks_per_sm = 4, order_mode = 1;  // 1: largest tube first
  double cfl = 0.8, cfl_max_var = 1.1;
  int graph_nsteps = -1;
  cudaGraphExec_t graph = nullptr;
  int sms = 0;
};

namespace {
thread_local std::string b_err;
int bfail(int code, const char* msg) {
  b_err = msg;
  set_last_error(msg);
  return code;
}
#define BCK(call)                                                      \
  do {                                                                 \
    cudaError_t _e = (call);                                           \
    if (_e != cudaSuccess) return bfail(PG_ERR_CUDA, cudaGetErrorString(_e)); \
  } while (0)

template <class T>
BatchArgs<T> bargs(pg_batch* B) {
  BatchArgs<T> a;
  memset(&a, 0, sizeof a);
  a.ntubes = B->ntubes;
  a.order = B->d_order;
  a.nx = B->d_nx;
  a.off = B->d_off;
  a.inv_dx = B->d_inv_dx;
  a.dxv = B->d_dx;
  for (int s = 0; s < 2; s++)
    for (int nv = 0; nv < 8; nv++) a.V[s][nv] = (T*)B->V[s][nv];
  for (int nv = 0; nv < 8; nv++) {
    a.U0[nv] = B->U0[nv];
    a.U1[nv] = B->U1[nv];
  }
  a.dt = B->d_dt;
  a.time = B->d_time;
  a.nfail = B->d_nfail;
  a.cur = B->d_cur;
  a.status = B->d_status;
  a.counter = B->d_counter;
  a.gamma = B->cfg.gamma;
  a.cfl = B->cfl;
  a.cfl_max_var = B->cfl_max_var;
  a.small_rho = B->cfg.small_density > 0 ? B->cfg.small_density : 1e-12;
  a.small_p = B->cfg.small_pressure > 0 ? B->cfg.small_pressure : 1e-12;
  a.ng = B->ng;
  a.bc = B->cfg.bc[0];
  a.limiter = B->cfg.limiter;
  a.solver = B->cfg.riemann;
  a.ncomp = B->cfg.components;
  return a;
}

int enqueue_batch(pg_batch* B, int nsteps) {
  cudaError_t e = cudaMemsetAsync(B->d_counter, 0, sizeof(unsigned int), B->stream);
  if (e != cudaSuccess) return bfail(PG_ERR_CUDA, cudaGetErrorString(e));
  int grid = std::min(B->ntubes, std::max(1, B->sms * B->blocks_per_sm));
  const int nst = B->cfg.time_stepping == PG_RK3 ? 3 : 2;
  if (B->f64) e = launch_batch_f64(bargs<double>(B), B->rs, B->cfg.riemann, nst, nsteps, grid, B->threads, B->stream);
  else
    e = launch_batch_mixed(bargs<float>(B), B->cfg.precision == PG_MIXED_DW, B->rs, B->cfg.riemann, nst, nsteps,
                           grid, B->threads, B->stream);
  if (e != cudaSuccess) return bfail(PG_ERR_CUDA, cudaGetErrorString(e));
  return PG_OK;
}

// Mixed path: the resident conserved state from the primitives (after an
// upload or a restored snapshot).
int init_conserved(pg_batch* B) {
  if (B->f64) return PG_OK;
  cudaError_t e = launch_batch_cons_init(bargs<float>(B), B->cfg.precision == PG_MIXED_DW, B->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(B->stream);
  if (e != cudaSuccess) return bfail(PG_ERR_CUDA, cudaGetErrorString(e));
  return PG_OK;
}

int set_order(pg_batch* B) {
  std::vector<int> order(B->ntubes);
  std::iota(order.begin(), order.end(), 0);
  if (B->order_mode == 1)
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return B->nx[a] > B->nx[b]; });
  BCK(cudaMemcpy(B->d_order, order.data(), sizeof(int) * B->ntubes, cudaMemcpyHostToDevice));
  return PG_OK;
}

void free_batch(pg_batch* B) {
  auto f = [](void* p) {
    if (p) cudaFree(p);
  };
  if (B->graph) cudaGraphExecDestroy(B->graph);
  f(B->d_order); f(B->d_nx); f(B->d_cur); f(B->d_status); f(B->d_off); f(B->d_inv_dx); f(B->d_dx);
  f(B->d_dt); f(B->d_time); f(B->d_nfail); f(B->d_counter);
  for (int s = 0; s < 2; s++)
    for (int nv = 0; nv < 8; nv++) f(B->V[s][nv]);
  for (int nv = 0; nv < 8; nv++) { f(B->U0[nv]); f(B->U1[nv]); }
  if (B->stream) cudaStreamDestroy(B->stream);
}
}  // namespace

extern "C" int pg_batch_create(const pg_config* cfg, int ntubes, const int* nx, const double* dx, pg_batch** out) {
  if (!cfg || !nx || !dx || !out || ntubes < 1) return bfail(PG_ERR_INVALID, "pg_batch_create: bad argument");
  *out = nullptr;
  pg_config c = *cfg;
  c.nx[0] = 8;
  c.dx[0] = 1.0;
  c.nx[1] = c.nx[2] = 1;
  int rc = validate_config(&c);
  if (rc) return rc;
  if (c.dims != 1 || c.divb != PG_DIVB_NONE) return bfail(PG_ERR_INVALID, "pg_batch_create: 1D problems without CT");
  if (c.precision != PG_FP64 && c.precision != PG_MIXED && c.precision != PG_MIXED_DW)
    return bfail(PG_ERR_INVALID, "pg_batch_create: PG_FP64, PG_MIXED or PG_MIXED_DW");
  if (c.time_stepping != PG_RK2 && c.time_stepping != PG_RK3)
    return bfail(PG_ERR_INVALID, "pg_batch_create: batches take RK2 or RK3 time stepping");
  if (c.bc[0] == PG_USERDEF || (c.bc_sides && c.bc_hi[0] == PG_USERDEF))
    return bfail(PG_ERR_INVALID, "pg_batch_create: user-defined boundaries are not batched");
  if (c.char_limiting) return bfail(PG_ERR_INVALID, "pg_batch_create: CHAR_LIMITING is not batched");
  int rs;
  if (c.reconstruction == PG_PARABOLIC) rs = 4;
  else if (c.limiter == PG_MINMOD_LIM) rs = 1;
  else if (c.limiter == PG_MC_LIM) rs = 0;
  else return bfail(PG_ERR_INVALID, "pg_batch_create: batch supports PLM minmod/MC and PPM");
  pack_bc(&c);
  pg_batch* B = new pg_batch();
  B->cfg = c;
  B->rs = rs;
  B->ntubes = ntubes;
  B->f64 = c.precision == PG_FP64;
  B->ng = c.reconstruction == PG_PARABOLIC ? 3 : 2;
  B->nx.assign(nx, nx + ntubes);
  B->dx.assign(dx, dx + ntubes);
  B->off.resize(ntubes);
  long long o = 0;
  for (int t = 0; t < ntubes; t++) {
    if (nx[t] < 4 || !(dx[t] > 0)) {
      delete B;
      return bfail(PG_ERR_INVALID, "pg_batch_create: tube sizes must be >= 4 and dx > 0");
    }
    B->off[t] = o;
    o += nx[t] + 2 * B->ng;
  }
  B->total = o;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&B->sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t es = B->f64 ? sizeof(double) : sizeof(float);
  auto al = [&](void** p, size_t bytes) { return cudaMalloc(p, bytes) == cudaSuccess; };
  bool ok = cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking) == cudaSuccess;
  ok = ok && al((void**)&B->d_order, sizeof(int) * ntubes) && al((void**)&B->d_nx, sizeof(int) * ntubes) &&
       al((void**)&B->d_cur, sizeof(int) * ntubes) && al((void**)&B->d_status, sizeof(int)) &&
       al((void**)&B->d_off, sizeof(long long) * ntubes) && al((void**)&B->d_inv_dx, sizeof(double) * ntubes) &&
       al((void**)&B->d_dx, sizeof(double) * ntubes) && al((void**)&B->d_dt, sizeof(double) * ntubes) &&
       al((void**)&B->d_time, sizeof(double) * ntubes) &&
       al((void**)&B->d_nfail, sizeof(unsigned long long) * ntubes) && al((void**)&B->d_counter, sizeof(unsigned));
  for (int s = 0; s < 2 && ok; s++)
    for (int nv = 0; nv < 8 && ok; nv++) ok = al(&B->V[s][nv], es * o);
  for (int nv = 0; nv < 8 && ok; nv++) ok = al(&B->U0[nv], 8 * o) && al(&B->U1[nv], 8 * o);
  if (!ok) {
    free_batch(B);
    delete B;
    return bfail(PG_ERR_NOMEM, "pg_batch_create: device allocation failed");
  }
  std::vector<double> inv(ntubes);
  for (int t = 0; t < ntubes; t++) inv[t] = 1.0 / dx[t];  // Src/set_geometry.c:244
  cudaMemcpy(B->d_nx, nx, sizeof(int) * ntubes, cudaMemcpyHostToDevice);
  cudaMemcpy(B->d_off, B->off.data(), sizeof(long long) * ntubes, cudaMemcpyHostToDevice);
  cudaMemcpy(B->d_dx, dx, sizeof(double) * ntubes, cudaMemcpyHostToDevice);
  cudaMemcpy(B->d_inv_dx, inv.data(), sizeof(double) * ntubes, cudaMemcpyHostToDevice);
  cudaMemset(B->d_cur, 0, sizeof(int) * ntubes);
  cudaMemset(B->d_status, 0, sizeof(int));
  cudaMemset(B->d_nfail, 0, sizeof(unsigned long long) * ntubes);
  cudaMemset(B->d_time, 0, sizeof(double) * ntubes);
  cudaMemset(B->d_dt, 0, sizeof(double) * ntubes);
  for (int s = 0; s < 2; s++)
    for (int nv = 0; nv < 8; nv++) cudaMemset(B->V[s][nv], 0, es * o);
  rc = set_order(B);
  if (rc || cudaDeviceSynchronize() != cudaSuccess) {
    free_batch(B);
    delete B;
    return rc ? rc : bfail(PG_ERR_CUDA, "pg_batch_create: CUDA error");
  }
  *out = B;
  return PG_OK;
}

extern "C" int pg_batch_destroy(pg_batch* B) {
  if (!B) return PG_OK;
  free_batch(B);
  delete B;
  return PG_OK;
}

// vars: tubes one after the other, each [8][nx_t] (interior zones).
extern "C" int pg_batch_upload(pg_batch* B, const double* vars) {
  if (!B || !vars) return bfail(PG_ERR_INVALID, "pg_batch_upload: null argument");
  const size_t es = B->f64 ? sizeof(double) : sizeof(float);
  std::vector<char> h(es * B->total, 0);
  std::vector<int> cur(B->ntubes, 0);
  for (int nv = 0; nv < 8; nv++) {
    long long q = 0;
    for (int t = 0; t < B->ntubes; t++) {
      const double* src = vars + q + (long long)nv * B->nx[t];
      long long dst = B->off[t] + B->ng;
      for (int i = 0; i < B->nx[t]; i++) {
        if (B->f64) ((double*)h.data())[dst + i] = src[i];
        else ((float*)h.data())[dst + i] = (float)src[i];
      }
      q += 8LL * B->nx[t];
    }
    BCK(cudaMemcpy(B->V[0][nv], h.data(), es * B->total, cudaMemcpyHostToDevice));
  }
  BCK(cudaMemcpy(B->d_cur, cur.data(), sizeof(int) * B->ntubes, cudaMemcpyHostToDevice));
  BCK(cudaMemset(B->d_nfail, 0, sizeof(unsigned long long) * B->ntubes));
  return init_conserved(B);
}

extern "C" int pg_batch_download(pg_batch* B, double* vars) {
  if (!B || !vars) return bfail(PG_ERR_INVALID, "pg_batch_download: null argument");
  const size_t es = B->f64 ? sizeof(double) : sizeof(float);
  std::vector<int> cur(B->ntubes);
  BCK(cudaMemcpy(cur.data(), B->d_cur, sizeof(int) * B->ntubes, cudaMemcpyDeviceToHost));
  std::vector<char> h0(es * B->total), h1(es * B->total);
  for (int nv = 0; nv < 8; nv++) {
    BCK(cudaMemcpy(h0.data(), B->V[0][nv], es * B->total, cudaMemcpyDeviceToHost));
    BCK(cudaMemcpy(h1.data(), B->V[1][nv], es * B->total, cudaMemcpyDeviceToHost));
    long long q = 0;
    for (int t = 0; t < B->ntubes; t++) {
      const char* h = cur[t] ? h1.data() : h0.data();
      double* dst = vars + q + (long long)nv * B->nx[t];
      long long src = B->off[t] + B->ng;
      for (int i = 0; i < B->nx[t]; i++)
        dst[i] = B->f64 ? ((const double*)h)[src + i] : (double)((const float*)h)[src + i];
      q += 8LL * B->nx[t];
    }
  }
  return PG_OK;
}

// Per-tube time, next dt and floor count after the last run (any may be NULL).
extern "C" int pg_batch_get(pg_batch* B, double* time, double* dt, int64_t* nfail) {
  if (!B) return bfail(PG_ERR_INVALID, "pg_batch_get: null batch");
  if (time) BCK(cudaMemcpy(time, B->d_time, sizeof(double) * B->ntubes, cudaMemcpyDeviceToHost));
  if (dt) BCK(cudaMemcpy(dt, B->d_dt, sizeof(double) * B->ntubes, cudaMemcpyDeviceToHost));
  if (nfail) BCK(cudaMemcpy(nfail, B->d_nfail, sizeof(int64_t) * B->ntubes, cudaMemcpyDeviceToHost));
  return PG_OK;
}

static int batch_prepare(pg_batch* B, int nsteps, double first_dt, double cfl, double cfl_max_var) {
  if (cfl != B->cfl || cfl_max_var != B->cfl_max_var) {
    B->cfl = cfl;
    B->cfl_max_var = cfl_max_var;
    B->graph_nsteps = -1;
  }
  if (first_dt > 0) {
    std::vector<double> v(B->ntubes, first_dt);
    BCK(cudaMemcpy(B->d_dt, v.data(), sizeof(double) * B->ntubes, cudaMemcpyHostToDevice));
    BCK(cudaMemset(B->d_time, 0, sizeof(double) * B->ntubes));
  }
  if (B->graph && B->graph_nsteps == nsteps) return PG_OK;
  if (B->graph) cudaGraphExecDestroy(B->graph);
  B->graph = nullptr;
  cudaGraph_t g;
  BCK(cudaStreamBeginCapture(B->stream, cudaStreamCaptureModeThreadLocal));
  int rc = enqueue_batch(B, nsteps);
  cudaError_t e = cudaStreamEndCapture(B->stream, &g);
  if (rc) return rc;
  if (e != cudaSuccess) return bfail(PG_ERR_CUDA, cudaGetErrorString(e));
  e = cudaGraphInstantiate(&B->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return bfail(PG_ERR_CUDA, cudaGetErrorString(e));
  B->graph_nsteps = nsteps;
  return PG_OK;
}

// Run nsteps steps of every tube (each with its own dt) as one graph launch.
// first_dt > 0 restarts every tube's clock at t = 0 with that dt.
extern "C" int pg_batch_run(pg_batch* B, int nsteps, double first_dt, double cfl, double cfl_max_var,
                            double* elapsed_ms) {
  if (!B || nsteps < 0) return bfail(PG_ERR_INVALID, "pg_batch_run: bad argument");
  int rc = batch_prepare(B, nsteps, first_dt, cfl, cfl_max_var);
  if (rc) return rc;
  cudaEvent_t e0, e1;
  BCK(cudaEventCreate(&e0));
  BCK(cudaEventCreate(&e1));
  BCK(cudaEventRecord(e0, B->stream));
  BCK(cudaGraphLaunch(B->graph, B->stream));
  BCK(cudaEventRecord(e1, B->stream));
  BCK(cudaEventSynchronize(e1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (elapsed_ms) *elapsed_ms = ms;
  int st = 0;
  BCK(cudaMemcpy(&st, B->d_status, sizeof(int), cudaMemcpyDeviceToHost));
  if (st & 2) return bfail(PG_ERR_NAN, "pg_batch_run: Roe solver met a negative sound speed squared");
  if (st) return bfail(PG_ERR_NAN, "pg_batch_run: non-finite dt in a tube");
  return PG_OK;
}

// Autotuner: times trial_steps of the batch for every schedule candidate
// (threads per CTA, i.e. warps per tube team, x CTAs per SM), tubes queued
// largest first, from the same starting state; each candidate runs twice and
// keeps its faster time (the first trial also brings the clocks up), the
// fastest candidate wins and the state is restored.  Every tube runs all
// trial_steps steps, so the trial has the makespan structure of a full run.
// Results: threads, CTAs/SM, order (1 = largest tube first), best time (ms).
extern "C" int pg_batch_autotune(pg_batch* B, int trial_steps, double first_dt, double cfl, double cfl_max_var,
                                 int* best_threads, int* best_blocks_per_sm, int* best_order, double* best_ms) {
  if (!B || trial_steps < 1) return bfail(PG_ERR_INVALID, "pg_batch_autotune: bad argument");
  const size_t es = B->f64 ? sizeof(double) : sizeof(float);
  // snapshot of the state the trials start from
  std::vector<void*> snap(16, nullptr);
  double *dt0 = nullptr, *t0 = nullptr;
  int* cur0 = nullptr;
  for (int s = 0; s < 2; s++)
    for (int nv = 0; nv < 8; nv++) {
      BCK(cudaMalloc(&snap[s * 8 + nv], es * B->total));
      BCK(cudaMemcpy(snap[s * 8 + nv], B->V[s][nv], es * B->total, cudaMemcpyDeviceToDevice));
    }
  BCK(cudaMalloc(&dt0, sizeof(double) * B->ntubes));
  BCK(cudaMalloc(&t0, sizeof(double) * B->ntubes));
  BCK(cudaMalloc(&cur0, sizeof(int) * B->ntubes));
  if (first_dt > 0) {
    std::vector<double> v(B->ntubes, first_dt);
    BCK(cudaMemcpy(B->d_dt, v.data(), sizeof(double) * B->ntubes, cudaMemcpyHostToDevice));
  }
  BCK(cudaMemcpy(dt0, B->d_dt, sizeof(double) * B->ntubes, cudaMemcpyDeviceToDevice));
  BCK(cudaMemcpy(t0, B->d_time, sizeof(double) * B->ntubes, cudaMemcpyDeviceToDevice));
  BCK(cudaMemcpy(cur0, B->d_cur, sizeof(int) * B->ntubes, cudaMemcpyDeviceToDevice));
  auto restore = [&]() -> int {
    for (int s = 0; s < 2; s++)
      for (int nv = 0; nv < 8; nv++)
        BCK(cudaMemcpy(B->V[s][nv], snap[s * 8 + nv], es * B->total, cudaMemcpyDeviceToDevice));
    BCK(cudaMemcpy(B->d_dt, dt0, sizeof(double) * B->ntubes, cudaMemcpyDeviceToDevice));
    BCK(cudaMemcpy(B->d_time, t0, sizeof(double) * B->ntubes, cudaMemcpyDeviceToDevice));
    BCK(cudaMemcpy(B->d_cur, cur0, sizeof(int) * B->ntubes, cudaMemcpyDeviceToDevice));
    return init_conserved(B);
  };
  const int cand_threads[] = {64, 128, 256};
  const int cand_bps[] = {2, 4, 8, 16};
  double best = 1e300;
  int bt = B->threads, bb = B->blocks_per_sm;
  B->order_mode = 1;
  if (set_order(B)) return PG_ERR_CUDA;
  for (int th : cand_threads)
    for (int bps : cand_bps) {
      if (th * bps > 2048) continue;
      B->threads = th;
      B->blocks_per_sm = bps;
      B->graph_nsteps = -1;
      double t_best = 1e300;
      for (int rep = 0; rep < 2; rep++) {
        if (restore()) return PG_ERR_CUDA;
        double ms = 0;
        if (pg_batch_run(B, trial_steps, 0.0, cfl, cfl_max_var, &ms)) break;  // e.g. resource limits
        t_best = ms < t_best ? ms : t_best;
      }
      if (t_best < best) {
        best = t_best;
        bt = th;
        bb = bps;
      }
    }
  B->threads = bt;
  B->blocks_per_sm = bb;
  B->graph_nsteps = -1;
  int rc = restore();
  for (void* p : snap) cudaFree(p);
  cudaFree(dt0);
  cudaFree(t0);
  cudaFree(cur0);
  cudaMemset(B->d_status, 0, sizeof(int));
  if (best_threads) *best_threads = bt;
  if (best_blocks_per_sm) *best_blocks_per_sm = bb;
  if (best_order) *best_order = 1;
  if (best_ms) *best_ms = best;
  return rc;
}

// Fix a schedule explicitly (threads per CTA, CTAs per SM, queue order).
extern "C" int pg_batch_set_schedule(pg_batch* B, int threads, int blocks_per_sm, int order) {
  if (!B || threads < 32 || threads % 32 || threads > 256 || blocks_per_sm < 1)
    return bfail(PG_ERR_INVALID, "pg_batch_set_schedule: bad argument");
  B->threads = threads;
  B->blocks_per_sm = blocks_per_sm;
  B->order_mode = order ? 1 : 0;
  B->graph_nsteps = -1;
  return set_order(B);
}
