// Mixed-precision instantiations of the batched 1D kernel (FP32 storage and
// fluxes; conserved accumulation in FP64 or FP32 double-word pairs).
#include "pg_batch.cuh"

namespace pg {

template <class A>
static cudaError_t launch_mixed_a(const BatchArgs<float>& b, int rs, int solver, int nstage, int nsteps, int grid,
                                  int threads, cudaStream_t st) {
#define PG_BATCH_CASE(RS_, SOLV_, NST_)                                                               \
  if (rs == RS_ && solver == SOLV_ && nstage == NST_) {                                               \
    k_batch<float, A, RS_, SOLV_, NST_><<<grid, threads, 0, st>>>(b, nsteps);                         \
    return cudaGetLastError();                                                                        \
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

cudaError_t launch_batch_cons_init(const BatchArgs<float>& b, bool use_dw, cudaStream_t st) {
  if (use_dw) k_batch_cons_init<pg::dw><<<b.ntubes, 128, 0, st>>>(b);
  else k_batch_cons_init<pg::f64hw><<<b.ntubes, 128, 0, st>>>(b);
  return cudaGetLastError();
}

cudaError_t launch_batch_mixed(const BatchArgs<float>& b, bool use_dw, int rs, int solver, int nstage, int nsteps,
                               int grid, int threads, cudaStream_t st) {
  if (use_dw) return launch_mixed_a<pg::dw>(b, rs, solver, nstage, nsteps, grid, threads, st);
  return launch_mixed_a<pg::f64hw>(b, rs, solver, nstage, nsteps, grid, threads, st);
}

}  // namespace pg
