// FP64 step in double-double arithmetic (PG_FP64_DD): the kernels of the
// plain FP64 path (pg_fp64_kernels.cuh) instantiated with the double-double
// type of pg_dd.cuh, for high-precision reference evaluations (central
// differences that check the adjoint).  RK time stepping only.  Compiled
// without multiply-add contraction.
#include "pg_fp64_kernels.cuh"
#include "pg_dd.cuh"

namespace pg {

int dd_enqueue_step(Solver* S) {
  F64A<DD> a = make_args<DD>(S);
  if (S->cfg.time_stepping == PG_RK3) enqueue_rk<DD, 3>(S, a);
  else if (S->cfg.time_stepping == PG_EULER) enqueue_rk<DD, 1>(S, a);
  else enqueue_rk<DD, 2>(S, a);
  return cudaGetLastError() == cudaSuccess ? PG_OK : PG_ERR_CUDA;
}

}  // namespace pg
