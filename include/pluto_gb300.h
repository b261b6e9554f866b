/*
 * pluto_gb300 -- C ABI of the GB300 implementation of PLUTO 4.3's unsplit
 * finite-volume step for ideal MHD on a uniform Cartesian grid.
 *
 * Plain C types only; every call returns an int status (PG_OK == 0).
 * One solver object owns the device copy of one PLUTO domain (cell-centred
 * primitives Vc, staggered fields Vs) and one CUDA stream.  Not thread safe:
 * like PLUTO's own globals (Src/globals.h), a solver is driven from a single
 * host thread.
 *
 * Reference interfaces replaced (paths inside the PLUTO source tree):
 *   pg_advance       int AdvanceStep(Data*, Riemann_Solver*, timeStep*, Grid*)
 *                    Src/prototypes.h:5, Src/Time_Stepping/rk_step.c:27
 *   pg_run           the step loop of main(), Src/main.c:133-243, with
 *                    NextTimeStep(), Src/main.c:389-575
 *   pg_upload /      the host arrays d->Vc, d->Vs (Src/structs.h:29-88)
 *   pg_download      read and written by AdvanceStep
 *   pg_config        definitions.h scheme macros (Src/pluto.h:300-445,
 *                    Src/MHD/CT/ct.h:43-49) + pluto.ini [Grid]/[Time]
 *                    (Src/runtime_setup.c:22) + SetSolver()
 *                    (Src/MHD/set_solver.c:13-80)
 */
#ifndef PLUTO_GB300_H
#define PLUTO_GB300_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

#define PG_ABI_VERSION 3  /* 2: pg_config gained bc_hi / bc_sides; 3: char_limiting */

/* status codes */
enum {
  PG_OK = 0,
  PG_ERR_INVALID = 1,      /* bad argument or unsupported configuration   */
  PG_ERR_CUDA = 2,         /* CUDA runtime error (message via pg_last_error) */
  PG_ERR_NOMEM = 3,        /* device allocation failed                    */
  PG_ERR_NAN = 4,          /* non-finite state detected                   */
  PG_ERR_DT_TOO_SMALL = 5, /* dt < 1e-9*first_dt, Src/main.c:534-543       */
  PG_ERR_TIMEOUT = 6,      /* a bounded device wait ran out               */
  PG_ERR_TOO_LARGE = 7     /* size beyond a stated maximum                */
};

/* definitions.h / pluto.ini choices */
enum { PG_LINEAR = 0, PG_PARABOLIC = 1 };                         /* RECONSTRUCTION */
enum { PG_FLAT_LIM = 0, PG_MINMOD_LIM = 1, PG_VANLEER_LIM = 2,
       PG_MC_LIM = 3, PG_DEFAULT_LIM = 4 };                       /* LIMITER */
enum { PG_HLL = 0, PG_HLLD = 1, PG_ROE = 2 };                     /* [Solver] */
enum { PG_EULER = 1, PG_RK2 = 2, PG_RK3 = 3,                      /* TIME_STEPPING */
       PG_HANCOCK = 4, PG_CHAR_TRACING = 5, PG_HANCOCK_CONS = 6 };
/* EULER: the RK predictor alone (rk_step.c); HANCOCK: CTU (ctu_step.c) with the
   primitive MUSCL-Hancock predictor; CHAR_TRACING: TIME_STEPPING
   CHARACTERISTIC_TRACING, CTU with the characteristic tracing predictor
   (char_tracing.c, linear reconstruction); HANCOCK_CONS: TIME_STEPPING
   HANCOCK with PRIMITIVE_HANCOCK NO, CTU with the conservative MUSCL-Hancock
   predictor (hancock.c:159-434) */
enum { PG_DIVB_NONE = 0, PG_CONSTRAINED_TRANSPORT = 1 };          /* DIVB_CONTROL */
enum { PG_ARITHMETIC = 1, PG_UCT0 = 2, PG_UCT_CONTACT = 3, PG_UCT_HLL = 4 }; /* CT_EMF_AVERAGE */
enum { PG_PERIODIC = 0, PG_OUTFLOW = 1, PG_REFLECTIVE = 2,
       PG_EQTSYMMETRIC = 3, PG_USERDEF = 4 };                     /* [Boundary] */
/* arithmetic: PG_FP64 bit-compatible with the reference C path;
   PG_MIXED FP32 storage and fluxes, FP64 accumulation / pressure recovery /
   face update / dt reduction; PG_MIXED_DW the same with the FP64 parts done
   as FP32 double-word pairs (48-bit significand) on the FP32 pipes.
   PG_FP64_TANGENT: the FP64 step together with its tangent-linear model
   (each value carries one directional derivative; see pg_tangent_upload).
   PG_FP64_DD: the FP64 step in double-double arithmetic (about 106 bits;
   no reference counterpart), for high-precision reference evaluations such
   as central differences that check the adjoint: pg_upload / pg_download
   move the high parts (the upload zeroes the low parts), pg_tangent_upload /
   pg_tangent_download the low parts.  EULER/RK2/RK3, no user-defined sides,
   no CHAR_LIMITING; no output files or batches. */
enum { PG_FP64 = 0, PG_MIXED = 1, PG_MIXED_DW = 2, PG_FP64_TANGENT = 3, PG_FP64_DD = 4 };
enum { PG_LAYOUT_INTERIOR = 0, PG_LAYOUT_PLUTO = 1 };             /* host array layout */

typedef struct {
  int dims;             /* DIMENSIONS 1..3 */
  int components;       /* COMPONENTS 2 or 3 */
  int nx[3];            /* interior zones per axis (1 on inactive axes) */
  double dx[3];         /* uniform zone widths, grid->dx[d][IBEG] */
  double gamma;         /* g_gamma */
  int reconstruction;
  int limiter;
  int riemann;
  int time_stepping;
  int divb;
  int emf_average;      /* CT_EMF_AVERAGE under CT (Src/MHD/CT/ct_emf.c:210-291):
                           RK takes all four, CTU all but UCT_HLL (ct_emf.c:196-200);
                           ARITHMETIC/UCT0/UCT_CONTACT on PG_FP64 and PG_FP64_TANGENT */
  int bc[3];            /* boundary type per axis (the beginning side, X*_BEG,
                           and the end side too unless bc_sides is 1) */
  int precision;        /* PG_FP64: bit-compatible with the reference C path */
  int compute_mach;     /* 1: also reduce g_maxMach (two extra sqrt per face) */
  double small_density; /* g_smallDensity (0 -> 1e-12) */
  double small_pressure;/* g_smallPressure (0 -> 1e-12) */
  int bc_hi[3];         /* type of the end side (X*_END) when bc_sides is 1 */
  int bc_sides;         /* 0: bc[d] on both sides; 1: bc[d] / bc_hi[d] per side
                           (PERIODIC must then be on both sides of an axis) */
  int char_limiting;    /* CHAR_LIMITING YES: states limited in characteristic
                           variables (Src/States/plm_states.c:446-705,
                           ppm_states.c:258-560); PG_FP64 solvers (RK and CTU) */
} pg_config;

typedef struct {
  double inv_dt_hyp;    /* Dts->invDt_hyp after the step */
  double max_mach;      /* g_maxMach (0 unless compute_mach) */
  int64_t nfail;        /* zones floored by ConsToPrim this step */
} pg_step_info;

typedef struct pg_solver pg_solver;

/* PG_USERDEF sides (PLUTO's UserDefBoundary).  side: 0..5 = X1_BEG, X1_END,
   X2_BEG, X2_END, X3_BEG, X3_END; vpos: 0 the cell box (CENTER), 1..3 the
   box of staggered component 1..3 (X1FACE..X3FACE); stage: 1-based index of
   the boundary fill within the step (g_intStage).  Called on a CUDA host
   thread, in stream order inside the step: it must not call CUDA. */
typedef void (*pg_userdef_fn)(void *user, int side, int vpos, int stage);

/* Create a solver; the device state is zero until pg_upload. */
int pg_create(const pg_config *cfg, pg_solver **out);
int pg_destroy(pg_solver *s);

/* Host <-> device state.  vars[8] point to RHO, VX1, VX2, VX3, BX1, BX2,
   BX3, PRS (NULL for a slot the problem does not have, e.g. VX3/BX3 with
   COMPONENTS 2: zero on upload, skipped on download).  faces[d] point to the
   staggered component d (NULL without CT).
   PG_LAYOUT_INTERIOR: interior zones only, the order of a .dbl dump
     (Src/bin_io.c:216): cells [nz][ny][nx], faces one longer along d.
   PG_LAYOUT_PLUTO: PLUTO's in-memory arrays including ghost zones,
     d->Vc[nv] = [NX3_TOT][NX2_TOT][NX1_TOT] and d->Vs[d] allocated as an
     ArrayBox with index origin -1 along d (Src/initialize.c:448-453); pass
     the pointer to element [-1] (i.e. the start of the allocation).
   pg_upload also clears the sticky error state of earlier steps (a step that
   returned PG_ERR_NAN or PG_ERR_TIMEOUT left invalid results; upload a valid
   state to continue). */
int pg_upload(pg_solver *s, const double *const vars[8], const double *const faces[3],
              int layout);
int pg_download(pg_solver *s, double *const vars[8], double *const faces[3], int layout);

/* One AdvanceStep with time step dt (host value of g_dt).  Blocks until the
   step is complete and fills info (may be NULL).  PG_ERR_TIMEOUT: a bounded
   device-side wait ran out (the mixed paths' TMA tile waits; the environment
   variable PLUTO_GB300_TILE_WAIT_TRIES, read when a step is enqueued, sets
   their try limit -- 0 makes every such wait time out, for testing the
   error path); the kernels return, the context stays usable. */
int pg_advance(pg_solver *s, double dt, pg_step_info *info);

/* The reference main loop for nsteps steps without host round trips:
   dt(0) = first_dt (or the dt carried over from a previous pg_run when
   first_dt <= 0), dt(n+1) = min(cfl/invDt_hyp, cfl_max_var*dt(n)) computed
   on the device.  One CUDA graph per step.  Returns the time advanced and
   the next dt. */
int pg_run(pg_solver *s, int nsteps, double first_dt, double cfl, double cfl_max_var,
           double *t_out, double *next_dt_out);

/* Asynchronous variant of pg_run: enqueues nsteps graph launches on the
   solver's stream and returns; pg_sync waits for them. */
int pg_run_async(pg_solver *s, int nsteps, double first_dt, double cfl, double cfl_max_var);
int pg_sync(pg_solver *s);

/* Timing: run nsteps as in pg_run_async and return the elapsed time between
   two CUDA events recorded on the solver's stream around the launches. */
int pg_run_timed(pg_solver *s, int nsteps, double first_dt, double cfl, double cfl_max_var,
                 double *elapsed_ms);

/* Per-kernel profile of nsteps eagerly launched steps: CUDA events around
   every launch, aggregated per kernel family.  names receives n_kernels
   NUL-terminated strings of name_stride bytes each. */
int pg_profile_kernels(pg_solver *s, int nsteps, double first_dt, double cfl, double cfl_max_var,
                       char *names, int name_stride, double *total_ms, int *launches,
                       int max_kernels, int *n_kernels);

/* ---------------------------------------------------------------------
   Differentiation (no reference counterpart: PLUTO has no adjoint).
   The step is differentiated for a given, frozen dt; the derivative follows
   the limiter, Riemann-solver and floor branches the forward step takes.
   --------------------------------------------------------------------- */
/* PG_FP64_TANGENT solvers: pg_upload sets the state with a zero tangent;
   these set / read the tangent (direction) of the same arrays, same layouts.
   pg_advance then moves state and tangent together. */
int pg_tangent_upload(pg_solver *s, const double *const vars[8], const double *const faces[3],
                      int layout);
int pg_tangent_download(pg_solver *s, double *const vars[8], double *const faces[3], int layout);
/* Kink margin of the tangent-linear step (PG_FP64_TANGENT, no reference
   counterpart): enable = 1 starts recording, enable = 0 stops it and returns
   in *margin the smallest |a - b| / |a' - b'| over every comparison the
   steps made in between (limiter signs, MIN/MAX, Riemann-fan regions,
   floors, |x|), a' the derivative along the uploaded tangent direction: the
   perturbation size along that direction at which, to first order, some
   branch of the computation would switch (+inf: none depends on it). */
int pg_tangent_kink(pg_solver *s, int enable, double *margin);

/* PG_FP64 solvers with EULER/RK2/RK3: adjoint of one step.  pg_adjoint_set loads the
   adjoint (gradient of a scalar with respect to the state after the step)
   into device buffers; pg_adjoint_step(dt) replaces it, on the device, with
   the gradient with respect to the state before a step of length dt taken
   from the solver's current state (which it leaves unchanged);
   pg_adjoint_get reads it back.  Adjoint values on ghost zones are ignored
   on set and zero on get.  Covered: PLM/PPM (no characteristic limiting),
   HLL/HLLD/Roe, constrained transport with the UCT_HLL average, periodic,
   outflow, reflective and equatorial-symmetric sides; PG_ERR_INVALID for
   user-defined sides and the other configurations. */
int pg_adjoint_set(pg_solver *s, const double *const vars[8], const double *const faces[3],
                   int layout);
int pg_adjoint_step(pg_solver *s, double dt);
int pg_adjoint_get(pg_solver *s, double *const vars[8], double *const faces[3], int layout);

/* The same step split in two, for reversing a run of steps without
   recomputing each one twice: pg_adjoint_slots(n) (after pg_adjoint_set)
   allocates n slots (n in 0..PG_MAX_CHECKPOINTS), each holding what one step's forward recomputation
   saves (its start state, stage inputs and results, reconstructed states,
   wave speeds and slopes); PG_ERR_NOMEM, with nothing allocated, when they
   would take more than half of the free device memory; n = 0 frees them.
   pg_adjoint_forward(dt, slot) takes a step of length dt from the solver's
   state, saving into slot, and leaves the solver at the step's end;
   pg_adjoint_reverse(dt, slot) does what pg_adjoint_step does for the step
   saved in slot (the same kernels; like any two runs of the reversal, whose
   scatter adds are FP64 atomics, equal to round-off) and leaves the solver
   at that step's start.  Forward steps q0..q1-1 into slots 0..q1-q0-1, then
   reverse them in the opposite order. */
int pg_adjoint_slots(pg_solver *s, int nslots);
int pg_adjoint_forward(pg_solver *s, double dt, int slot);
int pg_adjoint_reverse(pg_solver *s, double dt, int slot);

/* Device-resident state checkpoints (PG_FP64 / PG_FP64_TANGENT): copy the
   whole state into slot (0..PG_MAX_CHECKPOINTS-1, allocated on first use)
   or back. */
#define PG_MAX_CHECKPOINTS 256
int pg_checkpoint_save(pg_solver *s, int slot);
int pg_checkpoint_load(pg_solver *s, int slot);

/* ---------------------------------------------------------------------
   Batched independent 1D problems ("tubes"), each an independent PLUTO run
   (Src/main.c step loop with its own NextTimeStep dt), all advanced by one
   persistent, CUDA-graph-captured launch.  cfg supplies the scheme (dims 1,
   no constrained transport; PLM minmod/MC or PPM; HLL/HLLD; RK2/RK3;
   PG_FP64 / PG_MIXED / PG_MIXED_DW; nx/dx are taken per tube).
   --------------------------------------------------------------------- */
typedef struct pg_batch pg_batch;
int pg_batch_create(const pg_config *cfg, int ntubes, const int *nx, const double *dx,
                    pg_batch **out);
int pg_batch_destroy(pg_batch *b);
/* vars: the tubes one after the other, each [8][nx_t] interior zones. */
int pg_batch_upload(pg_batch *b, const double *vars);
int pg_batch_download(pg_batch *b, double *vars);
/* nsteps steps of every tube; first_dt > 0 restarts each tube at t = 0;
   cfl <= 0 keeps every tube's dt fixed (no NextTimeStep update). */
int pg_batch_run(pg_batch *b, int nsteps, double first_dt, double cfl, double cfl_max_var,
                 double *elapsed_ms);
int pg_batch_get(pg_batch *b, double *time, double *dt, int64_t *nfail);
/* Schedule autotuner: times trial_steps for each (threads per CTA = warps
   sharing one tube, CTAs per SM) candidate from the same state, tubes queued
   largest first, each candidate twice (the faster time counts); keeps the
   fastest and restores the state.  *best_order is always 1. */
int pg_batch_autotune(pg_batch *b, int trial_steps, double first_dt, double cfl, double cfl_max_var,
                      int *best_threads, int *best_blocks_per_sm, int *best_order, double *best_ms);
/* threads: 32..256, a multiple of 32 (the warps of a CTA share one tube). */
int pg_batch_set_schedule(pg_batch *b, int threads, int blocks_per_sm, int largest_first);

/* Allocation-free variant of one 1D AdvanceStep (no reference counterpart;
   an addition of this library).  For callers that may not allocate device
   memory while they run -- hosts whose own pool allocator owns all device
   memory, real-time loops that cannot take the implicit device
   synchronisation of cudaMalloc/cudaFree.  The step's work arrays live in
   one file-scope device array of about 13.4 MB, held by every GPU that
   loads the library, sized for PG_STATIC_MAX_ZONES zones; larger problems
   return PG_ERR_TOO_LARGE.  cfg: dims 1, no constrained transport, PG_FP64,
   EULER/RK2/RK3 (CTU returns PG_ERR_INVALID), no PG_USERDEF side (returns
   PG_ERR_INVALID).  v_in / v_out: device pointers to the interior state
   [8][nx] (RHO, VX1..3, BX1..3, PRS; may alias).  cuda_stream: cudaStream_t
   or NULL.  Blocks until the step is done (it reads the step's scalars back
   and synchronises the stream).  Calls share the array: calls that overlap
   on the GPU race.  The first call on a device looks up the array's device
   address with that device current and keeps it for the process. */
#define PG_STATIC_MAX_ZONES 32768
int pg_tube_step_static(const pg_config *cfg, const double *v_in, double *v_out, double dt,
                        void *cuda_stream, pg_step_info *info);

/* USERDEF sides: fn is called for every such side at every boundary fill,
   in the reference's order (Src/boundary.c:258-288: the cell box, then each
   staggered box; FillMagneticField follows under CT).  vars[8] / faces[3]
   are the caller's host arrays in PG_LAYOUT_PLUTO (null slots skipped).
   Before the calls for a side the library writes into them the side's slab
   -- its ghost layers and as many interior layers, over the whole transverse
   extent (faces with their -1 layer) -- and after the calls it reads back
   the boxes the reference hands to UserDefBoundary for that side.  The
   arrays must stay valid for the solver's life; arrays the device cannot
   reach are pinned here (cudaHostRegister) and unpinned by pg_destroy.  Not
   for PG_FP64_TANGENT solvers, batches or the adjoint. */
int pg_set_userdef(pg_solver *s, pg_userdef_fn fn, void *user, double *const vars[8], double *const faces[3]);

/* INTERNAL_BOUNDARY YES (Src/boundary.c:90-92): at the start of every
   boundary fill the callback of pg_set_userdef is called with side
   PG_SIDE_INTERNAL (UserDefBoundary with a null box) after the library wrote
   the whole state into its host arrays and the zone flags into flags[]
   (PG_LAYOUT_PLUTO, one byte per zone, cleared at the start of each step as
   Src/main.c:329 does); afterwards it reads the whole state and the flags
   back.  Zones flagged PG_FLAG_INTERNAL_BOUNDARY get a zero right-hand side
   (Src/int_bound_reset.c).  Each fill moves the whole state across the host
   link.  EULER/RK2/RK3 time stepping on the FP64 and mixed paths; call
   pg_set_userdef first. */
#define PG_SIDE_INTERNAL 6
#define PG_FLAG_INTERNAL_BOUNDARY 32  /* Src/pluto.h:197 */
int pg_set_internal_boundary(pg_solver *s, unsigned char *flags);

/* ---- Output files written from the device ----
   Replaces the .dbl / .flt / .vtk branches of WriteData (Src/write_data.c:29-330;
   FileWriteData Src/bin_io.c:216-259, Convert_dbl2flt Src/bin_io.c:51-83,
   WriteVTK_Header / WriteVTK_Vector / WriteVTK_Scalar Src/write_vtk.c) and its
   ".out" record (Src/write_data.c:360-385): the same file names and bytes as a
   serial reference run writes, for the state pg_download returns.
   pg_write_output packs the dumped variables on the device in file order
   (doubles; single precision rounded to nearest; big-endian single precision
   for VTK), copies them to pinned host memory on a separate stream and writes
   the files on a background thread; it returns once the packing is enqueued,
   so the next steps overlap the copy and the file writes.  Outputs complete
   in call order.  pg_output_wait blocks until every pending output is on
   disk and returns the first error met (PG_ERR_INVALID for an I/O error, the
   message via pg_last_error).  pg_destroy waits too.  FP64 and mixed
   precisions; the tangent-linear solver returns PG_ERR_INVALID. */
enum { PG_OUT_DBL = 0, PG_OUT_FLT = 1, PG_OUT_VTK = 2 };
#define PG_OUT_MAX_VARS 16
#define PG_OUT_FACE(d) (8 + (d))   /* var id of the staggered component d (Bx1s..) */
#define PG_OUT_VECTOR 5            /* dump value VTK_VECTOR (Src/pluto.h:97)       */
typedef struct {
  int format;                         /* PG_OUT_DBL / PG_OUT_FLT / PG_OUT_VTK          */
  int single_file;                    /* output->mode "single_file" (else one per var) */
  int nfile;                          /* file number NNNN (after WriteData's ++)       */
  int nvar;                           /* entries below, in output->var order           */
  int var[PG_OUT_MAX_VARS];           /* 0..7: cell slot RHO..PRS; PG_OUT_FACE(d)      */
  int dump[PG_OUT_MAX_VARS];          /* output->dump_var: 0, 1 or PG_OUT_VECTOR       */
  const char *name[PG_OUT_MAX_VARS];  /* output->var_name                              */
  double unit[PG_OUT_MAX_VARS];       /* multiplier for .flt/.vtk (1, or c.g.s units)  */
  const char *dir;                    /* output->dir                                   */
  const double *xnode[3];             /* VTK: grid->xl_glob[d] + BEG, nx+1 entries on
                                         an active axis, 1 otherwise                   */
  double time, dt;                    /* g_time, g_dt for the .out record              */
  long step;                          /* g_stepNumber                                  */
  int write_record;                   /* 1: update dir/<ext>.out                       */
} pg_output;
int pg_write_output(pg_solver *s, const pg_output *out);
int pg_output_wait(pg_solver *s);
/* Asynchronous download (interior layout, as pg_download with
   PG_LAYOUT_INTERIOR): enqueues a device-side snapshot of the state and its
   copy into the caller's host arrays on a second stream, and returns; steps
   enqueued afterwards run while the copy proceeds (pinned host arrays make it
   asynchronous).  pg_download_wait blocks until the arrays hold the
   snapshot; a further pg_download_async first waits for the previous copy.
   The host arrays must not be touched until then.  FP64 and mixed
   precisions. */
int pg_download_async(pg_solver *s, double *const vars[8], double *const faces[3]);
int pg_download_wait(pg_solver *s);

/* Restart from a .dbl written as above (RestartFromFile's data part,
   Src/restart.c:17-150): reads the files named by out (format PG_OUT_DBL;
   dump, var, single_file, nfile, dir; native little-endian doubles) and
   uploads their interior like pg_upload with PG_LAYOUT_INTERIOR: cell slots
   not in the list are set to zero, and under constrained transport every
   staggered component must be listed. */
int pg_read_output(pg_solver *s, const pg_output *out);

/* Diagnostics */
int pg_get_stream(pg_solver *s, void **cuda_stream);
int pg_get_info(pg_solver *s, pg_step_info *info, double *time, double *dt);
int pg_kernel_launches_per_step(pg_solver *s);
const char *pg_last_error(void);
int pg_abi_version(void);

/* Self-test of the integer float<->double conversions the mixed path uses
   in place of the hardware ones (no reference counterpart): counts[0] =
   float bit patterns whose widening differs from the IEEE conversion
   (PTX cvt.f64.f32 without flush-to-zero; all 2^32 checked), counts[1] =
   doubles whose round-to-nearest-even narrowing differs from cvt.rn.f32.f64 (5 * 2^32 near-float and 2^32 wide-exponent patterns,
   ties included).  NaN matches any NaN.  Both are 0 on a correct build.
   Runs on the current device, about a second. */
int pg_selftest_conversions(unsigned long long counts[2]);

#ifdef __cplusplus
}
#endif
#endif
