/* ///////////////////////////////////////////////////////////////////// */
/*!
  \file
  \brief GB300 replacement for PLUTO's unsplit AdvanceStep() (RK and CTU).

  Link this object instead of rk_step.o and update_stage.o (the objects the
  setup tool lists for an unsplit RK scheme; ctu_step.o for CTU) and add
  -lpluto_gb300 -lcudart.
  It defines the same symbol PLUTO's Integrate() calls,

      int AdvanceStep (Data *d, Riemann_Solver *Riemann,
                       timeStep *Dts, Grid *grid)      (Src/prototypes.h:5)

  and forwards the step to libpluto_gb300 through its C ABI
  (include/pluto_gb300.h).  The scheme is read from the same definitions.h
  macros the reference uses, the Riemann solver from the function pointer
  SetSolver() returned (Src/MHD/set_solver.c:40-47).

  Device residency: the state lives on the GPU between steps.  It is
  uploaded on the first call and whenever the environment variable
  PLUTO_GPU_UPLOAD_EVERY says so (e.g. after a restart or when init code
  changed d->Vc).  The host copy d->Vc / d->Vs is refreshed on demand by the
  two readers of it between steps in Src/main.c, both defined here:
    WriteData   (Src/write_data.c:29): .dbl, .flt and .vtk files are written
                from the device by pg_write_output (asynchronously: the next
                steps overlap the copy and the file writes); every other
                format, user-defined output variables and anything the
                device writer does not take download the state first and
                call the reference's writer, compiled as pg_host_WriteData;
    Analysis    (the problem's init.c, compiled as pg_user_Analysis):
                downloads the state first.
  Makefile.gpu renames the two reference definitions (-DWriteData=... on
  write_data.o, -DAnalysis=... on init.o).  PLUTO_GPU_SYNC_EVERY=n > 0
  also downloads after every n-th step (the former behaviour).
  Pending output files are complete when the program exits (atexit).

  Errors: a non-zero status from the library is fatal, as the reference's
  own fatal conditions are (QUIT_PLUTO).
*/
/* ///////////////////////////////////////////////////////////////////// */
#include <stdlib.h>
#include <string.h>

#include "pluto.h"
#include "pluto_gb300.h"

/* the reference definitions these wrap (renamed by Makefile.gpu) */
void pg_host_WriteData (const Data *, Output *, Grid *);
void pg_user_Analysis (const Data *, Grid *);

static pg_solver *s_gpu = NULL;
static long s_calls = 0;
static int s_host_stale = 0;  /* d->Vc / d->Vs older than the device state */
static Data *s_data = NULL;   /* for UserDefBoundary on USERDEF sides */
static Grid *s_grid = NULL;

static int gpu_riemann(Riemann_Solver *R)
{
  if (R == HLL_Solver)  return PG_HLL;
  if (R == HLLD_Solver) return PG_HLLD;
  if (R == Roe_Solver)  return PG_ROE;
  return -1;
}

static int gpu_bc(int t)
{
  if (t == PERIODIC) return PG_PERIODIC;
  if (t == OUTFLOW)  return PG_OUTFLOW;
  if (t == REFLECTIVE)   return PG_REFLECTIVE;
  if (t == EQTSYMMETRIC) return PG_EQTSYMMETRIC;
  if (t == USERDEF)      return PG_USERDEF;
  return -1;
}

static void gpu_config(pg_config *c, Riemann_Solver *Riemann, Grid *grid)
{
  int d;
  const char *prec = getenv("PLUTO_GPU_PRECISION");

  memset(c, 0, sizeof *c);
  c->dims       = DIMENSIONS;
  c->components = COMPONENTS;
  for (d = 0; d < 3; d++) {
    c->nx[d] = d < DIMENSIONS ? grid->np_int[d] : 1;
    c->dx[d] = d < DIMENSIONS ? grid->dx[d][grid->nghost[d]] : 1.0;
    c->bc[d]    = d < DIMENSIONS ? gpu_bc(grid->lbound[d]) : PG_PERIODIC;
    c->bc_hi[d] = d < DIMENSIONS ? gpu_bc(grid->rbound[d]) : PG_PERIODIC;
    if (c->bc_hi[d] != c->bc[d]) c->bc_sides = 1;
  }
  c->gamma = g_gamma;
#if RECONSTRUCTION == PARABOLIC
  c->reconstruction = PG_PARABOLIC;
#else
  c->reconstruction = PG_LINEAR;
#endif
#if LIMITER == MC_LIM
  c->limiter = PG_MC_LIM;
#elif LIMITER == MINMOD_LIM
  c->limiter = PG_MINMOD_LIM;
#elif LIMITER == VANLEER_LIM
  c->limiter = PG_VANLEER_LIM;
#elif LIMITER == FLAT_LIM
  c->limiter = PG_FLAT_LIM;
#else
  c->limiter = PG_DEFAULT_LIM;
#endif
  c->riemann = gpu_riemann(Riemann);
#if CHAR_LIMITING == YES
  c->char_limiting = 1;
#endif
#if TIME_STEPPING == RK3
  c->time_stepping = PG_RK3;
#elif TIME_STEPPING == EULER
  c->time_stepping = PG_EULER;
#elif TIME_STEPPING == HANCOCK && PRIMITIVE_HANCOCK == NO
  c->time_stepping = PG_HANCOCK_CONS;
#elif TIME_STEPPING == HANCOCK
  c->time_stepping = PG_HANCOCK;
#elif TIME_STEPPING == CHARACTERISTIC_TRACING
  c->time_stepping = PG_CHAR_TRACING;
#else
  c->time_stepping = PG_RK2;
#endif
#ifdef STAGGERED_MHD
  c->divb = PG_CONSTRAINED_TRANSPORT;
  #if CT_EMF_AVERAGE == ARITHMETIC
  c->emf_average = PG_ARITHMETIC;
  #elif CT_EMF_AVERAGE == UCT_CONTACT
  c->emf_average = PG_UCT_CONTACT;
  #elif CT_EMF_AVERAGE == UCT0
  c->emf_average = PG_UCT0;
  #else
  c->emf_average = PG_UCT_HLL;
  #endif
#else
  c->divb = PG_DIVB_NONE;
#endif
  c->precision = PG_FP64;
  if (prec && !strcmp(prec, "mixed"))    c->precision = PG_MIXED;
  if (prec && !strcmp(prec, "mixed_dw")) c->precision = PG_MIXED_DW;
  c->compute_mach = 1;
  c->small_density  = g_smallDensity;
  c->small_pressure = g_smallPressure;
}

/* Pointers to PLUTO's host arrays in the 8-slot order of the C ABI. */
static void gpu_host_arrays(Data *d, double *vars[8], double *faces[3])
{
  int q;
  for (q = 0; q < 8; q++) vars[q] = NULL;
  faces[0] = faces[1] = faces[2] = NULL;
  vars[0] = d->Vc[RHO][0][0];
  EXPAND(vars[1] = d->Vc[VX1][0][0];  ,
         vars[2] = d->Vc[VX2][0][0];  ,
         vars[3] = d->Vc[VX3][0][0];)
  EXPAND(vars[4] = d->Vc[BX1][0][0];  ,
         vars[5] = d->Vc[BX2][0][0];  ,
         vars[6] = d->Vc[BX3][0][0];)
  vars[7] = d->Vc[PRS][0][0];
#ifdef STAGGERED_MHD
  /* ArrayBox storage is contiguous; pass the first element (index -1
     along the staggered axis), Src/initialize.c:448-453. */
  D_EXPAND(faces[0] = &d->Vs[BX1s][0][0][-1];  ,
           faces[1] = &d->Vs[BX2s][0][-1][0];  ,
           faces[2] = &d->Vs[BX3s][-1][0][0];)
#endif
}

/* USERDEF sides: the library calls this, in stream order inside the step,
   for every such side at every boundary fill, after writing the side's slab
   into d->Vc / d->Vs; it hands UserDefBoundary the box the reference builds
   for that side and variable position (Src/boundary.c:144-164, 279-283). */
static void gpu_userdef(void *user, int side, int vpos, int stage)
{
  static const int sides[6] = {X1_BEG, X1_END, X2_BEG, X2_END, X3_BEG, X3_END};
  int ib = 0, ie = NX1_TOT - 1, jb = 0, je = NX2_TOT - 1, kb = 0, ke = NX3_TOT - 1;
  RBox box;

  (void)user;
  g_intStage = stage;
  if (side == PG_SIDE_INTERNAL) {  /* INTERNAL_BOUNDARY, Src/boundary.c:90-92 */
    UserDefBoundary (s_data, NULL, 0, s_grid);
    return;
  }
  if      (side == 0) {ib = IBEG - 1; ie = 0;}
  else if (side == 1) {ib = IEND + 1; ie = NX1_TOT - 1;}
  else if (side == 2) {jb = JBEG - 1; je = 0;}
  else if (side == 3) {jb = JEND + 1; je = NX2_TOT - 1;}
  else if (side == 4) {kb = KBEG - 1; ke = 0;}
  else                {kb = KEND + 1; ke = NX3_TOT - 1;}
  if (vpos == 0) RBoxDefine (ib, ie, jb, je, kb, ke, CENTER, &box);
  else if (vpos == 1) {
    if (ib < ie) RBoxDefine (ib-1, ie, jb, je, kb, ke, X1FACE, &box);
    else         RBoxDefine (ib, ie-1, jb, je, kb, ke, X1FACE, &box);
  } else if (vpos == 2) {
    if (jb < je) RBoxDefine (ib, ie, jb-1, je, kb, ke, X2FACE, &box);
    else         RBoxDefine (ib, ie, jb, je-1, kb, ke, X2FACE, &box);
  } else {
    if (kb < ke) RBoxDefine (ib, ie, jb, je, kb-1, ke, X3FACE, &box);
    else         RBoxDefine (ib, ie, jb, je, kb, ke-1, X3FACE, &box);
  }
  g_intStage = stage;
  UserDefBoundary (s_data, &box, sides[side], s_grid);
}

static void gpu_check(int rc, const char *where)
{
  if (rc != PG_OK) {
    print ("! AdvanceStep (GPU): %s failed (%d): %s\n", where, rc, pg_last_error());
    QUIT_PLUTO(1);
  }
}

/* Refresh d->Vc / d->Vs from the device when a step made them stale. */
static void gpu_sync_host(const Data *d)
{
  double *vars[8], *faces[3];
  if (s_gpu == NULL || !s_host_stale) return;
  gpu_host_arrays((Data *)d, vars, faces);
  gpu_check(pg_download(s_gpu, vars, faces, PG_LAYOUT_PLUTO), "pg_download");
  s_host_stale = 0;
}

static void gpu_atexit(void)
{
  if (s_gpu == NULL) return;
  if (pg_output_wait(s_gpu) != PG_OK)
    print ("! WriteData (GPU): %s\n", pg_last_error());
  pg_destroy(s_gpu);
  s_gpu = NULL;
}

/* The output request for pg_write_output, or 0 when the device writer does
   not take this output (the reference's writer then runs on host data). */
static int gpu_output_spec(const Data *d, Output *output, Grid *grid, pg_output *o)
{
  int nv, q, slot[NVAR];
  static double units[MAX_OUTPUT_VARS];

  if (output->type != DBL_OUTPUT && output->type != FLT_OUTPUT && output->type != VTK_OUTPUT) return 0;
  if (d->Vuser != NULL || output->nvar > PG_OUT_MAX_VARS) return 0;
  for (q = 0; q < NVAR; q++) slot[q] = -1;
  slot[RHO] = 0;
  EXPAND(slot[VX1] = 1;  , slot[VX2] = 2;  , slot[VX3] = 3;)
  EXPAND(slot[BX1] = 4;  , slot[BX2] = 5;  , slot[BX3] = 6;)
  slot[PRS] = 7;
  memset(o, 0, sizeof *o);
  o->format = output->type == DBL_OUTPUT ? PG_OUT_DBL : (output->type == FLT_OUTPUT ? PG_OUT_FLT : PG_OUT_VTK);
  o->single_file = strcmp(output->mode, "single_file") == 0;
  o->nvar = output->nvar;
  for (nv = 0; nv < MAX_OUTPUT_VARS; nv++) units[nv] = 1.0;
  if (output->cgs) GetCGSUnits(units);
  for (nv = 0; nv < output->nvar; nv++) {
    int id = -1;
    for (q = 0; q < NVAR; q++)
      if (output->V[nv] == d->Vc[q]) id = slot[q];
  #ifdef STAGGERED_MHD
    for (q = 0; q < DIMENSIONS; q++)
      if (output->V[nv] == d->Vs[q]) id = 8 + q;
  #endif
    o->dump[nv] = output->dump_var[nv];
    o->var[nv]  = id < 0 ? 0 : id;
    o->name[nv] = output->var_name[nv];
    o->unit[nv] = units[nv];
    if (o->dump[nv] && (id < 0 || (id >= 8 && output->type != DBL_OUTPUT))) return 0;
  }
  o->dir = output->dir;
  o->xnode[0] = grid->xl_glob[IDIR] + IBEG;
  o->xnode[1] = grid->xl_glob[JDIR] + JBEG;
  o->xnode[2] = grid->xl_glob[KDIR] + KBEG;
  o->time = g_time;
  o->dt   = g_dt;
  o->step = g_stepNumber;
  o->write_record = (prank == 0);
  return 1;
}

/* ********************************************************************* */
void WriteData (const Data *d, Output *output, Grid *grid)
/*!
 * WriteData (Src/write_data.c:29) with the .dbl, .flt and .vtk files
 * written from the device copy of the state.
 *********************************************************************** */
{
  pg_output o;
  if (s_gpu != NULL && gpu_output_spec(d, output, grid, &o)) {
    output->nfile++;
    print ("> Writing file #%d (%s) to disk...", output->nfile, output->ext);
    o.nfile = output->nfile;
    gpu_check(pg_write_output(s_gpu, &o), "pg_write_output");
    print ("\n");
    return;
  }
  gpu_sync_host(d);
  pg_host_WriteData(d, output, grid);
}

/* ********************************************************************* */
void Analysis (const Data *d, Grid *grid)
/*!
 * The problem's Analysis() (compiled as pg_user_Analysis) on current host
 * data.
 *********************************************************************** */
{
  gpu_sync_host(d);
  pg_user_Analysis(d, grid);
}

/* ********************************************************************* */
int AdvanceStep (Data *d, Riemann_Solver *Riemann, timeStep *Dts, Grid *grid)
/*!
 * Advance the solution by one unsplit RK step on the GPU.
 *
 * \param [in,out]      d  pointer to Data structure
 * \param [in]    Riemann  pointer to a Riemann solver function
 * \param [in,out]    Dts  pointer to time step structure
 * \param [in]       grid  pointer to Grid structure
 *********************************************************************** */
{
  double *vars[8], *faces[3];
  pg_step_info info;
  const char *env;
  long up_every = 0, sync_every = 0;

  if ((env = getenv("PLUTO_GPU_UPLOAD_EVERY")) != NULL) up_every = atol(env);
  if ((env = getenv("PLUTO_GPU_SYNC_EVERY")) != NULL)   sync_every = atol(env);
  if (sync_every < 0) sync_every = 0;
  /* a re-upload pushes the host copy: keep it current for host-side edits */
  if (up_every > 0 && sync_every == 0) sync_every = up_every;

  gpu_host_arrays(d, vars, faces);
  s_data = d;
  s_grid = grid;
  if (s_gpu == NULL) {
    pg_config cfg;
    int dd, ud = 0;
    gpu_config(&cfg, Riemann, grid);
    gpu_check(pg_create(&cfg, &s_gpu), "pg_create");
    atexit(gpu_atexit);
    for (dd = 0; dd < DIMENSIONS; dd++)
      ud |= grid->lbound[dd] == USERDEF || grid->rbound[dd] == USERDEF;
  #if INTERNAL_BOUNDARY == YES
    ud = 1;
  #endif
    if (ud) gpu_check(pg_set_userdef(s_gpu, gpu_userdef, NULL, vars, faces), "pg_set_userdef");
  #if INTERNAL_BOUNDARY == YES
    gpu_check(pg_set_internal_boundary(s_gpu, d->flag[0][0]), "pg_set_internal_boundary");
  #endif
    gpu_check(pg_upload(s_gpu, (const double *const *)vars, (const double *const *)faces,
                        PG_LAYOUT_PLUTO), "pg_upload");
  } else if (up_every > 0 && s_calls % up_every == 0) {
    gpu_check(pg_upload(s_gpu, (const double *const *)vars, (const double *const *)faces,
                        PG_LAYOUT_PLUTO), "pg_upload");
  }

  gpu_check(pg_advance(s_gpu, g_dt, &info), "pg_advance");
  s_calls++;

/* -- the quantities NextTimeStep() and the log read (Src/main.c:389-575) -- */

  Dts->invDt_hyp = MAX(Dts->invDt_hyp, info.inv_dt_hyp);
  g_maxMach      = MAX(g_maxMach, info.max_mach);

  s_host_stale = 1;
  if (sync_every > 0 && s_calls % sync_every == 0) gpu_sync_host(d);
  return 0;
}
