/*
 * CPU oracle for the unsplit ideal-MHD finite-volume step of PLUTO 4.3.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithm (Src/Time_Stepping/rk_step.c, update_stage.c, the Src/States,
 * Src/MHD and Src/MHD/CT directories), written so that every floating-point operation
 * happens in the reference's order.  Built with -ffp-contract=off it agrees
 * bit for bit with the reference binary on the golden problems.  Only the
 * test suite, the smoke check and the CPU-baseline leg of the benchmark use
 * it; the product (libpluto_gb300.so) never links or calls it.
 *
 * State layout (interior only, the layout of a PLUTO .dbl dump):
 *   vc : 8 primitive variables [RHO,VX1,VX2,VX3,BX1,BX2,BX3,PRS][nz][ny][nx]
 *        (two-component problems carry zero VX3/BX3),
 *   bs : staggered fields, bs[d] of shape [nz+(d==2)][ny+(d==1)][nx+(d==0)],
 *        face index 0 is the left face of the first interior cell.
 */
#ifndef MHD_ORACLE_H
#define MHD_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

enum { OC_RHO = 0, OC_VX1, OC_VX2, OC_VX3, OC_BX1, OC_BX2, OC_BX3, OC_PRS, OC_NVAR };
enum { OC_LINEAR = 0, OC_PARABOLIC = 1 };
enum { OC_FLAT_LIM = 0, OC_MINMOD_LIM, OC_VANLEER_LIM, OC_MC_LIM, OC_DEFAULT_LIM };
enum { OC_HLL = 0, OC_HLLD = 1, OC_ROE = 2 };
enum { OC_EULER = 1, OC_RK2 = 2, OC_RK3 = 3, OC_HANCOCK = 4, OC_CHARTR = 5, OC_HANCOCK_CONS = 6 };
/* OC_HANCOCK_CONS: CTU with the conservative Hancock predictor (PRIMITIVE_HANCOCK NO) */
/* OC_CHARTR: CTU with CharTracingStep (TIME_STEPPING CHARACTERISTIC_TRACING,
   LINEAR reconstruction) */
#define IS_CTU(s) ((s) == OC_HANCOCK || (s) == OC_CHARTR || (s) == OC_HANCOCK_CONS) /* HANCOCK: CTU with the primitive Hancock predictor */
enum { OC_ARITHMETIC = 1, OC_UCT0 = 2, OC_UCT_CONTACT = 3, OC_UCT_HLL = 4 }; /* CT_EMF_AVERAGE, Src/MHD/CT/ct.h:17-21 */
enum { OC_PERIODIC = 0, OC_OUTFLOW = 1, OC_REFLECTIVE = 2, OC_EQTSYMMETRIC = 3, OC_USERDEF = 4 };

/* USERDEF sides: called in Boundary's order with side 0..5 (X1_BEG..X3_END),
   vpos 0 (cell box) then 1..3 (staggered boxes, under CT), stage = index of
   the boundary fill within the step; writes the problem's own arrays. */
typedef void (*oc_userdef_fn)(void *user, int side, int vpos, int stage);

typedef struct {
  int dims;            /* DIMENSIONS 1..3 */
  int components;      /* COMPONENTS 2 or 3 */
  int nx[3];           /* interior cells (1 for inactive dims) */
  double dx[3];        /* uniform spacing */
  double gamma;
  int recon, limiter, solver, stepping;
  int ct;              /* 1: constrained transport (EMF average in emf) */
  int bc[3];           /* boundary type per dim, beginning side (X*-beg) */
  int nthreads;        /* OpenMP threads (0: runtime default) */
  int emf;             /* CT_EMF_AVERAGE (0 = UCT_HLL) */
  int bc_hi[3];        /* end side (X*-end) */
  int char_limiting;   /* CHAR_LIMITING YES (LINEAR reconstruction) */
} oc_config;

typedef struct oc_problem oc_problem;

oc_problem *oc_create(const oc_config *cfg);
void oc_set_userdef(oc_problem *p, oc_userdef_fn fn, void *user);
/* the problem's own arrays in PLUTO's layout: vc[8] ghosted cell arrays,
   bs[3] face arrays (one longer along their axis, -1 layer first) */
void oc_arrays(oc_problem *p, double **vc, double **bs);
/* INTERNAL_BOUNDARY: the userdef callback also runs with side 6 at the start
   of every boundary fill; zones flagged FLAG_INTERNAL_BOUNDARY (32) in the
   flag array (oc_flags, PLUTO layout, cleared every step) are not updated. */
void oc_set_internal(oc_problem *p, int on);
unsigned char *oc_flags(oc_problem *p);
void oc_destroy(oc_problem *p);
void oc_set_state(oc_problem *p, const double *vc, const double *bs0,
                  const double *bs1, const double *bs2);
void oc_get_state(const oc_problem *p, double *vc, double *bs0, double *bs1,
                  double *bs2);
/* One AdvanceStep with time step dt (returns 0; 1 when the Roe solver met a
   negative sound speed squared, where the reference stops); gives invDt_hyp (pre-division by
   DIMENSIONS already applied as in the reference) and the floor count. */
int oc_advance(oc_problem *p, double dt, double *inv_dt_hyp, double *max_mach,
               int64_t *nfail);
/* The reference main loop for nsteps steps: dt(0) = first_dt,
   dt(n+1) = min(cfl/invDt_hyp, cfl_max_var*dt(n)).  dts receives each dt. */
int oc_run(oc_problem *p, int nsteps, double first_dt, double cfl,
           double cfl_max_var, double *dts, double *t_final);

#ifdef __cplusplus
}
#endif
#endif
