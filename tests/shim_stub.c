/*
 * Host stand-in for libpluto_gb300, for running the PLUTO-side shim
 * (pluto_gb300/shim/gpu_step.c) without a GPU.  TEST INFRASTRUCTURE ONLY.
 *
 * It implements the part of the C ABI (include/pluto_gb300.h) the shim
 * calls, following the ABI's contract -- PG_LAYOUT_PLUTO host arrays with
 * the -1 face layer first, one AdvanceStep per pg_advance with
 * Dts->invDt_hyp handed back, user-defined sides and the internal boundary
 * called back with the state written into the caller's host arrays, .dbl
 * files written by pg_write_output -- on top of the CPU oracle
 * (oracle/mhd_oracle.c), which reproduces the reference bit for bit.  A PLUTO
 * executable linked with the shim and this library therefore writes the
 * reference's own dumps exactly when the shim passes the right arrays,
 * layout, time step and output requests.
 *
 * Every call is also appended to the file named by PG_STUB_LOG (when set):
 *   create dims nx ny nz divb time_stepping precision
 *   upload layout
 *   advance dt inv_dt_hyp max_mach
 *   download layout
 *   output nfile time step
 */
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mhd_oracle.h"
#include "pluto_gb300.h"

struct pg_solver {
  oc_problem *p;
  pg_config cfg;
  int nt[3];
  pg_userdef_fn ud_fn;
  void *ud_user;
  double *ud_vars[8];
  double *ud_faces[3];
  unsigned char *ud_flags;
};

static char s_err[256] = "";

static int stub_fail(int code, const char *msg)
{
  snprintf(s_err, sizeof s_err, "%s", msg);
  return code;
}

static void stub_log(const char *fmt, ...)
{
  const char *path = getenv("PG_STUB_LOG");
  FILE *fp;
  va_list ap;
  if (!path || !(fp = fopen(path, "a"))) return;
  va_start(ap, fmt);
  vfprintf(fp, fmt, ap);
  va_end(ap);
  fputc('\n', fp);
  fclose(fp);
}

static long cell_count(const pg_solver *s) { return (long)s->nt[0] * s->nt[1] * s->nt[2]; }

static long face_count(const pg_solver *s, int d)
{
  return (long)(s->nt[0] + (d == 0)) * (s->nt[1] + (d == 1)) * (s->nt[2] + (d == 2));
}

static int has_faces(const pg_solver *s, int d)
{
  return s->cfg.divb == PG_CONSTRAINED_TRANSPORT && d < s->cfg.dims;
}

const char *pg_last_error(void) { return s_err; }

int pg_create(const pg_config *cfg, pg_solver **out)
{
  oc_config c;
  pg_solver *s;
  int d, ng;
  if (!cfg || !out) return stub_fail(PG_ERR_INVALID, "pg_create: null argument");
  if (cfg->precision != PG_FP64) return stub_fail(PG_ERR_INVALID, "stub: PG_FP64 only");
  memset(&c, 0, sizeof c);
  c.dims = cfg->dims;
  c.components = cfg->components;
  for (d = 0; d < 3; d++) {
    c.nx[d] = cfg->nx[d];
    c.dx[d] = cfg->dx[d];
    c.bc[d] = cfg->bc[d];  /* PG_PERIODIC..PG_USERDEF == OC_PERIODIC..OC_USERDEF */
    c.bc_hi[d] = cfg->bc_sides ? cfg->bc_hi[d] : cfg->bc[d];
  }
  c.gamma = cfg->gamma;
  c.recon = cfg->reconstruction == PG_PARABOLIC ? OC_PARABOLIC : OC_LINEAR;
  c.limiter = cfg->limiter;          /* FLAT, MINMOD, VANLEER, MC, DEFAULT: same order */
  c.solver = cfg->riemann;           /* HLL, HLLD, ROE: same order */
  c.stepping = cfg->time_stepping;   /* EULER..HANCOCK_CONS: same values */
  c.ct = cfg->divb == PG_CONSTRAINED_TRANSPORT;
  c.emf = c.ct ? cfg->emf_average : 0;
  c.char_limiting = cfg->char_limiting;
  c.nthreads = 1;
  s = (pg_solver *)calloc(1, sizeof *s);
  s->p = oc_create(&c);
  if (!s->p) {
    free(s);
    return stub_fail(PG_ERR_INVALID, "stub: the oracle rejected the configuration");
  }
  s->cfg = *cfg;
  ng = cfg->reconstruction == PG_PARABOLIC ? 3 : 2;
  if (IS_CTU(cfg->time_stepping) && c.ct) ng++;
  for (d = 0; d < 3; d++) s->nt[d] = d < cfg->dims ? cfg->nx[d] + 2 * ng : 1;
  stub_log("create %d %d %d %d %d %d %d", cfg->dims, cfg->nx[0], cfg->nx[1], cfg->nx[2], cfg->divb,
           cfg->time_stepping, cfg->precision);
  *out = s;
  return PG_OK;
}

int pg_destroy(pg_solver *s)
{
  if (!s) return PG_OK;
  oc_destroy(s->p);
  free(s);
  return PG_OK;
}

/* host arrays (PLUTO layout) <-> the oracle's own arrays (the same layout) */
static void copy_state(pg_solver *s, double *const vars[8], double *const faces[3], int to_oracle)
{
  double *vc[8], *bs[3];
  int q, d;
  oc_arrays(s->p, vc, bs);
  for (q = 0; q < 8; q++) {
    if (!vars[q]) continue;
    if (to_oracle) memcpy(vc[q], vars[q], sizeof(double) * cell_count(s));
    else memcpy(vars[q], vc[q], sizeof(double) * cell_count(s));
  }
  for (d = 0; d < 3; d++) {
    if (!has_faces(s, d) || !faces || !faces[d]) continue;
    if (to_oracle) memcpy(bs[d], faces[d], sizeof(double) * face_count(s, d));
    else memcpy(faces[d], bs[d], sizeof(double) * face_count(s, d));
  }
}

int pg_upload(pg_solver *s, const double *const vars[8], const double *const faces[3], int layout)
{
  stub_log("upload %d", layout);
  if (layout != PG_LAYOUT_PLUTO) return stub_fail(PG_ERR_INVALID, "stub: PG_LAYOUT_PLUTO expected");
  copy_state(s, (double *const *)vars, (double *const *)faces, 1);
  return PG_OK;
}

int pg_download(pg_solver *s, double *const vars[8], double *const faces[3], int layout)
{
  stub_log("download %d", layout);
  if (layout != PG_LAYOUT_PLUTO) return stub_fail(PG_ERR_INVALID, "stub: PG_LAYOUT_PLUTO expected");
  copy_state(s, vars, faces, 0);
  return PG_OK;
}

int pg_advance(pg_solver *s, double dt, pg_step_info *info)
{
  double inv = 0.0, mach = 0.0;
  int64_t nf = 0;
  if (oc_advance(s->p, dt, &inv, &mach, &nf)) return stub_fail(PG_ERR_NAN, "stub: negative sound speed");
  stub_log("advance %.17g %.17g %.17g", dt, inv, mach);
  if (info) {
    info->inv_dt_hyp = inv;
    info->max_mach = mach;
    info->nfail = nf;
  }
  return PG_OK;
}

/* user-defined sides and the internal boundary: the caller sees the state in
   its host arrays during the call, as the library's contract says */
static void stub_userdef(void *user, int side, int vpos, int stage)
{
  pg_solver *s = (pg_solver *)user;
  unsigned char *fl = oc_flags(s->p);
  copy_state(s, s->ud_vars, s->ud_faces, 0);
  if (s->ud_flags) memcpy(s->ud_flags, fl, (size_t)cell_count(s));
  s->ud_fn(s->ud_user, side, vpos, stage);
  copy_state(s, s->ud_vars, s->ud_faces, 1);
  if (s->ud_flags) memcpy(fl, s->ud_flags, (size_t)cell_count(s));
}

int pg_set_userdef(pg_solver *s, pg_userdef_fn fn, void *user, double *const vars[8], double *const faces[3])
{
  int q;
  if (!s || !fn || !vars) return stub_fail(PG_ERR_INVALID, "pg_set_userdef: null argument");
  s->ud_fn = fn;
  s->ud_user = user;
  for (q = 0; q < 8; q++) s->ud_vars[q] = vars[q];
  for (q = 0; q < 3; q++) s->ud_faces[q] = faces ? faces[q] : NULL;
  oc_set_userdef(s->p, stub_userdef, s);
  stub_log("userdef");
  return PG_OK;
}

int pg_set_internal_boundary(pg_solver *s, unsigned char *flags)
{
  if (!s || !flags || !s->ud_fn) return stub_fail(PG_ERR_INVALID, "pg_set_internal_boundary: call pg_set_userdef first");
  s->ud_flags = flags;
  oc_set_internal(s->p, 1);
  stub_log("internal");
  return PG_OK;
}

/* .dbl files only: each dumped variable's interior, in the request's order */
int pg_write_output(pg_solver *s, const pg_output *o)
{
  const int nx = s->cfg.nx[0], ny = s->cfg.dims > 1 ? s->cfg.nx[1] : 1, nz = s->cfg.dims > 2 ? s->cfg.nx[2] : 1;
  const long ncell = (long)nx * ny * nz;
  double *vc, *bs[3] = {NULL, NULL, NULL};
  char path[4096];
  FILE *fp = NULL;
  int nv, d;
  if (o->format != PG_OUT_DBL) return stub_fail(PG_ERR_INVALID, "stub: .dbl output only");
  vc = (double *)malloc(sizeof(double) * 8 * ncell);
  for (d = 0; d < 3; d++)
    if (has_faces(s, d)) bs[d] = (double *)malloc(sizeof(double) * (ncell / (d == 0 ? nx : d == 1 ? ny : nz)) *
                                                  ((d == 0 ? nx : d == 1 ? ny : nz) + 1));
  oc_get_state(s->p, vc, bs[0], bs[1], bs[2]);
  if (o->single_file) {
    snprintf(path, sizeof path, "%s/data.%04d.dbl", o->dir, o->nfile);
    fp = fopen(path, "wb");
  }
  for (nv = 0; nv < o->nvar; nv++) {
    const double *src;
    long n;
    if (!o->dump[nv]) continue;
    if (o->var[nv] >= 8) {
      d = o->var[nv] - 8;
      src = bs[d];
      n = ncell / (d == 0 ? nx : d == 1 ? ny : nz) * ((d == 0 ? nx : d == 1 ? ny : nz) + 1);
    } else {
      src = vc + (long)o->var[nv] * ncell;
      n = ncell;
    }
    if (!o->single_file) {
      snprintf(path, sizeof path, "%s/%s.%04d.dbl", o->dir, o->name[nv], o->nfile);
      fp = fopen(path, "wb");
    }
    if (fp) fwrite(src, sizeof(double), (size_t)n, fp);
    if (!o->single_file && fp) {
      fclose(fp);
      fp = NULL;
    }
  }
  if (fp) fclose(fp);
  free(vc);
  for (d = 0; d < 3; d++) free(bs[d]);
  stub_log("output %d %.17g %ld", o->nfile, o->time, o->step);
  return PG_OK;
}

int pg_output_wait(pg_solver *s)
{
  (void)s;
  return PG_OK;
}
