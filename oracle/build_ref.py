#!/usr/bin/env python3
"""Compile and run the reference PLUTO 4.3 C code on small problems.

Test infrastructure only.  This recipe compiles the reference's own C sources
where they lie (``$PLUTO_REF/Src``, default ``/root/reference``) with plain
``gcc`` -- it does not run the reference's ``setup.py`` or makefile -- into
``oracle/_ref/<setup>/pluto``, then runs each binary for a fixed number of
steps and returns the ``.dbl`` dumps.  The problem setups (``definitions.h``,
``pluto.ini``, ``init.c``) are written by this script; they follow the
reference's user-hook interface (``Src/Templates/init.c:17,65,78,91,110``) and
its runtime file format (``Src/Templates/pluto.ini``).

The object list mirrors what the reference's setup tool links for an
unsplit RK + CT ideal-MHD problem (``Src/Templates/makefile`` base list plus
``Src/MHD/makefile``, ``Src/MHD/CT/makefile``, ``Src/EOS/Ideal/makefile``,
``Src/Math_Tools/makefile``; per-scheme extras chosen as in
``Tools/Python/define_problem.py:509-556``).

Everything is built with ``-O3 -ffp-contract=off`` so that no multiply-add is
fused: the CPU restatement in ``oracle/`` and the FP64 CUDA path follow the
same operation order and therefore the same rounding.

The golden fixtures in ``tests/golden/`` are produced by
``tests/golden/make_golden.py`` which drives this module.
"""
from __future__ import annotations

import concurrent.futures as cf
import math
import os
import shutil
import subprocess
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REF = Path(os.environ.get("PLUTO_REF", "/root/reference"))
OUT = HERE / "_ref"

BASE_SRC = """adv_flux arrays boundary check_states cmd_line_opt entropy_switch
flag_shock flatten get_nghost int_bound_reset input_data mappers3D
mean_mol_weight parse_file plm_coeffs rbox set_indexes set_geometry set_output
tools var_names bin_io colortable initialize jet_domain main output_log
restart runtime_setup set_image show_config set_grid startup split_source
userdef_output write_data write_tab write_img write_vtk write_vtk_proc
math_interp math_lu_decomp math_qr_decomp math_misc math_ode math_quadrature
math_random math_root_finders math_table2D
bckgrnd_field eigenv fluxes get_current hll hllc hlld hll_speed mappers
prim_eqn rhs roe set_solver source tvdlf rhs_source eos
vec_pot_diff vec_pot_update""".split()
CT_SRC = "ct_field_average ct_emf ct_emf_average emf_userdef ct_update ct_fill_mag_field ct_stag_slopes".split()
SRC_DIRS = ["Src", "Src/Time_Stepping", "Src/States", "Src/Math_Tools",
            "Src/MHD", "Src/MHD/CT", "Src/EOS/Ideal"]
INC_DIRS = ["Src", "Src/MHD", "Src/EOS/Ideal", "Src/Math_Tools", "Src/MHD/CT"]


@dataclass
class Setup:
    """One reference problem: compile-time scheme + runtime file + init code."""
    name: str
    dims: int
    components: int
    recon: str = "LINEAR"          # LINEAR | PARABOLIC
    limiter: str = "MC_LIM"
    stepping: str = "RK2"          # EULER | RK2 | RK3 | HANCOCK | CHARACTERISTIC_TRACING | HANCOCK_CONS
    ct: bool = True
    emf: str = "UCT_HLL"
    vecpot: bool = False
    solver: str = "hlld"
    n: tuple = (32, 32, 1)
    lo: tuple = (0.0, 0.0, 0.0)
    hi: tuple = (1.0, 1.0, 1.0)
    bc: object = "periodic"       # one type, or a (beg, end) pair per axis
    cfl: float = 0.4
    first_dt: float = 1e-4
    steps: int = 20
    params: dict = field(default_factory=dict)
    init_body: str = ""
    userdef_body: str = ""          # body of UserDefBoundary (USERDEF sides)
    internal_boundary: bool = False  # INTERNAL_BOUNDARY YES
    dbl_mode: str = "single_file"    # [Static Grid Output] dbl mode
    out_modes: tuple = ()            # extra outputs written at the dbl cadence: ((fmt, mode), ...)
    vtk_vector: bool = False         # VTK_VECTOR_DUMP YES
    char_limiting: bool = False      # CHAR_LIMITING YES
    analysis_body: str = ""          # body of Analysis (called every analysis_every steps)
    analysis_every: int = -1


def _fmt(x: float) -> str:
    return repr(float(x))


def definitions_h(s: Setup) -> str:
    lines = [
        ("PHYSICS", "MHD"), ("DIMENSIONS", s.dims), ("COMPONENTS", s.components),
        ("GEOMETRY", "CARTESIAN"), ("BODY_FORCE", "NO"), ("FORCED_TURB", "NO"),
        ("COOLING", "NO"), ("RECONSTRUCTION", s.recon),
        ("TIME_STEPPING", "HANCOCK" if s.stepping == "HANCOCK_CONS" else s.stepping),
        ("DIMENSIONAL_SPLITTING", "NO"),
        ("NTRACER", 0), ("USER_DEF_PARAMETERS", len(s.params)),
        ("EOS", "IDEAL"), ("ENTROPY_SWITCH", "NO"),
        ("DIVB_CONTROL", "CONSTRAINED_TRANSPORT" if s.ct else "NO"),
        ("BACKGROUND_FIELD", "NO"), ("AMBIPOLAR_DIFFUSION", "NO"),
        ("RESISTIVITY", "NO"), ("HALL_MHD", "NO"),
        ("THERMAL_CONDUCTION", "NO"), ("VISCOSITY", "NO"),
        ("ROTATING_FRAME", "NO"),
    ]
    if s.internal_boundary:
        lines.append(("INTERNAL_BOUNDARY", "YES"))
    if s.vtk_vector:
        lines.append(("VTK_VECTOR_DUMP", "YES"))
    out = [f"#define  {k:<30} {v}" for k, v in lines]
    for idx, key in enumerate(s.params):
        out.append(f"#define  {key:<30} {idx}")
    out.append("/* [Beg] user-defined constants (do not change this line) */")
    out.append(f"#define  LIMITER                        {s.limiter}")
    if s.char_limiting:
        out.append("#define  CHAR_LIMITING                  YES")
    if s.stepping == "HANCOCK_CONS":  # the conservative MUSCL-Hancock predictor (pluto.h:484-495)
        out.append("#define  PRIMITIVE_HANCOCK              NO")
    if s.ct:
        out.append(f"#define  CT_EMF_AVERAGE                 {s.emf}")
        out.append(f"#define  ASSIGN_VECTOR_POTENTIAL        {'YES' if s.vecpot else 'NO'}")
    out.append("/* [End] user-defined constants (do not change this line) */")
    return "\n".join(out) + "\n"


def pluto_ini(s: Setup) -> str:
    g = []
    for d in range(3):
        n = s.n[d] if d < s.dims else 1
        lo = s.lo[d] if d < s.dims else 0.0
        hi = s.hi[d] if d < s.dims else 1.0
        g.append(f"X{d+1}-grid    1    {_fmt(lo)}    {n}    u    {_fmt(hi)}")
    bcs = []
    for d in range(3):
        if d >= s.dims:
            lo = hi = "outflow"
        elif isinstance(s.bc, (list, tuple)):
            lo, hi = s.bc[d]
        else:
            lo = hi = s.bc
        bcs.append(f"X{d+1}-beg        {lo}\nX{d+1}-end        {hi}")
    par = "\n".join(f"{k}    {_fmt(v)}" for k, v in s.params.items())
    extra = {fmt: (str(s.steps), mode) for fmt, mode in s.out_modes}
    return f"""[Grid]

{chr(10).join(g)}

[Chombo Refinement]

Levels           4
Ref_ratio        2 2 2 2 2
Regrid_interval  2 2 2 2
Refine_thresh    0.3
Tag_buffer_size  3
Block_factor     8
Max_grid_size    64
Fill_ratio       0.75

[Time]

CFL              {_fmt(s.cfl)}
CFL_max_var      1.1
tstop            1.0e30
first_dt         {_fmt(s.first_dt)}

[Solver]

Solver         {s.solver}

[Boundary]

{chr(10).join(bcs)}

[Static Grid Output]

uservar    0
dbl       -1.0  {s.steps}   {s.dbl_mode}
flt       -1.0  {extra.get("flt", ("-1", "single_file"))[0]}   {extra.get("flt", ("-1", "single_file"))[1]}
vtk       -1.0  {extra.get("vtk", ("-1", "single_file"))[0]}   {extra.get("vtk", ("-1", "single_file"))[1]}
dbl.h5    -1.0  -1
flt.h5    -1.0  -1
tab       -1.0  -1
ppm       -1.0  -1
png       -1.0  -1
log        100000
analysis  -1.0  {s.analysis_every}

[Chombo HDF5 output]

Checkpoint_interval  -1.0  0
Plot_interval         1.0  0

[Parameters]

{par}
"""


INIT_TEMPLATE = r"""#include "pluto.h"

void Init (double *v, double x1, double x2, double x3)
{
  int nv;
  for (nv = 0; nv < NVAR; nv++) v[nv] = 0.0;
#if PHYSICS == MHD
  v[AX1] = v[AX2] = v[AX3] = 0.0;
#endif
%s
}

void InitDomain (Data *d, Grid *grid) {}
void Analysis (const Data *d, Grid *grid)
{
%s
}
#if PHYSICS == MHD
void BackgroundField (double x1, double x2, double x3, double *B0)
{ B0[0] = B0[1] = B0[2] = 0.0; }
#endif
void UserDefBoundary (const Data *d, RBox *box, int side, Grid *grid)
{
%s
}
"""


def build(s: Setup, jobs: int = 8) -> Path:
    """Compile the reference sources for setup ``s``; return the run dir."""
    if not (REF / "Src" / "main.c").exists():
        raise FileNotFoundError(f"reference tree not found at {REF}")
    run = OUT / s.name
    obj = run / "obj"
    obj.mkdir(parents=True, exist_ok=True)
    (run / "definitions.h").write_text(definitions_h(s))
    (run / "pluto.ini").write_text(pluto_ini(s))
    (run / "init.c").write_text(INIT_TEMPLATE % (s.init_body, s.analysis_body, s.userdef_body))
    names = list(BASE_SRC)
    names += ["plm_states"] if s.recon == "LINEAR" else ["ppm_states", "ppm_coeffs"]
    # time stepping: RK (rk_step + update_stage) or CTU (ctu_step + hancock,
    # or char_tracing for CHARACTERISTIC_TRACING)
    if s.stepping in ("HANCOCK", "HANCOCK_CONS"):
        names += ["ctu_step", "hancock"]
    elif s.stepping == "CHARACTERISTIC_TRACING":
        names += ["ctu_step", "char_tracing"]
    else:
        names += ["rk_step", "update_stage"]
    if s.ct:
        names += CT_SRC
    srcs = [run / "init.c"]
    for nm in names:
        for d in SRC_DIRS:
            p = REF / d / f"{nm}.c"
            if p.exists():
                srcs.append(p)
                break
        else:
            raise FileNotFoundError(nm)
    inc = ["-I", str(run)] + sum((["-I", str(REF / d)] for d in INC_DIRS), [])
    flags = ["-c", "-O3", "-ffp-contract=off", "-w"]

    def cc(src: Path) -> Path:
        o = obj / (src.stem + ".o")
        subprocess.run(["gcc", *flags, *inc, str(src), "-o", str(o)], check=True,
                       capture_output=True)
        return o

    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(cc, srcs))
    subprocess.run(["gcc", *map(str, objs), "-lm", "-o", str(run / "pluto")],
                   check=True, capture_output=True)
    return run


def read_dbl(run: Path, index: int) -> dict:
    """Read ``data.NNNN.dbl`` (single_file) written by the reference.

    Layout per ``Src/write_data.c`` / ``Src/bin_io.c``: each listed variable in
    turn, cell arrays over the interior ``[k][j][i]``, staggered fields with one
    extra face along their own axis; native little-endian doubles.
    """
    lines = (run / "dbl.out").read_text().split("\n")
    rec = [l.split() for l in lines if l.strip()]
    row = [r for r in rec if int(r[0]) == index][0]
    t, dt, step = float(row[1]), float(row[2]), int(row[3])
    names = row[6:]
    ini = (run / "pluto.ini").read_text().split("\n")
    n = [int(l.split()[3]) for l in ini if l.startswith("X") and "-grid" in l]
    raw = np.fromfile(run / f"data.{index:04d}.dbl", dtype="<f8")
    out, off = {"t": t, "dt": dt, "step": step}, 0
    for nm in names:
        shp = [n[2], n[1], n[0]]
        if nm.endswith("s") and nm.startswith("Bx"):
            ax = int(nm[2]) - 1
            shp[2 - ax] += 1
        sz = int(np.prod(shp))
        out[nm] = raw[off:off + sz].reshape(shp).copy()
        off += sz
    assert off == raw.size, (off, raw.size)
    return out


def run(s: Setup) -> tuple:
    """Build, run ``s.steps`` steps, return (initial, final) dumps."""
    d = build(s)
    for f in d.glob("data.*.dbl"):
        f.unlink()
    subprocess.run(["./pluto", "-maxsteps", str(s.steps + 1)], cwd=d, check=True,
                   capture_output=True)
    return read_dbl(d, 0), read_dbl(d, 1)


# --------------------------------------------------------------------------
#  Problem setups (initial conditions written for this project)
# --------------------------------------------------------------------------

OT_INIT = r"""
  double B0 = 1.0/sqrt(4.0*CONST_PI);
  g_gamma = 5.0/3.0;
  v[RHO] = 25.0/(36.0*CONST_PI);
  v[PRS] = 5.0/(12.0*CONST_PI);
  v[VX1] = -sin(2.0*CONST_PI*x2);
  v[VX2] =  sin(2.0*CONST_PI*x1);
  v[BX1] = -B0*sin(2.0*CONST_PI*x2);
  v[BX2] =  B0*sin(4.0*CONST_PI*x1);
  v[AX3] =  B0*(cos(2.0*CONST_PI*x2)/(2.0*CONST_PI) + cos(4.0*CONST_PI*x1)/(4.0*CONST_PI));
"""

BLAST_INIT = r"""
  double r = sqrt(x1*x1 + x2*x2 + x3*x3);
  double r0 = g_inputParam[P_R0], dr = g_inputParam[P_DR];
  double b = g_inputParam[P_BMAG]/sqrt(3.0);
  g_gamma = 5.0/3.0;
  v[RHO] = 1.0;
  if (r < r0) v[PRS] = g_inputParam[P_PIN];
  else if (r < r0 + dr) v[PRS] = g_inputParam[P_PIN]
                                  + (g_inputParam[P_POUT] - g_inputParam[P_PIN])*(r - r0)/dr;
  else v[PRS] = g_inputParam[P_POUT];
  v[BX1] = v[BX2] = v[BX3] = b;
"""

TUBE_INIT = r"""
  g_gamma = 2.0;
  if (x1 < 0.5) {
    v[RHO] = g_inputParam[P_RL]; v[PRS] = g_inputParam[P_PL];
    v[VX1] = g_inputParam[P_UL]; v[VX2] = g_inputParam[P_VL]; v[VX3] = g_inputParam[P_WL];
    v[BX2] = g_inputParam[P_BYL]; v[BX3] = g_inputParam[P_BZL];
  } else {
    v[RHO] = g_inputParam[P_RR]; v[PRS] = g_inputParam[P_PR];
    v[VX1] = g_inputParam[P_UR]; v[VX2] = g_inputParam[P_VR]; v[VX3] = g_inputParam[P_WR];
    v[BX2] = g_inputParam[P_BYR]; v[BX3] = g_inputParam[P_BZR];
  }
  v[BX1] = g_inputParam[P_BX];
"""

CPA_INIT = r"""
  double ca = cos(g_inputParam[P_ALPHA]), sa = sin(g_inputParam[P_ALPHA]);
  double lam = g_inputParam[P_LAMBDA], eps = g_inputParam[P_EPS];
  double xpar = x1*ca + x2*sa, xperp = -x1*sa + x2*ca;
  double phi = 2.0*CONST_PI*xpar/lam;
  double bperp = eps*sin(phi), vperp = eps*sin(phi);
  g_gamma = 5.0/3.0;
  v[RHO] = 1.0;
  v[PRS] = 0.1;
  v[VX1] = -vperp*sa;
  v[VX2] =  vperp*ca;
  v[VX3] =  eps*cos(phi);
  v[BX1] = ca - bperp*sa;
  v[BX2] = sa + bperp*ca;
  v[BX3] = eps*cos(phi);
  v[AX3] = xperp + eps*lam/(2.0*CONST_PI)*cos(phi);
"""

TURB_INIT = r"""
  double tp = 2.0*CONST_PI;
  g_gamma = 5.0/3.0;
  v[RHO] = 1.0 + 0.1*sin(tp*(x1 + 2.0*x3));
  v[PRS] = 1.0;
  v[VX1] = 0.6*sin(tp*x2 + 0.3) + 0.2*cos(tp*2.0*x3 + 1.1);
  v[VX2] = 0.6*sin(tp*x3 + 0.7) + 0.2*cos(tp*2.0*x1 + 0.4);
  v[VX3] = 0.6*sin(tp*x1 + 1.9) + 0.2*cos(tp*2.0*x2 + 2.3);
  v[AX1] = 0.05*sin(tp*x2 + 0.2) + 0.02*cos(tp*(x3 + x2));
  v[AX2] = 0.05*sin(tp*x3 + 1.2) + 0.02*cos(tp*(x1 + x3));
  v[AX3] = 0.05*sin(tp*x1 + 2.2) + 0.02*cos(tp*(x2 + x1));
"""


def ot_setup(solver="hlld", n=32, steps=20):
    return Setup(name=f"ot_{solver}_{n}", dims=2, components=2, solver=solver,
                 n=(n, n, 1), vecpot=True, cfl=0.4, steps=steps, init_body=OT_INIT)


def blast_setup(n=16, steps=10, pin=10.0, name=None, bmag=10.0):
    dx = 1.0 / n
    return Setup(name=name or f"blast_{n}", dims=3, components=3, n=(n, n, n),
                 lo=(-0.5, -0.5, -0.5), hi=(0.5, 0.5, 0.5), cfl=0.3, steps=steps,
                 params={"P_R0": 0.1, "P_DR": 2 * dx, "P_PIN": pin, "P_POUT": 0.1,
                         "P_BMAG": bmag / math.sqrt(4 * math.pi)},
                 init_body=BLAST_INIT)


def tube_setup(seed=0, n=256, steps=100):
    rng = np.random.default_rng(seed)
    lu = lambda a, b: float(np.exp(rng.uniform(np.log(a), np.log(b))))
    p = {"P_BX": float(rng.uniform(0.25, 1.0))}
    for side in "LR":
        p["P_R" + side] = lu(0.1, 1.0)
        p["P_P" + side] = lu(0.05, 1.0)
        p["P_U" + side] = float(rng.uniform(-1, 1))
        p["P_V" + side] = float(rng.uniform(-1, 1))
        p["P_W" + side] = float(rng.uniform(-1, 1))
        p["P_BY" + side] = float(rng.uniform(-1, 1))
        p["P_BZ" + side] = float(rng.uniform(-1, 1))
    return Setup(name=f"tube_{seed}_{n}", dims=1, components=3, ct=False,
                 limiter="MINMOD_LIM", n=(n, 1, 1), bc="outflow", cfl=0.8,
                 first_dt=1e-4, steps=steps, params=p, init_body=TUBE_INIT)


def cpa_setup(n=32, steps=20):
    alpha = math.pi / 6.0
    ly = 1.0 / math.tan(alpha)
    return Setup(name=f"cpa_{n}", dims=2, components=3, n=(n, n, 1),
                 hi=(1.0, ly, 1.0), vecpot=True, cfl=0.4, steps=steps,
                 params={"P_ALPHA": alpha, "P_LAMBDA": math.cos(alpha), "P_EPS": 0.1},
                 init_body=CPA_INIT)


def turb_setup(n=12, steps=10):
    return Setup(name=f"turb_{n}", dims=3, components=3, recon="PARABOLIC",
                 stepping="RK3", n=(n, n, n), vecpot=True, cfl=0.3, steps=steps,
                 init_body=TURB_INIT)


if __name__ == "__main__":
    import sys
    s = ot_setup()
    a, b = run(s)
    print(sorted(a), a["t"], b["t"], b["dt"], b["step"])
