#!/usr/bin/env python3
"""Generate the golden fixtures by running the reference PLUTO 4.3 binary.

Run in a container that has the reference tree (``PLUTO_REF``, default
``/root/reference``) and gcc:

    python tests/golden/make_golden.py [name ...]
    python tests/golden/make_golden.py --large [name ...]   # tests/golden/large/

Each fixture ``<name>.npz`` holds the reference's own initial dump (step 0)
and its dump after ``steps`` steps, as written by the reference (``.dbl``,
double precision), plus the problem description.  Variables are stored in the
8-slot order RHO, VX1, VX2, VX3, BX1, BX2, BX3, PRS (two-component problems
get zero VX3/BX3 slots); staggered fields as ``bs0``.. with one extra face
along their own axis.
"""
from __future__ import annotations

import json
import sys
from dataclasses import replace
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle import build_ref as br  # noqa: E402

GOLDEN = Path(__file__).resolve().parent
NAMES = ["rho", "vx1", "vx2", "vx3", "Bx1", "Bx2", "Bx3", "prs"]


def to_arrays(dump: dict, s: br.Setup):
    n = [s.n[d] if d < s.dims else 1 for d in range(3)]
    vc = np.zeros((8, n[2], n[1], n[0]))
    for q, nm in enumerate(NAMES):
        if nm in dump:
            vc[q] = dump[nm]
    bs = {}
    for d in range(s.dims if s.ct else 0):
        bs[f"bs{d}"] = dump[f"Bx{d+1}s"]
    return vc, bs


def spec_of(s: br.Setup) -> dict:
    n = [s.n[d] if d < s.dims else 1 for d in range(3)]
    dx = [(s.hi[d] - s.lo[d]) / n[d] if d < s.dims else 1.0 for d in range(3)]
    gamma = 2.0 if s.name.startswith("tube") else 5.0 / 3.0
    return dict(name=s.name, dims=s.dims, components=s.components, nx=n, dx=dx,
                lo=list(s.lo), hi=list(s.hi), gamma=gamma, recon=s.recon,
                limiter=s.limiter, solver=s.solver, stepping=s.stepping, ct=s.ct, emf=s.emf,
                bc=s.bc, cfl=s.cfl, first_dt=s.first_dt, steps=s.steps,
                internal_boundary=s.internal_boundary,
                char_limiting=s.char_limiting,
                params=s.params)


# UserDefBoundary of the USERDEF fixtures (the same rules, in numpy, are in
# tests/userdef_cases.py): an X1_BEG nozzle -- a fixed inflow state on the
# middle half of the rows, a mirror wall (vx, Bx negated) elsewhere; the
# staggered By and Bz of the side's x2face / x3face boxes likewise -- and an
# X3_END side copied from the last interior plane (cells with vz = 0 and
# p = 0.1, the staggered Bx and By of its boxes).  Every transverse staggered
# component of a side's boxes is set, so nothing depends on ghost values that
# only the initial condition wrote.
USERDEF_C = r"""
  int i, j, k, nv;
  if (side == X1_BEG) {
    if (box->vpos == CENTER) {
      BOX_LOOP(box, k, j, i) {
        if (j >= JBEG + NX2/4 && j < JBEG + (3*NX2)/4) {
          d->Vc[RHO][k][j][i] = 2.0;
          d->Vc[VX1][k][j][i] = 0.5;
          d->Vc[VX2][k][j][i] = 0.0;
          d->Vc[PRS][k][j][i] = 0.3;
          d->Vc[BX1][k][j][i] = 0.2;
          d->Vc[BX2][k][j][i] = 0.1;
#if COMPONENTS == 3
          d->Vc[VX3][k][j][i] = 0.0;
          d->Vc[BX3][k][j][i] = 0.0;
#endif
        } else {
          NVAR_LOOP(nv) d->Vc[nv][k][j][i] = d->Vc[nv][k][j][2*IBEG - 1 - i];
          d->Vc[VX1][k][j][i] = -d->Vc[VX1][k][j][i];
          d->Vc[BX1][k][j][i] = -d->Vc[BX1][k][j][i];
        }
      }
    }
#ifdef STAGGERED_MHD
    else if (box->vpos == X2FACE) {
      BOX_LOOP(box, k, j, i) {
        if (j >= JBEG + NX2/4 && j < JBEG + (3*NX2)/4) d->Vs[BX2s][k][j][i] = 0.1;
        else d->Vs[BX2s][k][j][i] = d->Vs[BX2s][k][j][2*IBEG - 1 - i];
      }
    }
  #if DIMENSIONS == 3
    else if (box->vpos == X3FACE) {
      BOX_LOOP(box, k, j, i) {
        if (j >= JBEG + NX2/4 && j < JBEG + (3*NX2)/4) d->Vs[BX3s][k][j][i] = 0.0;
        else d->Vs[BX3s][k][j][i] = d->Vs[BX3s][k][j][2*IBEG - 1 - i];
      }
    }
  #endif
#endif
  }
#if INTERNAL_BOUNDARY == YES
  if (side == 0) {  /* internal boundary: a dense block that is not updated */
    TOT_LOOP(k, j, i) {
      if (i >= IBEG + NX1/4 && i < IBEG + NX1/4 + 3 && j >= JBEG + NX2/2 - 2 && j < JBEG + NX2/2 + 2) {
        d->Vc[RHO][k][j][i] = 10.0;
        d->Vc[VX1][k][j][i] = 0.0;
        d->Vc[VX2][k][j][i] = 0.0;
        d->Vc[PRS][k][j][i] = 1.0;
        d->flag[k][j][i] |= FLAG_INTERNAL_BOUNDARY;
      }
    }
  }
#endif
#if DIMENSIONS == 3
  if (side == X3_END) {
    if (box->vpos == CENTER) {
      BOX_LOOP(box, k, j, i) {
        NVAR_LOOP(nv) d->Vc[nv][k][j][i] = d->Vc[nv][KEND][j][i];
        d->Vc[VX3][k][j][i] = 0.0;
        d->Vc[PRS][k][j][i] = 0.1;
      }
    }
  #ifdef STAGGERED_MHD
    else if (box->vpos == X1FACE) {
      BOX_LOOP(box, k, j, i) d->Vs[BX1s][k][j][i] = d->Vs[BX1s][KEND][j][i];
    } else if (box->vpos == X2FACE) {
      BOX_LOOP(box, k, j, i) d->Vs[BX2s][k][j][i] = d->Vs[BX2s][KEND][j][i];
    }
  #endif
  }
#endif
"""


def setups():
    out = [
        br.ot_setup("hlld", 32, 30),
        br.ot_setup("hll", 32, 30),
        br.blast_setup(16, 12),
        br.blast_setup(16, 12, pin=1000.0, name="blast_floor_16", bmag=30.0),
        br.tube_setup(0, 256, 100),
        br.tube_setup(1, 200, 120),
        br.tube_setup(2, 160, 80),
        br.cpa_setup(32, 20),
        br.turb_setup(12, 10),
        br.ot_setup("roe", 32, 30),
        replace(br.cpa_setup(32, 20), solver="roe", name="cpa_roe_32"),
        replace(br.blast_setup(16, 12), solver="roe", name="blast_roe_16"),
        replace(br.tube_setup(0, 256, 100), solver="roe", name="tube_roe_0_256"),
        replace(br.ot_setup("hlld", 32, 30), bc="outflow", name="ot_outflow_32"),
        replace(br.turb_setup(12, 10), bc="outflow", name="turb_outflow_12"),
        replace(br.ot_setup("hlld", 32, 30), stepping="HANCOCK", emf="UCT_CONTACT", name="ot_ctu_uctc_32"),
        replace(br.ot_setup("roe", 32, 30), stepping="HANCOCK", emf="ARITHMETIC", name="ot_ctu_arith_roe_32"),
        replace(br.turb_setup(12, 10), recon="LINEAR", stepping="HANCOCK", emf="UCT_CONTACT",
                name="turb_ctu_uctc_12"),
        replace(br.tube_setup(1, 200, 120), stepping="HANCOCK", name="tube_ctu_1_200"),
        replace(br.cpa_setup(32, 20), stepping="HANCOCK", emf="UCT_CONTACT", bc="outflow",
                name="cpa_ctu_outflow_32"),
        replace(br.blast_setup(16, 12), bc="reflective", name="blast_reflective_16"),
        replace(br.ot_setup("hlld", 32, 30), bc="reflective", name="ot_reflective_32"),
        replace(br.cpa_setup(32, 20), bc="eqtsymmetric", name="cpa_eqtsym_32"),
        replace(br.tube_setup(0, 256, 100), bc="reflective", name="tube_reflective_0_256"),
        replace(br.ot_setup("hlld", 32, 30), stepping="HANCOCK", emf="UCT_CONTACT", bc="reflective",
                name="ot_ctu_reflective_32"),
        # a different type on each side of an axis (pluto.ini X*-beg / X*-end)
        replace(br.blast_setup(16, 12), name="blast_sides_16",
                bc=(("reflective", "outflow"), ("outflow", "eqtsymmetric"), ("periodic", "periodic"))),
        replace(br.ot_setup("hlld", 32, 30), name="ot_sides_32",
                bc=(("reflective", "outflow"), ("eqtsymmetric", "reflective"), ("outflow", "outflow"))),
        replace(br.ot_setup("hlld", 32, 30), stepping="HANCOCK", emf="UCT_CONTACT", name="ot_ctu_sides_32",
                bc=(("outflow", "reflective"), ("reflective", "outflow"), ("outflow", "outflow"))),
        replace(br.tube_setup(0, 256, 100), name="tube_sides_0_256",
                bc=(("reflective", "outflow"), ("outflow", "outflow"), ("outflow", "outflow"))),
        # user-defined sides (UserDefBoundary above)
        replace(br.ot_setup("hlld", 32, 30), name="ot_userdef_32", userdef_body=USERDEF_C,
                bc=(("userdef", "outflow"), ("periodic", "periodic"), ("outflow", "outflow"))),
        replace(br.blast_setup(16, 12), name="blast_userdef_16", userdef_body=USERDEF_C, ct=False,
                bc=(("periodic", "periodic"), ("outflow", "outflow"), ("reflective", "userdef"))),
        replace(br.blast_setup(16, 12), name="blast_userdef_ct_16", userdef_body=USERDEF_C,
                bc=(("userdef", "outflow"), ("periodic", "periodic"), ("reflective", "userdef"))),
        # INTERNAL_BOUNDARY (UserDefBoundary with side 0 before every fill)
        replace(br.ot_setup("hlld", 32, 30), name="ot_internal_32", userdef_body=USERDEF_C,
                internal_boundary=True),
        # TIME_STEPPING EULER (the RK predictor alone)
        replace(br.ot_setup("hlld", 32, 10), stepping="EULER", cfl=0.2, name="ot_euler_32"),
        replace(br.tube_setup(0, 256, 60), stepping="EULER", name="tube_euler_0_256"),
        # TIME_STEPPING CHARACTERISTIC_TRACING (CTU with CharTracingStep)
        replace(br.ot_setup("hlld", 32, 30), stepping="CHARACTERISTIC_TRACING", emf="UCT_CONTACT",
                name="ot_chtr_uctc_32"),
        replace(br.ot_setup("roe", 32, 30), stepping="CHARACTERISTIC_TRACING", emf="ARITHMETIC",
                name="ot_chtr_arith_roe_32"),
        replace(br.cpa_setup(32, 20), stepping="CHARACTERISTIC_TRACING", emf="UCT_CONTACT",
                name="cpa_chtr_32"),
        replace(br.turb_setup(12, 10), recon="LINEAR", stepping="CHARACTERISTIC_TRACING",
                emf="UCT_CONTACT", name="turb_chtr_12"),
        replace(br.tube_setup(1, 200, 120), stepping="CHARACTERISTIC_TRACING", name="tube_chtr_1_200"),
        replace(br.blast_setup(16, 12), stepping="CHARACTERISTIC_TRACING", emf="UCT_CONTACT",
                bc="outflow", name="blast_chtr_outflow_16"),
        replace(br.blast_setup(16, 12), stepping="CHARACTERISTIC_TRACING", ct=False, name="blast_chtr_noct_16"),
        replace(br.blast_setup(16, 12), stepping="HANCOCK", ct=False, name="blast_ctu_noct_16"),
        # CHAR_LIMITING YES (limiting in characteristic variables, plm_states.c:446-705)
        replace(br.ot_setup("hlld", 32, 30), char_limiting=True, name="ot_charlim_32"),
        replace(br.blast_setup(16, 12), char_limiting=True, limiter="DEFAULT", name="blast_charlim_default_16"),
        replace(br.tube_setup(1, 200, 120), char_limiting=True, limiter="MINMOD_LIM", name="tube_charlim_1_200"),
        replace(br.cpa_setup(32, 20), char_limiting=True, limiter="VANLEER_LIM", stepping="RK3",
                name="cpa_charlim_rk3_32"),
        replace(br.ot_setup("hlld", 32, 30), char_limiting=True, stepping="CHARACTERISTIC_TRACING",
                emf="UCT_CONTACT", name="ot_chtr_charlim_32"),
        replace(br.blast_setup(16, 12), char_limiting=True, stepping="HANCOCK", emf="ARITHMETIC",
                name="blast_ctu_charlim_16"),
        # PARABOLIC + CHARACTERISTIC_TRACING (CTU-PPM, char_tracing.c:46-279)
        replace(br.ot_setup("hlld", 32, 30), recon="PARABOLIC", stepping="CHARACTERISTIC_TRACING",
                emf="UCT_CONTACT", name="ot_ppm_chtr_32"),
        replace(br.turb_setup(12, 10), stepping="CHARACTERISTIC_TRACING", emf="UCT_CONTACT",
                name="turb_ppm_chtr_12"),
        replace(br.tube_setup(1, 200, 120), recon="PARABOLIC", stepping="CHARACTERISTIC_TRACING",
                name="tube_ppm_chtr_1_200"),
        replace(br.cpa_setup(32, 20), recon="PARABOLIC", stepping="CHARACTERISTIC_TRACING", emf="ARITHMETIC",
                solver="roe", bc="outflow", name="cpa_ppm_chtr_roe_32"),
        replace(br.blast_setup(16, 12), recon="PARABOLIC", stepping="CHARACTERISTIC_TRACING", ct=False,
                name="blast_ppm_chtr_noct_16"),
        # PARABOLIC + CHAR_LIMITING (ppm_states.c:258-560), RK and CTU (reference state 2)
        replace(br.ot_setup("hlld", 32, 30), recon="PARABOLIC", char_limiting=True, name="ot_ppm_charlim_32"),
        replace(br.turb_setup(12, 10), char_limiting=True, name="turb_ppm_charlim_12"),
        replace(br.tube_setup(1, 200, 120), recon="PARABOLIC", char_limiting=True, name="tube_ppm_charlim_1_200"),
        replace(br.ot_setup("hlld", 32, 30), recon="PARABOLIC", char_limiting=True,
                stepping="CHARACTERISTIC_TRACING", emf="UCT_CONTACT", name="ot_ppm_chtr_charlim_32"),
        replace(br.blast_setup(16, 12), recon="PARABOLIC", char_limiting=True, stepping="CHARACTERISTIC_TRACING",
                emf="ARITHMETIC", bc="outflow", name="blast_ppm_chtr_charlim_16"),
        # the other CT_EMF_AVERAGE choices: ARITHMETIC, UCT_CONTACT and UCT0 under RK; UCT0 under CTU
        replace(br.ot_setup("hlld", 32, 30), emf="UCT_CONTACT", name="ot_uctc_32"),
        replace(br.ot_setup("roe", 32, 30), emf="ARITHMETIC", name="ot_arith_roe_32"),
        replace(br.ot_setup("hlld", 32, 30), emf="UCT0", name="ot_uct0_32"),
        replace(br.blast_setup(16, 12), emf="UCT0", name="blast_uct0_16"),
        replace(br.turb_setup(12, 10), emf="UCT_CONTACT", name="turb_uctc_12"),
        replace(br.cpa_setup(32, 20), emf="ARITHMETIC", bc="outflow", name="cpa_arith_outflow_32"),
        replace(br.ot_setup("hlld", 32, 30), stepping="HANCOCK", emf="UCT0", name="ot_ctu_uct0_32"),
        replace(br.blast_setup(16, 12), stepping="CHARACTERISTIC_TRACING", emf="UCT0",
                name="blast_chtr_uct0_16"),
        # TIME_STEPPING HANCOCK with PRIMITIVE_HANCOCK NO (conservative predictor, hancock.c:159-434)
        replace(br.ot_setup("hlld", 32, 30), stepping="HANCOCK_CONS", emf="UCT_CONTACT", name="ot_ctu_cons_32"),
        replace(br.blast_setup(16, 12), stepping="HANCOCK_CONS", emf="ARITHMETIC", name="blast_ctu_cons_16"),
        replace(br.blast_setup(16, 12, pin=1000.0, bmag=30.0), stepping="HANCOCK_CONS", emf="UCT0",
                name="blast_ctu_cons_floor_16"),
        replace(br.tube_setup(1, 200, 120), stepping="HANCOCK_CONS", name="tube_ctu_cons_1_200"),
        replace(br.cpa_setup(32, 20), stepping="HANCOCK_CONS", emf="UCT0", bc="outflow", name="cpa_ctu_cons_32"),
    ]
    for s in out:
        s.first_dt = 1e-3 if not s.name.startswith("tube") else 1e-4
    return out


# ---------------------------------------------------------------------------
# Fixtures at the benchmark configurations' own sizes (tests/golden/large/).
# The final states are too large to commit; each fixture keeps the reference's
# initial dump (it compresses well) and, of the dump after ``steps`` steps,
# the SHA-256 of every variable's bytes (little-endian doubles in the dump's
# order) and of the whole file, with per-variable sums for diagnosis.
# ---------------------------------------------------------------------------
LARGE = GOLDEN / "large"
TUBE_FAMILY = (32, 400)  # the first 32 tubes of the batched family (seed 0), 400 steps each


def large_setups():
    return [
        # 2D Orszag-Tang 256^2, PLM/MC + HLLD + RK2 + CT(UCT_HLL), CFL 0.4, 200 steps
        replace(br.ot_setup("hlld", 256, 200), name="ot_hlld_256_200", first_dt=1e-4),
        # the 3D blast scheme (PLM/MC + HLLD + RK2 + CT, CFL 0.3) at 64^3: the pressure
        # floor fires from step ~16 on
        replace(br.blast_setup(64, 21), name="blast_64_21", first_dt=1e-4),
        # rotated circularly polarised Alfven wave 128^2, 256 steps (the adjoint problem's forward run)
        replace(br.cpa_setup(128, 256), name="cpa_128_256", first_dt=1e-4),
    ]


def _digest(arrays):
    import hashlib
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a, dtype="<f8").tobytes())
    return h.hexdigest()


def large_record(final: dict, names) -> dict:
    import math as _m
    return {"names": list(names), "sha256": _digest([final[nm] for nm in names]),
            "sha256_per_variable": {nm: _digest([final[nm]]) for nm in names},
            "sums": {nm: _m.fsum(final[nm].ravel().tolist()) for nm in names}}


def dump_names(run_dir: Path, index: int = 1):
    rec = [l.split() for l in (run_dir / "dbl.out").read_text().split("\n") if l.strip()]
    return [r for r in rec if int(r[0]) == index][0][6:]


def make_large(only=()):
    import hashlib
    LARGE.mkdir(exist_ok=True)
    for s in large_setups():
        if only and s.name not in only:
            continue
        a, b = br.run(s)
        run_dir = br.OUT / s.name
        names = dump_names(run_dir)
        rec = large_record(b, names)
        assert rec["sha256"] == hashlib.sha256((run_dir / "data.0001.dbl").read_bytes()).hexdigest()
        vc0, bs0 = to_arrays(a, s)
        arrs = {"vc0": vc0}
        arrs.update({k + "_0": v for k, v in bs0.items()})
        meta = spec_of(s)
        meta.update(t_final=b["t"], dt_final=b["dt"], step_final=b["step"], final=rec)
        np.savez_compressed(LARGE / f"{s.name}.npz", meta=json.dumps(meta), **arrs)
        print(f"{s.name}: t={b['t']:.6e} dt={b['dt']:.6e} step={b['step']} sha={rec['sha256'][:16]}")
    name = f"tubes_family0_{TUBE_FAMILY[0]}x{TUBE_FAMILY[1]}"
    if only and name not in only:
        return
    from pluto_gb300.batch import tube_family
    ntubes, steps = TUBE_FAMILY
    _, ns, _, _ = tube_family(4096, 0, 128, 4096)
    ns = ns[:ntubes]
    tubes = [replace(br.tube_setup(t, int(ns[t]), steps), name=f"tubefam_{t}_{int(ns[t])}") for t in range(ntubes)]
    import concurrent.futures as cf
    with cf.ThreadPoolExecutor(8) as ex:
        res = list(ex.map(br.run, tubes))
    v0 = np.concatenate([to_arrays(a, s)[0].reshape(8, -1) for (a, _), s in zip(res, tubes)], axis=1)
    v1 = np.concatenate([to_arrays(b, s)[0].reshape(8, -1) for (_, b), s in zip(res, tubes)], axis=1)
    t1 = np.array([b["t"] for _, b in res])
    dt1 = np.array([b["dt"] for _, b in res])
    meta = spec_of(tubes[0])
    meta.update(name=name, nx_tubes=[int(n) for n in ns], steps=steps, family_seed=0)
    np.savez_compressed(LARGE / f"{name}.npz", meta=json.dumps(meta), v0=v0, v1=v1, t1=t1, dt1=dt1)
    print(f"{name}: {ntubes} tubes, {int(ns.sum())} cells, t in [{t1.min():.4f}, {t1.max():.4f}]")


def main():
    args = sys.argv[1:]
    if args and args[0] == "--large":
        make_large(set(args[1:]))
        return
    only = set(args)  # fixture names to (re)make; all when empty
    for s in setups():
        if only and s.name not in only:
            continue
        a, b = br.run(s)
        vc0, bs0 = to_arrays(a, s)
        vc1, bs1 = to_arrays(b, s)
        arrs = {"vc0": vc0, "vc1": vc1}
        arrs.update({k + "_0": v for k, v in bs0.items()})
        arrs.update({k + "_1": v for k, v in bs1.items()})
        meta = spec_of(s)
        meta.update(t_final=b["t"], dt_final=b["dt"], step_final=b["step"])
        np.savez_compressed(GOLDEN / f"{s.name}.npz", meta=json.dumps(meta), **arrs)
        print(f"{s.name}: t={b['t']:.6e} dt={b['dt']:.6e} step={b['step']}")


if __name__ == "__main__":
    main()
