"""Host-side mirror of PLUTO's AdvanceStep interface over the C ABI.

A problem is described with the names PLUTO uses in ``definitions.h`` and
``pluto.ini`` (Src/pluto.h:300-445, Src/Templates/pluto.ini):

    spec = dict(dims=2, components=2, nx=(256, 256, 1), dx=(1/256, 1/256, 1.0),
                gamma=5/3, recon="LINEAR", limiter="MC_LIM", solver="hlld",
                stepping="RK2", ct=True, bc="periodic")

``Solver.advance(dt)`` is one AdvanceStep (Src/Time_Stepping/rk_step.c:27);
``Solver.run(n, first_dt, cfl)`` is n passes of the main loop with
NextTimeStep (Src/main.c:133-243, 389-575) kept on the device.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L

RECON = {"LINEAR": L.PG_LINEAR, "PARABOLIC": L.PG_PARABOLIC}
LIMITER = {"FLAT_LIM": L.PG_FLAT_LIM, "MINMOD_LIM": L.PG_MINMOD_LIM,
           "VANLEER_LIM": L.PG_VANLEER_LIM, "MC_LIM": L.PG_MC_LIM, "DEFAULT": L.PG_DEFAULT_LIM}
RIEMANN = {"hll": L.PG_HLL, "hlld": L.PG_HLLD, "roe": L.PG_ROE}
STEPPING = {"EULER": L.PG_EULER, "RK2": L.PG_RK2, "RK3": L.PG_RK3, "HANCOCK": L.PG_HANCOCK,
            "CHARACTERISTIC_TRACING": L.PG_CHAR_TRACING, "HANCOCK_CONS": L.PG_HANCOCK_CONS}
CTU_STEPPING = ("HANCOCK", "CHARACTERISTIC_TRACING", "HANCOCK_CONS")
EMF = {"ARITHMETIC": L.PG_ARITHMETIC, "UCT0": L.PG_UCT0, "UCT_CONTACT": L.PG_UCT_CONTACT,
       "UCT_HLL": L.PG_UCT_HLL}
BC = {"periodic": L.PG_PERIODIC, "outflow": L.PG_OUTFLOW, "reflective": L.PG_REFLECTIVE,
      "eqtsymmetric": L.PG_EQTSYMMETRIC, "userdef": L.PG_USERDEF}
PRECISION = {"fp64": L.PG_FP64, "mixed": L.PG_MIXED, "mixed_dw": L.PG_MIXED_DW,
             "fp64_tangent": L.PG_FP64_TANGENT, "fp64_dd": L.PG_FP64_DD}
NVAR = 8


def make_config(spec: dict, precision: str = "fp64", compute_mach: bool = False) -> L.PgConfig:
    c = L.PgConfig()
    c.dims = int(spec["dims"])
    c.components = int(spec["components"])
    for d in range(3):
        c.nx[d] = int(spec["nx"][d]) if d < c.dims else 1
        c.dx[d] = float(spec["dx"][d]) if d < c.dims else 1.0
        # "bc": one type for every side, one per axis, or a (beg, end) pair per axis
        bc = spec.get("bc", "periodic")
        t = bc[d] if isinstance(bc, (list, tuple)) else bc
        lo, hi = (t[0], t[1]) if isinstance(t, (list, tuple)) else (t, t)
        c.bc[d] = BC[lo]
        c.bc_hi[d] = BC[hi]
        if lo != hi:
            c.bc_sides = 1
    c.gamma = float(spec["gamma"])
    c.reconstruction = RECON[spec.get("recon", "LINEAR")]
    c.limiter = LIMITER[spec.get("limiter", "MC_LIM")]
    c.riemann = RIEMANN[spec.get("solver", "hlld")]
    c.time_stepping = STEPPING[spec.get("stepping", "RK2")]
    c.divb = L.PG_CONSTRAINED_TRANSPORT if spec.get("ct", True) else L.PG_DIVB_NONE
    c.emf_average = EMF[spec.get("emf", "UCT_HLL")]
    c.char_limiting = int(bool(spec.get("char_limiting", False)))
    c.precision = PRECISION[precision]
    c.compute_mach = int(bool(compute_mach))
    c.small_density = 1e-12
    c.small_pressure = 1e-12
    return c


# SetDefaultVarNames (Src/var_names.c) names of the 8 slots
OUTPUT_NAMES = ["rho", "vx1", "vx2", "vx3", "Bx1", "Bx2", "Bx3", "prs"]


def _ptrs(arrs, n):
    P = C.POINTER(C.c_double)
    out = (P * n)()
    for q, a in enumerate(arrs):
        out[q] = a.ctypes.data_as(P) if a is not None else None
    return out


class Solver:
    """One PLUTO domain resident on the GPU."""

    def __init__(self, spec: dict, precision: str = "fp64", compute_mach: bool = False):
        self.spec = dict(spec)
        self.precision = precision
        self.cfg = make_config(spec, precision, compute_mach)
        self.dims = self.cfg.dims
        self.ct = self.cfg.divb == L.PG_CONSTRAINED_TRANSPORT
        self.nx = tuple(self.cfg.nx[d] for d in range(3))
        h = C.c_void_p()
        L.check(L.lib().pg_create(C.byref(self.cfg), C.byref(h)), "pg_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            L.lib().pg_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def face_shape(self, d):
        nx, ny, nz = self.nx
        return (nz + (d == 2), ny + (d == 1), nx + (d == 0))

    # -- state transfer (interior layout, as in a .dbl dump) --
    def _put(self, fn: str, vc: np.ndarray, bs=(None, None, None)):
        nx, ny, nz = self.nx
        vc = np.ascontiguousarray(vc, dtype=np.float64).reshape(NVAR, nz, ny, nx)
        keep = [np.ascontiguousarray(vc[q]) for q in range(NVAR)]
        faces = [None, None, None]
        if self.ct:
            for d in range(self.dims):
                faces[d] = np.ascontiguousarray(bs[d], dtype=np.float64).reshape(self.face_shape(d))
        L.check(getattr(L.lib(), fn)(self.h, _ptrs(keep, 8), _ptrs(faces, 3), L.PG_LAYOUT_INTERIOR), fn)

    def _get(self, fn: str, out=None):
        nx, ny, nz = self.nx
        if out is None:
            vc = np.zeros((NVAR, nz, ny, nx))
            faces = [np.zeros(self.face_shape(d)) if (self.ct and d < self.dims) else None
                     for d in range(3)]
        else:
            vc, faces = self._check_out(out)
        views = [vc[q] for q in range(NVAR)]
        L.check(getattr(L.lib(), fn)(self.h, _ptrs(views, 8), _ptrs(faces, 3), L.PG_LAYOUT_INTERIOR), fn)
        return vc, faces

    def _check_out(self, out):
        """(vc, faces) of caller-provided arrays, shapes and layout checked."""
        nx, ny, nz = self.nx
        vc, faces = out[0], list(out[1]) + [None] * (3 - len(out[1]))
        if vc.shape != (NVAR, nz, ny, nx) or vc.dtype != np.float64 or not vc.flags.c_contiguous:
            raise ValueError("out[0] must be a C-contiguous float64 array of shape %s" % ((NVAR, nz, ny, nx),))
        for d in range(3):
            want = self.ct and d < self.dims
            f = faces[d]
            if want and (f is None or f.shape != self.face_shape(d) or f.dtype != np.float64
                         or not f.flags.c_contiguous):
                raise ValueError("out[1][%d] must be a C-contiguous float64 array of shape %s"
                                 % (d, self.face_shape(d)))
            if not want:
                faces[d] = None
        return vc, faces

    def ghost_shape(self):
        """(nt2, nt1, nt0): the ghosted cell-array shape (PLUTO layout)."""
        s = self.spec
        ng = 3 if s.get("recon", "LINEAR") == "PARABOLIC" else 2
        if s.get("stepping", "RK2") in CTU_STEPPING and self.ct:
            ng += 1
        return tuple(int(s["nx"][d]) + 2 * ng if d < self.dims else 1 for d in (2, 1, 0))

    def set_userdef(self, fn):
        """User-defined boundary sides (PLUTO's UserDefBoundary).  fn(side,
        vpos, stage, vc, faces) is called at every boundary fill for every
        "userdef" side (side 0..5 = X1_BEG..X3_END; vpos 0 the cell box, 1..3
        the box of face component 1..3); vc [8, nt2, nt1, nt0] and faces[d]
        (one longer along d, -1 layer first) are PLUTO-layout host arrays that
        hold the current state near the side; fn writes the side's ghost
        boxes.  It runs on a CUDA host thread while the step waits for it.
        A sixth argument, flags, is the zone-flag array (internal boundaries)."""
        nz, ny, nx = self.ghost_shape()
        self._ud_vc = np.zeros((NVAR, nz, ny, nx))
        self._ud_f = [np.zeros((nz + (d == 2), ny + (d == 1), nx + (d == 0)))
                      if (self.ct and d < self.dims) else None for d in range(3)]

        self._ud_flags = np.zeros((nz, ny, nx), dtype=np.uint8)

        def cb(user, side, vpos, stage):
            fn(side, vpos, stage, self._ud_vc, self._ud_f, self._ud_flags)

        self._ud_cb = L.USERDEF_FN(cb)
        views = [self._ud_vc[q] for q in range(NVAR)]
        L.check(L.lib().pg_set_userdef(self.h, self._ud_cb, None, _ptrs(views, 8), _ptrs(self._ud_f, 3)),
                "pg_set_userdef")

    def set_internal_boundary(self):
        """INTERNAL_BOUNDARY YES: the set_userdef function is also called with
        side 6 (PG_SIDE_INTERNAL) before every boundary fill, with the whole
        state and the zone flags (flags, uint8, PLUTO layout); zones flagged 32
        are not updated.  EULER/RK2/RK3 time stepping, FP64 or mixed."""
        ptr = self._ud_flags.ctypes.data_as(C.POINTER(C.c_ubyte))
        L.check(L.lib().pg_set_internal_boundary(self.h, ptr), "pg_set_internal_boundary")

    def upload(self, vc: np.ndarray, bs=(None, None, None)):
        self._put("pg_upload", vc, bs)

    def download(self, out=None):
        """State as (vc [8,nz,ny,nx], faces).  out=(vc, faces) writes into
        preallocated arrays instead (e.g. pinned host memory, which the
        device writes in place)."""
        return self._get("pg_download", out)

    def download_async(self, out):
        """Enqueue a snapshot of the state into out=(vc, faces) (pinned
        host arrays as for download(out=...)) and return; the copy runs on a
        second stream while later steps proceed.  download_wait() blocks
        until out holds the snapshot."""
        vc, faces = self._check_out(out)
        views = [vc[q] for q in range(NVAR)]
        self._async_keep = (vc, faces)
        L.check(L.lib().pg_download_async(self.h, _ptrs(views, 8), _ptrs(faces, 3)), "pg_download_async")

    def download_wait(self):
        L.check(L.lib().pg_download_wait(self.h), "pg_download_wait")
        self._async_keep = None

    # -- output files (WriteData's .dbl / .flt / .vtk) --
    def output_vars(self, fmt: str, vtk_vector: bool = False):
        """[(var id, name, dump)] in the order SetOutput lists them: the
        primitives (PLUTO's NVAR order), then Bx1s.. under CT (dumped in .dbl
        only); VTK_VECTOR_DUMP makes vx1 and Bx1 vector entries."""
        comps = self.cfg.components
        slots = [0, 1, 2] + ([3] if comps == 3 else []) + [4, 5] + ([6] if comps == 3 else []) + [7]
        out = [[q, OUTPUT_NAMES[q], 1] for q in slots]
        if self.ct:
            out += [[8 + d, f"Bx{d + 1}s", 1 if fmt == "dbl" else 0] for d in range(self.dims)]
        if fmt == "vtk" and vtk_vector:
            for first in (1, 4):
                for e in out:
                    if first <= e[0] < first + self.dims:
                        e[2] = L.PG_OUT_VECTOR if e[0] == first else 0
        return [tuple(e) for e in out]

    def _output_spec(self, directory, fmt, nfile, single_file, vars, units, xbeg, xend, time, dt, step,
                     write_record, vtk_vector):
        o = L.PgOutput()
        o.format = {"dbl": L.PG_OUT_DBL, "flt": L.PG_OUT_FLT, "vtk": L.PG_OUT_VTK}[fmt]
        o.single_file = int(bool(single_file))
        o.nfile = int(nfile)
        vars = list(vars if vars is not None else self.output_vars(fmt, vtk_vector))
        if len(vars) > L.PG_OUT_MAX_VARS:
            raise ValueError("too many output variables")
        o.nvar = len(vars)
        units = units or {}
        keep = []
        for m, (vid, name, dump) in enumerate(vars):
            o.var[m] = int(vid)
            o.dump[m] = int(dump)
            keep.append(name.encode())
            o.name[m] = keep[-1]
            o.unit[m] = float(units.get(name, 1.0))
        keep.append(str(directory).encode())
        o.dir = keep[-1]
        if fmt == "vtk":
            xbeg = xbeg if xbeg is not None else (0.0, 0.0, 0.0)
            xend = xend if xend is not None else tuple(xbeg[d] + self.cfg.nx[d] * self.cfg.dx[d] for d in range(3))
            for d in range(3):
                n = self.cfg.nx[d] if d < self.dims else 1
                dx = (xend[d] - xbeg[d]) / float(n)
                x = np.array([xbeg[d] + float(i) * dx for i in range(n)] + [0.0])
                x[n] = x[n - 1] + dx  # Src/set_grid.c:395-403, :60-64
                keep.append(x)
                o.xnode[d] = x.ctypes.data_as(C.POINTER(C.c_double))
        o.time, o.dt, o.step = float(time), float(dt), int(step)
        o.write_record = int(bool(write_record))
        return o, keep

    def write_output(self, directory, fmt: str = "dbl", nfile: int = 0, *, single_file: bool = True,
                     vars=None, units=None, xbeg=None, xend=None, time: float = 0.0, dt: float = 0.0,
                     step: int = 0, write_record: bool = True, vtk_vector: bool = False):
        """Write the current state as PLUTO's WriteData would (files
        data.NNNN.<fmt> or <var>.NNNN.<fmt> and the <fmt>.out record) from the
        device, asynchronously: returns once the state is packed on the
        device; output_wait() blocks until the files are written.  VTK needs
        the domain extents xbeg/xend (pluto.ini X*-grid) for the node
        coordinates; inactive axes take the reference's 0..1."""
        o, keep = self._output_spec(directory, fmt, nfile, single_file, vars, units, xbeg, xend, time, dt,
                                    step, write_record, vtk_vector)
        L.check(L.lib().pg_write_output(self.h, C.byref(o)), "pg_write_output")
        del keep

    def output_wait(self):
        L.check(L.lib().pg_output_wait(self.h), "pg_output_wait")

    def read_output(self, directory, nfile: int, *, single_file: bool = True, vars=None):
        """Restart: upload the state of a .dbl written as above."""
        o, keep = self._output_spec(directory, "dbl", nfile, single_file, vars, None, None, None, 0.0, 0.0, 0,
                                    False, False)
        L.check(L.lib().pg_read_output(self.h, C.byref(o)), "pg_read_output")
        del keep

    # -- differentiation (frozen dt) --
    def tangent_upload(self, dvc: np.ndarray, dbs=(None, None, None)):
        """Direction of the tangent-linear model (precision "fp64_tangent")."""
        self._put("pg_tangent_upload", dvc, dbs)

    def tangent_download(self):
        return self._get("pg_tangent_download")

    def tangent_kink(self, enable: bool):
        """Start (True) or stop (False) recording the kink margin of the
        tangent-linear steps; stopping returns the smallest perturbation along
        the tangent direction at which, to first order, a branch switches."""
        m = C.c_double(0.0)
        L.check(L.lib().pg_tangent_kink(self.h, 1 if enable else 0, C.byref(m)), "pg_tangent_kink")
        return m.value

    def adjoint_set(self, lvc: np.ndarray, lbs=(None, None, None)):
        """Adjoint (gradient) on the state after the step to be reversed."""
        self._put("pg_adjoint_set", lvc, lbs)

    def adjoint_step(self, dt: float):
        """Adjoint through one step of length dt from the current state."""
        L.check(L.lib().pg_adjoint_step(self.h, float(dt)), "pg_adjoint_step")

    def adjoint_get(self):
        return self._get("pg_adjoint_get")

    def adjoint_slots(self, nslots: int) -> bool:
        """Allocate nslots per-step slots for adjoint_forward/adjoint_reverse
        (after adjoint_set); False, with nothing allocated, when they would
        take more than half of the free device memory."""
        rc = L.lib().pg_adjoint_slots(self.h, int(nslots))
        if rc == L.PG_ERR_NOMEM:
            return False
        L.check(rc, "pg_adjoint_slots")
        return True

    def adjoint_forward(self, dt: float, slot: int):
        """One step of length dt from the current state, saving what its
        reversal needs into slot; the state advances."""
        L.check(L.lib().pg_adjoint_forward(self.h, float(dt), int(slot)), "pg_adjoint_forward")

    def adjoint_reverse(self, dt: float, slot: int):
        """adjoint_step for the step saved in slot (the same kernels); the
        state goes back to that step's start."""
        L.check(L.lib().pg_adjoint_reverse(self.h, float(dt), int(slot)), "pg_adjoint_reverse")

    def checkpoint_save(self, slot: int):
        L.check(L.lib().pg_checkpoint_save(self.h, int(slot)), "pg_checkpoint_save")

    def checkpoint_load(self, slot: int):
        L.check(L.lib().pg_checkpoint_load(self.h, int(slot)), "pg_checkpoint_load")

    # -- stepping --
    def advance(self, dt: float):
        info = L.PgStepInfo()
        L.check(L.lib().pg_advance(self.h, float(dt), C.byref(info)), "pg_advance")
        return info.inv_dt_hyp, info.max_mach, info.nfail

    def run(self, nsteps: int, first_dt: float, cfl: float, cfl_max_var: float = 1.1):
        t = C.c_double()
        dt = C.c_double()
        L.check(L.lib().pg_run(self.h, int(nsteps), float(first_dt), float(cfl),
                               float(cfl_max_var), C.byref(t), C.byref(dt)), "pg_run")
        return t.value, dt.value

    def run_async(self, nsteps: int, first_dt: float, cfl: float, cfl_max_var: float = 1.1):
        L.check(L.lib().pg_run_async(self.h, int(nsteps), float(first_dt), float(cfl),
                                     float(cfl_max_var)), "pg_run_async")

    def run_timed(self, nsteps: int, first_dt: float, cfl: float, cfl_max_var: float = 1.1) -> float:
        """Run nsteps; return milliseconds between CUDA events on the solver stream."""
        ms = C.c_double()
        L.check(L.lib().pg_run_timed(self.h, int(nsteps), float(first_dt), float(cfl),
                                     float(cfl_max_var), C.byref(ms)), "pg_run_timed")
        return ms.value

    def profile_kernels(self, nsteps: int, first_dt: float, cfl: float, cfl_max_var: float = 1.1):
        """Per-kernel-family device time (ms) and launch counts over nsteps eager steps."""
        stride, cap = 64, 64
        names = C.create_string_buffer(stride * cap)
        tot = (C.c_double * cap)()
        cnt = (C.c_int * cap)()
        n = C.c_int()
        L.check(L.lib().pg_profile_kernels(self.h, int(nsteps), float(first_dt), float(cfl),
                                           float(cfl_max_var), names, stride, tot, cnt, cap,
                                           C.byref(n)), "pg_profile_kernels")
        out = {}
        for u in range(n.value):
            nm = names.raw[u * stride:(u + 1) * stride].split(b"\0", 1)[0].decode()
            out[nm] = (tot[u], cnt[u])
        return out

    def sync(self):
        L.check(L.lib().pg_sync(self.h), "pg_sync")

    def info(self):
        inf = L.PgStepInfo()
        t = C.c_double()
        dt = C.c_double()
        L.check(L.lib().pg_get_info(self.h, C.byref(inf), C.byref(t), C.byref(dt)), "pg_get_info")
        return dict(inv_dt_hyp=inf.inv_dt_hyp, max_mach=inf.max_mach, nfail=inf.nfail,
                    time=t.value, dt=dt.value)

    def stream(self) -> int:
        p = C.c_void_p()
        L.check(L.lib().pg_get_stream(self.h, C.byref(p)), "pg_get_stream")
        return p.value or 0

    def launches_per_step(self) -> int:
        return int(L.lib().pg_kernel_launches_per_step(self.h))
