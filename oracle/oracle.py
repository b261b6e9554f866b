"""ctypes wrapper for the CPU oracle (test infrastructure only).

Used by the test suite, the smoke check and the CPU-baseline leg of the
benchmark, never by the product path.  ``build()`` compiles ``liboracle.so``
from ``mhd_oracle.c`` with the committed Makefile.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"

NVAR = 8
RECON = {"LINEAR": 0, "PARABOLIC": 1}
LIMITER = {"FLAT_LIM": 0, "MINMOD_LIM": 1, "VANLEER_LIM": 2, "MC_LIM": 3, "DEFAULT": 4}
SOLVER = {"hll": 0, "hlld": 1, "roe": 2}
STEPPING = {"EULER": 1, "RK2": 2, "RK3": 3, "HANCOCK": 4, "CHARACTERISTIC_TRACING": 5, "HANCOCK_CONS": 6}
CTU_STEPPING = ("HANCOCK", "CHARACTERISTIC_TRACING", "HANCOCK_CONS")
BC = {"periodic": 0, "outflow": 1, "reflective": 2, "eqtsymmetric": 3, "userdef": 4}
EMF = {"ARITHMETIC": 1, "UCT0": 2, "UCT_CONTACT": 3, "UCT_HLL": 4}


class OcConfig(C.Structure):
    _fields_ = [("dims", C.c_int), ("components", C.c_int), ("nx", C.c_int * 3),
                ("dx", C.c_double * 3), ("gamma", C.c_double), ("recon", C.c_int),
                ("limiter", C.c_int), ("solver", C.c_int), ("stepping", C.c_int),
                ("ct", C.c_int), ("bc", C.c_int * 3), ("nthreads", C.c_int), ("emf", C.c_int),
                ("bc_hi", C.c_int * 3), ("char_limiting", C.c_int)]


_lib = None


def build(force: bool = False) -> Path:
    if force or not LIB.exists() or LIB.stat().st_mtime < (HERE / "mhd_oracle.c").stat().st_mtime:
        subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


USERDEF_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_int, C.c_int, C.c_int)


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        L.oc_create.restype = C.c_void_p
        L.oc_create.argtypes = [C.POINTER(OcConfig)]
        L.oc_destroy.argtypes = [C.c_void_p]
        dp = C.POINTER(C.c_double)
        L.oc_set_state.argtypes = [C.c_void_p, dp, dp, dp, dp]
        L.oc_get_state.argtypes = [C.c_void_p, dp, dp, dp, dp]
        L.oc_advance.argtypes = [C.c_void_p, C.c_double, dp, dp, C.POINTER(C.c_int64)]
        L.oc_run.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_double, dp, dp]
        L.oc_set_userdef.argtypes = [C.c_void_p, USERDEF_FN, C.c_void_p]
        L.oc_arrays.argtypes = [C.c_void_p, C.POINTER(dp), C.POINTER(dp)]
        L.oc_set_internal.argtypes = [C.c_void_p, C.c_int]
        L.oc_flags.argtypes = [C.c_void_p]
        L.oc_flags.restype = C.POINTER(C.c_ubyte)
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


class _VarStack:
    """vc[q] -> the view of variable q (the oracle's cell arrays are separate
    allocations, so they cannot form one numpy array without a copy)."""

    def __init__(self, views):
        self.views = views

    def __getitem__(self, q):
        return self.views[q]


class Oracle:
    """One problem instance held by the C oracle.

    ``spec`` keys: dims, components, nx (3-tuple), dx (3-tuple), gamma,
    recon, limiter, solver, stepping, ct, bc.
    """

    def __init__(self, spec: dict, nthreads: int = 0):
        self.spec = dict(spec)
        c = OcConfig()
        c.dims = spec["dims"]
        c.components = spec["components"]
        for d in range(3):
            c.nx[d] = int(spec["nx"][d]) if d < spec["dims"] else 1
            c.dx[d] = float(spec["dx"][d])
            # one type for every side, one per axis, or a (beg, end) pair per axis
            bc = spec.get("bc", "periodic")
            t = bc[d] if isinstance(bc, (list, tuple)) else bc
            lo, hi = (t[0], t[1]) if isinstance(t, (list, tuple)) else (t, t)
            c.bc[d] = BC[lo]
            c.bc_hi[d] = BC[hi]
        c.gamma = float(spec["gamma"])
        c.recon = RECON[spec["recon"]]
        c.limiter = LIMITER[spec["limiter"]]
        c.solver = SOLVER[spec["solver"]]
        c.stepping = STEPPING[spec["stepping"]]
        c.ct = int(bool(spec["ct"]))
        c.nthreads = nthreads
        c.emf = EMF[spec.get("emf", "UCT_HLL")]
        c.char_limiting = int(bool(spec.get("char_limiting", False)))
        self.h = lib().oc_create(C.byref(c))
        if not self.h:
            raise ValueError("oracle rejected the configuration")
        self.nx = tuple(c.nx[d] for d in range(3))

    def __del__(self):
        if getattr(self, "h", None):
            lib().oc_destroy(self.h)
            self.h = None

    def face_shape(self, d):
        nx, ny, nz = self.nx
        return (nz + (d == 2), ny + (d == 1), nx + (d == 0))

    def set_userdef(self, fn):
        """USERDEF sides: fn(side, vpos, stage, vc, faces) on numpy views of
        the oracle's own PLUTO-layout arrays (vc [8, nt2, nt1, nt0], faces[d]
        one longer along d with the -1 layer first)."""
        ng = 3 if self.spec["recon"] == "PARABOLIC" else 2
        if self.spec["stepping"] in CTU_STEPPING and self.spec["ct"]:
            ng += 1
        nt = [self.nx[d] + 2 * ng if d < self.spec["dims"] else 1 for d in range(3)]
        dp = C.POINTER(C.c_double)
        vp, bp = (dp * NVAR)(), (dp * 3)()
        lib().oc_arrays(self.h, vp, bp)
        vviews = [np.ctypeslib.as_array(vp[q], shape=(nt[2], nt[1], nt[0])) for q in range(NVAR)]
        faces = [np.ctypeslib.as_array(bp[d], shape=(nt[2] + (d == 2), nt[1] + (d == 1), nt[0] + (d == 0)))
                 if (self.spec["ct"] and d < self.spec["dims"]) else None for d in range(3)]
        flags = np.ctypeslib.as_array(lib().oc_flags(self.h), shape=(nt[2], nt[1], nt[0]))
        self._ud_views = (_VarStack(vviews), faces, flags)

        def cb(user, side, vpos, stage):
            fn(side, vpos, stage, self._ud_views[0], self._ud_views[1], self._ud_views[2])

        self._ud_cb = USERDEF_FN(cb)
        lib().oc_set_userdef(self.h, self._ud_cb, None)

    def set_internal_boundary(self):
        """INTERNAL_BOUNDARY YES: the userdef callback also runs with side 6
        before every boundary fill and sees the zone flags (set_userdef first)."""
        lib().oc_set_internal(self.h, 1)

    def set_state(self, vc: np.ndarray, bs=(None, None, None)):
        vc = np.ascontiguousarray(vc, dtype=np.float64)
        b = [None if x is None else np.ascontiguousarray(x, dtype=np.float64) for x in bs]
        lib().oc_set_state(self.h, _ptr(vc), _ptr(b[0]), _ptr(b[1]), _ptr(b[2]))

    def get_state(self):
        nx, ny, nz = self.nx
        vc = np.zeros((NVAR, nz, ny, nx))
        bs = [np.zeros(self.face_shape(d)) if (self.spec["ct"] and d < self.spec["dims"]) else None
              for d in range(3)]
        lib().oc_get_state(self.h, _ptr(vc), _ptr(bs[0]), _ptr(bs[1]), _ptr(bs[2]))
        return vc, bs

    def advance(self, dt: float):
        inv = C.c_double()
        mach = C.c_double()
        nf = C.c_int64()
        if lib().oc_advance(self.h, dt, C.byref(inv), C.byref(mach), C.byref(nf)):
            raise RuntimeError("oracle: Roe solver met a negative sound speed squared")
        return inv.value, mach.value, nf.value

    def run(self, nsteps: int, first_dt: float, cfl: float, cfl_max_var: float = 1.1):
        dts = np.zeros(max(nsteps, 1))
        t = C.c_double()
        if lib().oc_run(self.h, nsteps, first_dt, cfl, cfl_max_var, _ptr(dts), C.byref(t)):
            raise RuntimeError("oracle: Roe solver met a negative sound speed squared")
        return dts[:nsteps], t.value
