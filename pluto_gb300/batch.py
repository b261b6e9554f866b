"""Batched independent 1D MHD problems over the C ABI (pg_batch_*).

Each tube is an independent PLUTO 1D run (own grid, own dt sequence); all
tubes advance in one persistent, graph-captured launch.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .solver import make_config


class Batch:
    def __init__(self, spec: dict, nx, dx, precision: str = "fp64"):
        nx = np.ascontiguousarray(nx, dtype=np.int32)
        dx = np.ascontiguousarray(dx, dtype=np.float64)
        s = dict(spec)
        s.setdefault("nx", (8, 1, 1))
        s.setdefault("dx", (1.0, 1.0, 1.0))
        self.cfg = make_config(s, precision)
        self.nx = nx
        self.ntubes = len(nx)
        h = C.c_void_p()
        L.check(L.lib().pg_batch_create(C.byref(self.cfg), self.ntubes,
                                        nx.ctypes.data_as(C.POINTER(C.c_int)),
                                        dx.ctypes.data_as(C.POINTER(C.c_double)), C.byref(h)),
                "pg_batch_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            L.lib().pg_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, states):
        """states: list of [8][nx_t] arrays (or one concatenated flat array)."""
        flat = np.concatenate([np.ascontiguousarray(s, dtype=np.float64).ravel() for s in states]) \
            if isinstance(states, (list, tuple)) else np.ascontiguousarray(states, dtype=np.float64)
        assert flat.size == 8 * int(self.nx.sum())
        L.check(L.lib().pg_batch_upload(self.h, flat.ctypes.data_as(C.POINTER(C.c_double))), "pg_batch_upload")

    def download(self):
        flat = np.zeros(8 * int(self.nx.sum()))
        L.check(L.lib().pg_batch_download(self.h, flat.ctypes.data_as(C.POINTER(C.c_double))), "pg_batch_download")
        out, q = [], 0
        for n in self.nx:
            out.append(flat[q:q + 8 * n].reshape(8, n))
            q += 8 * n
        return out

    def run(self, nsteps, first_dt, cfl, cfl_max_var=1.1):
        ms = C.c_double()
        L.check(L.lib().pg_batch_run(self.h, int(nsteps), float(first_dt), float(cfl), float(cfl_max_var),
                                     C.byref(ms)), "pg_batch_run")
        return ms.value

    def get(self):
        t = np.zeros(self.ntubes)
        dt = np.zeros(self.ntubes)
        nf = np.zeros(self.ntubes, dtype=np.int64)
        L.check(L.lib().pg_batch_get(self.h, t.ctypes.data_as(C.POINTER(C.c_double)),
                                     dt.ctypes.data_as(C.POINTER(C.c_double)),
                                     nf.ctypes.data_as(C.POINTER(C.c_int64))), "pg_batch_get")
        return t, dt, nf

    def autotune(self, trial_steps, first_dt, cfl, cfl_max_var=1.1):
        th, bps, order = C.c_int(), C.c_int(), C.c_int()
        ms = C.c_double()
        L.check(L.lib().pg_batch_autotune(self.h, int(trial_steps), float(first_dt), float(cfl),
                                          float(cfl_max_var), C.byref(th), C.byref(bps), C.byref(order),
                                          C.byref(ms)), "pg_batch_autotune")
        return dict(threads=th.value, blocks_per_sm=bps.value, largest_first=order.value, trial_ms=ms.value)

    def set_schedule(self, threads, blocks_per_sm, largest_first=True):
        L.check(L.lib().pg_batch_set_schedule(self.h, int(threads), int(blocks_per_sm), int(largest_first)),
                "pg_batch_set_schedule")


def tube_family(ntubes=4096, seed=0, nmin=128, nmax=4096):
    """The batched Riemann-tube family: N log-uniform in [nmin, nmax] from the
    seed, one problems.riemann_tube per tube (seeded per tube)."""
    from . import problems
    rng = np.random.default_rng(seed)
    ns = np.rint(np.exp(rng.uniform(np.log(nmin), np.log(nmax), ntubes))).astype(np.int32)
    states, dxs, spec = [], [], None
    for t, n in enumerate(ns):
        spec, vc, _ = problems.riemann_tube(int(n), seed=seed * 1_000_003 + t)
        states.append(vc.reshape(8, int(n)))
        dxs.append(spec["dx"][0])
    return spec, ns, np.array(dxs), states
