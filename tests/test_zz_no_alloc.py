"""Allocation-free 1D step (pg_tube_step_static) against the regular entry point.

pg_tube_step_static serves callers that may not allocate device memory while
they run (an application whose pool allocator owns the device memory, loops
that cannot take the device synchronisation of cudaMalloc/cudaFree): its
work arrays are one file-scope device array.  Here it must reproduce
pg_create/pg_upload/pg_advance/pg_download on two consecutive calls, the
second one fed with the first one's output, with the tolerance of the other
FP64 tests (it runs the same kernels, so the results are in fact identical).
Configurations it cannot run (CTU, user-defined sides, constrained
transport, more than one dimension, sizes above the array) are rejected
before any CUDA call, so those checks also run without a GPU.  This file is
collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_l1

TOL = 1e-10


def _static_step(lib, cfg, d_in, d_out, dt, stream):
    from pluto_gb300 import _lib as L
    info = L.PgStepInfo()
    rc = lib.pg_tube_step_static(C.byref(cfg), C.c_void_p(d_in.data_ptr()), C.c_void_p(d_out.data_ptr()),
                                 float(dt), C.c_void_p(stream), C.byref(info))
    assert rc == 0, lib.pg_last_error()
    return info


@pytest.mark.gpu
@pytest.mark.parametrize("n,seed,recon,bc", [(3000, 3, "LINEAR", "outflow"), (1500, 5, "PARABOLIC", "outflow"),
                                             (2048, 7, "LINEAR", "periodic")])
def test_static_step_matches_regular_entry_point_on_two_calls(n, seed, recon, bc):
    import torch
    from pluto_gb300 import Solver, problems
    from pluto_gb300 import _lib as L
    spec, vc, _ = problems.riemann_tube(n, seed)
    spec["recon"] = recon
    spec["bc"] = bc
    lib = L.lib()
    ref = Solver(spec, precision="fp64")
    ref.upload(vc)
    dt1 = 2e-4
    inv1, _, nf1 = ref.advance(dt1)
    dt2 = min(spec["cfl"] / inv1, 1.1 * dt1)
    inv2, _, nf2 = ref.advance(dt2)
    want, _ = ref.download()

    cfg = ref.cfg
    stream = torch.cuda.current_stream().cuda_stream
    d_a = torch.tensor(vc.reshape(8, n), dtype=torch.float64, device="cuda")
    d_b = torch.empty_like(d_a)
    i1 = _static_step(lib, cfg, d_a, d_b, dt1, stream)
    i2 = _static_step(lib, cfg, d_b, d_a, dt2, stream)
    got = d_a.cpu().numpy().reshape(want.shape)
    errs = [rel_l1(got[q], want[q]) for q in range(8) if np.abs(want[q]).sum() > 0]
    assert max(errs) <= TOL, errs
    assert i1.inv_dt_hyp == inv1 and i2.inv_dt_hyp == inv2
    assert i1.nfail == nf1 and i2.nfail == nf2


def _rejected(spec_changes, msg):
    """Calls the entry point with a configuration it must refuse; the pointers
    are never dereferenced because the refusal comes before any CUDA call."""
    from pluto_gb300 import _lib as L
    from pluto_gb300 import problems
    from pluto_gb300.solver import make_config
    spec, _, _ = problems.riemann_tube(64, 0)
    spec.update(spec_changes)
    cfg = make_config(spec)
    lib = L.lib()
    info = L.PgStepInfo()
    rc = lib.pg_tube_step_static(C.byref(cfg), C.c_void_p(16), C.c_void_p(16), 1e-4, None, C.byref(info))
    return rc, lib.pg_last_error()


def test_static_step_rejects_oversize():
    from pluto_gb300 import _lib as L
    rc, err = _rejected({"nx": (L.PG_STATIC_MAX_ZONES + 1, 1, 1)}, "")
    assert rc == L.PG_ERR_TOO_LARGE and b"PG_STATIC_MAX_ZONES" in err


@pytest.mark.parametrize("changes,word", [
    ({"stepping": "HANCOCK"}, b"CTU"),
    ({"stepping": "CHARACTERISTIC_TRACING"}, b"CTU"),
    ({"stepping": "HANCOCK_CONS"}, b"CTU"),
    ({"bc": "userdef"}, b"user-defined"),
    ({"bc": [("outflow", "userdef"), "periodic", "periodic"]}, b"user-defined"),
    ({"dims": 2, "nx": (64, 64, 1), "dx": (1 / 64, 1 / 64, 1.0), "ct": True}, b"1D"),
    ({"dims": 2, "nx": (64, 64, 1), "dx": (1 / 64, 1 / 64, 1.0)}, b"1D"),
])
def test_static_step_rejects_unsupported_configs(changes, word):
    from pluto_gb300 import _lib as L
    rc, err = _rejected(changes, word)
    assert rc == L.PG_ERR_INVALID and word in err, err
