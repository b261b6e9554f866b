"""The CUDA paths at the benchmark configurations' sizes.

Plain FP64 path against the reference's own dumps (tests/golden/large/: the
2D Orszag-Tang vortex 256^2 x 200 steps, the 3D blast scheme at 64^3 x 21
steps with 222 pressure-floor events, the rotated CP Alfven wave 128^2 x 256
steps, 32 tubes of the batched family x 400 steps): bit for bit, checked by
the SHA-256 of every variable.  Mixed precision (both accumulator forms)
against the FP64 path from the same initial state: relative L1 per variable
(faces included) <= 1e-5.
"""
import numpy as np
import pytest

from conftest import check_against_large, load_large, rel_l1

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-5
NAMES = ["ot_hlld_256_200", "blast_64_21", "cpa_128_256"]


def _run(meta, vc0, bs0, precision):
    from pluto_gb300 import Solver
    s = Solver(meta, precision=precision)
    s.upload(vc0, bs0)
    t, _ = s.run(meta["steps"], meta["first_dt"], meta["cfl"])
    vc, bs = s.download()
    return vc, bs, t


@pytest.mark.parametrize("name", NAMES)
def test_fp64_bitwise_at_config_size(name):
    meta, vc0, bs0 = load_large(name)
    vc, bs, t = _run(meta, vc0, bs0, "fp64")
    assert check_against_large(meta, vc, bs) == []
    assert abs(t - meta["t_final"]) <= 1e-6 * meta["t_final"]


def test_fp64_floor_events_at_config_size():
    """The blast scheme at 64^3: the pressure floor fires 222 times in 21
    steps in the reference; the FP64 path counts the same events."""
    from pluto_gb300 import Solver
    meta, vc0, bs0 = load_large("blast_64_21")
    s = Solver(meta, precision="fp64")
    s.upload(vc0, bs0)
    dt, floors = meta["first_dt"], 0
    for _ in range(meta["steps"]):
        inv, _, nf = s.advance(dt)
        floors += nf
        dt = min((1.0 / inv) * meta["cfl"], 1.1 * dt)
    assert floors == 222
    vc, bs = s.download()
    assert check_against_large(meta, vc, bs) == []


@pytest.mark.parametrize("precision", ["mixed", "mixed_dw"])
@pytest.mark.parametrize("name", NAMES)
def test_mixed_within_bar_at_config_size(name, precision):
    meta, vc0, bs0 = load_large(name)
    ref, rbs, _ = _run(meta, vc0, bs0, "fp64")
    vc, bs, _ = _run(meta, vc0, bs0, precision)
    errs = {q: rel_l1(vc[q], ref[q]) for q in range(8) if np.abs(ref[q]).sum() > 0}
    for d in range(3):
        if rbs[d] is not None:
            errs[f"b{d}"] = rel_l1(bs[d], rbs[d])
    assert max(errs.values()) <= MIXED_TOL, errs


def test_fp64_batch_bitwise_on_tube_family():
    from pluto_gb300.batch import Batch
    meta, z = load_large("tubes_family0_32x400")
    ns = np.array(meta["nx_tubes"], dtype=np.int32)
    v0, v1 = z["v0"], z["v1"]
    states, off = [], 0
    for n in ns:
        states.append(v0[:, off:off + n])
        off += n
    b = Batch(meta, ns, 1.0 / ns, "fp64")
    b.upload(states)
    b.run(meta["steps"], meta["first_dt"], meta["cfl"])
    out = b.download()
    t, _, _ = b.get()
    off = 0
    for q, n in enumerate(ns):
        assert np.array_equal(out[q], v1[:, off:off + n]), q
        off += n
    assert np.allclose(t, z["t1"], rtol=1e-6, atol=0)  # dbl.out keeps 7 digits
