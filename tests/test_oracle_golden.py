"""The CPU oracle reproduces the reference PLUTO binary bit for bit.

The fixtures were written by the reference itself (tests/golden/make_golden.py
compiles PLUTO 4.3's C sources with -ffp-contract=off and runs them); the
oracle restates the same algorithm and must match every double exactly.
"""
import numpy as np
import pytest

import userdef_cases
from conftest import GOLDEN_NAMES, load_golden, rel_l1
from oracle.oracle import Oracle


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_oracle_matches_reference_bitwise(name):
    meta, vc0, bs0, vc1, bs1 = load_golden(name)
    o = Oracle(meta, nthreads=2)
    if userdef_cases.has_userdef(meta):
        o.set_userdef(userdef_cases.make(meta))
        if meta.get("internal_boundary"):
            o.set_internal_boundary()
    o.set_state(vc0, bs0)
    dts, t = o.run(meta["steps"], meta["first_dt"], meta["cfl"])
    vc, bs = o.get_state()
    assert np.array_equal(vc, vc1), [rel_l1(vc[q], vc1[q]) for q in range(8)]
    for d in range(3):
        if bs1[d] is not None:
            assert np.array_equal(bs[d], bs1[d])
    assert abs(t - meta["t_final"]) <= 1e-6 * meta["t_final"]  # dbl.out keeps 7 digits


def test_oracle_floor_branch_is_exercised():
    meta, vc0, bs0, _, _ = load_golden("blast_floor_16")
    o = Oracle(meta, nthreads=2)
    o.set_state(vc0, bs0)
    dt, total = meta["first_dt"], 0
    for _ in range(meta["steps"]):
        inv, _, nf = o.advance(dt)
        total += nf
        dt = min((1.0 / inv) * meta["cfl"], 1.1 * dt)
    assert total > 0


def test_oracle_threads_are_deterministic():
    meta, vc0, bs0, _, _ = load_golden("blast_16")
    out = []
    for nt in (1, 4):
        o = Oracle(meta, nthreads=nt)
        o.set_state(vc0, bs0)
        o.run(4, meta["first_dt"], meta["cfl"])
        out.append(o.get_state()[0])
    assert np.array_equal(out[0], out[1])


@pytest.mark.parametrize("stepping,emf", [("RK2", "UCT_HLL"), ("RK2", "ARITHMETIC"), ("RK3", "UCT_CONTACT"),
                                          ("RK2", "UCT0"), ("HANCOCK", "UCT0"), ("HANCOCK_CONS", "UCT_CONTACT"),
                                          ("CHARACTERISTIC_TRACING", "ARITHMETIC")])
def test_oracle_ct_keeps_divergence_at_roundoff(stepping, emf):
    """Constrained transport keeps the face field divergence-free to round-off
    for every edge average and predictor (a property independent of the grid
    size; here a 3D blast at 24^3 with a uniform oblique field, 6 steps)."""
    from pluto_gb300 import problems
    spec, vc, faces = problems.blast3d(24)
    spec = dict(spec, stepping=stepping, emf=emf)
    o = Oracle(spec, nthreads=4)
    o.set_state(vc, faces)
    o.run(6, spec["first_dt"], spec["cfl"])
    _, b = o.get_state()
    div = (b[0][:, :, 1:] - b[0][:, :, :-1]) + (b[1][:, 1:, :] - b[1][:, :-1, :]) + (b[2][1:] - b[2][:-1])
    assert np.isfinite(b[0]).all()
    assert np.abs(div).max() <= 1e-12 * np.abs(b[0]).max()  # undivided differences, relative to |B|
