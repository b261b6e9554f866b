"""The CPU oracle against the reference at the benchmark configurations' sizes.

Fixtures (tests/golden/large/, written by ``make_golden.py --large`` from the
reference compiled with -ffp-contract=off): the 2D Orszag-Tang vortex at
256^2 for 200 steps, the 3D blast scheme at 64^3 for 21 steps (the pressure
floor fires 222 times), the rotated circularly polarised Alfven wave at 128^2
for 256 steps, and the first 32 tubes of the batched Riemann-tube family at
their drawn sizes for 400 steps.  The oracle must give the reference's final
dump bit for bit (SHA-256 of every variable).
"""
import os

import numpy as np
import pytest

from conftest import check_against_large, load_large
from oracle.oracle import Oracle

THREADS = max(1, min(8, os.cpu_count() or 1))


def _run(meta, vc0, bs0):
    o = Oracle(meta, nthreads=THREADS)
    o.set_state(vc0, bs0)
    dt, floors = meta["first_dt"], 0
    for _ in range(meta["steps"]):
        inv, _, nf = o.advance(dt)
        floors += nf
        dt = min((1.0 / inv) * meta["cfl"], 1.1 * dt)
    return o.get_state(), floors


@pytest.mark.parametrize("name", ["ot_hlld_256_200", "blast_64_21", "cpa_128_256"])
def test_oracle_matches_reference_at_config_size(name):
    meta, vc0, bs0 = load_large(name)
    (vc, bs), floors = _run(meta, vc0, bs0)
    assert check_against_large(meta, vc, bs) == []
    if name == "blast_64_21":
        assert floors == 222  # the pressure-floor branch at scale (Src/MHD/mappers.c:188-200)


def test_oracle_matches_reference_tube_family():
    meta, z = load_large("tubes_family0_32x400")
    v0, v1 = z["v0"], z["v1"]
    off = 0
    for n in meta["nx_tubes"]:
        spec = dict(meta, nx=(n, 1, 1), dx=(1.0 / n, 1.0, 1.0))
        o = Oracle(spec, nthreads=1)
        o.set_state(v0[:, off:off + n].reshape(8, 1, 1, n), [None, None, None])
        o.run(meta["steps"], meta["first_dt"], meta["cfl"])
        vc, _ = o.get_state()
        assert np.array_equal(vc.reshape(8, n), v1[:, off:off + n]), n
        off += n
