"""Batched 1D tubes: every tube of the persistent launch against the oracle
(FP64 bit-for-bit through 1e-10) and the mixed batch within 1e-5."""
import numpy as np
import pytest

from conftest import load_golden, rel_l1

pytestmark = pytest.mark.gpu


def _family(ntubes, seed, nmin, nmax):
    from pluto_gb300.batch import tube_family
    return tube_family(ntubes, seed, nmin, nmax)


def _oracle_run(spec, n, dx, state, nsteps, first_dt):
    from oracle.oracle import Oracle
    s = dict(spec)
    s["nx"] = (int(n), 1, 1)
    s["dx"] = (float(dx), 1.0, 1.0)
    o = Oracle(s, nthreads=1)
    o.set_state(state.reshape(8, 1, 1, int(n)))
    dts, t = o.run(nsteps, first_dt, s["cfl"])
    return o.get_state()[0].reshape(8, int(n)), t


@pytest.mark.parametrize("recon,stepping,bc", [("LINEAR", "RK2", "outflow"), ("PARABOLIC", "RK3", "outflow"),
                                               ("LINEAR", "RK2", "reflective"),
                                               ("PARABOLIC", "RK2", "eqtsymmetric"),
                                               ("LINEAR", "RK3", [("reflective", "outflow"), "outflow", "outflow"])])
def test_batch_fp64_matches_oracle_per_tube(recon, stepping, bc):
    from pluto_gb300.batch import Batch
    spec, ns, dxs, states = _family(24, 7, 16, 300)
    spec = dict(spec, recon=recon, stepping=stepping, bc=bc)
    b = Batch(spec, ns, dxs, "fp64")
    b.upload(states)
    b.run(60, 1e-4, spec["cfl"])
    out = b.download()
    times, _, _ = b.get()
    for t in range(len(ns)):
        want, tw = _oracle_run(spec, ns[t], dxs[t], states[t], 60, 1e-4)
        assert np.array_equal(out[t], want), (t, max(rel_l1(out[t][q], want[q]) for q in range(8)))
        assert times[t] == tw


def test_batch_fp64_matches_golden_tubes():
    from pluto_gb300.batch import Batch
    names = ["tube_0_256", "tube_1_200", "tube_2_160", "tube_roe_0_256", "tube_reflective_0_256",
             "tube_sides_0_256"]
    metas, st0, st1 = [], [], []
    for nm in names:
        meta, vc0, _, vc1, _ = load_golden(nm)
        metas.append(meta)
        st0.append(vc0.reshape(8, -1))
        st1.append(vc1.reshape(8, -1))
    # the goldens differ in step count: run each as its own batch
    for meta, a, want in zip(metas, st0, st1):
        b = Batch(meta, [meta["nx"][0]], [meta["dx"][0]], "fp64")
        b.upload([a])
        b.run(meta["steps"], meta["first_dt"], meta["cfl"])
        got = b.download()[0]
        assert np.array_equal(got, want)


@pytest.mark.parametrize("prec", ["mixed", "mixed_dw"])
def test_batch_mixed_close_to_fp64(prec):
    """Mixed batch against the FP64 batch at equal times (fixed dt 1e-4, 200
    steps), every tube and variable within relative L1 1e-5: the mixed batch
    keeps each tube's conserved state resident in the accumulator type.  (With
    the CFL dt each precision takes its own dt sequence, and on shock tubes
    the time offset alone moves the discontinuities.)"""
    from pluto_gb300.batch import Batch
    spec, ns, dxs, states = _family(64, 3, 64, 600)
    out, meta = {}, {}
    for p in ("fp64", prec):
        b = Batch(spec, ns, dxs, p)
        b.upload(states)
        b.run(200, 1e-4, 0.0)
        out[p] = b.download()
        meta[p] = b.get()
    errs = sorted((rel_l1(out[prec][t][q], out["fp64"][t][q]), t, q, int(ns[t]))
                  for t in range(len(ns)) for q in range(8) if np.abs(out["fp64"][t][q]).sum() > 0)
    print(prec, "worst (rel L1, tube, var, n):", errs[-5:], "median", errs[len(errs) // 2][0])
    w = errs[-1][1]
    print("worst tube time/dt/nfail fp64:", [m[w] for m in meta["fp64"]], prec, [m[w] for m in meta[prec]])
    q = errs[-1][2]
    d = np.abs(out[prec][w][q] - out["fp64"][w][q])
    print("worst tube |diff| profile max at", int(d.argmax()), "max", float(d.max()),
          "cells with |diff|>1e-4:", int((d > 1e-4).sum()))
    assert np.array_equal(meta["fp64"][0], meta[prec][0])  # same times
    assert errs[len(errs) // 2][0] <= 1e-6
    assert errs[-1][0] <= 1e-5, errs[-1]


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_batch_autotune_keeps_results(prec):
    from pluto_gb300.batch import Batch
    spec, ns, dxs, states = _family(40, 11, 32, 400)
    b = Batch(spec, ns, dxs, prec)
    b.upload(states)
    tun = b.autotune(5, 1e-4, spec["cfl"])
    assert tun["threads"] in (64, 128, 256) and tun["largest_first"] == 1
    b.run(30, 1e-4, spec["cfl"])
    got = b.download()
    ref = Batch(spec, ns, dxs, prec)
    ref.upload(states)
    ref.run(30, 1e-4, spec["cfl"])
    want = ref.download()
    for t in range(len(ns)):
        assert np.array_equal(got[t], want[t])


@pytest.mark.parametrize("prec", ["fp64", "mixed", "mixed_dw"])
def test_batch_schedule_does_not_change_results(prec):
    """Every zone's arithmetic is the same whichever warps of the team take
    its chunk and however many teams share an SM."""
    from pluto_gb300.batch import Batch
    spec, ns, dxs, states = _family(50, 13, 16, 700)
    outs = []
    for threads, bps, order in ((32, 1, 0), (256, 8, 1), (96, 3, 1)):
        b = Batch(spec, ns, dxs, prec)
        b.set_schedule(threads, bps, order)
        b.upload(states)
        b.run(40, 1e-4, spec["cfl"])
        outs.append((b.download(), b.get()))
    for got, info in outs[1:]:
        for t in range(len(ns)):
            assert np.array_equal(got[t], outs[0][0][t])
        assert np.array_equal(info[0], outs[0][1][0]) and np.array_equal(info[1], outs[0][1][1])
