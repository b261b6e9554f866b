"""FP64 CUDA path vs the reference (golden dumps) and vs the CPU oracle.

Bar: relative L1 <= 1e-10 per variable after the fixed number of steps
(the FP64 path is built without FMA contraction and is expected to agree
bit for bit, which ``test_fp64_bitwise_on_goldens`` checks).
"""
import numpy as np
import pytest

import userdef_cases
from conftest import GOLDEN_NAMES, load_golden, rel_l1

pytestmark = pytest.mark.gpu

TOL = 1e-10


def _solver(meta, precision="fp64", **kw):
    from pluto_gb300 import Solver
    s = Solver(meta, precision=precision, **kw)
    if userdef_cases.has_userdef(meta):
        s.set_userdef(userdef_cases.make(meta))
        if meta.get("internal_boundary"):
            s.set_internal_boundary()
    return s


def _errors(vc, bs, vc_ref, bs_ref):
    errs = {f"v{q}": rel_l1(vc[q], vc_ref[q]) for q in range(8)}
    for d in range(3):
        if bs_ref[d] is not None:
            errs[f"b{d}"] = rel_l1(bs[d], bs_ref[d])
    return errs


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_fp64_matches_reference_goldens(name):
    meta, vc0, bs0, vc1, bs1 = load_golden(name)
    s = _solver(meta)
    s.upload(vc0, bs0)
    t, _ = s.run(meta["steps"], meta["first_dt"], meta["cfl"])
    vc, bs = s.download()
    errs = _errors(vc, bs, vc1, bs1)
    assert max(errs.values()) <= TOL, errs
    assert abs(t - meta["t_final"]) <= 1e-6 * meta["t_final"]


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_fp64_bitwise_on_goldens(name):
    meta, vc0, bs0, vc1, bs1 = load_golden(name)
    s = _solver(meta)
    s.upload(vc0, bs0)
    s.run(meta["steps"], meta["first_dt"], meta["cfl"])
    vc, bs = s.download()
    assert np.array_equal(vc, vc1)
    for d in range(3):
        if bs1[d] is not None:
            assert np.array_equal(bs[d], bs1[d])


def test_advance_matches_oracle_step_by_step():
    """pg_advance (the AdvanceStep drop-in): host dt in, invDt_hyp out."""
    from oracle.oracle import Oracle
    meta, vc0, bs0, _, _ = load_golden("blast_floor_16")
    s = _solver(meta)
    o = Oracle(meta, nthreads=4)
    s.upload(vc0, bs0)
    o.set_state(vc0, bs0)
    dt = meta["first_dt"]
    for step in range(6):
        inv_g, _, nf_g = s.advance(dt)
        inv_o, _, nf_o = o.advance(dt)
        assert inv_g == inv_o, (step, inv_g, inv_o)
        assert nf_g == nf_o
        dt = min((1.0 / inv_o) * meta["cfl"], 1.1 * dt)
    vc, bs = s.download()
    vo, bo = o.get_state()
    assert np.array_equal(vc, vo)


def _random_blast(n, seed):
    rng = np.random.default_rng(seed)
    x = (np.arange(n) + 0.5) / n - 0.5
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    r = np.sqrt(X**2 + Y**2 + Z**2)
    vc = np.zeros((8, n, n, n))
    vc[0] = 1.0 + 0.1 * rng.random((n, n, n))
    vc[7] = np.where(r < 0.15, 10.0, 0.1) * (1 + 0.05 * rng.random((n, n, n)))
    vc[1:4] = 0.2 * (rng.random((3, n, n, n)) - 0.5)
    b0 = 10.0 / np.sqrt(3.0) / np.sqrt(4 * np.pi)
    bs = [np.full((n, n, n + 1), b0), np.full((n, n + 1, n), b0), np.full((n + 1, n, n), b0)]
    vc[4] = 0.5 * (bs[0][:, :, 1:] + bs[0][:, :, :-1])
    vc[5] = 0.5 * (bs[1][:, 1:, :] + bs[1][:, :-1, :])
    vc[6] = 0.5 * (bs[2][1:, :, :] + bs[2][:-1, :, :])
    spec = dict(dims=3, components=3, nx=(n, n, n), dx=(1 / n, 1 / n, 1 / n), gamma=5 / 3,
                recon="LINEAR", limiter="MC_LIM", solver="hlld", stepping="RK2", ct=True,
                bc="periodic")
    return spec, vc, bs


@pytest.mark.parametrize("solver,recon,stepping", [("hlld", "LINEAR", "RK2"), ("hll", "PARABOLIC", "RK3"),
                                                   ("hlld", "PARABOLIC", "RK2"), ("roe", "PARABOLIC", "RK3")])
def test_fp64_vs_oracle_random_3d(solver, recon, stepping):
    from oracle.oracle import Oracle
    spec, vc, bs = _random_blast(24, seed=7)
    spec.update(solver=solver, recon=recon, stepping=stepping)
    s = _solver(spec)
    o = Oracle(spec, nthreads=4)
    s.upload(vc, bs)
    o.set_state(vc, bs)
    s.run(4, 1e-3, 0.3)
    o.run(4, 1e-3, 0.3)
    a, ab = s.download()
    b, bb = o.get_state()
    errs = _errors(a, ab, b, bb)
    assert max(errs.values()) <= TOL, errs


@pytest.mark.parametrize("bc", [("outflow", "outflow", "outflow"), ("outflow", "periodic", "outflow"),
                                ("periodic", "outflow", "periodic"), ("reflective", "eqtsymmetric", "reflective"),
                                ("eqtsymmetric", "periodic", "outflow"),
                                (("reflective", "outflow"), ("outflow", "eqtsymmetric"), ("eqtsymmetric", "reflective")),
                                (("userdef", "outflow"), "periodic", ("reflective", "userdef"))])
def test_fp64_vs_oracle_outflow_ct_3d(bc):
    """Outflow, reflective and equatorial-symmetric sides under CT
    (FillMagneticField, normal averaging on outflow sides, FlipSign mirror
    signs), mixed with periodic axes, on a random 3D state against the
    oracle."""
    from oracle.oracle import Oracle
    spec, vc, bs = _random_blast(20, seed=5)
    spec.update(bc=list(bc), solver="roe", recon="PARABOLIC", stepping="RK3")
    s = _solver(spec)
    o = Oracle(spec, nthreads=4)
    if userdef_cases.has_userdef(spec):
        o.set_userdef(userdef_cases.make(spec))
    s.upload(vc, bs)
    o.set_state(vc, bs)
    s.run(4, 1e-3, 0.3)
    o.run(4, 1e-3, 0.3)
    a, ab = s.download()
    b, bb = o.get_state()
    assert np.array_equal(a, b), _errors(a, ab, b, bb)
    for d in range(3):
        assert np.array_equal(ab[d], bb[d])


@pytest.mark.parametrize("emf,solver,stepping,bc", [
    ("ARITHMETIC", "hlld", "RK2", "periodic"),
    ("UCT_CONTACT", "roe", "RK3", "periodic"),
    ("UCT0", "hll", "RK2", "periodic"),
    ("UCT_CONTACT", "hlld", "RK2", [("reflective", "outflow"), "periodic", ("outflow", "eqtsymmetric")]),
    ("UCT0", "hlld", "EULER", ["outflow", "outflow", "periodic"]),
    ("ARITHMETIC", "roe", "RK2", [("userdef", "outflow"), "periodic", ("reflective", "userdef")])])
def test_rk_emf_averages_vs_oracle_random_3d(emf, solver, stepping, bc):
    """RK time stepping with the ARITHMETIC, UCT0 and UCT_CONTACT edge
    averages (face EMFs stored by the Riemann kernel, corner integration in
    every stage) on a random 3D state against the oracle, bit for bit."""
    from oracle.oracle import Oracle
    spec, vc, bs = _random_blast(16, seed=21)
    spec.update(emf=emf, solver=solver, stepping=stepping, bc=bc)
    s = _solver(spec)
    o = Oracle(spec, nthreads=4)
    if userdef_cases.has_userdef(spec):
        o.set_userdef(userdef_cases.make(spec))
    s.upload(vc, bs)
    o.set_state(vc, bs)
    s.run(4, 1e-3, 0.3)
    o.run(4, 1e-3, 0.3)
    a, ab = s.download()
    b, bb = o.get_state()
    assert np.array_equal(a, b), _errors(a, ab, b, bb)
    for d in range(3):
        assert np.array_equal(ab[d], bb[d])


def test_divergence_free_under_ct():
    spec, vc, bs = _random_blast(24, seed=3)
    s = _solver(spec)
    s.upload(vc, bs)
    s.run(8, 1e-3, 0.3)
    _, b = s.download()
    n = spec["nx"][0]
    div = (b[0][:, :, 1:] - b[0][:, :, :-1] + b[1][:, 1:, :] - b[1][:, :-1, :] + b[2][1:, :, :] - b[2][:-1, :, :]) * n
    bmag = np.abs(b[0]).max()
    assert np.abs(div).max() * (1.0 / n) <= 1e-12 * bmag


def test_fp64_deterministic():
    spec, vc, bs = _random_blast(16, seed=11)
    out = []
    for _ in range(2):
        s = _solver(spec)
        s.upload(vc, bs)
        s.run(3, 1e-3, 0.3)
        out.append(s.download()[0])
    assert np.array_equal(out[0], out[1])


def test_upload_download_roundtrip():
    spec, vc, bs = _random_blast(12, seed=5)
    s = _solver(spec)
    s.upload(vc, bs)
    v2, b2 = s.download()
    assert np.array_equal(v2, vc)
    for d in range(3):
        assert np.array_equal(b2[d], bs[d])


def test_nan_state_reported_not_trapped():
    """A corrupted state yields an error status from the step, not a fault."""
    from pluto_gb300._lib import PgError
    spec, vc, bs = _random_blast(12, seed=5)
    vc[7, 3, 3, 3] = np.nan
    s = _solver(spec)
    s.upload(vc, bs)
    with pytest.raises(PgError) as e:
        s.advance(1e-3)
    assert e.value.code == 4


@pytest.mark.parametrize("emf,solver,bc,stepping", [
    ("UCT_CONTACT", "hlld", "periodic", "HANCOCK"), ("ARITHMETIC", "hll", "outflow", "HANCOCK"),
    ("UCT_CONTACT", "roe", "outflow", "HANCOCK"),
    ("UCT_CONTACT", "hlld", ["reflective", "periodic", "eqtsymmetric"], "HANCOCK"),
    ("ARITHMETIC", "roe", [("outflow", "reflective"), "periodic", ("eqtsymmetric", "outflow")], "HANCOCK"),
    ("UCT_CONTACT", "hlld", [("userdef", "outflow"), "periodic", ("outflow", "userdef")], "HANCOCK"),
    ("UCT0", "hlld", "periodic", "HANCOCK"),
    ("UCT0", "roe", [("outflow", "reflective"), "periodic", "outflow"], "HANCOCK"),
    ("UCT_CONTACT", "hlld", "periodic", "HANCOCK_CONS"),
    ("ARITHMETIC", "roe", "outflow", "HANCOCK_CONS"),
    ("UCT0", "hll", [("reflective", "outflow"), "periodic", ("eqtsymmetric", "userdef")], "HANCOCK_CONS")])
def test_ctu_vs_oracle_random_3d(emf, solver, bc, stepping):
    """CTU (primitive or conservative Hancock predictor, corner-coupled
    corrector) with CT on a random 3D state against the oracle, bit for bit."""
    from oracle.oracle import Oracle
    spec, vc, bs = _random_blast(16, seed=9)
    spec.update(stepping=stepping, emf=emf, solver=solver, bc=bc, limiter="MC_LIM")
    s = _solver(spec)
    o = Oracle(spec, nthreads=4)
    if userdef_cases.has_userdef(spec):
        o.set_userdef(userdef_cases.make(spec))
    s.upload(vc, bs)
    o.set_state(vc, bs)
    s.run(4, 1e-3, 0.3)
    o.run(4, 1e-3, 0.3)
    a, ab = s.download()
    b, bb = o.get_state()
    assert np.array_equal(a, b), _errors(a, ab, b, bb)
    for d in range(3):
        assert np.array_equal(ab[d], bb[d])


@pytest.mark.parametrize("emf,solver,bc", [("UCT_CONTACT", "hlld", "periodic"), ("ARITHMETIC", "roe", "outflow"),
                                           ("UCT_CONTACT", "hll", [("reflective", "outflow"), "periodic",
                                                                   ("eqtsymmetric", "outflow")]),
                                           ("UCT_CONTACT", "hlld", [("userdef", "outflow"), "periodic",
                                                                    ("outflow", "userdef")])])
def test_char_tracing_vs_oracle_random_3d(emf, solver, bc):
    """CTU with the characteristic tracing predictor on a random 3D state
    against the oracle, bit for bit."""
    from oracle.oracle import Oracle
    spec, vc, bs = _random_blast(16, seed=12)
    spec.update(stepping="CHARACTERISTIC_TRACING", emf=emf, solver=solver, bc=bc, limiter="MC_LIM")
    s = _solver(spec)
    o = Oracle(spec, nthreads=4)
    if userdef_cases.has_userdef(spec):
        o.set_userdef(userdef_cases.make(spec))
    s.upload(vc, bs)
    o.set_state(vc, bs)
    s.run(4, 1e-3, 0.3)
    o.run(4, 1e-3, 0.3)
    a, ab = s.download()
    b, bb = o.get_state()
    assert np.array_equal(a, b), _errors(a, ab, b, bb)
    for d in range(3):
        assert np.array_equal(ab[d], bb[d])


@pytest.mark.parametrize("limiter,stepping,extra", [("MC_LIM", "RK2", {}), ("DEFAULT", "RK3", {}),
                                                    ("MINMOD_LIM", "RK2", {"ct": False}),
                                                    ("VANLEER_LIM", "CHARACTERISTIC_TRACING",
                                                     {"emf": "UCT_CONTACT", "bc": "outflow"}),
                                                    ("DEFAULT", "HANCOCK", {"emf": "ARITHMETIC"}),
                                                    ("MC_LIM", "RK3", {"recon": "PARABOLIC"}),
                                                    ("MC_LIM", "CHARACTERISTIC_TRACING",
                                                     {"recon": "PARABOLIC", "emf": "UCT_CONTACT"})])
def test_char_limiting_vs_oracle_random_3d(limiter, stepping, extra):
    """CHAR_LIMITING YES on a random 3D state against the oracle, bit for bit."""
    from oracle.oracle import Oracle
    spec, vc, bs = _random_blast(16, seed=21)
    spec.update(char_limiting=True, limiter=limiter, stepping=stepping, **extra)
    s = _solver(spec)
    o = Oracle(spec, nthreads=4)
    s.upload(vc, bs)
    o.set_state(vc, bs)
    s.run(4, 1e-3, 0.3)
    o.run(4, 1e-3, 0.3)
    a, ab = s.download()
    b, bb = o.get_state()
    assert np.array_equal(a, b), _errors(a, ab, b, bb)
    if spec.get("ct", True):
        for d in range(3):
            assert np.array_equal(ab[d], bb[d])


@pytest.mark.parametrize("emf,solver,bc", [("UCT_CONTACT", "hlld", "periodic"), ("ARITHMETIC", "hll", "outflow"),
                                           ("UCT_CONTACT", "roe", [("reflective", "outflow"), "periodic",
                                                                   ("eqtsymmetric", "outflow")])])
def test_ppm_char_tracing_vs_oracle_random_3d(emf, solver, bc):
    """CTU with parabolic states and characteristic tracing on a random 3D
    state against the oracle, bit for bit."""
    from oracle.oracle import Oracle
    spec, vc, bs = _random_blast(16, seed=31)
    spec.update(recon="PARABOLIC", stepping="CHARACTERISTIC_TRACING", emf=emf, solver=solver, bc=bc)
    s = _solver(spec)
    o = Oracle(spec, nthreads=4)
    s.upload(vc, bs)
    o.set_state(vc, bs)
    s.run(4, 1e-3, 0.3)
    o.run(4, 1e-3, 0.3)
    a, ab = s.download()
    b, bb = o.get_state()
    assert np.array_equal(a, b), _errors(a, ab, b, bb)
    for d in range(3):
        assert np.array_equal(ab[d], bb[d])


def test_char_tracing_without_ct_vs_oracle_3d():
    """Characteristic tracing with cell-centred fields only (no CT)."""
    from oracle.oracle import Oracle
    spec, vc, bs = _random_blast(16, seed=13)
    spec.update(stepping="CHARACTERISTIC_TRACING", ct=False, solver="hlld", limiter="MINMOD_LIM")
    s = _solver(spec)
    o = Oracle(spec, nthreads=4)
    s.upload(vc, bs)
    o.set_state(vc, bs)
    s.run(4, 1e-3, 0.3)
    o.run(4, 1e-3, 0.3)
    a, _ = s.download()
    b, _ = o.get_state()
    assert np.array_equal(a, b)


@pytest.mark.parametrize("stepping,emf", [("HANCOCK", "UCT_CONTACT"), ("HANCOCK", "UCT0"), ("RK2", "UCT_CONTACT"),
                                          ("HANCOCK_CONS", "UCT_CONTACT"),
                                          ("RK3", "UCT0"), ("RK2", "ARITHMETIC")])
def test_ctu_tangent_value_part_is_the_fp64_step(stepping, emf):
    """The value part of the tangent-linear build (dual numbers) is the
    plain FP64 step, for CTU and for RK with the non-UCT_HLL averages."""
    from pluto_gb300.adjoint import tangent_linear
    spec, vc, bs = _random_blast(12, seed=4)
    spec.update(stepping=stepping, emf=emf)
    s = _solver(spec)
    s.upload(vc, bs)
    dts = [1e-3] * 3
    for dt in dts:
        s.advance(dt)
    want, wb = s.download()
    rng = np.random.default_rng(3)
    (got, gb), _ = tangent_linear(spec, dts, vc, bs, rng.normal(size=vc.shape),
                                  [rng.normal(size=f.shape) for f in bs])
    assert np.array_equal(got, want)
    for d in range(3):
        assert np.array_equal(gb[d], wb[d])
