"""Mixed-precision path (FP32 storage/fluxes, FP64 accumulation) vs FP64.

Bar (the benchmark's): per-variable relative L1 <= 1e-5 against the FP64
path on the 3D blast; looser bounds on the small golden problems, where a
few FP32-rounded steps of strongly non-linear flows are compared with the
reference binary directly.
"""
import numpy as np
import pytest

import userdef_cases
from conftest import GOLDEN_NAMES, load_golden, rel_l1

pytestmark = pytest.mark.gpu


def _s(spec, precision):
    from pluto_gb300 import Solver
    s = Solver(spec, precision=precision)
    if userdef_cases.has_userdef(spec):
        s.set_userdef(userdef_cases.make(spec))
        if spec.get("internal_boundary"):
            s.set_internal_boundary()
    return s


MIXED = ["mixed", "mixed_dw"]


def test_integer_conversions_match_hardware():
    """The mixed path's integer float<->double conversions (they keep the
    FP64 pipe free for the accumulation) give the IEEE conversions' bits
    (subnormals included): all 2^32 floats widened, 6 * 2^32 doubles
    narrowed (ties included)."""
    import ctypes as C
    from pluto_gb300 import _lib as L
    counts = (C.c_ulonglong * 2)()
    L.check(L.lib().pg_selftest_conversions(counts), "pg_selftest_conversions")
    assert list(counts) == [0, 0]


def _tma_cases():
    from pluto_gb300 import problems as P
    out = {}
    spec, vc, f = P.blast3d(32)                                 # PLM/MC + HLLD + CT, pitch 36
    out["blast3d_plm_ct"] = (spec, vc, f)
    spec, vc, f = P.turbulence3d(26)                             # PPM + RK3 + CT, pitch 32
    out["turb3d_ppm_rk3"] = (spec, vc, f)
    spec, vc, f = P.orszag_tang(36)                              # 2D, y sweep only
    out["ot2d_roe_minmod"] = (dict(spec, solver="roe", limiter="MINMOD_LIM"), vc, f)
    spec, vc, f = P.blast3d(28)
    out["blast3d_noct_hll_outflow"] = (dict(spec, ct=False, solver="hll", bc="outflow"), vc, f)
    return out


@pytest.mark.parametrize("prec", MIXED)
@pytest.mark.parametrize("case", ["blast3d_plm_ct", "turb3d_ppm_rk3", "ot2d_roe_minmod",
                                  "blast3d_noct_hll_outflow"])
def test_tma_sweeps_match_plain_sweeps(case, prec, monkeypatch):
    """The TMA-staged persistent sweeps are deterministic and compute what the
    directly-loading sweeps compute: same tiles and arithmetic, equal to FP32
    round-off (the compiler may contract a multiply-add differently in the
    two kernels, so single ulps can differ and then spread)."""
    spec, vc, f = _tma_cases()[case]
    out, names = {}, {}
    monkeypatch.setenv("PLUTO_GB300_SWEEP", "tile")  # y/z tiles, not the marching columns
    for tma in ("1", "1b", "0"):
        monkeypatch.setenv("PLUTO_GB300_SWEEP_TMA", tma[0])
        s = _s(spec, prec)
        s.upload(vc, f)
        names[tma] = set(s.profile_kernels(1, spec["first_dt"], spec["cfl"]))
        s.upload(vc, f)
        s.run(6, spec["first_dt"], spec["cfl"])
        out[tma] = s.download()
    for k in ("mixed_sweep_x_tma", "mixed_sweep_y_tma"):
        assert k in names["1"] and k not in names["0"], names
    assert np.array_equal(out["1"][0], out["1b"][0])
    errs = {q: rel_l1(out["1"][0][q], out["0"][0][q]) for q in range(8) if np.abs(out["0"][0][q]).sum() > 0}
    for d in range(3):
        if out["0"][1][d] is not None:
            assert np.array_equal(out["1"][1][d], out["1b"][1][d])
            errs[f"b{d}"] = rel_l1(out["1"][1][d], out["0"][1][d])
    assert max(errs.values()) <= 1e-6, errs


@pytest.mark.parametrize("prec", MIXED)
@pytest.mark.parametrize("case", ["blast3d_plm_ct", "turb3d_ppm_rk3", "ot2d_roe_minmod",
                                  "blast3d_noct_hll_outflow"])
@pytest.mark.parametrize("seg", ["0", "5"])
def test_marching_sweeps_match_tile_sweeps(case, prec, seg, monkeypatch):
    """The y/z sweeps that march along columns (the default) compute what the
    TMA tiles compute, to FP32 round-off, deterministically, for any segment
    length (5: segments that do not divide the grid)."""
    spec, vc, f = _tma_cases()[case]
    out, names = {}, {}
    monkeypatch.setenv("PLUTO_GB300_MARCH_SEG", seg)
    for mode in ("march", "march_b", "tile"):
        monkeypatch.setenv("PLUTO_GB300_SWEEP", mode.split("_")[0])
        s = _s(spec, prec)
        s.upload(vc, f)
        names[mode] = set(s.profile_kernels(1, spec["first_dt"], spec["cfl"]))
        s.upload(vc, f)
        s.run(6, spec["first_dt"], spec["cfl"])
        out[mode] = s.download()
    assert "mixed_sweep_y_march" in names["march"] and "mixed_sweep_y_march" not in names["tile"], names
    assert all(np.array_equal(out["march"][0][q], out["march_b"][0][q]) for q in range(8))
    errs = {q: rel_l1(out["march"][0][q], out["tile"][0][q]) for q in range(8)
            if np.abs(out["tile"][0][q]).sum() > 0}
    for d in range(3):
        if out["tile"][1][d] is not None:
            assert np.array_equal(out["march"][1][d], out["march_b"][1][d])
            errs[f"b{d}"] = rel_l1(out["march"][1][d], out["tile"][1][d])
    assert max(errs.values()) <= 1e-6, errs


@pytest.mark.parametrize("prec", MIXED)
@pytest.mark.parametrize("case", ["blast3d_plm_ct", "turb3d_ppm_rk3", "ot2d_roe_minmod"])
def test_marching_sweeps_independent_of_segment_length(case, prec, monkeypatch):
    """Conservation across segments: the interface two column segments share
    is solved by the same instructions from the same inputs in both, so the
    result does not depend on where the segments start -- bit for bit."""
    spec, vc, f = _tma_cases()[case]
    out = {}
    monkeypatch.setenv("PLUTO_GB300_SWEEP", "march")
    for seg in ("5", "7", "0"):
        monkeypatch.setenv("PLUTO_GB300_MARCH_SEG", seg)
        s = _s(spec, prec)
        s.upload(vc, f)
        s.run(6, spec["first_dt"], spec["cfl"])
        out[seg] = s.download()
    for seg in ("7", "0"):
        for q in range(8):
            assert np.array_equal(out["5"][0][q], out[seg][0][q]), (seg, q)
        for d in range(3):
            if out["5"][1][d] is not None:
                assert np.array_equal(out["5"][1][d], out[seg][1][d]), (seg, d)


def _mixed_scheme(name):
    """the mixed solvers take RK time stepping without CHAR_LIMITING and, under
    CT, the UCT_HLL edge average (CTU, characteristic limiting and the other
    averages run on the FP64 path)"""
    meta = load_golden(name)[0]
    return (meta["stepping"] in ("EULER", "RK2", "RK3") and not meta.get("char_limiting")
            and (not meta["ct"] or meta.get("emf", "UCT_HLL") == "UCT_HLL"))


RK_GOLDENS = [n for n in GOLDEN_NAMES if _mixed_scheme(n)]


@pytest.mark.parametrize("prec", MIXED)
@pytest.mark.parametrize("name", RK_GOLDENS)
def test_mixed_close_to_reference_goldens(name, prec):
    meta, vc0, bs0, vc1, bs1 = load_golden(name)
    s = _s(meta, prec)
    s.upload(vc0, bs0)
    s.run(meta["steps"], meta["first_dt"], meta["cfl"])
    vc, bs = s.download()
    errs = [rel_l1(vc[q], vc1[q]) for q in range(8) if np.abs(vc1[q]).sum() > 0]
    tol = 5e-3 if "floor" in name else 2e-4
    assert max(errs) <= tol, errs


@pytest.mark.parametrize("prec", MIXED)
def test_mixed_vs_fp64_blast_l1(prec):
    from pluto_gb300 import problems
    spec, vc, faces = problems.blast3d(48)
    out = {}
    for p in ("fp64", prec):
        s = _s(spec, p)
        s.upload(vc, faces)
        s.run(40, spec["first_dt"], spec["cfl"])
        out[p] = s.download()
    m = out[prec]
    errs = {q: rel_l1(m[0][q], out["fp64"][0][q]) for q in (0, 1, 2, 3, 4, 5, 6, 7)}
    for d in range(3):
        errs[f"b{d}"] = rel_l1(m[1][d], out["fp64"][1][d])
    assert max(errs.values()) <= 1e-5, errs


@pytest.mark.parametrize("prec", MIXED)
def test_mixed_divergence_free_to_fp32_roundoff(prec):
    from pluto_gb300 import problems
    spec, vc, faces = problems.blast3d(32)
    s = _s(spec, prec)
    s.upload(vc, faces)
    s.run(20, spec["first_dt"], spec["cfl"])
    _, b = s.download()
    div = (np.diff(b[0], axis=2) + np.diff(b[1], axis=1) + np.diff(b[2], axis=0))
    assert np.abs(div).max() <= 1e-5 * np.abs(b[0]).max()


def test_mixed_upload_roundtrip_is_fp32_rounding():
    from pluto_gb300 import problems
    spec, vc, faces = problems.blast3d(16)
    vc = vc + 1e-3 * np.random.default_rng(0).random(vc.shape)
    s = _s(spec, "mixed")
    s.upload(vc, faces)
    v2, b2 = s.download()
    assert np.array_equal(v2, vc.astype(np.float32).astype(np.float64))


@pytest.mark.parametrize("prec", MIXED)
def test_mixed_rk3_ppm_turbulence_small(prec):
    from pluto_gb300 import problems
    spec, vc, faces = problems.turbulence3d(24, seed=1)
    out = {}
    for p in ("fp64", prec):
        s = _s(spec, p)
        s.upload(vc, faces)
        s.run(10, spec["first_dt"], spec["cfl"])
        out[p] = s.download()[0]
    errs = [rel_l1(out[prec][q], out["fp64"][q]) for q in range(8)]
    assert max(errs) <= 1e-5, errs


def _padded_cases():
    """Grids whose ghosted rows are not a multiple of 4 floats: the mixed
    solvers pad the row pitch (TMA sweeps) unless the TMA sweeps are off."""
    from pluto_gb300 import problems as P
    out = {}
    spec, vc, f = P.blast3d(30)                                  # rows 34 -> pitch 36
    out["blast3d_30"] = (spec, vc, f)
    spec, vc, f = P.turbulence3d(24)                             # PPM: rows 30 -> pitch 32
    out["turb3d_24_ppm_rk3"] = (spec, vc, f)
    meta = load_golden("ot_userdef_32")[0]                       # USERDEF side + CT, 2D
    spec, vc, f = P.orszag_tang(30)
    out["ot2d_30_userdef"] = (dict(meta, nx=spec["nx"], dx=spec["dx"]), vc, f)
    meta = load_golden("ot_internal_32")[0]                      # INTERNAL_BOUNDARY, flags moved
    out["ot2d_30_internal"] = (dict(meta, nx=spec["nx"], dx=spec["dx"]), vc, f)
    meta = load_golden("blast_userdef_ct_16")[0]                 # 3D USERDEF sides + CT
    spec, vc, f = P.blast3d(18)
    out["blast3d_18_userdef_ct"] = (dict(meta, nx=spec["nx"], dx=spec["dx"]), vc, f)
    return out


@pytest.mark.parametrize("prec", MIXED)
@pytest.mark.parametrize("case", ["blast3d_30", "turb3d_24_ppm_rk3", "ot2d_30_userdef", "ot2d_30_internal",
                                  "blast3d_18_userdef_ct"])
def test_padded_rows_match_unpadded(case, prec, monkeypatch):
    """With padded rows the TMA sweeps run (and every transfer, boundary,
    user callback and flag copy maps the pitch); the result equals the
    unpadded direct-load solver to FP32 round-off, and stays within the
    mixed bar of the FP64 path."""
    spec, vc, f = _padded_cases()[case]
    out, names = {}, {}
    monkeypatch.setenv("PLUTO_GB300_SWEEP", "tile")  # y/z tiles, not the marching columns
    for tma in ("1", "0"):
        monkeypatch.setenv("PLUTO_GB300_SWEEP_TMA", tma)
        s = _s(spec, prec)
        s.upload(vc, f)
        names[tma] = set(s.profile_kernels(1, spec["first_dt"], spec["cfl"]))
        s.upload(vc, f)
        s.run(6, spec["first_dt"], spec["cfl"])
        out[tma] = s.download()
    assert "mixed_sweep_y_tma" in names["1"] and "mixed_sweep_y_tma" not in names["0"], names
    ref = _s(spec, "fp64")
    ref.upload(vc, f)
    ref.run(6, spec["first_dt"], spec["cfl"])
    want = ref.download()
    for other, bar in ((out["0"], 1e-6), (want, 1e-5)):
        errs = {q: rel_l1(out["1"][0][q], other[0][q]) for q in range(8) if np.abs(other[0][q]).sum() > 0}
        for d in range(3):
            if other[1][d] is not None:
                errs[f"b{d}"] = rel_l1(out["1"][1][d], other[1][d])
        assert max(errs.values()) <= bar, errs


@pytest.mark.parametrize("prec", MIXED)
def test_tile_wait_timeout_is_reported_and_recoverable(prec, monkeypatch):
    """A TMA tile wait that runs out (forced: a try limit of 0 through
    PLUTO_GB300_TILE_WAIT_TRIES; the waits that drain copies in flight keep
    their normal limit) makes the sweep kernels return, pg_advance report
    PG_ERR_TIMEOUT, and leaves the solver usable: after a new upload the next
    step equals a fresh solver's step bit for bit."""
    from pluto_gb300 import Solver, problems
    from pluto_gb300._lib import PG_ERR_TIMEOUT, PgError
    spec, vc, f = problems.blast3d(32)
    dt = spec["first_dt"]
    s = _s(spec, prec)
    s.upload(vc, f)
    monkeypatch.setenv("PLUTO_GB300_TILE_WAIT_TRIES", "0")
    with pytest.raises(PgError) as err:
        s.advance(dt)
    assert err.value.code == PG_ERR_TIMEOUT
    monkeypatch.delenv("PLUTO_GB300_TILE_WAIT_TRIES")
    s.upload(vc, f)
    got = s.advance(dt), s.download()
    ref = _s(spec, prec)
    ref.upload(vc, f)
    want = ref.advance(dt), ref.download()
    assert got[0] == want[0]
    assert np.array_equal(got[1][0], want[1][0])
    for d in range(3):
        assert np.array_equal(got[1][1][d], want[1][1][d])
