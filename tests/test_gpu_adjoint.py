"""Differentiated FP64 path: tangent-linear model and hand-written adjoint.

Checks, all with a frozen dt sequence:
- the tangent-linear value part is the plain FP64 step bit for bit;
- dot-product test <lambda, TL(delta)> == <adjoint(lambda), delta> for PLM
  and PPM, HLL and HLLD, 1D outflow / 2D / 3D constrained transport,
  outflow / reflective / equatorial-symmetric sides under constrained
  transport, RK2, RK3 and EULER stepping;
- TL against central finite differences of the state;
- the CP-Alfven objective (128^2, 256 steps, checkpoint every 16): the
  autograd gradient against the tangent-linear derivative (exact transpose)
  and against central differences taken with the double-double step inside
  the kink margin (the distance to the nearest branch switch), <= 1e-6;
- at the CP-Alfven initial condition itself the kink margin is 0.
"""
import math

import numpy as np
import pytest

from conftest import load_golden, rel_l1

pytestmark = pytest.mark.gpu


def _inner(a_vc, a_f, b_vc, b_f):
    s = float(np.dot(a_vc.ravel(), b_vc.ravel()))
    for d in range(3):
        if a_f[d] is not None and b_f[d] is not None:
            s += float(np.dot(a_f[d].ravel(), b_f[d].ravel()))
    return s


def _random_like(rng, vc, faces):
    return rng.normal(size=vc.shape), [rng.normal(size=f.shape) if f is not None else None for f in faces]


def _case(name):
    from pluto_gb300 import problems as P
    if name == "cpa2d_plm_hlld":
        spec, vc, f = P.cp_alfven(24)
        return spec, vc, f, [2e-3] * 5
    if name == "ot2d_plm_hll":
        spec, vc, f = P.orszag_tang(20)
        return dict(spec, solver="hll"), vc, f, [1e-3] * 4
    if name == "turb3d_ppm_hlld":
        spec, vc, f = P.turbulence3d(10)
        return dict(spec, stepping="RK2"), vc, f, [1e-3] * 3
    if name == "turb3d_plm_minmod_hll":
        spec, vc, f = P.turbulence3d(8, seed=3)
        return dict(spec, stepping="RK2", recon="LINEAR", limiter="MINMOD_LIM", solver="hll"), vc, f, [1e-3] * 3
    if name == "tube1d_outflow":
        spec, vc, f = P.riemann_tube(64, 5)
        return spec, vc, f, [1e-3] * 6
    if name == "cpa2d_plm_roe":
        spec, vc, f = P.cp_alfven(20)
        return dict(spec, solver="roe"), vc, f, [2e-3] * 4
    if name == "tube1d_ppm_outflow":
        spec, vc, f = P.riemann_tube(48, 2)
        return dict(spec, recon="PARABOLIC", limiter="MC_LIM"), vc, f, [1e-3] * 6
    if name == "tube1d_reflective":
        spec, vc, f = P.riemann_tube(48, 1)
        return dict(spec, bc="reflective"), vc, f, [1e-3] * 5
    if name == "tube1d_sides":
        spec, vc, f = P.riemann_tube(48, 0)
        return dict(spec, bc=[("reflective", "outflow"), "outflow", "outflow"]), vc, f, [1e-3] * 5
    if name == "ot2d_mirror_noct":
        spec, vc, f = P.orszag_tang(16)
        return dict(spec, ct=False, bc=["reflective", "eqtsymmetric", "periodic"]), vc, f, [1e-3] * 3
    # non-periodic sides under CT: the axis-by-axis fill with the normal field
    # from div B = 0 (and its cell averages on outflow sides), transposed
    if name == "ot2d_outflow_ct":
        spec, vc, f = P.orszag_tang(16)
        return dict(spec, bc="outflow"), vc, f, [1e-3] * 4
    if name == "cpa2d_mirror_ct":
        spec, vc, f = P.cp_alfven(16)
        return dict(spec, bc=["reflective", "eqtsymmetric", "periodic"]), vc, f, [2e-3] * 3
    if name == "blast3d_outflow_ct":
        spec, vc, f = P.blast3d(10)
        return dict(spec, bc="outflow"), vc, f, [1e-3] * 3
    if name == "turb3d_sides_ct":
        spec, vc, f = P.turbulence3d(8, seed=5)
        return (dict(spec, stepping="RK2", recon="LINEAR", bc=[("outflow", "reflective"), "periodic", "outflow"]),
                vc, f, [1e-3] * 3)
    # RK3 (the turbulence configuration's stepping) and EULER
    if name == "turb3d_ppm_rk3":
        spec, vc, f = P.turbulence3d(8, seed=2)
        return spec, vc, f, [1e-3] * 3
    if name == "blast3d_outflow_rk3":
        spec, vc, f = P.blast3d(8)
        return dict(spec, stepping="RK3", bc="outflow"), vc, f, [1e-3] * 2
    if name == "ot2d_euler":
        spec, vc, f = P.orszag_tang(16)
        return dict(spec, stepping="EULER"), vc, f, [5e-4] * 4
    raise KeyError(name)


CASES = ["cpa2d_plm_hlld", "ot2d_plm_hll", "turb3d_ppm_hlld", "turb3d_plm_minmod_hll",
         "tube1d_outflow", "tube1d_ppm_outflow", "cpa2d_plm_roe", "tube1d_reflective", "ot2d_mirror_noct",
         "tube1d_sides", "ot2d_outflow_ct", "cpa2d_mirror_ct", "blast3d_outflow_ct", "turb3d_sides_ct",
         "turb3d_ppm_rk3", "blast3d_outflow_rk3", "ot2d_euler"]


def _smooth(vc):
    """Non-constant smooth density and pressure: the limiters of a state with
    exactly constant fields sit on their kinks (zero slopes), where central
    differences do not converge to the derivative of either branch."""
    out = vc.copy()
    idx = np.indices(vc.shape[1:])
    phase = sum((k + 1) * 2 * np.pi * idx[a] / vc.shape[1 + a] for k, a in enumerate(range(idx.shape[0])))
    out[0] = vc[0] * (1 + 0.1 * np.sin(phase + 0.3))
    out[7] = vc[7] * (1 + 0.1 * np.cos(phase + 0.7))
    return out


def _generic_2d(vc, f, rng, sigma, dx, dy):
    """A nearby generic point of a 2D CT state: seeded noise on density,
    velocity and pressure, and on the faces the discrete curl of a noisy
    corner vector potential (divergence stays zero; cell B = face average).
    Symmetric initial conditions put limiters exactly on their kinks (equal
    neighbours, zero slopes); there central differences converge to the mean
    of the one-sided derivatives instead of the derivative of the branch."""
    v = vc.copy()
    for q in (0, 1, 2, 3, 7):
        v[q] = v[q] + sigma * rng.normal(size=v[q].shape)
    ny, nx = v.shape[2], v.shape[3]
    az = sigma * min(dx, dy) * rng.normal(size=(ny, nx))  # corner (i+1/2, j+1/2), periodic
    bx = f[0].copy()
    by = f[1].copy()
    bx[0, :, 1:] += (az - np.roll(az, 1, axis=0)) / dy   # dAz/dy
    bx[0, :, 0] = bx[0, :, -1]
    by[0, 1:, :] -= (az - np.roll(az, 1, axis=1)) / dx   # -dAz/dx
    by[0, 0, :] = by[0, -1, :]
    v[4, 0] = 0.5 * (bx[0, :, 1:] + bx[0, :, :-1])
    v[5, 0] = 0.5 * (by[0, 1:, :] + by[0, :-1, :])
    return v, [bx, by, None]


def _smooth_generic_2d(vc, f, rng, sigma, dx, dy, kmax=3):
    """A smooth generic point next to a 2D CT state: random low-wavenumber
    periodic modes (seeded) of amplitude sigma on density, velocity and
    pressure, and on the faces the discrete curl of such a corner vector
    potential.  It leaves no exact ties in the limiters (as the symmetric
    initial condition has) and few near-ties (as a noisy state has)."""
    v = vc.copy()
    ny, nx = v.shape[2], v.shape[3]

    def field(xs, ys):
        X, Y = np.meshgrid(xs, ys, indexing="xy")
        out = np.zeros_like(X)
        for kx in range(1, kmax + 1):
            for ky in range(1, kmax + 1):
                out += rng.normal() * np.sin(2 * np.pi * (kx * X + ky * Y) + rng.uniform(0, 2 * np.pi))
        return out / kmax

    xc, yc = (np.arange(nx) + 0.5) / nx, (np.arange(ny) + 0.5) / ny
    for q in (0, 1, 2, 3, 6, 7):  # every cell variable that has no face (Bz too)
        v[q, 0] = v[q, 0] + sigma * field(xc, yc)
    az = sigma * min(dx, dy) * nx / (2 * np.pi) * field((np.arange(nx) + 1.0) / nx, (np.arange(ny) + 1.0) / ny)
    bx = f[0].copy()
    by = f[1].copy()
    bx[0, :, 1:] += (az - np.roll(az, 1, axis=0)) / dy
    bx[0, :, 0] = bx[0, :, -1]
    by[0, 1:, :] -= (az - np.roll(az, 1, axis=1)) / dx
    by[0, 0, :] = by[0, -1, :]
    v[4, 0] = 0.5 * (bx[0, :, 1:] + bx[0, :, :-1])
    v[5, 0] = 0.5 * (by[0, 1:, :] + by[0, :-1, :])
    return v, [bx, by, None]


def _faces(spec, f):
    return [f[d] if (spec.get("ct", True) and d < spec["dims"]) else None for d in range(3)]


@pytest.mark.parametrize("name", ["cpa2d_plm_hlld", "turb3d_ppm_hlld"])
def test_tangent_value_part_is_the_fp64_step(name):
    from pluto_gb300 import Solver
    from pluto_gb300.adjoint import tangent_linear
    spec, vc, f, dts = _case(name)
    f = _faces(spec, f)
    s = Solver(spec, "fp64")
    s.upload(vc, f)
    for dt in dts:
        s.advance(dt)
    want_vc, want_f = s.download()
    rng = np.random.default_rng(1)
    dvc, df = _random_like(rng, vc, f)
    (got_vc, got_f), _ = tangent_linear(spec, dts, vc, f, dvc, df)
    assert np.array_equal(got_vc, want_vc)
    for d in range(3):
        if want_f[d] is not None:
            assert np.array_equal(got_f[d], want_f[d])


@pytest.mark.parametrize("name", CASES)
def test_adjoint_dot_product(name):
    from pluto_gb300.adjoint import Rollout, tangent_linear
    spec, vc, f, dts = _case(name)
    f = _faces(spec, f)
    rng = np.random.default_rng(11)
    dvc, df = _random_like(rng, vc, f)
    lvc, lf = _random_like(rng, vc, f)
    _, (tvc, tf) = tangent_linear(spec, dts, vc, f, dvc, df)
    r = Rollout(spec, dts, every=2)
    r.run(vc, f, checkpoint=True)
    avc, af = r.gradient(lvc, lf)
    lhs = _inner(lvc, lf, tvc, tf)
    rhs = _inner(avc, af, dvc, df)
    assert abs(lhs - rhs) <= 1e-11 * max(abs(lhs), abs(rhs)), (lhs, rhs)


@pytest.mark.parametrize("name", ["cpa2d_plm_hlld", "turb3d_ppm_rk3", "ot2d_euler", "blast3d_outflow_ct",
                                  "tube1d_ppm_outflow"])
def test_gradient_from_step_slots_matches_per_step_recomputation(name):
    """The gradient that recomputes each step once into per-step slots
    (adjoint_forward / adjoint_reverse) equals the one that rebuilds the step
    states and lets every adjoint_step recompute its step, to round-off: the
    forward states are identical, and the reversal's scatter adds (FP64
    atomics) make any two runs differ in the last bits (2.7e-16 relative seen
    here).  Segments of 2 steps over an odd count, so the last segment is
    partial."""
    from pluto_gb300.adjoint import Rollout
    spec, vc, f, dts = _case(name)
    f = _faces(spec, f)
    dts = (list(dts) * 3)[:5]
    rng = np.random.default_rng(3)
    lvc, lf = _random_like(rng, vc, f)
    out = {}
    for slots in (True, False):
        r = Rollout(spec, dts, every=2)
        r.run(vc, f, checkpoint=True)
        out[slots] = r.gradient(lvc, lf, slots=slots)
    assert r.solver.adjoint_slots(1)  # small grids: the slots fit
    r.solver.adjoint_slots(0)
    (av, af), (bv, bf) = out[True], out[False]
    scale = np.abs(bv).max()
    assert np.abs(av - bv).max() <= 1e-12 * scale
    for d in range(3):
        if bf[d] is not None:
            assert np.abs(af[d] - bf[d]).max() <= 1e-12 * max(scale, np.abs(bf[d]).max()), d


@pytest.mark.parametrize("name,emf", [("cpa2d_plm_hlld", None), ("turb3d_ppm_hlld", None),
                                     ("cpa2d_plm_hlld", "UCT0"), ("cpa2d_plm_hlld", "ARITHMETIC"),
                                     ("turb3d_ppm_rk3", None)])
def test_tangent_matches_central_differences(name, emf):
    """Tangent-linear step against central differences; also with the UCT0
    and ARITHMETIC edge averages of the RK path (no branch of their own) and
    with RK3 stepping. Periodic cases only: zero-gradient ghost copies make the
    one-sided slope at an outflow side exactly 0, a kink of the limiter for
    every perturbation, where central differences return the mean of the two
    branches (relative error ~4e-4 at every h on the 2D Orszag-Tang outflow
    case); the outflow adjoint is covered by the dot-product test."""
    from pluto_gb300 import Solver
    from pluto_gb300.adjoint import tangent_linear
    spec, vc, f, dts = _case(name)
    if emf:
        spec = dict(spec, emf=emf)
    f = _faces(spec, f)
    vc = _smooth(vc)
    rng = np.random.default_rng(5)
    if spec["dims"] == 2:
        vc, f = _generic_2d(vc, f, rng, 1e-3, spec["dx"][0], spec["dx"][1])
    dvc, df = _random_like(rng, vc, f)
    norm = math.sqrt(_inner(dvc, df, dvc, df))
    dvc = dvc / norm
    df = [x / norm if x is not None else None for x in df]
    _, (tvc, tf) = tangent_linear(spec, dts, vc, f, dvc, df)
    s = Solver(spec, "fp64")

    def run(h):
        s.upload(vc + h * dvc, [f[d] + h * df[d] if f[d] is not None else None for d in range(3)])
        for dt in dts:
            s.advance(dt)
        return s.download()

    errs = {}
    for h in (1e-5, 1e-6, 1e-7):
        (pv, pf), (mv, mf) = run(h), run(-h)
        num = float(np.abs((pv - mv) / (2 * h) - tvc).sum())
        den = float(np.abs(tvc).sum())
        for d in range(3):
            if tf[d] is not None:
                num += float(np.abs((pf[d] - mf[d]) / (2 * h) - tf[d]).sum())
                den += float(np.abs(tf[d]).sum())
        errs[h] = num / den
    print(name, "relative L1 |central FD - TL| per h:", errs)
    assert min(errs.values()) < 1e-6, errs


def _dd_central_difference(spec, dts, vc, f, dvc, df, h, tgt_vc):
    """(J(x + h delta) - J(x - h delta)) / 2h of the CP-Alfven objective
    J = 1/2 |rho - rho*|^2 + 1/2 |B - B*|^2, the two runs in double-double and
    the difference of the objectives formed from the difference of the states
    (J+ - J- = 1/2 sum (v+ - v-)(v+ + v- - 2 v*)), so that nothing cancels in
    double precision."""
    from pluto_gb300.adjoint import dd_perturbed_run
    hp, lp = dd_perturbed_run(spec, dts, vc, f, dvc, df, h)
    hm, lm = dd_perturbed_run(spec, dts, vc, f, dvc, df, -h)
    diff = 0.0
    for q in (0, 4, 5, 6):
        dv = (hp[q] - hm[q]) + (lp[q] - lm[q])
        diff += 0.5 * float((dv * (hp[q] + hm[q] - 2.0 * tgt_vc[q])).sum())
    return diff / (2.0 * h)


def _cp_alfven_setup(nsteps):
    from pluto_gb300 import problems as P
    from pluto_gb300.adjoint import Rollout, cfl_dt_sequence
    spec, vc, f = P.cp_alfven(128)
    f = _faces(spec, f)
    dts = cfl_dt_sequence(spec, vc, f, nsteps, spec["first_dt"], spec["cfl"])
    # target: the forward result from a seeded Gaussian perturbation (sigma 1e-3)
    rng = np.random.default_rng(2024)
    vt = vc.copy()
    for q in (0, 1, 2, 3, 7):
        vt[q] = vt[q] + 1e-3 * rng.normal(size=vt[q].shape)
    tgt_vc, _ = Rollout(spec, dts, every=16).run(vt, f)
    return spec, vc, f, dts, tgt_vc


def _autograd_gradient(spec, dts, vc, f, tgt_vc):
    import torch
    from pluto_gb300.adjoint import Rollout, rollout
    r = Rollout(spec, dts, every=16)
    tv = torch.from_numpy(vc.copy()).requires_grad_(True)
    tfx = torch.from_numpy(f[0].copy()).requires_grad_(True)
    tfy = torch.from_numpy(f[1].copy()).requires_grad_(True)
    out = rollout(r, tv, tfx, tfy)
    tgt = torch.from_numpy(tgt_vc)
    J = 0.5 * (((out[0][0] - tgt[0]) ** 2).sum() + ((out[0][4:7] - tgt[4:7]) ** 2).sum())
    J.backward()
    return r, float(J.detach()), out[0].detach().numpy(), tv.grad.numpy(), [tfx.grad.numpy(), tfy.grad.numpy(), None]


def test_cp_alfven_gradient_against_tangent_and_finite_differences():
    """Headline differentiation check on the 128^2 circularly polarised
    Alfven wave (30 degrees), PLM/MC, HLLD, RK2, CT, 256 FP64 steps with a
    checkpoint every 16.  The gradient (torch.autograd over the hand-written
    adjoint) is taken at a smooth generic point next to the initial condition
    (_smooth_generic_2d); the target is the forward result of the initial
    condition with seeded Gaussian noise (sigma 1e-3) on density, velocity,
    pressure.

    * against the FP64 tangent-linear model along 16 random directions: the
      adjoint is its exact transpose (<= 1e-9);
    * against central differences, <= 1e-6: the map is only piecewise smooth
      -- the kink margin of the tangent-linear run shows a branch switch
      (limiter, Riemann fan, MIN/MAX) within about 1e-10 of the point along
      every direction, so FP64 differences (which need h >~ 1e-7 to beat
      round-off) cross thousands of kinks.  The differences are therefore
      taken with the double-double step (PG_FP64_DD) at h = 1e-12, at least
      ten times inside the kink margin, where round-off is negligible."""
    from pluto_gb300.adjoint import tangent_linear
    spec, vc0, f0, dts, tgt_vc = _cp_alfven_setup(256)
    vc, f = _smooth_generic_2d(vc0, f0, np.random.default_rng(99), 2e-2, spec["dx"][0], spec["dx"][1])
    r, J, out_vc, g_vc, g_f = _autograd_gradient(spec, dts, vc, f, tgt_vc)

    def objective(v_T):
        return 0.5 * float(((v_T[0] - tgt_vc[0]) ** 2).sum() + ((v_T[4:7] - tgt_vc[4:7]) ** 2).sum())

    assert abs(J - objective(r.run(vc, f)[0])) <= 1e-12 * J
    lam_vc = np.zeros_like(vc)
    lam_vc[0] = out_vc[0] - tgt_vc[0]
    lam_vc[4:7] = out_vc[4:7] - tgt_vc[4:7]

    h = 1e-12
    worst_tl, worst_fd = 0.0, 0.0
    drng = np.random.default_rng(7)
    for n in range(16):
        dvc, df = _random_like(drng, vc, f)
        norm = math.sqrt(_inner(dvc, df, dvc, df))
        dvc = dvc / norm
        df = [x / norm if x is not None else None for x in df]
        adj = _inner(g_vc, g_f, dvc, df)
        _, (tvc, _), margin = tangent_linear(spec, dts, vc, f, dvc, df, kink=True)
        tl = float(np.dot(lam_vc.ravel(), tvc.ravel()))
        worst_tl = max(worst_tl, abs(adj - tl) / abs(tl))
        line = f"direction {n:2d}: adjoint {adj:.9e}  TL {tl:.9e}  kink margin {margin:.2e}"
        if n < 8:  # double-double central differences (2 x 256 steps each)
            assert margin >= 10 * h, margin
            fd = _dd_central_difference(spec, dts, vc, f, dvc, df, h, tgt_vc)
            worst_fd = max(worst_fd, abs(fd - adj) / abs(adj))
            line += f"  DD central difference {fd:.9e}"
        print(line)
    print(f"cp_alfven 128^2 x 256: max rel |adjoint - TL| = {worst_tl:.3e}, "
          f"max rel |adjoint - DD central difference (h=1e-12)| = {worst_fd:.3e}")
    assert worst_tl <= 1e-9
    assert worst_fd <= 1e-6


@pytest.mark.parametrize("nsteps", [16, 64])
def test_cp_alfven_initial_condition_sits_on_kinks(nsteps):
    """At the CP-Alfven initial condition itself (uniform density and
    pressure, a wave commensurate with the grid) limiters sit exactly on their
    kinks: the kink margin along directions that perturb only the velocity and
    the faces is exactly 0, so central differences there return a mean of
    one-sided derivatives, not the derivative of the branch the step takes.
    The adjoint is still the exact transpose of the tangent-linear model."""
    from pluto_gb300.adjoint import tangent_linear
    spec, vc, f, dts, tgt_vc = _cp_alfven_setup(nsteps)
    _, _, out_vc, g_vc, g_f = _autograd_gradient(spec, dts, vc, f, tgt_vc)
    lam_vc = np.zeros_like(vc)
    lam_vc[0] = out_vc[0] - tgt_vc[0]
    lam_vc[4:7] = out_vc[4:7] - tgt_vc[4:7]
    drng = np.random.default_rng(11)
    for _ in range(2):
        dvc, df = _random_like(drng, vc, f)
        dvc[[0, 4, 5, 6, 7]] = 0.0
        norm = math.sqrt(_inner(dvc, df, dvc, df))
        dvc = dvc / norm
        df = [x / norm if x is not None else None for x in df]
        adj = _inner(g_vc, g_f, dvc, df)
        _, (tvc, _), margin = tangent_linear(spec, dts, vc, f, dvc, df, kink=True)
        tl = float(np.dot(lam_vc.ravel(), tvc.ravel()))
        assert abs(adj - tl) <= 1e-9 * abs(tl)
        assert margin == 0.0


def test_double_double_step_matches_reference():
    """The double-double FP64 step (PG_FP64_DD) against the reference's dump:
    equal to FP64 round-off (it is more accurate than the reference, not
    identical), with non-zero low parts."""
    from pluto_gb300 import Solver
    meta, vc0, bs0, vc1, bs1 = load_golden("ot_hlld_32")
    s = Solver(meta, "fp64_dd")
    s.upload(vc0, bs0)
    s.run(meta["steps"], meta["first_dt"], meta["cfl"])
    hv, hb = s.download()
    lv, _ = s.tangent_download()
    errs = [rel_l1(hv[q], vc1[q]) for q in range(8) if np.abs(vc1[q]).sum() > 0]
    assert max(errs) <= 1e-13, errs
    assert np.abs(lv).max() > 0.0
    assert np.all(np.abs(lv) <= 1e-15 * np.abs(hv) + 1e-300)
