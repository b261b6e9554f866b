"""Differentiated FP64 path: tangent-linear model and hand-written adjoint.

Checks, all with a frozen dt sequence:
- the tangent-linear value part is the plain FP64 step bit for bit;
- dot-product test <lambda, TL(delta)> == <adjoint(lambda), delta> for PLM
  and PPM, HLL and HLLD, 1D outflow / 2D / 3D constrained transport;
- TL against central finite differences of the state;
- the CP-Alfven objective (128^2, 256 steps, checkpoint every 16): the
  autograd gradient against the tangent-linear derivative (exact transpose)
  and against central differences along 16 random unit directions (limited
  by the kinks of the limiters and Riemann branches crossed inside [-h, h]).
"""
import math

import numpy as np
import pytest

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
    raise KeyError(name)


CASES = ["cpa2d_plm_hlld", "ot2d_plm_hll", "turb3d_ppm_hlld", "turb3d_plm_minmod_hll",
         "tube1d_outflow", "tube1d_ppm_outflow", "cpa2d_plm_roe", "tube1d_reflective", "ot2d_mirror_noct",
         "tube1d_sides"]


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


@pytest.mark.parametrize("name,emf", [("cpa2d_plm_hlld", None), ("turb3d_ppm_hlld", None),
                                     ("cpa2d_plm_hlld", "UCT0"), ("cpa2d_plm_hlld", "ARITHMETIC")])
def test_tangent_matches_central_differences(name, emf):
    """Tangent-linear step against central differences; also with the UCT0
    and ARITHMETIC edge averages of the RK path (no branch of their own)."""
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


def test_cp_alfven_gradient_against_tangent_and_finite_differences():
    """Headline differentiation check on the 128^2 circularly polarised
    Alfven wave (30 degrees), PLM/MC, HLLD, RK2, CT, 256 FP64 steps.  The
    gradient is taken at a smooth generic point next to the initial condition
    (see _smooth_generic_2d); the target is the forward result of the initial condition
    with seeded Gaussian noise (sigma 1e-3) on density, velocity, pressure."""
    import torch
    from pluto_gb300 import problems as P
    from pluto_gb300.adjoint import Rollout, cfl_dt_sequence, rollout, tangent_linear
    spec, vc, f = P.cp_alfven(128)
    f = _faces(spec, f)
    nsteps = 256
    dts = cfl_dt_sequence(spec, vc, f, nsteps, spec["first_dt"], spec["cfl"])
    # target: the forward result from a seeded Gaussian perturbation (sigma 1e-3)
    rng = np.random.default_rng(2024)
    vt = vc.copy()
    for q in (0, 1, 2, 3, 7):
        vt[q] = vt[q] + 1e-3 * rng.normal(size=vt[q].shape)
    r = Rollout(spec, dts, every=16)
    tgt_vc, _ = r.run(vt, f)
    vc, f = _smooth_generic_2d(vc, f, np.random.default_rng(99), 2e-2, spec["dx"][0], spec["dx"][1])

    def objective(v_T):
        return 0.5 * float(((v_T[0] - tgt_vc[0]) ** 2).sum() + ((v_T[4:7] - tgt_vc[4:7]) ** 2).sum())

    # gradient through torch.autograd
    tv = torch.from_numpy(vc.copy()).requires_grad_(True)
    tfx = torch.from_numpy(f[0].copy()).requires_grad_(True)
    tfy = torch.from_numpy(f[1].copy()).requires_grad_(True)
    out = rollout(r, tv, tfx, tfy)
    tgt = torch.from_numpy(tgt_vc)
    J = 0.5 * (((out[0][0] - tgt[0]) ** 2).sum() + ((out[0][4:7] - tgt[4:7]) ** 2).sum())
    J.backward()
    g_vc, g_f = tv.grad.numpy(), [tfx.grad.numpy(), tfy.grad.numpy(), None]
    assert abs(float(J.detach()) - objective(r.run(vc, f)[0])) <= 1e-12 * float(J.detach())
    lam_vc = np.zeros_like(vc)
    out_vc = out[0].detach().numpy()
    lam_vc[0] = out_vc[0] - tgt_vc[0]
    lam_vc[4:7] = out_vc[4:7] - tgt_vc[4:7]

    worst_tl, fd_best = 0.0, []
    drng = np.random.default_rng(7)
    for _ in range(16):
        dvc, df = _random_like(drng, vc, f)
        norm = math.sqrt(_inner(dvc, df, dvc, df))
        dvc = dvc / norm
        df = [x / norm if x is not None else None for x in df]
        adj = _inner(g_vc, g_f, dvc, df)
        _, (tvc, _) = tangent_linear(spec, dts, vc, f, dvc, df)
        tl = float(np.dot(lam_vc.ravel(), tvc.ravel()))
        worst_tl = max(worst_tl, abs(adj - tl) / abs(tl))
        errs = []
        for h in (1e-5, 1e-6, 1e-7, 1e-8):
            jp = objective(r.run(vc + h * dvc, [f[0] + h * df[0], f[1] + h * df[1], None])[0])
            jm = objective(r.run(vc - h * dvc, [f[0] - h * df[0], f[1] - h * df[1], None])[0])
            errs.append(abs((jp - jm) / (2 * h) - adj) / abs(adj))
        print(f"direction: adjoint {adj:.6e}  TL {tl:.6e}  rel FD error for h=1e-5..1e-8: "
              + ", ".join(f"{e:.2e}" for e in errs))
        fd_best.append(min(errs))
    fd_best.sort()
    print(f"cp_alfven 128^2 x 256: max rel |adjoint - TL| = {worst_tl:.3e}, "
          f"rel |adjoint - central FD| (best h per direction): median {fd_best[8]:.3e}, max {fd_best[-1]:.3e}")
    # The adjoint is the exact transpose of the tangent-linear model.
    assert worst_tl <= 1e-9
    # Central differences of this piecewise-smooth map: error from limiter
    # and Riemann-branch kinks crossed inside [-h, h] (proportional to h)
    # plus round-off (proportional to 1/h); no h gets it under ~1e-6 for
    # all 16 directions at 256 steps.
    assert fd_best[8] <= 2e-5
    assert fd_best[-1] <= 2e-4
