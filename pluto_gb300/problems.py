"""Initial conditions of the benchmark problems (the role of a PLUTO init.c).

Each function returns ``(spec, vc, faces)``: the scheme/grid description used
by ``Solver``, the 8 cell-centred primitives ``[RHO,VX1,VX2,VX3,BX1,BX2,BX3,PRS]``
over the interior, and the staggered field components (one longer along their
own axis), in the layout of a PLUTO ``.dbl`` dump.  Cell-centred B is the
average of the two faces, as Src/startup.c:230-236 sets it.
"""
from __future__ import annotations

import math

import numpy as np


def _centres(n, lo, hi):
    dx = (hi - lo) / n
    return lo + (np.arange(n) + 0.5) * dx, dx


def _faces_from_az(az_edges, dx, dy):
    """2D face fields from the corner vector potential A_z[j+1/2][i+1/2]
    (faces bx = dA/dy, by = -dA/dx, as Src/vec_pot_diff.c does)."""
    bx = (az_edges[1:, :] - az_edges[:-1, :]) / dy          # [ny][nx+1]
    by = -(az_edges[:, 1:] - az_edges[:, :-1]) / dx         # [ny+1][nx]
    return bx, by


def _cell_b(faces, dims):
    out = []
    for d in range(dims):
        f = faces[d]
        if d == 0:
            out.append(0.5 * (f[..., 1:] + f[..., :-1]))
        elif d == 1:
            out.append(0.5 * (f[..., 1:, :] + f[..., :-1, :]))
        else:
            out.append(0.5 * (f[1:] + f[:-1]))
    return out


def blast3d(n=512, p_in=10.0, p_out=0.1, r0=0.1, bmag=10.0, dtype=np.float64, nz=None):
    """3D MHD blast wave on [-0.5,0.5]^3, periodic; taper over two zones.

    ``nz`` < n keeps only the central nz layers in z (an n x n x nz periodic
    slab with the n^3 grid's spacing; the cut is mirror-symmetric about z=0,
    so the periodic wrap joins equal states)."""
    x, dx = _centres(n, -0.5, 0.5)
    nz = n if nz is None else nz
    if not 1 <= nz <= n:
        raise ValueError(f"nz={nz} outside [1, {n}]")
    z = x[(n - nz) // 2:(n - nz) // 2 + nz]
    vc = np.zeros((8, nz, n, n), dtype=dtype)
    vc[0] = 1.0
    r2 = (x[None, None, :] ** 2 + x[None, :, None] ** 2 + z[:, None, None] ** 2)
    r = np.sqrt(r2)
    dr = 2 * dx
    p = np.where(r < r0, p_in, np.where(r < r0 + dr, p_in + (p_out - p_in) * (r - r0) / dr, p_out))
    vc[7] = p
    b = bmag / math.sqrt(3.0) / math.sqrt(4.0 * math.pi)
    faces = [np.full((nz, n, n + 1), b), np.full((nz, n + 1, n), b), np.full((nz + 1, n, n), b)]
    vc[4:7] = b
    name = f"blast3d_{n}" if nz == n else f"blast3d_{n}_slab{nz}"
    spec = dict(name=name, dims=3, components=3, nx=(n, n, nz), dx=(dx, dx, dx),
                gamma=5.0 / 3.0, recon="LINEAR", limiter="MC_LIM", solver="hlld",
                stepping="RK2", ct=True, bc="periodic", cfl=0.3, first_dt=1e-4)
    return spec, vc, faces


def orszag_tang(n=256):
    """2D Orszag-Tang vortex on [0,1]^2 (COMPONENTS 2), vector potential IC."""
    x, dx = _centres(n, 0.0, 1.0)
    xe = np.arange(n + 1) * dx  # edges
    B0 = 1.0 / math.sqrt(4.0 * math.pi)
    tp = 2.0 * math.pi
    X, Y = np.meshgrid(xe, xe, indexing="xy")
    az = B0 * (np.cos(tp * Y) / tp + np.cos(2 * tp * X) / (2 * tp))
    bx, by = _faces_from_az(az, dx, dx)
    vc = np.zeros((8, 1, n, n))
    Xc, Yc = np.meshgrid(x, x, indexing="xy")
    vc[0, 0] = 25.0 / (36.0 * math.pi)
    vc[7, 0] = 5.0 / (12.0 * math.pi)
    vc[1, 0] = -np.sin(tp * Yc)
    vc[2, 0] = np.sin(tp * Xc)
    faces = [bx[None], by[None], None]
    cb = _cell_b(faces, 2)
    vc[4], vc[5] = cb[0], cb[1]
    spec = dict(name=f"ot_{n}", dims=2, components=2, nx=(n, n, 1), dx=(dx, dx, 1.0),
                gamma=5.0 / 3.0, recon="LINEAR", limiter="MC_LIM", solver="hlld",
                stepping="RK2", ct=True, bc="periodic", cfl=0.4, first_dt=1e-4)
    return spec, vc, faces


def cp_alfven(n=128, eps=0.1, alpha=math.pi / 6):
    """Circularly polarised Alfven wave rotated by alpha on [0,1]x[0,1/tan(alpha)]
    (periodic for that aspect), rho=1, p=0.1, B_par=1, gamma=5/3."""
    lx, ly = 1.0, 1.0 / math.tan(alpha)
    x, dx = _centres(n, 0.0, lx)
    y, dy = _centres(n, 0.0, ly)
    ca, sa = math.cos(alpha), math.sin(alpha)
    lam = ca
    tp = 2 * math.pi
    xe = np.arange(n + 1) * dx
    ye = np.arange(n + 1) * dy
    XE, YE = np.meshgrid(xe, ye, indexing="xy")
    xpar = XE * ca + YE * sa
    xperp = -XE * sa + YE * ca
    az = xperp + eps * lam / tp * np.cos(tp * xpar / lam)
    bx, by = _faces_from_az(az, dx, dy)
    X, Y = np.meshgrid(x, y, indexing="xy")
    phi = tp * (X * ca + Y * sa) / lam
    vc = np.zeros((8, 1, n, n))
    vc[0, 0] = 1.0
    vc[7, 0] = 0.1
    vperp = eps * np.sin(phi)
    vc[1, 0] = -vperp * sa
    vc[2, 0] = vperp * ca
    vc[3, 0] = eps * np.cos(phi)
    vc[6, 0] = eps * np.cos(phi)
    faces = [bx[None], by[None], None]
    cb = _cell_b(faces, 2)
    vc[4], vc[5] = cb[0], cb[1]
    spec = dict(name=f"cpa_{n}", dims=2, components=3, nx=(n, n, 1), dx=(dx, dy, 1.0),
                gamma=5.0 / 3.0, recon="LINEAR", limiter="MC_LIM", solver="hlld",
                stepping="RK2", ct=True, bc="periodic", cfl=0.4, first_dt=1e-4)
    return spec, vc, faces


def riemann_tube(n, seed, gamma=2.0):
    """One 1D MHD Riemann problem (batched-tube family): states drawn from the
    seed; discontinuity at x=0.5 on [0,1], outflow."""
    rng = np.random.default_rng(seed)
    lu = lambda a, b: float(np.exp(rng.uniform(np.log(a), np.log(b))))
    bx = float(rng.uniform(0.25, 1.0))
    st = []
    for _ in range(2):
        st.append(dict(rho=lu(0.1, 1.0), p=lu(0.05, 1.0), v=rng.uniform(-1, 1, 3),
                       b=rng.uniform(-1, 1, 2)))
    x, dx = _centres(n, 0.0, 1.0)
    vc = np.zeros((8, 1, 1, n))
    for side, sel in ((0, x < 0.5), (1, x >= 0.5)):
        s = st[side]
        vc[0, 0, 0, sel] = s["rho"]
        vc[7, 0, 0, sel] = s["p"]
        for c in range(3):
            vc[1 + c, 0, 0, sel] = s["v"][c]
        vc[5, 0, 0, sel] = s["b"][0]
        vc[6, 0, 0, sel] = s["b"][1]
    vc[4] = bx
    spec = dict(name=f"tube_{seed}_{n}", dims=1, components=3, nx=(n, 1, 1), dx=(dx, 1.0, 1.0),
                gamma=gamma, recon="LINEAR", limiter="MINMOD_LIM", solver="hlld", stepping="RK2",
                ct=False, bc="outflow", cfl=0.8, first_dt=1e-4)
    return spec, vc, [None, None, None]


def _modes_on_grid(modes, n, which, comp, shift):
    """sum over the modes of amp * vec[comp] * cos(2 pi k.x + phase) at the
    points x = j dx + shift (j = 0..n-1 per axis, array [z][y][x]), by one
    inverse FFT of the mode coefficients (cuFFT on the device when there is
    one, else numpy); equal to the direct sum up to round-off."""
    dx = 1.0 / n
    coef = {}
    for kv, amp, a1, ph1, a2, ph2 in modes:
        if which == "v":
            c = amp * a1[comp] * np.exp(1j * ph1)
        else:
            c = amp * a2[comp] / np.linalg.norm(kv) * np.exp(1j * ph2)
        c *= np.exp(2j * np.pi * float(kv @ np.asarray(shift)))
        idx = (int(kv[2]) % n, int(kv[1]) % n, int(kv[0]) % n)
        coef[idx] = coef.get(idx, 0.0) + c
    try:
        import torch
        dev = "cuda" if torch.cuda.is_available() else None
    except Exception:
        dev = None
    if dev:
        F = torch.zeros((n, n, n), dtype=torch.complex128, device=dev)
        ii = torch.tensor(list(coef.keys()), dtype=torch.long, device=dev)
        F[ii[:, 0], ii[:, 1], ii[:, 2]] = torch.tensor(list(coef.values()), dtype=torch.complex128, device=dev)
        out = torch.fft.ifftn(F, norm="forward").real.cpu().numpy()
        del F, ii
        torch.cuda.empty_cache()
        return out
    F = np.zeros((n, n, n), dtype=np.complex128)
    for idx, c in coef.items():
        F[idx] = c
    return np.fft.ifftn(F, norm="forward").real


def _wrap(a, axes):
    """append the first layer along each periodic axis (face/edge grids of n+1 points)"""
    for ax in axes:
        a = np.concatenate([a, np.take(a, [0], axis=ax)], axis=ax)
    return a


def turbulence3d(n=768, seed=0, kmin=1, kmax=4, mach=1.0, beta=10.0, fft=None):
    """Decaying MHD turbulence: random-phase solenoidal v and vector potential
    A with E(k) ~ k^-2 on shells kmin<=|k|<=kmax; B = curl A on the faces.
    fft (default: n >= 64) evaluates the mode sums by inverse FFT instead of
    term by term (the same fields up to round-off; the term-by-term sum takes
    hours at 768^3)."""
    if fft is None:
        fft = n >= 64
    rng = np.random.default_rng(seed)
    dx = 1.0 / n
    ks = [(kx, ky, kz) for kx in range(-kmax, kmax + 1) for ky in range(-kmax, kmax + 1)
          for kz in range(-kmax, kmax + 1) if kmin ** 2 <= kx * kx + ky * ky + kz * kz <= kmax ** 2]
    modes = []
    for k in ks:
        kv = np.array(k, float)
        km = np.linalg.norm(kv)
        amp = km ** -2.0 / km  # |v_k| ~ k^-1 so that E(k) dk ~ k^-2 over the shell
        a1 = rng.normal(size=3)
        a1 -= kv * (a1 @ kv) / (km * km)
        a1 /= np.linalg.norm(a1) + 1e-30
        a2 = rng.normal(size=3)
        modes.append((kv, amp, a1, rng.uniform(0, 2 * np.pi), a2, rng.uniform(0, 2 * np.pi)))
    x = (np.arange(n) + 0.5) * dx
    xe = np.arange(n + 1) * dx
    tp = 2 * np.pi

    def field(coords, which):
        X, Y, Z = coords
        out = np.zeros((3,) + X.shape)
        for kv, amp, a1, ph1, a2, ph2 in modes:
            if which == "v":
                out += (amp * a1)[:, None, None, None] * np.cos(tp * (kv[0] * X + kv[1] * Y + kv[2] * Z) + ph1)
            else:
                out += (amp * a2 / np.linalg.norm(kv))[:, None, None, None] * \
                    np.cos(tp * (kv[0] * X + kv[1] * Y + kv[2] * Z) + ph2)
        return out

    if fft:
        h = 0.5 * dx
        v = np.stack([_modes_on_grid(modes, n, "v", c, (h, h, h)) for c in range(3)])
        ax = _wrap(_modes_on_grid(modes, n, "a", 0, (h, 0.0, 0.0)), (0, 1))
        ay = _wrap(_modes_on_grid(modes, n, "a", 1, (0.0, h, 0.0)), (0, 2))
        az = _wrap(_modes_on_grid(modes, n, "a", 2, (0.0, 0.0, h)), (1, 2))
    else:
        Zc, Yc, Xc = np.meshgrid(x, x, x, indexing="ij")
        v = field((Xc, Yc, Zc), "v")
        del Zc, Yc, Xc
    cs = math.sqrt(5.0 / 3.0)
    v *= mach * cs / math.sqrt((v ** 2).sum(0).mean())
    # edge-centred A components: Ax at (i, j+1/2, k+1/2), Ay at (i+1/2, j, k+1/2), Az at (i+1/2, j+1/2, k)
    if not fft:
        Z, Y, X = np.meshgrid(xe, xe, x, indexing="ij")
        ax = field((X, Y, Z), "a")[0]
        Z, Y, X = np.meshgrid(xe, x, xe, indexing="ij")
        ay = field((X, Y, Z), "a")[1]
        Z, Y, X = np.meshgrid(x, xe, xe, indexing="ij")
        az = field((X, Y, Z), "a")[2]
        del Z, Y, X
    # faces: bx = dAz/dy - dAy/dz at (i+1/2, j, k) etc.
    bx = (az[:, 1:, :] - az[:, :-1, :]) / dx - (ay[1:, :, :] - ay[:-1, :, :]) / dx
    by = (ax[1:, :, :] - ax[:-1, :, :]) / dx - (az[:, :, 1:] - az[:, :, :-1]) / dx
    bz = (ay[:, :, 1:] - ay[:, :, :-1]) / dx - (ax[:, 1:, :] - ax[:, :-1, :]) / dx
    del ax, ay, az
    faces = [bx, by, bz]
    cb = _cell_b(faces, 3)
    brms2 = float(sum((c ** 2).mean() for c in cb))
    del cb
    scale = math.sqrt(2.0 * 1.0 / beta / brms2)
    for f in faces:
        f *= scale
    vc = np.zeros((8, n, n, n))
    vc[0] = 1.0
    vc[7] = 1.0
    vc[1:4] = v
    del v
    vc[4], vc[5], vc[6] = _cell_b(faces, 3)
    spec = dict(name=f"turb3d_{n}", dims=3, components=3, nx=(n, n, n), dx=(dx, dx, dx),
                gamma=5.0 / 3.0, recon="PARABOLIC", limiter="MC_LIM", solver="hlld",
                stepping="RK3", ct=True, bc="periodic", cfl=0.3, first_dt=1e-4)
    return spec, vc, faces
