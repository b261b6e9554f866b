"""The user-defined boundary of the USERDEF fixtures, in numpy.

The same rules as the C UserDefBoundary the fixtures were made with
(tests/golden/make_golden.py, USERDEF_C): an X1_BEG nozzle -- a fixed inflow
state on the middle half of the rows, a mirror wall (vx, Bx negated)
elsewhere, and the staggered By and Bz of the side's x2face / x3face boxes
likewise -- and an X3_END side copied from the last interior plane (cells with
vz = 0 and p = 0.1, the staggered Bx and By of its boxes).
With INTERNAL_BOUNDARY, a dense block (rho 10, v 0, p 1) a quarter of the
way along x is set before every fill and flagged so it is not updated.
Only assignments and negations, so results match the C version bit for bit.

The callback signature is the one of Solver.set_userdef / Oracle.set_userdef:
fn(side, vpos, stage, vc, faces) with vc[q] a (nt2, nt1, nt0) PLUTO-layout
view and faces[d] one longer along d with the -1 layer first.
"""
import numpy as np

RHO, VX1, VX2, VX3, BX1, BX2, BX3, PRS = range(8)


def has_userdef(spec) -> bool:
    bc = spec.get("bc", "periodic")
    return "userdef" in repr(bc) or bool(spec.get("internal_boundary"))


def nghost(spec) -> int:
    ng = 3 if spec.get("recon", "LINEAR") == "PARABOLIC" else 2
    if spec.get("stepping", "RK2") in ("HANCOCK", "CHARACTERISTIC_TRACING", "HANCOCK_CONS") and spec.get("ct", True):
        ng += 1
    return ng


def make(spec):
    ng = nghost(spec)
    nx2 = int(spec["nx"][1]) if spec["dims"] > 1 else 1
    jbeg = ng if spec["dims"] > 1 else 0
    kend = ng + int(spec["nx"][2]) - 1 if spec["dims"] > 2 else 0
    lo, hi = jbeg + nx2 // 4, jbeg + (3 * nx2) // 4
    inflow = ((RHO, 2.0), (VX1, 0.5), (VX2, 0.0), (PRS, 0.3), (BX1, 0.2), (BX2, 0.1), (VX3, 0.0), (BX3, 0.0))

    nx1 = int(spec["nx"][0])
    i0, j0 = ng + nx1 // 4, jbeg + nx2 // 2 - 2

    def fn(side, vpos, stage, vc, faces, flags=None):
        if side == 6:  # internal boundary: a dense block that is not updated
            if flags is not None:
                for q, val in ((RHO, 10.0), (VX1, 0.0), (VX2, 0.0), (PRS, 1.0)):
                    vc[q][:, j0:j0 + 4, i0:i0 + 3] = val
                flags[:, j0:j0 + 4, i0:i0 + 3] |= 32
        elif side == 0:  # X1_BEG
            if vpos == 0:  # CENTER
                j = np.arange(vc[0].shape[1])
                noz = (j >= lo) & (j < hi)
                for i in range(ng):
                    src = 2 * ng - 1 - i
                    for q in range(8):
                        vc[q][:, :, i] = vc[q][:, :, src]
                    vc[VX1][:, :, i] = -vc[VX1][:, :, i]
                    vc[BX1][:, :, i] = -vc[BX1][:, :, i]
                    for q, val in inflow:
                        vc[q][:, noz, i] = val
            elif vpos == 2 and faces[1] is not None:  # X2FACE: rows j = -1 .. nt1-1
                f = faces[1]
                jj = np.arange(-1, f.shape[1] - 1)
                noz = (jj >= lo) & (jj < hi)
                for i in range(ng):
                    f[:, :, i] = f[:, :, 2 * ng - 1 - i]
                    f[:, noz, i] = 0.1
            elif vpos == 3 and faces[2] is not None:  # X3FACE: planes k = -1 .. nt2-1
                f = faces[2]
                j = np.arange(f.shape[1])
                noz = (j >= lo) & (j < hi)
                for i in range(ng):
                    f[:, :, i] = f[:, :, 2 * ng - 1 - i]
                    f[:, noz, i] = 0.0
        elif side == 5:  # X3_END
            nt2 = vc[0].shape[0]
            if vpos == 0:  # CENTER
                for k in range(kend + 1, nt2):
                    for q in range(8):
                        vc[q][k] = vc[q][kend]
                    vc[VX3][k] = 0.0
                    vc[PRS][k] = 0.1
            elif vpos in (1, 2) and faces[vpos - 1] is not None:  # X1FACE / X2FACE
                f = faces[vpos - 1]
                for k in range(kend + 1, nt2):
                    f[k] = f[kend]

    return fn
