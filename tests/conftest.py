import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def load_golden(name):
    z = np.load(GOLDEN / f"{name}.npz")
    meta = json.loads(str(z["meta"]))
    bs0 = [z[f"bs{d}_0"] if f"bs{d}_0" in z else None for d in range(3)]
    bs1 = [z[f"bs{d}_1"] if f"bs{d}_1" in z else None for d in range(3)]
    return meta, z["vc0"], bs0, z["vc1"], bs1


GOLDEN_NAMES = sorted(p.stem for p in GOLDEN.glob("*.npz"))


def rel_l1(a, b):
    """Relative L1 difference per variable: sum|a-b| / sum|b| (absolute when b == 0)."""
    den = np.abs(b).sum()
    num = np.abs(a - b).sum()
    return float(num / den) if den > 0 else float(num)


# ---------------------------------------------------------------------------
# fixtures at the benchmark configurations' sizes (tests/golden/large/): the
# reference's initial dump and SHA-256 digests of its dump after the steps
# ---------------------------------------------------------------------------
LARGE = GOLDEN / "large"
SLOT = {"rho": 0, "vx1": 1, "vx2": 2, "vx3": 3, "Bx1": 4, "Bx2": 5, "Bx3": 6, "prs": 7}


def load_large(name):
    z = np.load(LARGE / f"{name}.npz")
    meta = json.loads(str(z["meta"]))
    if "vc0" not in z:
        return meta, z
    bs0 = [z[f"bs{d}_0"] if f"bs{d}_0" in z else None for d in range(3)]
    return meta, z["vc0"], bs0


def dump_arrays(vc, bs, names):
    """The variables of a .dbl dump, in the dump's order, from the 8 cell
    slots and the face arrays."""
    out = []
    for nm in names:
        if nm.endswith("s") and nm.startswith("Bx"):
            out.append(bs[int(nm[2]) - 1])
        else:
            out.append(vc[SLOT[nm]])
    return out


def digest(arrays):
    import hashlib
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a, dtype="<f8").tobytes())
    return h.hexdigest()


def check_against_large(meta, vc, bs):
    """Compares a final state with a large fixture's digests; returns the
    names of the variables that differ (empty when bit-identical)."""
    fin = meta["final"]
    arrs = dump_arrays(vc, bs, fin["names"])
    bad = [nm for nm, a in zip(fin["names"], arrs) if digest([a]) != fin["sha256_per_variable"][nm]]
    if not bad:
        assert digest(arrs) == fin["sha256"]
    return bad
