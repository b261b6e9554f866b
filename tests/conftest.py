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
