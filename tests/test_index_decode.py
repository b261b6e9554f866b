"""Index decoding of the kernels (multiply-and-shift divisions by
host-prepared magic numbers, pg_internal.h) against exact 64-bit division,
on the host: tests/index_decode_check.cu is compiled by nvcc as a host
program and checks every thread index of the boundary-fill, per-zone and
box maps on 1D/2D/3D grids with 2-4 ghost layers, in both the 32-bit branch
and the 64-bit branch kept for 2^32 zones or more."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
NVCC = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def test_index_decode_matches_division(tmp_path):
    if not Path(NVCC).exists():
        pytest.skip("nvcc not found")
    exe = tmp_path / "index_decode_check"
    cmd = [NVCC, "-O2", "-std=c++17", "--expt-relaxed-constexpr", "-x", "cu",
           "-I", str(ROOT / "pluto_gb300" / "csrc"), "-I", str(ROOT / "include"),
           str(ROOT / "tests" / "index_decode_check.cu"), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "all ok" in r.stdout, r.stdout
