"""Hand-derived reverse-mode point functions of the adjoint (HLL / HLLD
Riemann outputs, edge EMF, PLM and PPM states, prim/cons maps) against forward-mode Dual<1> derivatives of the
same point functions, on the host: tests/adjoint_rev_check.cu is compiled by
nvcc as a host program and run on seeded random states that visit every HLLD
region (L / R flux, single-star L / R, double-star L / R, HLLC reversion L / R)
and every branch of the MC face-field slope."""
import re
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
NVCC = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
# relative difference of J^T lam, reverse vs Dual<1>: rounding of the two
# evaluation orders only (the largest seen is ~3e-13, on states close to a
# region boundary where terms cancel)
TOL = 1e-11


@pytest.fixture(scope="module")
def report(tmp_path_factory):
    if not Path(NVCC).exists():
        pytest.skip("nvcc not found")
    exe = tmp_path_factory.mktemp("rev") / "adjoint_rev_check"
    cmd = [NVCC, "-O2", "-std=c++17", "--expt-relaxed-constexpr", "-x", "cu",
           "-I", str(ROOT / "pluto_gb300" / "csrc"), "-I", str(ROOT / "include"),
           str(ROOT / "tests" / "adjoint_rev_check.cu"), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe), "20000"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return r.stdout


def _lines(report, kind):
    return [ln for ln in report.splitlines() if ln.startswith(kind)]


@pytest.mark.parametrize("solver", ["hlld", "hll"])
def test_riemann_reverse_matches_dual(report, solver):
    rows = [ln for ln in _lines(report, "riemann") if ln.split()[1] == solver]
    assert len(rows) == 3  # one per direction
    for ln in rows:
        worst = float(ln.split("worst")[1])
        assert worst < TOL, ln
        if solver == "hlld":
            regions = [int(x) for x in re.search(r"regions ((?:\d+ ){8})", ln + " ").group(1).split()]
            assert all(n > 0 for n in regions), f"an HLLD region was not visited: {ln}"


def test_plm_reverse_matches_dual(report):
    (ln,) = _lines(report, "plm")
    assert float(ln.split("worst")[1]) < TOL, ln
    branches = [int(x) for x in ln.split("branches")[1].split("worst")[0].split()]
    assert all(n > 0 for n in branches), ln


def test_ppm_reverse_matches_dual(report):
    (ln,) = _lines(report, "ppm")
    assert float(ln.split("worst")[1]) < TOL, ln
    branches = [int(x) for x in ln.split("branches")[1].split("worst")[0].split()]
    assert all(n > 0 for n in branches), ln


def test_prim_cons_maps_reverse_matches_dual(report):
    (ln,) = _lines(report, "maps")
    assert float(ln.split("worst")[1]) < TOL, ln
    branches = [int(x) for x in ln.split("branches")[1].split("worst")[0].split()]
    assert all(n > 0 for n in branches), ln  # no floor, density, energy and pressure floors


def test_emf_reverse_matches_dual(report):
    (ln,) = _lines(report, "emf")
    assert float(ln.split("worst")[1]) < TOL, ln
    branches = [int(x) for x in ln.split("branches")[1].split("worst")[0].split()]
    assert all(n > 0 for n in branches), ln
