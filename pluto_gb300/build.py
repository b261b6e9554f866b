"""Build libpluto_gb300.so in-tree with nvcc for sm_103a.

The FP64 translation unit is compiled with --fmad=false: the reference C
path rounds every multiply and add separately, and the FP64 kernels must
round the same way to reproduce it bit for bit.  The mixed-precision units
keep FMA contraction.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libpluto_gb300.so"
ROOT = PKG.parent

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", str(ROOT / "include"),
          "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]
UNITS = {
    "pg_api.cu": [],
    "pg_fp64.cu": ["--fmad=false"],
    "pg_mixed.cu": ["--use_fast_math"],
    "pg_batch.cu": ["--fmad=false"],
    "pg_batch_mixed.cu": ["--use_fast_math"],
    "pg_adjoint.cu": ["--fmad=false"],
    "pg_dd.cu": ["--fmad=false"],
    "pg_output.cu": [],
}


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and Path(c).exists():
            return c
    raise FileNotFoundError("nvcc not found")


def _sources():
    return [(CSRC / u, f) for u, f in UNITS.items() if (CSRC / u).exists()]


def _stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = list(CSRC.glob("*")) + [ROOT / "include" / "pluto_gb300.h", Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps if p.is_file())


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and not _stale():
        return LIB
    BUILD.mkdir(exist_ok=True)
    exe = nvcc()

    def compile_one(item):
        src, flags = item
        obj = BUILD / (src.stem + ".o")
        cmd = [exe, *ARCH, *COMMON, *flags, "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stderr}")
        if verbose and r.stderr.strip():
            print(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(len(UNITS)) as ex:
        objs = list(ex.map(compile_one, _sources()))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [exe, *ARCH, "-shared", *map(str, objs), "-o", str(tmp), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    build(force="-f" in sys.argv, verbose=True)
    print(LIB)
