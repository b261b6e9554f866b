#!/usr/bin/env python3
"""Record the reference's .dbl / .flt / .vtk output files for a few fixtures.

Run in a container that has the reference tree (``PLUTO_REF``, default
``/root/reference``) and gcc:

    python tests/golden/make_output_golden.py [name ...]

For each case the reference binary is rebuilt from the setup of the fixture
``<base>.npz`` (tests/golden/make_golden.py) with the listed output formats and
modes enabled at the dump cadence of that fixture, so its files 0000 and 0001
hold the fixture's ``vc0`` / ``vc1`` states.  ``output_<base>.json`` keeps,
per written file, its size and SHA-256, and the text of each ``<ext>.out``
record file, plus what a writer needs to reproduce them (grid extents for the
VTK node coordinates).
"""
from __future__ import annotations

import hashlib
import json
import subprocess
import sys
from dataclasses import replace
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(Path(__file__).resolve().parent))
from oracle import build_ref as br  # noqa: E402
import make_golden as mg  # noqa: E402

GOLDEN = Path(__file__).resolve().parent

# base fixture -> (dbl mode, extra outputs, VTK_VECTOR_DUMP)
CASES = {
    "ot_hlld_32": ("single_file", (("flt", "single_file"), ("vtk", "single_file")), False),
    # VTK_VECTOR_DUMP with multiple_files stops the reference (no "bx1" vector name)
    "blast_16": ("multiple_files", (("flt", "multiple_files"), ("vtk", "multiple_files")), False),
    "tube_0_256": ("single_file", (("flt", "multiple_files"), ("vtk", "single_file")), True),
    "cpa_32": ("single_file", (("flt", "single_file"), ("vtk", "single_file")), True),
}


def main():
    only = set(sys.argv[1:])
    base = {s.name: s for s in mg.setups()}
    for name, (dbl_mode, extra, vec) in CASES.items():
        if only and name not in only:
            continue
        s = replace(base[name], name=f"out_{name}", dbl_mode=dbl_mode, out_modes=extra, vtk_vector=vec)
        run = br.build(s)
        for f in list(run.glob("*.dbl")) + list(run.glob("*.flt")) + list(run.glob("*.vtk")) + list(run.glob("*.out")):
            f.unlink()
        subprocess.run(["./pluto", "-maxsteps", str(s.steps + 1)], cwd=run, check=True, capture_output=True)
        files = {}
        for f in sorted(run.iterdir()):
            if f.suffix in (".dbl", ".flt", ".vtk"):
                b = f.read_bytes()
                files[f.name] = [len(b), hashlib.sha256(b).hexdigest()]
        records = {ext: (run / f"{ext}.out").read_text() for ext in ("dbl", "flt", "vtk")
                   if (run / f"{ext}.out").exists()}
        meta = {"base": name, "dbl_mode": dbl_mode, "outputs": [list(e) for e in extra], "vtk_vector": vec,
                "dims": s.dims, "components": s.components, "ct": s.ct,
                "n": list(s.n), "lo": list(s.lo), "hi": list(s.hi),
                "files": files, "records": records}
        (GOLDEN / f"output_{name}.json").write_text(json.dumps(meta, indent=1) + "\n")
        print(f"output_{name}: {len(files)} files")


if __name__ == "__main__":
    main()
