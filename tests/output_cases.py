"""The reference output fixtures (tests/golden/output_<base>.json) as write jobs.

Each job is one WriteData call of the reference run: a format, its mode, the
file number, the state (the base fixture's vc0/bs0 for file 0, vc1/bs1 for
file 1) and the time / dt / step of its ".out" record.  ``check`` compares the
files a writer produced in a directory with the reference's sizes and SHA-256
sums, and the ".out" files with the reference's text.
"""
import hashlib
import json
from pathlib import Path

from conftest import GOLDEN, load_golden

CASES = sorted(p.stem[len("output_"):] for p in GOLDEN.glob("output_*.json"))


def jobs(case):
    meta = json.loads((GOLDEN / f"output_{case}.json").read_text())
    _, vc0, bs0, vc1, bs1 = load_golden(meta["base"])
    formats = [("dbl", meta["dbl_mode"])] + [tuple(e) for e in meta["outputs"]]
    out = []
    for fmt, mode in formats:
        for rec in meta["records"][fmt].splitlines():
            f = rec.split()
            nfile = int(f[0])
            vc, bs = (vc0, bs0) if nfile == 0 else (vc1, bs1)
            out.append(dict(fmt=fmt, single_file=mode == "single_file", nfile=nfile, vc=vc, bs=bs,
                            time=float(f[1]), dt=float(f[2]), step=int(f[3]),
                            vtk_vector=meta["vtk_vector"] and fmt == "vtk"))
    return meta, out


def extents(meta):
    dims = meta["dims"]
    lo = [meta["lo"][d] if d < dims else 0.0 for d in range(3)]
    hi = [meta["hi"][d] if d < dims else 1.0 for d in range(3)]
    return lo, hi


def check(meta, directory):
    d = Path(directory)
    got = {}
    for f in sorted(d.iterdir()):
        if f.suffix in (".dbl", ".flt", ".vtk"):
            b = f.read_bytes()
            got[f.name] = [len(b), hashlib.sha256(b).hexdigest()]
    want = meta["files"]
    assert sorted(got) == sorted(want), (sorted(set(got) ^ set(want)))
    bad = [n for n in want if got[n] != want[n]]
    assert not bad, {n: (got[n][0], want[n][0]) for n in bad}
    for ext, text in meta["records"].items():
        assert (d / f"{ext}.out").read_text() == text, ext
