"""The CPU restatement of PLUTO's writers (oracle/output_oracle.py) against
the reference's own .dbl / .flt / .vtk files and .out records, byte for byte."""
import pytest

import output_cases as oc
from oracle import output_oracle as ow


@pytest.mark.parametrize("case", oc.CASES)
def test_oracle_writer_matches_reference_files(case, tmp_path):
    meta, jobs = oc.jobs(case)
    lo, hi = oc.extents(meta)
    dims = meta["dims"]
    xnode = [ow.nodes(lo[d], hi[d], meta["n"][d] if d < dims else 1) for d in range(3)]
    for j in jobs:
        ow.write(tmp_path, j["fmt"], j["nfile"], j["vc"], j["bs"], dims, meta["components"], meta["ct"],
                 single_file=j["single_file"], vtk_vector=j["vtk_vector"], xnode=xnode,
                 time=j["time"], dt=j["dt"], step=j["step"])
    oc.check(meta, tmp_path)


def test_cases_cover_every_format_and_mode():
    seen = set()
    for case in oc.CASES:
        meta, jobs = oc.jobs(case)
        seen |= {(j["fmt"], j["single_file"], j["vtk_vector"]) for j in jobs}
    for fmt in ("dbl", "flt", "vtk"):
        assert (fmt, True, False) in seen or (fmt, True, True) in seen
        assert (fmt, False, False) in seen
    assert ("vtk", True, True) in seen
