"""Output files written from the device (pg_write_output / pg_read_output)
against the reference's own files and the CPU restatement of its writers."""
import hashlib
from pathlib import Path

import numpy as np
import pytest

import output_cases as oc
from conftest import load_golden
from oracle import output_oracle as ow

pytestmark = pytest.mark.gpu


def _files(d):
    return {f.name: hashlib.sha256(f.read_bytes()).hexdigest() for f in sorted(Path(d).iterdir())
            if f.suffix in (".dbl", ".flt", ".vtk", ".out")}


@pytest.mark.parametrize("case", oc.CASES)
def test_device_writer_matches_reference_files(case, tmp_path):
    from pluto_gb300 import Solver
    meta, jobs = oc.jobs(case)
    lo, hi = oc.extents(meta)
    s = Solver(load_golden(meta["base"])[0])
    for nfile in (0, 1):
        mine = [j for j in jobs if j["nfile"] == nfile]
        s.upload(mine[0]["vc"], mine[0]["bs"])
        for j in mine:  # no wait in between: the uploads queue behind the packing
            s.write_output(tmp_path, j["fmt"], nfile, single_file=j["single_file"], vtk_vector=j["vtk_vector"],
                           xbeg=lo, xend=hi, time=j["time"], dt=j["dt"], step=j["step"])
    s.output_wait()
    oc.check(meta, tmp_path)


@pytest.mark.parametrize("precision", ["mixed", "mixed_dw"])
def test_mixed_precision_output_is_the_downloaded_state(precision, tmp_path):
    """The mixed solvers write what pg_download returns (FP32 state widened)."""
    from pluto_gb300 import Solver
    meta, vc0, bs0, _, _ = load_golden("ot_hlld_32")
    s = Solver(meta, precision=precision)
    s.upload(vc0, bs0)
    s.run(3, 1e-3, 0.4)
    vc, bs = s.download()
    (tmp_path / "gpu").mkdir()
    for fmt in ("dbl", "flt", "vtk"):
        s.write_output(tmp_path / "gpu", fmt, 4, xbeg=(0, 0, 0), xend=(1, 1, 1), time=0.5, dt=0.01, step=3)
        ow.write(tmp_path / "cpu", fmt, 4, vc, bs, 2, 2, True,
                 xnode=[ow.nodes(0.0, 1.0, 32), ow.nodes(0.0, 1.0, 32), ow.nodes(0.0, 1.0, 1)],
                 time=0.5, dt=0.01, step=3)
    s.output_wait()
    assert _files(tmp_path / "gpu") == _files(tmp_path / "cpu")


def test_outputs_snapshot_the_state_at_the_call(tmp_path):
    """Steps enqueued after pg_write_output do not reach its files."""
    from pluto_gb300 import Solver
    meta, vc0, bs0, _, _ = load_golden("blast_16")
    spec = meta
    a, b = Solver(spec), Solver(spec)
    a.upload(vc0, bs0)
    b.upload(vc0, bs0)
    states = []
    (tmp_path / "gpu").mkdir()
    for n, steps in enumerate((0, 3, 2, 1)):
        for _ in range(steps):
            a.advance(1e-3)
            b.advance(1e-3)
        a.write_output(tmp_path / "gpu", "dbl", n, single_file=n % 2 == 0, time=n, dt=1e-3, step=n)
        states.append(b.download())
    a.output_wait()
    for n, (vc, bs) in enumerate(states):
        ow.write(tmp_path / "cpu", "dbl", n, vc, bs, 3, 3, True, single_file=n % 2 == 0, time=n, dt=1e-3, step=n)
    assert _files(tmp_path / "gpu") == _files(tmp_path / "cpu")


@pytest.mark.parametrize("precision,single", [("fp64", True), ("fp64", False), ("mixed", True)])
def test_restart_round_trip(precision, single, tmp_path):
    from pluto_gb300 import Solver
    meta, vc0, bs0, _, _ = load_golden("cpa_32")
    spec = meta
    s = Solver(spec, precision=precision)
    s.upload(vc0, bs0)
    s.run(4, 1e-3, 0.4)
    s.write_output(tmp_path, "dbl", 7, single_file=single)
    want = s.download()
    s.output_wait()  # another solver reads the files
    r = Solver(spec, precision=precision)
    r.read_output(tmp_path, 7, single_file=single)
    got = r.download()
    assert np.array_equal(got[0], want[0])
    for d in range(2):
        assert np.array_equal(got[1][d], want[1][d])
    if precision == "fp64":  # the mixed solvers also keep FP64 conserved accumulators, not in the file
        s.advance(1e-3)
        r.advance(1e-3)
        assert np.array_equal(s.download()[0], r.download()[0])


def test_output_errors(tmp_path):
    from pluto_gb300 import Solver
    from pluto_gb300._lib import PgError
    meta, vc0, bs0, _, _ = load_golden("ot_hlld_32")
    s = Solver(meta)
    s.upload(vc0, bs0)
    # staggered fields go to .dbl files only (Src/set_output.c:204-215)
    with pytest.raises(PgError):
        s.write_output(tmp_path, "flt", 0, vars=[(8, "Bx1s", 1)])
    # an unwritable directory is reported by the wait, and the solver goes on
    s.write_output(tmp_path / "missing" / "dir", "dbl", 0)
    with pytest.raises(PgError):
        s.output_wait()
    s.advance(1e-3)
    s.write_output(tmp_path, "dbl", 0)
    s.output_wait()
    assert (tmp_path / "data.0000.dbl").stat().st_size == 8 * (32 * 32 * 6 + 2 * 33 * 32)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_download_async_snapshots_each_step(precision):
    """pg_download_async copies the state at the call while the next steps
    run: each snapshot equals a synchronous download of the same state."""
    import torch
    from pluto_gb300 import Solver
    meta, vc0, bs0, _, _ = load_golden("blast_16")
    a, b = Solver(meta, precision=precision), Solver(meta, precision=precision)
    a.upload(vc0, bs0)
    b.upload(vc0, bs0)

    def pinned(shape):
        return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()

    bufs = [(pinned(vc0.shape), [pinned(f.shape) for f in bs0]) for _ in range(3)]
    want = []
    for n in range(3):
        a.advance(1e-3)
        b.advance(1e-3)
        a.download_async(bufs[n])  # waits for the previous copy, not for later steps
        want.append(b.download())
    a.advance(1e-3)
    a.download_wait()
    for (vc, bs), (wv, wb) in zip(bufs, want):
        assert np.array_equal(vc, wv)
        for d in range(3):
            assert np.array_equal(bs[d], wb[d])


def test_mixed_output_with_padded_rows(tmp_path):
    """A mixed solver whose device rows are padded (30 + 4 ghosts -> pitch
    36) writes the same files as the CPU writer fed with its download."""
    from pluto_gb300 import Solver, problems
    spec, vc0, f0 = problems.orszag_tang(30)
    s = Solver(spec, precision="mixed")
    s.upload(vc0, f0)
    s.run(3, 1e-3, 0.4)
    vc, bs = s.download()
    (tmp_path / "gpu").mkdir()
    for fmt in ("dbl", "flt", "vtk"):
        s.write_output(tmp_path / "gpu", fmt, 2, xbeg=(0, 0, 0), xend=(1, 1, 1), time=0.5, dt=0.01, step=3)
        ow.write(tmp_path / "cpu", fmt, 2, vc, bs, 2, 2, True,
                 xnode=[ow.nodes(0.0, 1.0, 30), ow.nodes(0.0, 1.0, 30), ow.nodes(0.0, 1.0, 1)],
                 time=0.5, dt=0.01, step=3)
    s.output_wait()
    assert _files(tmp_path / "gpu") == _files(tmp_path / "cpu")
