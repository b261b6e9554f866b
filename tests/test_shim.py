"""The PLUTO-side shim compiles against the reference's headers and links a
complete PLUTO executable with libpluto_gb300 in place of the RK objects.

The same executables, linked instead with a host stand-in for the library
(tests/shim_stub.c: the C ABI's contract on top of the CPU oracle), are run:
PLUTO's own main loop then drives the shim -- the device state uploaded from
d->Vc / d->Vs with the -1 origin of the faces, one pg_advance per step with
Dts->invDt_hyp and g_maxMach handed to NextTimeStep, the WriteData and
Analysis wrappers, user-defined and internal boundaries -- and its dumps and
analysis output must equal those of the reference binary bit for bit.

Needs the reference source tree (skipped where it is absent, e.g. on the GPU
machine); no GPU is used.
"""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
from oracle.build_ref import REF  # noqa: E402  (the reference tree, PLUTO_REF)

pytestmark = pytest.mark.skipif(not (REF / "Src" / "main.c").exists(), reason="reference tree absent")


def _link(setup_fn, tmp_path, libdir=None):
    """Link the shim into the scheme's PLUTO executable: against
    libpluto_gb300 (and the CUDA runtime), or against the library of the same
    name found in libdir (the host stand-in)."""
    from oracle import build_ref as br
    from pluto_gb300 import build as pb
    lib = pb.build() if libdir is None else Path(libdir) / "libpluto_gb300.so"
    s = setup_fn()
    run = br.build(s)  # reference objects for this scheme
    objs = [p for p in (run / "obj").glob("*.o")
            if p.stem not in ("rk_step", "update_stage", "ctu_step", "write_data", "init")]
    inc = ["-I", str(run)] + sum((["-I", str(REF / d)] for d in br.INC_DIRS), []) + ["-I", str(ROOT / "include")]
    # the two objects Makefile.gpu compiles with renamed definitions (wrapped by the shim)
    for src, define in ((REF / "Src" / "write_data.c", "-DWriteData=pg_host_WriteData"),
                        (run / "init.c", "-DAnalysis=pg_user_Analysis")):
        o = tmp_path / (src.stem + ".o")
        subprocess.run(["gcc", "-c", "-O2", "-ffp-contract=off", "-w", define, *inc, str(src), "-o", str(o)],
                       check=True, capture_output=True, text=True)
        objs.append(o)
    shim_o = tmp_path / "gpu_step.o"
    subprocess.run(["gcc", "-c", "-O2", "-Wall", "-Wno-unused-variable", *inc,
                    str(ROOT / "pluto_gb300" / "shim" / "gpu_step.c"), "-o", str(shim_o)],
                   check=True, capture_output=True, text=True)
    exe = tmp_path / "pluto_gpu"
    cuda = ["-L/usr/local/cuda/lib64", "-lcudart"] if libdir is None else []
    r = subprocess.run(["g++", *map(str, objs), str(shim_o), f"-L{lib.parent}", "-lpluto_gb300",
                        f"-Wl,-rpath,{lib.parent}", *cuda, "-lm", "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_shim_links_ot_ct(tmp_path):
    from oracle import build_ref as br
    assert _link(lambda: br.ot_setup("hlld", 32, 30), tmp_path).exists()


def test_shim_links_1d_no_ct(tmp_path):
    from oracle import build_ref as br
    assert _link(lambda: br.tube_setup(0, 64, 10), tmp_path).exists()


def test_shim_links_3d_ppm_rk3(tmp_path):
    from oracle import build_ref as br
    assert _link(lambda: br.turb_setup(12, 10), tmp_path).exists()


def test_enable_script_edits_the_template_makefile(tmp_path):
    """The build switch inserts the shim include after the template's
    object-file block, once, and removes it again."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("pg_enable", ROOT / "pluto_gb300" / "shim" / "enable.py")
    en = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(en)
    mk = tmp_path / "makefile"
    orig = (REF / "Src" / "Templates" / "makefile").read_text()
    mk.write_text(orig)
    assert en.main([str(tmp_path)]) == 0
    once = mk.read_text()
    assert once.count("include $(PG_ROOT)/pluto_gb300/shim/Makefile.gpu") == 1
    assert once.index("Additional_object_files_here") < once.index(en.BEGIN) < once.index("PLUTO target rule")
    en.main([str(mk)])
    assert mk.read_text() == once
    (tmp_path / "write_data.o").write_bytes(b"stale")
    (tmp_path / "init.o").write_bytes(b"stale")
    en.main([str(mk), "--disable"])
    assert mk.read_text() == orig
    assert not (tmp_path / "write_data.o").exists() and not (tmp_path / "init.o").exists()


def test_shim_links_internal_boundary(tmp_path):
    """INTERNAL_BOUNDARY YES: the shim registers the flag array and calls
    UserDefBoundary with a null box."""
    from dataclasses import replace
    from oracle import build_ref as br
    s = replace(br.ot_setup("hlld", 32, 30), name="ot_shim_internal", internal_boundary=True)
    assert _link(lambda: s, tmp_path).exists()


def _preprocessed_shim(s):
    """gpu_step.c after the preprocessor, against the scheme's definitions.h"""
    from oracle import build_ref as br
    run = br.build(s)
    inc = ["-I", str(run)] + sum((["-I", str(REF / d)] for d in br.INC_DIRS), []) + ["-I", str(ROOT / "include")]
    r = subprocess.run(["gcc", "-E", "-P", *inc, str(ROOT / "pluto_gb300" / "shim" / "gpu_step.c")],
                       check=True, capture_output=True, text=True)
    return " ".join(r.stdout.split())


@pytest.mark.parametrize("stepping,emf,want_ts,want_emf", [
    ("HANCOCK_CONS", "UCT0", "PG_HANCOCK_CONS", "PG_UCT0"),
    ("HANCOCK", "ARITHMETIC", "PG_HANCOCK", "PG_ARITHMETIC"),
    ("RK2", "UCT_CONTACT", "PG_RK2", "PG_UCT_CONTACT"),
    ("RK3", "UCT0", "PG_RK3", "PG_UCT0")])
def test_shim_maps_time_stepping_and_emf_average(stepping, emf, want_ts, want_emf):
    """definitions.h's TIME_STEPPING (with PRIMITIVE_HANCOCK NO for the
    conservative predictor) and CT_EMF_AVERAGE select the matching pg_config
    values in the shim."""
    from dataclasses import replace
    from oracle import build_ref as br
    s = replace(br.ot_setup("hlld", 32, 30), stepping=stepping, emf=emf, name=f"ot_shim_{stepping}_{emf}")
    text = _preprocessed_shim(s)
    assert f"c->time_stepping = {want_ts};" in text and text.count("c->time_stepping =") == 1
    assert f"c->emf_average = {want_emf};" in text and text.count("c->emf_average =") == 1


def test_shim_links_conservative_hancock(tmp_path):
    from dataclasses import replace
    from oracle import build_ref as br
    s = replace(br.ot_setup("hlld", 32, 30), stepping="HANCOCK_CONS", emf="UCT0", name="ot_shim_cons")
    assert _link(lambda: s, tmp_path).exists()


# ---------------------------------------------------------------------------
# running the shim against the host stand-in of the library
# ---------------------------------------------------------------------------
ANALYSIS_C = r"""
  int i, j, k;
  double s = 0.0;
  FILE *fp;
  DOM_LOOP(k, j, i) s += d->Vc[RHO][k][j][i]*d->Vc[PRS][k][j][i];
  fp = fopen("analysis.txt", "a");
  fprintf(fp, "%ld %.17e %.17e\n", (long)g_stepNumber, g_time, s);
  fclose(fp);
"""


def _stub_libdir(tmp_path):
    d = tmp_path / "stub"
    d.mkdir()
    subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-std=c99", "-Wall",
                    "-Wno-unused-function", "-I", str(ROOT / "oracle"), "-I", str(ROOT / "include"),
                    str(ROOT / "tests" / "shim_stub.c"), str(ROOT / "oracle" / "mhd_oracle.c"), "-lm",
                    "-o", str(d / "libpluto_gb300.so")], check=True, capture_output=True, text=True)
    return d


def _shim_setups():
    from dataclasses import replace
    from oracle import build_ref as br
    import userdef_cases  # noqa: F401  (the same USERDEF rules as the fixtures)
    sys_path_golden = ROOT / "tests" / "golden"
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", sys_path_golden / "make_golden.py")
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    out = {
        "ot_ct_analysis": replace(br.ot_setup("hlld", 32, 12), name="shimrun_ot", analysis_body=ANALYSIS_C,
                                  analysis_every=4, first_dt=1e-3),
        "tube_1d": replace(br.tube_setup(0, 128, 20), name="shimrun_tube"),
        "turb_ppm_rk3": replace(br.turb_setup(12, 6), name="shimrun_turb", first_dt=1e-3),
        "blast_userdef_ct": replace(br.blast_setup(16, 8), name="shimrun_blast_ud", userdef_body=mg.USERDEF_C,
                                    bc=(("userdef", "outflow"), ("periodic", "periodic"), ("reflective", "userdef")),
                                    first_dt=1e-3),
        "ot_internal": replace(br.ot_setup("hlld", 32, 10), name="shimrun_ot_internal", userdef_body=mg.USERDEF_C,
                               internal_boundary=True, first_dt=1e-3),
        "ot_ctu_sides": replace(br.ot_setup("hlld", 32, 10), name="shimrun_ot_ctu", stepping="HANCOCK",
                                emf="UCT_CONTACT", first_dt=1e-3,
                                bc=(("outflow", "reflective"), ("reflective", "outflow"), ("outflow", "outflow"))),
    }
    return out


@pytest.mark.parametrize("case", ["ot_ct_analysis", "tube_1d", "turb_ppm_rk3", "blast_userdef_ct", "ot_internal",
                                  "ot_ctu_sides"])
def test_shim_runs_plutos_main_loop_like_the_reference(case, tmp_path):
    import hashlib
    import os
    import shutil
    from oracle import build_ref as br
    s = _shim_setups()[case]
    ref_dir = br.OUT / s.name
    if (ref_dir / "analysis.txt").exists():  # Analysis appends
        (ref_dir / "analysis.txt").unlink()
    br.run(s)  # the reference binary: dumps after 0 and s.steps steps
    exe = _link(lambda: s, tmp_path, libdir=_stub_libdir(tmp_path))
    run = tmp_path / "run"
    run.mkdir()
    shutil.copy(ref_dir / "pluto.ini", run / "pluto.ini")
    log = run / "stub.log"
    env = dict(os.environ, PG_STUB_LOG=str(log))
    r = subprocess.run([str(exe), "-maxsteps", str(s.steps + 1)], cwd=run, env=env, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]

    def sha(p):
        return hashlib.sha256(p.read_bytes()).hexdigest()
    # step 0 comes from the reference's writer (nothing on the device yet),
    # step s.steps from pg_write_output; both equal the reference's files
    for f in ("data.0000.dbl", "data.0001.dbl"):
        assert sha(run / f) == sha(ref_dir / f), f
    if s.analysis_body:
        assert (run / "analysis.txt").read_text() == (ref_dir / "analysis.txt").read_text()
        assert len((run / "analysis.txt").read_text().splitlines()) >= 3
    calls = [ln.split() for ln in log.read_text().splitlines()]
    assert calls[0][0] == "create" and [c for c in calls if c[0] == "upload"] == [["upload", "1"]]
    adv = [c for c in calls if c[0] == "advance"]
    assert len(adv) == s.steps + 2  # -maxsteps N (here steps + 1) runs N+1 steps (Src/main.c:149-151)
    assert float(adv[0][1]) == s.first_dt
    for prev, nxt in zip(adv, adv[1:]):  # NextTimeStep from the handed-back invDt_hyp (Src/main.c:459-532)
        inv, dt = float(prev[2]), float(prev[1])
        want = min(s.cfl * (1.0 / inv), 1.1 * dt)
        assert float(nxt[1]) == want, (prev, nxt)
    outs = [c for c in calls if c[0] == "output"]
    assert outs[0][1] == "1" and int(outs[0][3]) == s.steps
    if s.userdef_body:
        assert ["userdef"] in calls
    if s.internal_boundary:
        assert ["internal"] in calls
