"""The PLUTO-side shim compiles against the reference's headers and links a
complete PLUTO executable with libpluto_gb300 in place of the RK objects.

Needs the reference source tree (skipped where it is absent, e.g. on the GPU
machine); no GPU is used: the binary is built, not run.
"""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
from oracle.build_ref import REF  # noqa: E402  (the reference tree, PLUTO_REF)

pytestmark = pytest.mark.skipif(not (REF / "Src" / "main.c").exists(), reason="reference tree absent")


def _link(setup_fn, tmp_path):
    from oracle import build_ref as br
    from pluto_gb300 import build as pb
    lib = pb.build()
    s = setup_fn()
    run = br.build(s)  # reference objects for this scheme
    objs = [p for p in (run / "obj").glob("*.o")
            if p.stem not in ("rk_step", "update_stage", "ctu_step", "write_data", "init")]
    inc = ["-I", str(run)] + sum((["-I", str(REF / d)] for d in br.INC_DIRS), []) + ["-I", str(ROOT / "include")]
    # the two objects Makefile.gpu compiles with renamed definitions (wrapped by the shim)
    for src, define in ((REF / "Src" / "write_data.c", "-DWriteData=pg_host_WriteData"),
                        (run / "init.c", "-DAnalysis=pg_user_Analysis")):
        o = tmp_path / (src.stem + ".o")
        subprocess.run(["gcc", "-c", "-O2", "-w", define, *inc, str(src), "-o", str(o)],
                       check=True, capture_output=True, text=True)
        objs.append(o)
    shim_o = tmp_path / "gpu_step.o"
    subprocess.run(["gcc", "-c", "-O2", "-Wall", "-Wno-unused-variable", *inc,
                    str(ROOT / "pluto_gb300" / "shim" / "gpu_step.c"), "-o", str(shim_o)],
                   check=True, capture_output=True, text=True)
    exe = tmp_path / "pluto_gpu"
    r = subprocess.run(["g++", *map(str, objs), str(shim_o), f"-L{lib.parent}", "-lpluto_gb300",
                        f"-Wl,-rpath,{lib.parent}", "-L/usr/local/cuda/lib64", "-lcudart", "-lm",
                        "-o", str(exe)], capture_output=True, text=True)
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
