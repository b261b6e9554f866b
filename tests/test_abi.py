"""The C ABI library builds, loads and exports every declared entry point.

No compute call is made here (no GPU on the build machine): only symbol
presence, the ABI version and argument validation, which runs before any
CUDA call.
"""
import ctypes as C
import re
from pathlib import Path

import pytest

from pluto_gb300 import _lib as L
from pluto_gb300.solver import make_config

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        names |= set(re.findall(r"^\s*(?:int|void|const\s+char\s*\*)\s*\**\s*(pg_\w+)\s*\(", h.read_text(), re.M))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    L.build()
    return L.lib()


def test_header_declares_expected_symbols():
    assert set(L.EXPORTS) <= set(declared_symbols())


def test_every_declared_symbol_is_exported(lib):
    for name in declared_symbols():
        assert hasattr(lib, name), name


def test_abi_version(lib):
    from pluto_gb300 import _lib as L
    assert lib.pg_abi_version() == L.PG_ABI_VERSION == 3


@pytest.mark.parametrize("field,value", [("dims", 4), ("components", 1), ("gamma", 1.0),
                                         ("riemann", 7), ("time_stepping", 7), ("precision", 9)])
def test_invalid_config_rejected_before_any_cuda_call(lib, field, value):
    spec = dict(dims=2, components=2, nx=(16, 16, 1), dx=(1 / 16, 1 / 16, 1.0), gamma=5 / 3)
    cfg = make_config(spec)
    setattr(cfg, field, value)
    h = C.c_void_p()
    rc = lib.pg_create(C.byref(cfg), C.byref(h))
    assert rc == 1 and not h.value
    assert lib.pg_last_error()


def test_ct_requires_2d_and_accepts_outflow(lib):
    spec = dict(dims=1, components=3, nx=(64, 1, 1), dx=(1 / 64, 1, 1), gamma=2.0, ct=True)
    h = C.c_void_p()
    assert lib.pg_create(C.byref(make_config(spec)), C.byref(h)) == 1
    # outflow sides under CT pass validation (without a GPU the create then
    # stops at the first CUDA call, not at PG_ERR_INVALID)
    spec = dict(dims=2, components=2, nx=(16, 16, 1), dx=(1 / 16, 1 / 16, 1), gamma=5 / 3, ct=True,
                bc=("outflow", "periodic", "periodic"))
    rc = lib.pg_create(C.byref(make_config(spec)), C.byref(h))
    assert rc != 1
    if rc == 0:
        lib.pg_destroy(h)


@pytest.mark.parametrize("extra,ok", [({}, True), ({"recon": "PARABOLIC"}, True),
                                      ({"recon": "PARABOLIC", "stepping": "HANCOCK"}, False),
                                      ({"precision": "mixed"}, False), ({"precision": "fp64_tangent"}, False),
                                      ({"ct": True, "emf": "UCT_HLL"}, False),
                                      ({"ct": True, "emf": "UCT_CONTACT"}, True),
                                      ({"ct": True, "emf": "ARITHMETIC"}, True)])
def test_char_tracing_validation(lib, extra, ok):
    """TIME_STEPPING CHARACTERISTIC_TRACING: linear or parabolic states (the
    Hancock predictor: linear only), the plain FP64 path, and under CT the
    ARITHMETIC or UCT_CONTACT emf average."""
    extra = dict(extra)
    precision = extra.pop("precision", "fp64")
    spec = dict(dims=2, components=2, nx=(16, 16, 1), dx=(1 / 16, 1 / 16, 1), gamma=5 / 3, ct=False,
                stepping="CHARACTERISTIC_TRACING")
    spec.update(extra)
    h = C.c_void_p()
    rc = lib.pg_create(C.byref(make_config(spec, precision)), C.byref(h))
    assert (rc != 1) == ok, lib.pg_last_error()
    if rc == 0:
        lib.pg_destroy(h)


@pytest.mark.parametrize("stepping,emf,precision,ok", [
    ("RK2", "UCT_HLL", "fp64", True), ("RK2", "ARITHMETIC", "fp64", True), ("RK3", "UCT0", "fp64", True),
    ("EULER", "UCT_CONTACT", "fp64", True), ("RK2", "UCT0", "fp64_tangent", True),
    ("RK2", "UCT_HLL", "mixed", True), ("RK2", "UCT_CONTACT", "mixed", False), ("RK2", "UCT0", "mixed_dw", False),
    ("HANCOCK", "UCT0", "fp64", True), ("HANCOCK", "UCT_HLL", "fp64", False),
    ("CHARACTERISTIC_TRACING", "UCT0", "fp64", True),
    ("HANCOCK_CONS", "UCT0", "fp64", True), ("HANCOCK_CONS", "ARITHMETIC", "fp64_tangent", True),
    ("HANCOCK_CONS", "UCT_HLL", "fp64", False), ("HANCOCK_CONS", "UCT_CONTACT", "mixed", False)])
def test_emf_average_validation(lib, stepping, emf, precision, ok):
    """CT_EMF_AVERAGE: all four averages under RK (ARITHMETIC, UCT0 and
    UCT_CONTACT on the FP64 and tangent-linear builds only), every one but
    UCT_HLL under CTU (Src/MHD/CT/ct_emf.c:196-200)."""
    spec = dict(dims=2, components=2, nx=(16, 16, 1), dx=(1 / 16, 1 / 16, 1), gamma=5 / 3, ct=True,
                stepping=stepping, emf=emf)
    h = C.c_void_p()
    rc = lib.pg_create(C.byref(make_config(spec, precision)), C.byref(h))
    assert (rc != 1) == ok, lib.pg_last_error()
    if rc == 0:
        lib.pg_destroy(h)


@pytest.mark.parametrize("extra,precision,ok", [({}, "fp64", True), ({"recon": "PARABOLIC"}, "fp64", True),
                                                 ({}, "mixed", False), ({}, "fp64_tangent", False),
                                                 ({"stepping": "HANCOCK"}, "fp64", True),
                                                 ({"char_limiting": 2}, "fp64", False)])
def test_char_limiting_validation(lib, extra, precision, ok):
    """CHAR_LIMITING YES: linear or parabolic states on the plain FP64 path."""
    spec = dict(dims=2, components=2, nx=(16, 16, 1), dx=(1 / 16, 1 / 16, 1), gamma=5 / 3, ct=False,
                char_limiting=True)
    spec.update(extra)
    c = make_config(spec, precision)
    if extra.get("char_limiting") == 2:
        c.char_limiting = 2
    h = C.c_void_p()
    rc = lib.pg_create(C.byref(c), C.byref(h))
    assert (rc != 1) == ok, lib.pg_last_error()
    if rc == 0:
        lib.pg_destroy(h)


@pytest.mark.parametrize("struct,cname", [("PgConfig", "pg_config"), ("PgOutput", "pg_output")])
def test_config_layout_matches_header(tmp_path, struct, cname):
    """The ctypes structures match the C header field by field (offsets and
    size, from a program compiled against include/pluto_gb300.h)."""
    import shutil
    import subprocess
    from pluto_gb300 import _lib as L
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    S = getattr(L, struct)
    names = [f[0] for f in S._fields_]
    src = tmp_path / "layout.c"
    src.write_text("#include <stdio.h>\n#include <stddef.h>\n#include \"pluto_gb300.h\"\nint main(void){\n"
                   + "".join(f'printf("%zu\\n", offsetof({cname}, {n}));\n' for n in names)
                   + f'printf("%zu\\n", sizeof({cname})); return 0; }}\n')
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    want = [getattr(S, n).offset for n in names] + [C.sizeof(S)]
    assert got == want, dict(zip(names + ["sizeof"], zip(got, want)))


@pytest.mark.parametrize("bc,ok", [((("reflective", "outflow"), "periodic", "periodic"), True),
                                   ((("outflow", "eqtsymmetric"), ("reflective", "outflow"), "periodic"), True),
                                   ((("periodic", "outflow"), "periodic", "periodic"), False),
                                   (("periodic", ("reflective", "periodic"), "periodic"), False)])
def test_boundary_types_per_side(lib, bc, ok):
    """A different type on each side of an axis is accepted, except that a
    periodic axis is periodic on both sides (as pluto.ini requires)."""
    spec = dict(dims=2, components=2, nx=(16, 16, 1), dx=(1 / 16, 1 / 16, 1), gamma=5 / 3, ct=True, bc=bc)
    c = make_config(spec)
    assert c.bc_sides == 1
    h = C.c_void_p()
    rc = lib.pg_create(C.byref(c), C.byref(h))
    assert (rc != 1) == ok
    if rc == 0:
        lib.pg_destroy(h)


def test_missing_library_fails_loudly(tmp_path):
    with pytest.raises(OSError):
        L.load(tmp_path / "libpluto_gb300.so")
