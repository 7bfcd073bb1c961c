"""The C-ABI library loads and exports every entry point its header declares
(no compute calls: this runs without a GPU)."""

import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(iso_\w+)\s*\(", src))
    return names


def test_library_exports_header_symbols():
    from isoext_gb300 import _build

    lib = ctypes.CDLL(str(_build.build()))
    names = _declared()
    assert "iso_mc_dense" in names
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_library_reports_abi_and_config():
    from isoext_gb300 import _ffi

    lib = _ffi.lib()
    assert lib.iso_abi_version() == 2
    t = ctypes.c_int()
    lib.iso_mc_get_config(ctypes.byref(t))
    assert t.value in (128, 256)
    assert lib.iso_mc_set_config(100) == 1  # not 128 / 256 -> ISO_ERR_ARG
    assert "threads" in _ffi.last_error()


def test_unknown_method_message():
    import isoext_gb300 as iso

    import pytest

    with pytest.raises(RuntimeError, match="Unknown method: foo"):
        iso.mc.method_id("foo")


def test_tunables_roundtrip_and_reject_bad_values():
    from isoext_gb300 import _ffi, tune

    lib = _ffi.lib()
    old = tune.current()
    assert set(old) == set(tune.KNOBS)
    for key, values in tune.KNOBS.items():
        for v in values:
            tune.set(key, v)
            assert tune.get(key) == v
    assert lib.iso_tune_set(b"mc.emit_threads", 100) == 1
    assert lib.iso_tune_set(b"dc.cell_threads", 96) == 1
    assert lib.iso_tune_set(b"mc.sign_ctas_per_sm", 0) == 1
    assert lib.iso_tune_set(b"no.such.key", 1) == 1 and "unknown" in _ffi.last_error()
    tune.apply(old)
    assert tune.current() == old


def test_library_has_no_unresolved_symbols_of_its_own():
    """Every symbol the library calls is defined in it or in the C / C++ runtime
    (a mismatched declaration between translation units would show up here)."""
    import shutil
    import subprocess

    import pytest

    from isoext_gb300 import _build

    nm = shutil.which("nm")
    if not nm:
        pytest.skip("nm not available")
    out = subprocess.run([nm, "-D", "--undefined-only", str(_build.build())], capture_output=True, text=True).stdout
    own = [ln.split()[-1] for ln in out.splitlines()
           if ln.strip() and "@" not in ln and not ln.split()[-1].startswith(("_ITM_", "__gmon_start__"))]
    assert not own, own


def _prototypes():
    """{name: [parameter declarations]} of the header's entry points."""
    protos = {}
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if not fn.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", fn)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        for m in re.finditer(r"\b(iso_\w+)\s*\(([^;{]*?)\)\s*;", src):
            params = " ".join(m.group(2).split())
            protos[m.group(1)] = [] if params in ("", "void") else [p.strip() for p in params.split(",")]
    return protos


def _kind_of_param(decl):
    if "*" in decl or "[" in decl:
        return "pointer"
    words = decl.replace("const ", "").split()[:-1]  # drop the parameter's name
    t = " ".join(words)
    return {"float": "float", "double": "double", "int": "int", "unsigned": "uint", "unsigned int": "uint",
            "long long": "longlong", "size_t": "size_t"}.get(t, t)


def _kind_of_ctype(t):
    if t in (ctypes.c_void_p, ctypes.c_char_p) or issubclass(t, (ctypes._Pointer, ctypes.Array)):
        return "pointer"
    for kind, ct in (("float", ctypes.c_float), ("double", ctypes.c_double), ("int", ctypes.c_int),
                     ("uint", ctypes.c_uint), ("longlong", ctypes.c_longlong), ("size_t", ctypes.c_size_t)):
        if t is ct:
            return kind
    return t.__name__


def test_bindings_match_the_header_prototypes():
    """Every entry point the package binds with argtypes takes, in the header,
    the same number of parameters of the same kinds (a mismatch would only show
    as a wrong call on a GPU)."""
    import importlib

    import isoext_gb300
    from isoext_gb300 import _ffi

    for mod in ("mc", "dc", "sparse", "diff", "serve", "grids", "tune"):
        try:
            importlib.import_module(f"isoext_gb300.{mod}")
        except ModuleNotFoundError:
            pass
    lib = _ffi.lib()
    _ffi._apply(lib, _ffi._EXTRA)
    protos = _prototypes()
    checked, bad = 0, []
    for name, params in sorted(protos.items()):
        fn = getattr(lib, name, None)
        if fn is None or fn.argtypes is None:
            continue
        checked += 1
        want = [_kind_of_param(p) for p in params]
        got = [_kind_of_ctype(t) for t in fn.argtypes]
        if want != got:
            bad.append((name, want, got))
    assert checked >= 30, checked
    assert not bad, bad


def test_failures_leave_a_message_of_their_own():
    """After a failure, iso_last_error describes that failure, not an earlier one.
    Each call here fails on its arguments or its workspace size, checked on the
    host before any device work: the placeholder device pointers are never read."""
    import importlib

    from isoext_gb300 import _ffi

    for mod in ("dc", "sparse"):
        importlib.import_module(f"isoext_gb300.{mod}")
    lib = _ffi.lib()
    _ffi._apply(lib, _ffi._EXTRA)
    lo, hi = (ctypes.c_float * 3)(-1, -1, -1), (ctypes.c_float * 3)(1, 1, 1)
    P = 1 << 20  # a placeholder device address, 16-byte aligned, never dereferenced

    def stale():
        assert lib.iso_mc_set_config(100) == 1 and "threads" in _ffi.last_error()

    stale()
    rc = lib.iso_dc_dense_ex(P, 8, 8, 8, lo, hi, 0.0, 1e-2, 1e-6, P, 16, P, 16, P, 0, None, None, None, None, None,
                             None)
    assert rc == 1 and _ffi.last_error() == "invalid argument"  # counts and status are required
    stale()
    rc = lib.iso_dc_dense_ex(P, 8, 8, 8, lo, hi, 0.0, 1e-2, 1e-6, P, 16, P, 16, P, 0, P, P, None, None, None, None)
    assert rc == 5 and _ffi.last_error() == "workspace too small"
    stale()
    rc = lib.iso_sparse_mc(P, P, 10, 8, 8, 8, lo, hi, 0.0, 7, P, 16, P, 16, P, 0, P, P, None)
    assert rc == 1 and _ffi.last_error() == "invalid argument"  # method 7
    stale()
    rc = lib.iso_sparse_mc(P, P, 10, 8, 8, 8, lo, hi, 0.0, 0, P, 16, P, 16, P, 0, P, P, None)
    assert rc == 5 and _ffi.last_error() == "workspace too small"
    stale()
    rc = lib.iso_weld_mesh(P, 10, P, 4, P, P, None, P, P, P, 0, None)
    assert rc == 5 and _ffi.last_error() == "workspace too small"
    stale()
    rc = lib.iso_sort_vertices(P, -1, P, 4, P, 0, None)
    assert rc == 1 and _ffi.last_error() == "invalid argument"
    import isoext_gb300.serve  # noqa: F401  (its bindings)

    _ffi._apply(lib, _ffi._EXTRA)
    out = ctypes.c_void_p()
    stale()
    assert lib.iso_serve_create(0, 1 << 30, None, 0, ctypes.byref(out)) == 1  # no slots
    assert _ffi.last_error() == "invalid argument" and not out.value
    stale()
    assert lib.iso_serve_set_bucket(None, 2) == 1 and _ffi.last_error() == "invalid argument"
    stale()
    assert lib.iso_serve_set_capacity_scale(None, 0.5) == 1 and _ffi.last_error() == "invalid argument"
