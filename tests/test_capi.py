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
