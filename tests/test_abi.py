"""The C-ABI library loads and exports every entry point include/*.h
declares (no compute call: runs without a GPU)."""

import glob
import os
import re
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\bint\s+(fqegpu_\w+)\s*\(", text))
    return names


@pytest.fixture(scope="module")
def libpath():
    import fqe_gb300
    return fqe_gb300.build()


def test_header_declares_entry_points():
    names = _declared()
    assert "fqegpu_apply" in names and "fqegpu_graph_create" in names
    assert len(names) >= 25


def test_library_exports_every_declared_symbol(libpath):
    out = subprocess.run(["nm", "-D", "--defined-only", libpath],
                         capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (fqegpu_\w+)", out))
    missing = _declared() - exported
    assert not missing, f"declared but not exported: {sorted(missing)}"


def test_ctypes_binding_covers_header(libpath):
    from fqe_gb300 import _lib
    lib = _lib.load(libpath)
    for name in _declared():
        assert hasattr(lib, name)
    assert set(_lib.exported_symbols()) <= _declared()
    assert lib.fqegpu_version() >= 100  # no CUDA call


def test_missing_library_fails_loudly(tmp_path):
    from fqe_gb300 import _lib
    saved = _lib._lib
    _lib._lib = None
    try:
        with pytest.raises(_lib.FqeGpuError):
            _lib.load(str(tmp_path / "absent.so"))
    finally:
        _lib._lib = saved


def test_status_codes_map_to_reference_exceptions(libpath):
    from fqe_gb300 import _lib
    _lib.load(libpath)
    with pytest.raises(ValueError):
        _lib.check(_lib.ERR_INVALID)
    with pytest.raises(MemoryError):
        _lib.check(_lib.ERR_NOMEM)
    with pytest.raises(NotImplementedError):
        _lib.check(_lib.ERR_UNSUPPORTED)
    with pytest.raises(TimeoutError):
        _lib.check(_lib.ERR_TIMEOUT)
    with pytest.raises(RuntimeError):
        _lib.check(_lib.ERR_NUMERIC)
    _lib.check(_lib.OK)


def test_invalid_graph_arguments_rejected_before_cuda(libpath):
    import ctypes
    from fqe_gb300 import _lib
    lib = _lib.load(libpath)
    h = ctypes.c_void_p()
    assert lib.fqegpu_graph_create(3, 4, 1, None, ctypes.byref(h)) == _lib.ERR_INVALID
    assert "nalpha" in _lib.last_error()
    assert lib.fqegpu_graph_create(70, 1, 1, None, ctypes.byref(h)) == _lib.ERR_INVALID
