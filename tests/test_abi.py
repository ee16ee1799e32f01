"""The C-ABI library loads and exports every function the headers declare."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    names = []
    for h in ("sagesim_gb300.h",):
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*int\s+(sg_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_every_declared_symbol_is_exported():
    from sagesim_gb300 import _native

    lib = _native.load()
    names = declared()
    assert len(names) > 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_bindings_cover_the_header():
    from sagesim_gb300 import _native

    missing = [n for n in declared() if n not in _native.SIGNATURES]
    assert not missing, missing


def test_create_without_gpu_reports_error_or_succeeds():
    """On a machine without a GPU, engine creation fails with a status, not a crash."""
    from sagesim_gb300 import _native

    lib = _native.load()
    cfg = _native.EngineCfg(0, 0, None)
    h = ctypes.c_void_p()
    rc = lib.sg_engine_create(ctypes.byref(cfg), ctypes.byref(h))
    if rc == 0:
        lib.sg_engine_destroy(h)
    else:
        assert rc == _native.SG_ERR_CUDA
        assert "CUDA" in _native.last_error(None) or "device" in _native.last_error(None)
