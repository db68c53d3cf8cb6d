"""CPU-side checks of the boundary: librast.so builds, loads without a GPU, and exports every
entry point declared in include/rast.h; the Python mirror binds all of them."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    with open(os.path.join(ROOT, "include", "rast.h")) as f:
        src = f.read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(rast_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from rusterizer_gb300 import build
    path = build.build()
    return ctypes.CDLL(path)


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("rast_create", "rast_destroy", "rast_mesh_upload", "rast_texture_upload",
              "rast_set_uniforms", "rast_draw", "rast_framebuffer", "rast_read_samples"):
        assert s in syms


def test_library_exports_every_declared_symbol(lib):
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_python_binding_covers_header():
    from rusterizer_gb300 import _lib
    missing = [s for s in declared_symbols() if s not in _lib.SIGNATURES]
    assert not missing, missing


def test_status_strings_without_gpu(lib):
    from rusterizer_gb300 import _lib
    L = _lib.load()
    for code, name in enumerate(_lib.STATUS_NAMES):
        assert L.rast_status_string(code)


def test_create_rejects_bad_arguments_without_touching_cuda(lib):
    from rusterizer_gb300 import _lib
    L = _lib.load()
    st = ctypes.c_int(-1)
    assert not L.rast_create(0, 10, 4, ctypes.byref(st))
    assert st.value == _lib.INVALID_ARG
    assert not L.rast_create(10, 10, 2, ctypes.byref(st))
    assert st.value == _lib.INVALID_ARG


def test_oracle_library_loads():
    import oracle
    assert oracle.lib() is not None
