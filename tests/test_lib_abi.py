"""CPU checks of the C ABI: the library builds, loads, exports every symbol declared in
include/*.h, and fails cleanly (no crash, a status + message) without a GPU."""

import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            txt = open(os.path.join(inc, f)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names.update(re.findall(r"\b(tn_\w+)\s*\(", txt))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from tenetgb import _lib

    if not os.path.exists(_lib.LIB_PATH):
        import importlib.util

        spec = importlib.util.spec_from_file_location("tn_build", os.path.join(ROOT, "tenet.jl_gb300", "build.py"))
        m = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(m)
        m.build()
    return _lib.load()


def test_exports_every_declared_symbol(lib):
    syms = declared_symbols()
    assert len(syms) > 30
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_python_binding_covers_header():
    from tenetgb import _lib

    assert set(declared_symbols()) <= set(_lib.SIGNATURES)


def test_version_and_clean_error_without_gpu(lib):
    import torch

    assert b"sm_103a" in lib.tn_version()
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    h = ctypes.c_void_p()
    st = lib.tn_create(ctypes.byref(h), 0)
    assert st != 0
    assert lib.tn_last_error_string(None)


def test_null_context_is_rejected(lib):
    assert lib.tn_sync(None) != 0
    assert lib.tn_permute(None, 3, 2, None, None, None, None, None, 0) != 0
