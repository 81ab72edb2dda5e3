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


def test_boundary_declares_the_muscle_entry_points(lib):
    """The C ABI carries the mode-labelled Muscle entry points (binary_einsum,
    tensor_qr_thin, tensor_svd_thin with compress!'s truncation, simple_update, hadamard)
    and the split-BF16 precision mode, and the library exports them."""
    syms = set(declared_symbols())
    for name in ("tn_contract", "tn_tensor_qr_thin", "tn_tensor_svd_thin", "tn_simple_update", "tn_hadamard",
                 "tn_set_split_slices", "tn_profile_enable", "tn_profile_read", "tn_pipe_peak"):
        assert name in syms and hasattr(lib, name), name
    hdr = open(os.path.join(ROOT, "include", "tenet_gb300.h")).read()
    decl = hdr[hdr.index("tn_status_t tn_tensor_svd_thin("):]
    decl = decl[: decl.index(";")]
    for arg in ("maxdim", "abs_threshold", "rank_out", "s_mode", "u_modes"):
        assert arg in decl, arg
    assert "TN_PREC_SPLIT_BF16 = 3" in hdr


def test_julia_binding_defines_the_muscle_methods():
    """TenetGB300.jl adds Muscle methods for Tensors backed by GB300Array, each reaching
    the C entry point of the same Muscle call."""
    src = open(os.path.join(ROOT, "tenet.jl_gb300", "julia", "TenetGB300.jl")).read()
    for method, entry in [("Muscle.binary_einsum(a::Tensor{T,Na,<:GB300Array}", ":tn_contract"),
                          ("Muscle.tensor_qr_thin(A::Tensor{T,N,<:GB300Array}", ":tn_tensor_qr_thin"),
                          ("Muscle.tensor_svd_thin(A::Tensor{T,N,<:GB300Array}", ":tn_tensor_svd_thin"),
                          ("Muscle.simple_update(A::Tensor{ComplexF64,Na,<:GB300Array}", ":tn_simple_update"),
                          ("Muscle.hadamard(t::Tensor{T,N,<:GB300Array}", ":tn_hadamard"),
                          ("Muscle.fuse(t::Tensor{T,N,<:GB300Array}", ":tn_permute")]:
        assert "function " + method in src or method in src, method
        assert entry in src, entry
