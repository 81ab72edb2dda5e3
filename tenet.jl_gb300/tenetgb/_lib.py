"""ctypes binding of libtenetgb.so (the C ABI declared in include/tenet_gb300.h).

The library is the only compute path: there is no CPU fallback.  Loading fails loudly
when the shared library has not been built, and every non-zero status is raised as the
Python counterpart of the Julia exception Tenet raises for it (ArgumentError →
ValueError, OutOfMemoryError → MemoryError, ErrorException → RuntimeError).
"""

from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libtenetgb.so")

TN_OK, TN_EINVAL, TN_ENOMEM, TN_ENOCONV, TN_ETIMEOUT, TN_ECUDA, TN_EUNSUPPORTED = range(7)
TN_F32, TN_F64, TN_C32, TN_C64 = range(4)
TN_PREC_NATIVE, TN_PREC_MIXED, TN_PREC_TF32, TN_PREC_SPLIT_BF16 = 0, 1, 2, 3
TN_FORM_NONCANONICAL, TN_FORM_MIXED, TN_FORM_BOND = 0, 1, 2
TN_MAX_RANK = 16


class TenetGBError(RuntimeError):
    pass


class NoConvergenceError(TenetGBError):
    pass


class DeviceTimeoutError(TenetGBError):
    pass


class tn_query(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("mps", C.c_int32),
        ("mps_b", C.c_int32),
        ("site", C.c_int32),
        ("data", C.c_void_p),
    ]


TN_Q_AMPLITUDE, TN_Q_EXPECTATION, TN_Q_OVERLAP = 0, 1, 2


class tn_tensor(C.Structure):
    _fields_ = [
        ("rank", C.c_int32),
        ("dims", C.c_int64 * TN_MAX_RANK),
        ("modes", C.c_int32 * TN_MAX_RANK),
        ("data", C.c_void_p),
    ]


_vp = C.c_void_p
_i32 = C.c_int32
_i64 = C.c_int64
_dbl = C.c_double
_sz = C.c_size_t
_pi64 = C.POINTER(C.c_int64)
_pi32 = C.POINTER(C.c_int32)
_pdbl = C.POINTER(C.c_double)
_st = C.c_int32

# name -> (restype, argtypes)
SIGNATURES = {
    "tn_create": (_st, [C.POINTER(_vp), C.c_int]),
    "tn_destroy": (_st, [_vp]),
    "tn_set_stream": (_st, [_vp, _vp]),
    "tn_get_stream": (_vp, [_vp]),
    "tn_sync": (_st, [_vp]),
    "tn_alloc": (_st, [_vp, _sz, C.POINTER(_vp)]),
    "tn_free": (_st, [_vp, _vp]),
    "tn_memcpy_h2d": (_st, [_vp, _vp, _vp, _sz]),
    "tn_memcpy_d2h": (_st, [_vp, _vp, _vp, _sz]),
    "tn_memcpy_d2d": (_st, [_vp, _vp, _vp, _sz]),
    "tn_set_hbm_budget": (_st, [_vp, _sz]),
    "tn_hbm_in_use": (_st, [_vp, C.POINTER(_sz)]),
    "tn_kernel_launches": (_st, [_vp, _pi64]),
    "tn_last_error_string": (C.c_char_p, [_vp]),
    "tn_version": (C.c_char_p, []),
    "tn_set_autotune": (_st, [_vp, _i32]),
    "tn_set_split_slices": (_st, [_vp, _i32]),
    "tn_tensor_qr_thin": (_st, [_vp, _i32, _i32, _vp, _i32, _vp, _i32, _vp, _vp]),
    "tn_tensor_svd_thin": (_st, [_vp, _i32, _i32, _vp, _i32, _vp, _i32, _i64, C.c_double, _vp, _vp, _vp, _vp]),
    "tn_profile_enable": (_st, [_vp, _i32]),
    "tn_profile_read": (_st, [_vp, _i32, _vp, _vp, _vp, _vp]),
    "tn_pipe_peak": (_st, [_vp, _i32, _vp]),
    "tn_tuning_dump": (_st, [_vp, C.c_char_p, _sz, C.POINTER(_sz)]),
    "tn_tuning_load": (_st, [_vp, C.c_char_p]),
    "tn_permute": (_st, [_vp, C.c_int, _i32, _pi64, _pi64, _pi32, _vp, _vp, _i32]),
    "tn_gemm": (
        _st,
        [_vp, C.c_int, C.c_int, C.c_char, C.c_char, _i64, _i64, _i64, _pdbl, _vp, _i64, _i64, _vp, _i64, _i64,
         _pdbl, _vp, _i64, _i64, _i64],
    ),
    "tn_contract": (_st, [_vp, C.c_int, C.c_int, C.POINTER(tn_tensor), C.POINTER(tn_tensor), C.POINTER(tn_tensor)]),
    "tn_qr_thin": (_st, [_vp, C.c_int, C.c_int, _i64, _i64, _vp, _i64, _i64, _vp, _i64, _vp, _i64, _i64]),
    "tn_svd_thin": (_st, [_vp, C.c_int, C.c_int, _i64, _i64, _vp, _i64, _i64, _vp, _i64, _vp, _i64, _vp, _i64, _i64]),
    "tn_svd_last_sweeps": (_st, [_vp, _pi32, _pi32, _pi32, _i32]),
    "tn_svd_last_ratios": (_st, [_vp, C.POINTER(C.c_float), _i32]),
    "tn_svd_refine_stats": (_st, [_vp, C.POINTER(C.c_int64), _i32]),
    "tn_svd_last_refine": (_st, [_vp, C.POINTER(C.c_float), _pi32, _pi32]),
    "tn_svd_thin_noalloc": (_st, [_vp, _i64, _i64, _vp, _i64, _vp, _vp, _vp]),
    "tn_truncation_rank": (_st, [_vp, _vp, _i64, _i64, _dbl, _pi64]),
    "tn_hadamard": (_st, [_vp, C.c_int, _i32, _pi64, _i32, _vp, _vp, _vp]),
    "tn_norm2": (_st, [_vp, C.c_int, _i64, _vp, _pdbl]),
    "tn_scale": (_st, [_vp, C.c_int, _i64, _vp, _dbl]),
    "tn_dotc": (_st, [_vp, _i64, _vp, _vp, _pdbl]),
    "tn_axpy": (_st, [_vp, _i64, _dbl, _dbl, _vp, _vp]),
    "tn_simple_update": (
        _st,
        [_vp, C.c_int, C.c_int, _i64, _i64, _i64, _i64, _i64, _vp, _vp, _vp, _i64, _dbl, _vp, _vp, _vp, _pi64],
    ),
    "tn_simple_update_absorb": (
        _st,
        [_vp, C.c_int, C.c_int, _i64, _i64, _i64, _i64, _i64, _vp, _vp, _vp, _i64, _dbl, _i32, _vp, _vp, _vp, _pi64],
    ),
    "tn_mps_create": (_st, [_vp, _i32, _i32, _pi64, _i64, C.c_int, C.POINTER(_vp)]),
    "tn_mps_create_batched": (_st, [_vp, _i32, _i32, _i32, _pi64, _i64, C.c_int, C.POINTER(_vp)]),
    "tn_mps_batch_size": (_st, [_vp, _pi32]),
    "tn_mps_set_instance_site": (_st, [_vp, _i32, _i32, _i64, _i64, _vp]),
    "tn_mps_get_instance_site": (_st, [_vp, _i32, _i32, _vp]),
    "tn_mps_destroy": (_st, [_vp]),
    "tn_mps_copy": (_st, [_vp, C.POINTER(_vp)]),
    "tn_mps_set_site": (_st, [_vp, _i32, _i64, _i64, _vp]),
    "tn_mps_get_site": (_st, [_vp, _i32, _vp]),
    "tn_mps_bond_dims": (_st, [_vp, _pi64]),
    "tn_mps_set_precision": (_st, [_vp, C.c_int]),
    "tn_mps_form": (_st, [_vp, _pi32, _pi32, _pi32]),
    "tn_mps_set_form": (_st, [_vp, _i32, _i32, _i32]),
    "tn_mps_get_lambda": (_st, [_vp, _pdbl, _pi64]),
    "tn_mps_canonize_mixed": (_st, [_vp, _i32, _i32]),
    "tn_mps_canonize_bond": (_st, [_vp, _i32]),
    "tn_mps_compress": (_st, [_vp, _i32, _i64, _dbl]),
    "tn_mps_simple_update": (_st, [_vp, _i32, _i32, _vp, _i64, _dbl]),
    "tn_mps_evolve_brickwork": (_st, [_vp, _i32, _pi32, _pi32, _vp, _i64, _dbl]),
    "tn_mps_evolve_layers": (_st, [_vp, _i32, _pi32, _pi32, _pi32, _vp, _i64, _dbl]),
    "tn_mps_overlap": (_st, [_vp, _vp, _pdbl]),
    "tn_mps_norm": (_st, [_vp, _pdbl]),
    "tn_mps_normalize": (_st, [_vp]),
    "tn_mps_amplitude": (_st, [_vp, _vp, _pdbl]),
    "tn_mps_local_expectations": (_st, [_vp, _vp, _pdbl]),
    "tn_mps_sample": (_st, [_vp, _i32, _i64, _pdbl, _pi32]),
    "tn_mps_evolve_mpo": (_st, [_vp, C.POINTER(_vp), _pi64, _i32, _i64, _dbl]),
    "tn_mps_set_instance_sites": (_st, [_vp, _i32, C.POINTER(_vp)]),
    "tn_mps_get_instance_sites": (_st, [_vp, _i32, C.POINTER(_vp)]),
    "tn_mps_dmrg": (_st, [_vp, C.POINTER(_vp), _pi64, _i32, _i32, _i32, _i64, _i32, _i32, _dbl, _pdbl, _pdbl]),
    "tn_dmrg_last_stats": (_st, [_vp, _pdbl, _pi64]),
    "tn_mps_save": (_st, [_vp, C.c_char_p]),
    "tn_mps_shape": (_st, [_vp, _pi32, _pi32, _pi32]),
    "tn_mps_load": (_st, [_vp, C.c_char_p, _i64, C.POINTER(_vp)]),
    # query server
    "tn_serve_create": (_st, [_i32, _sz, _sz, _i32, C.c_int, C.POINTER(_vp)]),
    "tn_serve_destroy": (_st, [_vp]),
    "tn_serve_add_mps": (_st, [_vp, _i32, _i32, _pi64, C.POINTER(_vp), _pi32]),
    "tn_serve_add_random_mps": (_st, [_vp, _i32, _i32, _i64, C.c_uint64, _pi32]),
    "tn_serve_remove_mps": (_st, [_vp, _i32]),
    "tn_serve_mps_info": (_st, [_vp, _i32, _pi32, _pi32, _pi64, _pdbl]),
    "tn_serve_get_site": (_st, [_vp, _i32, _i32, _vp]),
    "tn_serve_submit": (_st, [_vp, _vp, _pi64]),
    "tn_serve_wait": (_st, [_vp, _i64, _dbl, _pdbl, _pdbl]),
    "tn_serve_stats": (_st, [_vp, _pi64]),
    "tn_serve_last_error": (C.c_char_p, []),
    # grouped (ragged) MPS batches
    "tn_group_create": (_st, [_vp, _i32, _pi32, _i32, _pi64, C.POINTER(_vp)]),
    "tn_group_destroy": (_st, [_vp]),
    "tn_group_fill_random": (_st, [_vp, C.c_uint64]),
    "tn_group_set_site": (_st, [_vp, _i32, _i32, _vp]),
    "tn_group_get_site": (_st, [_vp, _i32, _i32, _vp]),
    "tn_group_bond_dims": (_st, [_vp, _i32, _pi64]),
    "tn_group_canonize_compress_norm": (_st, [_vp, _pi64, _pdbl]),
    "tn_group_lambda": (_st, [_vp, _i32, _pdbl, _pi64]),
}

_lib = None
_shutting_down = False


def _mark_shutdown():
    global _shutting_down
    _shutting_down = True


def shutting_down():
    """True once the interpreter is exiting: destructors then leave device memory to
    the process teardown instead of calling into the library."""
    return _shutting_down


import atexit  # noqa: E402

atexit.register(_mark_shutdown)


def load():
    """Load libtenetgb.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"libtenetgb.so not found at {LIB_PATH}; build it with `python tenet.jl_gb300/build.py`"
        )
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def check(status, ctx=None):
    if status == TN_OK:
        return
    lib = load()
    msg = lib.tn_last_error_string(ctx).decode(errors="replace")
    if status == TN_EINVAL:
        raise ValueError(msg)
    if status == TN_ENOMEM:
        raise MemoryError(msg)
    if status == TN_ENOCONV:
        raise NoConvergenceError(msg)
    if status == TN_ETIMEOUT:
        raise DeviceTimeoutError(msg)
    if status == TN_EUNSUPPORTED:
        raise NotImplementedError(msg)
    raise TenetGBError(f"status {status}: {msg}")
