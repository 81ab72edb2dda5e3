"""The allocation-free SVD entry point (tn_svd_thin_noalloc).

It exists for callers that cannot allocate device memory at the point where they need an
SVD (loops whose memory is fixed up front, a bare stream without an allocator or a
context).  It keeps its scratch in a file-scope device array instead of calling
cudaMalloc.  This test calls it through the C ABI twice in a row on the same inputs and
checks its outputs against tn_svd_thin, within the FP64 tolerance the other SVD tests use
(1e-12 relative).  The second call shows that whatever the first left in the shared
scratch does not leak into the result.  The file sorts last so that a failure here
does not stop the rest of a `-x` run.
"""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cgauss(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) / np.sqrt(2)


@pytest.mark.parametrize("m,n", [(200, 120), (512, 512), (96, 96), (1024, 512), (3000, 40), (4096, 64)])
def test_noalloc_svd_matches_tn_svd_thin_twice(m, n):
    import tenetgb

    ctx = tenetgb.Context(0)
    lib = ctx.lib
    rng = np.random.default_rng(m * 7 + n)
    A = _cgauss(rng, (m, n))
    dA = tenetgb.DeviceTensor.from_numpy(ctx, A, ["r", "c"])
    U, s, V = tenetgb.tensor_svd_thin(dA, ["r"], ["c"], "s")
    s_ref, u_ref, vh_ref = s.numpy(), U.numpy(), V.numpy()
    # buffers for the allocation-free call (allocated here by the caller, not by it)
    dU = tenetgb.DeviceTensor(ctx, (m, n), np.complex128)
    dS = tenetgb.DeviceTensor(ctx, (n,), np.float64)
    dVh = tenetgb.DeviceTensor(ctx, (n, n), np.complex128)
    ctx.sync()
    before = ctx.hbm_in_use()
    for call in range(2):
        st = lib.tn_svd_thin_noalloc(None, m, n, C.c_void_p(dA.ptr), m, C.c_void_p(dU.ptr), C.c_void_p(dS.ptr),
                                     C.c_void_p(dVh.ptr))
        assert st == 0, lib.tn_last_error_string(None).decode()
        u, sv, vh = dU.numpy(), dS.numpy(), dVh.numpy()
        assert np.abs(sv - s_ref).max() <= 1e-12 * s_ref.max(), call
        assert np.abs((u * sv) @ vh - A).max() <= 1e-12 * s_ref.max(), call
        np.testing.assert_allclose(u.conj().T @ u, np.eye(n), atol=1e-12)
        np.testing.assert_allclose(vh @ vh.conj().T, np.eye(n), atol=1e-12)
        # same decomposition as tn_svd_thin up to column phases: compare U diag(s) Vh
        assert np.abs((u * sv) @ vh - (u_ref * s_ref) @ vh_ref).max() <= 1e-12 * s_ref.max(), call
        # scrub the outputs between the two calls
        ctx.h2d(dU.ptr, np.zeros((m, n), np.complex128))
        ctx.h2d(dS.ptr, np.zeros(n))
        ctx.h2d(dVh.ptr, np.zeros((n, n), np.complex128))
    assert ctx.hbm_in_use() == before  # the context allocated nothing on its behalf


def test_noalloc_svd_rejects_sizes_beyond_its_scratch():
    import tenetgb

    lib = tenetgb._lib.load()
    # 2048 x 1024 needs (2M + 1M) * 16 bytes > 16 MiB; rejected before any launch
    st = lib.tn_svd_thin_noalloc(None, 2048, 1024, C.c_void_p(16), 2048, C.c_void_p(16), C.c_void_p(16),
                                 C.c_void_p(16))
    assert st == tenetgb._lib.TN_EINVAL
    assert b"16 MiB" in lib.tn_last_error_string(None)
    st = lib.tn_svd_thin_noalloc(None, 10, 20, C.c_void_p(16), 10, C.c_void_p(16), C.c_void_p(16), C.c_void_p(16))
    assert st == tenetgb._lib.TN_EINVAL
    # 8192 x 64 fits the scratch (8.4 MB) but the Jacobi step holds at most 4096 rows
    st = lib.tn_svd_thin_noalloc(None, 8192, 64, C.c_void_p(16), 8192, C.c_void_p(16), C.c_void_p(16),
                                 C.c_void_p(16))
    assert st == tenetgb._lib.TN_EUNSUPPORTED
    assert b"4096" in lib.tn_last_error_string(None)
