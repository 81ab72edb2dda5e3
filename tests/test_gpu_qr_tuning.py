"""Every launch configuration the QR autotuner may pick (panel width 4/8/16 × block-
reflector slab 1/2/4, forced through the tuning table) and the autotuner itself give the
same factorisation: A = QR to FP64 accuracy, QᴴQ = I, R upper triangular with a real
diagonal.  Shapes of the TEBD gauge moves (512×256, B = 1 and 16) and
ragged ones.  Called through the C ABI (tn_qr_thin)."""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def cgauss(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) / np.sqrt(2)


def run_qr(ctx, A):
    import tenetgb

    batch, m, n = A.shape
    k = min(m, n)
    dA = tenetgb.DeviceTensor.from_numpy(ctx, np.transpose(A, (1, 2, 0)))
    dQ = tenetgb.DeviceTensor(ctx, (m, k, batch), np.complex128)
    dR = tenetgb.DeviceTensor(ctx, (k, n, batch), np.complex128)
    ctx.check(ctx.lib.tn_qr_thin(ctx.h, 3, 0, m, n, C.c_void_p(dA.ptr), m, m * n, C.c_void_p(dQ.ptr), m * k,
                                 C.c_void_p(dR.ptr), k * n, batch))
    return np.transpose(dQ.numpy(), (2, 0, 1)), np.transpose(dR.numpy(), (2, 0, 1))


def check(A, Q, R):
    for b in range(A.shape[0]):
        assert np.linalg.norm(Q[b] @ R[b] - A[b]) <= 1e-13 * np.linalg.norm(A[b])
        assert np.abs(Q[b].conj().T @ Q[b] - np.eye(Q.shape[2])).max() <= 1e-13
        assert np.allclose(np.tril(R[b], -1), 0)
        d = np.diag(R[b])
        assert np.all(np.abs(d.imag) <= 1e-13 * np.abs(d).max())


def bucket(batch):
    return 1 if batch <= 1 else 4 if batch <= 4 else 16 if batch <= 16 else 64


@pytest.mark.parametrize("m,n,batch", [(512, 256, 1), (512, 256, 16), (300, 77, 3), (64, 64, 2), (8, 64, 2),
                                       (256, 512, 1), (4, 2, 16)])
@pytest.mark.parametrize("nb,slab", [(nb, s) for nb in (4, 8, 16) for s in (1, 2, 4)])
def test_forced_configuration(m, n, batch, nb, slab):
    import tenetgb

    ctx = tenetgb.Context(0)
    ctx.load_tuning(f"qr16:{m}:{n}:{bucket(batch)} {nb} {slab}\n")
    rng = np.random.default_rng(m + n + batch)
    A = cgauss(rng, (batch, m, n))
    Q, R = run_qr(ctx, A)
    check(A, Q, R)


@pytest.mark.parametrize("m,n,batch", [(512, 256, 1), (512, 256, 16)])
def test_autotuned(m, n, batch):
    import tenetgb

    ctx = tenetgb.Context(0)
    ctx.set_autotune(True)
    rng = np.random.default_rng(2 * m + n + batch)
    A = cgauss(rng, (batch, m, n))
    for rep in range(2):  # the first call tunes, the second uses the table
        Q, R = run_qr(ctx, A)
        check(A, Q, R)


def test_autotuned_in_place():
    """Q written over A (the MPS gauge move factors a site in place): the autotuner's
    candidate runs must all factor the original A, not a previous candidate's Q."""
    import tenetgb

    ctx = tenetgb.Context(0)
    ctx.set_autotune(True)
    rng = np.random.default_rng(41)
    batch, m, n = 4, 512, 256
    A = cgauss(rng, (batch, m, n))
    dA = tenetgb.DeviceTensor.from_numpy(ctx, np.transpose(A, (1, 2, 0)))
    dR = tenetgb.DeviceTensor(ctx, (n, n, batch), np.complex128)
    ctx.check(ctx.lib.tn_qr_thin(ctx.h, 3, 0, m, n, C.c_void_p(dA.ptr), m, m * n, C.c_void_p(dA.ptr), m * n,
                                 C.c_void_p(dR.ptr), n * n, batch))
    Q = np.transpose(dA.numpy(), (2, 0, 1))
    R = np.transpose(dR.numpy(), (2, 0, 1))
    check(A, Q, R)
