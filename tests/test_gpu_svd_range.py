"""Thin SVD of matrices whose singular values span the whole FP64 range (ground-state
Schmidt spectra of gapped chains decay past 1e-300): the Jacobi sweeps must converge,
the representable values must be accurate, and U must stay orthonormal — the columns
whose squared norms fall below the floor of the rotations get an orthonormal
completion, as a Householder SVD's U has."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def haar(rng, n):
    z = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / np.sqrt(2)
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


def wide_range_matrix(rng, m, n, zeros=0):
    s = np.logspace(0, -300, n)
    if zeros:
        s[-zeros:] = 0.0
    U = haar(rng, m)[:, :n]
    V = haar(rng, n)
    return (U * s) @ V.conj().T, s


@pytest.mark.parametrize("shape,zeros", [((256, 256), 0), ((256, 256), 40), ((300, 200), 0), ((64, 64), 8)])
@pytest.mark.parametrize("precision", ["native", "mixed"])
def test_svd_wide_dynamic_range(shape, zeros, precision):
    import tenetgb

    rng = np.random.default_rng(17 + shape[0] + zeros)
    m, n = shape
    A, s = wide_range_matrix(rng, m, n, zeros)
    T = tenetgb.DeviceTensor.from_numpy(tenetgb.default_context(), A, ["r", "c"])
    U, S, V = tenetgb.tensor_svd_thin(T, ["r"], ["c"], "s", precision=precision)
    U, S, V = U.numpy(), S.numpy(), V.numpy()
    # values in the normal range are relatively accurate where the matrix itself is
    # (entries of A are exact only to ε·‖A‖): compare the leading ones to 1e-12
    big = s > 1e-3
    assert np.allclose(S[big], s[big], rtol=1e-12, atol=0)
    assert np.all(np.diff(S) <= 0)
    assert np.abs(U.conj().T @ U - np.eye(n)).max() < 1e-12
    assert np.abs(V @ V.conj().T - np.eye(n)).max() < 1e-12
    assert np.linalg.norm((U * S) @ V - A) < 1e-13
