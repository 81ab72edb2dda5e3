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


@pytest.mark.parametrize("spectrum", ["near_degenerate", "cluster_at_cut", "rank_deficient", "graded"])
@pytest.mark.parametrize("precision", ["native", "mixed"])
def test_truncated_gate_svd_on_designed_spectra(spectrum, precision):
    """The truncated SVD of a gate (Muscle.simple_update, θ 512×512 kept to 256) on a
    θ = U·diag(s)·Vᴴ of designed spectrum: near-degenerate kept pairs (relative gaps
    1e-9), a cluster straddling the cut, exact zeros, and a graded decay.  In mixed
    precision this is the FP32 pre-pass + matrix-product refinement path.  The kept values
    must match s to 1e-12 of s_max and θ' = A'·B' the rank-256 truncation of θ to 1e-12
    relative (for the straddling cluster, any orthonormal split of the cluster is right,
    so there the kept weight and the subspace are compared instead)."""
    import tenetgb

    rng = np.random.default_rng({"near_degenerate": 1, "cluster_at_cut": 2, "rank_deficient": 3, "graded": 4}[spectrum])
    n = 512
    s = np.sort(rng.uniform(0.01, 1.0, n))[::-1]
    if spectrum == "near_degenerate":
        for k in (10, 100, 200):
            s[k + 1] = s[k] * (1 - 1e-9)
    elif spectrum == "cluster_at_cut":
        s[250:262] = s[250]
    elif spectrum == "rank_deficient":
        s[300:] = 0.0
    else:
        s = np.logspace(0, -14, n)
    U, V = haar(rng, n), haar(rng, n)
    ctx = tenetgb.Context(0)
    # θ as A (512, 1, 512) · B (512, 1, 512) with the identity gate on d = 1
    A = tenetgb.DeviceTensor.from_numpy(ctx, (U * s).reshape(n, 1, n), ["l", "a", "m"])
    B = tenetgb.DeviceTensor.from_numpy(ctx, V.conj().T.reshape(n, 1, n), ["m", "b", "r"])
    G = tenetgb.DeviceTensor.from_numpy(ctx, np.ones((1, 1, 1, 1), np.complex128), ["ao", "bo", "a", "b"])
    An, Bn = tenetgb.simple_update(A, "a", B, "b", "m", G, "ao", "bo", maxdim=256, threshold=1e-12,
                                   precision=precision)
    an, bn = An.numpy().reshape(n, -1), Bn.numpy().reshape(-1, n)
    assert an.shape[1] == 256
    if precision == "mixed":
        # the refinement converges on every spectrum the FP32 pre-pass resolves; the
        # graded one (kept values down to 1e-7 of the largest) leaves the quadratic
        # regime at once and is finished by FP64 sweeps from the pre-pass basis
        trace, outcome = ctx.last_refine()
        assert outcome == ("diverged" if spectrum == "graded" else "converged"), (outcome, trace)
        if outcome == "converged":
            assert trace[-1][0] <= 1e-8 and trace[-1][1] <= 1e-8, trace
    s_dev = np.sort(np.linalg.svd(an, compute_uv=False) ** 2)[::-1]
    assert np.abs(s_dev - s[:256]).max() <= 1e-12 * s[0]
    th = an @ bn
    if spectrum == "cluster_at_cut":
        assert abs(np.linalg.norm(th) ** 2 - np.sum(s[:256] ** 2)) <= 1e-12 * np.sum(s[:256] ** 2)
        P = U[:, :262] @ U[:, :262].conj().T
        assert np.linalg.norm(th - P @ th) <= 1e-12 * np.linalg.norm(th)
    else:
        ref = (U[:, :256] * s[:256]) @ V[:, :256].conj().T
        assert np.linalg.norm(th - ref) <= 1e-12 * np.linalg.norm(ref)
