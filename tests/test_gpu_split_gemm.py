"""The ComplexF64 split-BF16 GEMM (TN_PREC_SPLIT_BF16, and the C64 GEMMs of the mixed
form): every operand is cut into exact BF16 digit planes whose products run on the
tcgen05 tensor pipe, and the levels are recombined in FP64.

Parity bar: with the default 8 planes the products agree with numpy's complex128 GEMM to
≤ 1e-13 relative (normwise, ‖C − C_ref‖_F / ‖C_ref‖_F, and elementwise against the
|A|·|B| bound); the error shrinks like 2^(-7·planes) down to FP64 rounding; integer
operands whose digits fit the planes give bit-identical results.  Called through the
C ABI (tn_gemm)."""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SPLIT = 3  # TN_PREC_SPLIT_BF16


@pytest.fixture(scope="module")
def ctx():
    import tenetgb

    return tenetgb.Context(0)


def cgauss(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) / np.sqrt(2)


def op(X, o):
    return X if o == "N" else (np.swapaxes(X, -1, -2) if o == "T" else np.swapaxes(X, -1, -2).conj())


def run_gemm(ctx, A, B, Cm, opa, opb, alpha, beta, prec=SPLIT):
    """C = alpha op(A) op(B) + beta C over a batch (leading axis) through tn_gemm."""
    import tenetgb

    batch, ra, ca = A.shape
    _, rb, cb = B.shape
    m, k = (ra, ca) if opa == "N" else (ca, ra)
    n = cb if opb == "N" else rb
    dA = tenetgb.DeviceTensor.from_numpy(ctx, np.transpose(A, (1, 2, 0)))
    dB = tenetgb.DeviceTensor.from_numpy(ctx, np.transpose(B, (1, 2, 0)))
    dC = tenetgb.DeviceTensor.from_numpy(ctx, np.transpose(Cm, (1, 2, 0)))
    al = (C.c_double * 2)(alpha.real, alpha.imag)
    be = (C.c_double * 2)(beta.real, beta.imag)
    l0 = ctx.launches()
    ctx.check(ctx.lib.tn_gemm(ctx.h, 3, prec, opa.encode(), opb.encode(), m, n, k, al, C.c_void_p(dA.ptr), ra, ra * ca,
                              C.c_void_p(dB.ptr), rb, rb * cb, be, C.c_void_p(dC.ptr), m, m * n, batch))
    return np.transpose(dC.numpy(), (2, 0, 1)), ctx.launches() - l0


@pytest.mark.parametrize("opa,opb", [("N", "N"), ("C", "N"), ("N", "C"), ("T", "T")])
@pytest.mark.parametrize("m,n,k,batch", [(512, 512, 256, 2), (130, 70, 90, 3), (1024, 96, 512, 1), (64, 200, 1500, 1)])
def test_split_gemm_matches_complex128(ctx, opa, opb, m, n, k, batch):
    rng = np.random.default_rng(m + 3 * n + 7 * k)
    A = cgauss(rng, (batch,) + ((m, k) if opa == "N" else (k, m)))
    B = cgauss(rng, (batch,) + ((k, n) if opb == "N" else (n, k)))
    Cm = cgauss(rng, (batch, m, n))
    alpha, beta = 0.7 - 0.2j, 0.3 + 0.1j
    out, launches = run_gemm(ctx, A, B, Cm, opa, opb, alpha, beta)
    assert launches >= 5  # scales, digit planes and the tensor-core kernel: the split path ran
    ref = alpha * op(A, opa) @ op(B, opb) + beta * Cm
    rel = np.linalg.norm(out - ref) / np.linalg.norm(ref)
    bound = np.abs(alpha) * np.abs(op(A, opa)) @ np.abs(op(B, opb)) + np.abs(beta) * np.abs(Cm)
    assert rel <= 1e-13, rel
    assert (np.abs(out - ref) / bound).max() <= 1e-13


def test_split_gemm_error_falls_with_the_planes(ctx):
    """Error against complex128 for 3…8 planes: ~2^(-7·planes) until FP64 rounding."""
    rng = np.random.default_rng(11)
    m, n, k = 256, 192, 384
    A, B = cgauss(rng, (1, m, k)), cgauss(rng, (1, k, n))
    Z = np.zeros((1, m, n), np.complex128)
    ref = A[0] @ B[0]
    errs = {}
    for s in range(3, 9):
        ctx.check(ctx.lib.tn_set_split_slices(ctx.h, s))
        out, _ = run_gemm(ctx, A, B, Z, "N", "N", 1.0 + 0j, 0j)
        errs[s] = np.linalg.norm(out[0] - ref) / np.linalg.norm(ref)
    ctx.check(ctx.lib.tn_set_split_slices(ctx.h, 8))
    for s in range(3, 8):
        assert errs[s] <= 2.0 ** (-6 * s + 8), errs
        assert errs[s + 1] < errs[s] or errs[s + 1] < 1e-15, errs
    assert errs[8] <= 1e-14, errs
    with pytest.raises(ValueError):
        ctx.check(ctx.lib.tn_set_split_slices(ctx.h, 9))


def test_split_gemm_integer_operands_are_exact(ctx):
    """Gaussian integers of magnitude ≤ 31 at a power-of-two scale fit in the first digit
    plane: every product is an exact integer sum and the result equals the exact one."""
    rng = np.random.default_rng(5)
    m, n, k = 200, 150, 1024
    A = (rng.integers(-31, 32, (1, m, k)) + 1j * rng.integers(-31, 32, (1, m, k))) * 0.25
    B = (rng.integers(-31, 32, (1, k, n)) + 1j * rng.integers(-31, 32, (1, k, n))) * 8.0
    out, _ = run_gemm(ctx, A, B, np.zeros((1, m, n), np.complex128), "N", "N", 1.0 + 0j, 0j)
    np.testing.assert_array_equal(out[0], A[0] @ B[0])


def test_split_gemm_graded_rows_and_zero_blocks(ctx):
    """Rows and columns spanning 60 orders of magnitude, and an all-zero row and column:
    each row and column is scaled by its own power of two, so every entry keeps its own
    relative accuracy."""
    rng = np.random.default_rng(6)
    m, n, k = 96, 80, 64
    A = cgauss(rng, (1, m, k)) * np.logspace(-30, 30, m)[None, :, None]
    B = cgauss(rng, (1, k, n)) * np.logspace(20, -20, n)[None, None, :]
    A[0, 5, :] = 0
    B[0, :, 7] = 0
    out, _ = run_gemm(ctx, A, B, np.zeros((1, m, n), np.complex128), "N", "N", 1.0 + 0j, 0j)
    ref = A[0] @ B[0]
    bound = np.abs(A[0]) @ np.abs(B[0])
    assert np.all(out[0][5, :] == 0) and np.all(out[0][:, 7] == 0)
    mask = bound > 0
    assert (np.abs(out[0] - ref)[mask] / bound[mask]).max() <= 1e-13


def test_small_shapes_stay_on_fp64(ctx):
    """Below the split path's size bounds the FP64 CUDA-core kernel runs (one launch)."""
    rng = np.random.default_rng(7)
    A, B, Cm = cgauss(rng, (2, 20, 9)), cgauss(rng, (2, 9, 13)), cgauss(rng, (2, 20, 13))
    out, launches = run_gemm(ctx, A, B, Cm, "N", "N", 1.0 + 0j, 1.0 + 0j)
    assert launches == 1
    np.testing.assert_allclose(out, A @ B + Cm, rtol=0, atol=1e-13)
