"""GPU parity of the individual kernels (K1 permute, K2 GEMM, K3 QR, K4 SVD, K5 ops)
against numpy/LAPACK on the same seeded inputs, through the C ABI.

Tolerances: integer-exact for the permutation (it moves bits); FP64 results within
1e-12 relative (the plain-form bar); FP32 within 1e-5.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import tenetgb

    return tenetgb.Context(0)


def cgauss(rng, shape, dtype=np.complex128):
    return ((rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) / np.sqrt(2)).astype(dtype)


@pytest.mark.parametrize("shape,perm", [
    ((64, 2, 64), (2, 1, 0)),
    ((3, 5, 7, 11), (1, 3, 0, 2)),
    ((256, 2, 256), (0, 2, 1)),
    ((33, 65), (1, 0)),
    ((1, 17, 1, 9), (3, 2, 1, 0)),
    ((8, 8, 8, 8, 8), (4, 0, 3, 1, 2)),
    ((96, 3, 5, 2), (0, 3, 1, 2)),
    ((1000, 7, 3), (0, 2, 1)),
])
@pytest.mark.parametrize("dtype", [np.complex128, np.complex64, np.float64, np.float32])
def test_permute_bit_exact(ctx, shape, perm, dtype):
    import tenetgb

    rng = np.random.default_rng(0)
    x = cgauss(rng, shape, np.complex128)
    x = (x if np.iscomplexobj(np.zeros(1, dtype)) else x.real).astype(dtype)
    labels = [f"i{k}" for k in range(len(shape))]
    t = tenetgb.DeviceTensor.from_numpy(ctx, x, labels)
    out = tenetgb.permute(t, [labels[p] for p in perm]).numpy()
    assert out.dtype == x.dtype
    np.testing.assert_array_equal(out, np.transpose(x, perm))


def test_permute_conj(ctx):
    import tenetgb

    rng = np.random.default_rng(1)
    x = cgauss(rng, (40, 3, 50))
    t = tenetgb.DeviceTensor.from_numpy(ctx, x, ["a", "b", "c"])
    out = tenetgb.permute(t, ["c", "a", "b"], conj=True).numpy()
    np.testing.assert_array_equal(out, np.transpose(x, (2, 0, 1)).conj())
    out = tenetgb.permute(t, ["a", "c", "b"], conj=True).numpy()  # contiguous mode kept: row copies
    np.testing.assert_array_equal(out, np.transpose(x, (0, 2, 1)).conj())


@pytest.mark.parametrize("opa,opb", [("N", "N"), ("N", "C"), ("C", "N"), ("T", "T"), ("T", "N")])
@pytest.mark.parametrize("m,n,k,batch", [(130, 70, 90, 1), (8, 512, 256, 1), (37, 11, 5, 3), (512, 512, 512, 1)])
def test_gemm_c64(ctx, opa, opb, m, n, k, batch):
    import ctypes as C

    import tenetgb

    rng = np.random.default_rng(2)
    ra, ca = (m, k) if opa == "N" else (k, m)
    rb, cb = (k, n) if opb == "N" else (n, k)
    A = cgauss(rng, (batch, ra, ca))
    B = cgauss(rng, (batch, rb, cb))
    Cm = cgauss(rng, (batch, m, n))

    def op(X, o):
        return X if o == "N" else (np.swapaxes(X, -1, -2) if o == "T" else np.swapaxes(X, -1, -2).conj())

    alpha, beta = 0.7 - 0.2j, 0.3 + 0.1j
    ref = alpha * op(A, opa) @ op(B, opb) + beta * Cm
    dA = tenetgb.DeviceTensor.from_numpy(ctx, np.transpose(A, (1, 2, 0)))
    dB = tenetgb.DeviceTensor.from_numpy(ctx, np.transpose(B, (1, 2, 0)))
    dC = tenetgb.DeviceTensor.from_numpy(ctx, np.transpose(Cm, (1, 2, 0)))
    al = (C.c_double * 2)(alpha.real, alpha.imag)
    be = (C.c_double * 2)(beta.real, beta.imag)
    ctx.check(ctx.lib.tn_gemm(ctx.h, 3, 0, opa.encode(), opb.encode(), m, n, k, al, C.c_void_p(dA.ptr), ra, ra * ca,
                              C.c_void_p(dB.ptr), rb, rb * cb, be, C.c_void_p(dC.ptr), m, m * n, batch))
    out = np.transpose(dC.numpy(), (2, 0, 1))
    err = np.abs(out - ref).max() / np.abs(ref).max()
    assert err < 1e-13, err


def test_gemm_real_and_c32(ctx):
    import ctypes as C

    import tenetgb

    rng = np.random.default_rng(3)
    for dt, code, tol in [(np.float64, 1, 1e-13), (np.float32, 0, 1e-5), (np.complex64, 2, 1e-5)]:
        A = cgauss(rng, (70, 50)).astype(dt) if np.iscomplexobj(np.zeros(1, dt)) else rng.standard_normal((70, 50)).astype(dt)
        B = cgauss(rng, (50, 40)).astype(dt) if np.iscomplexobj(np.zeros(1, dt)) else rng.standard_normal((50, 40)).astype(dt)
        dA = tenetgb.DeviceTensor.from_numpy(ctx, A)
        dB = tenetgb.DeviceTensor.from_numpy(ctx, B)
        dC = tenetgb.DeviceTensor(ctx, (70, 40), dt)
        one = (C.c_double * 2)(1, 0)
        zero = (C.c_double * 2)(0, 0)
        ctx.check(ctx.lib.tn_gemm(ctx.h, code, 0, b"N", b"N", 70, 40, 50, one, C.c_void_p(dA.ptr), 70, 0,
                                  C.c_void_p(dB.ptr), 50, 0, zero, C.c_void_p(dC.ptr), 70, 0, 1))
        ref = A.astype(np.complex128) @ B.astype(np.complex128)
        assert np.abs(dC.numpy() - ref).max() / np.abs(ref).max() < tol


@pytest.mark.parametrize("m,n", [(128, 64), (512, 256), (64, 128), (1024, 512), (7, 7), (300, 1), (2, 4)])
def test_qr_thin(ctx, m, n):
    import tenetgb

    rng = np.random.default_rng(4)
    A = cgauss(rng, (m, n))
    dA = tenetgb.DeviceTensor.from_numpy(ctx, A, ["r", "c"])
    Q, R = tenetgb.tensor_qr_thin(dA, ["r"], ["c"], "v")
    q, r = Q.numpy(), R.numpy()
    k = min(m, n)
    assert q.shape == (m, k) and r.shape == (k, n)
    np.testing.assert_allclose(q.conj().T @ q, np.eye(k), atol=1e-13)
    assert np.abs(q @ r - A).max() <= 1e-13 * np.abs(A).max() * max(1, np.sqrt(n))
    assert np.abs(np.tril(r, -1)).max() == 0
    assert np.abs(np.diagonal(r).imag).max() == 0


def test_qr_rank_deficient(ctx):
    """Integer fixture of the reference tests (reshape(1:64, 4, 4, 4)) is rank 2."""
    import tenetgb

    A = np.arange(1, 65, dtype=np.float64).reshape(16, 4, order="F").astype(np.complex128)
    dA = tenetgb.DeviceTensor.from_numpy(ctx, A, ["r", "c"])
    Q, R = tenetgb.tensor_qr_thin(dA, ["r"], ["c"], "v")
    q, r = Q.numpy(), R.numpy()
    np.testing.assert_allclose(q.conj().T @ q, np.eye(4), atol=1e-13)
    np.testing.assert_allclose(q @ r, A, atol=1e-12 * np.abs(A).max())


@pytest.mark.parametrize("precision", ["native", "mixed"])
@pytest.mark.parametrize("m,n", [(128, 64), (64, 128), (512, 512), (300, 260), (40, 40), (1024, 16), (3, 1)])
def test_svd_thin(ctx, m, n, precision):
    import tenetgb

    rng = np.random.default_rng(5)
    A = cgauss(rng, (m, n))
    dA = tenetgb.DeviceTensor.from_numpy(ctx, A, ["r", "c"])
    U, s, V = tenetgb.tensor_svd_thin(dA, ["r"], ["c"], "s", precision=precision)
    u, sv, vh = U.numpy(), s.numpy(), V.numpy()
    ref = np.linalg.svd(A, compute_uv=False)
    assert np.all(np.diff(sv) <= 0)
    assert np.abs(sv - ref).max() <= 1e-12 * ref.max()
    k = min(m, n)
    np.testing.assert_allclose(u.conj().T @ u, np.eye(k), atol=1e-12)
    np.testing.assert_allclose(vh @ vh.conj().T, np.eye(k), atol=1e-12)
    assert np.abs((u * sv) @ vh - A).max() <= 1e-12 * ref.max()


def test_svd_c32(ctx):
    import tenetgb

    rng = np.random.default_rng(6)
    A = cgauss(rng, (96, 80), np.complex64)
    dA = tenetgb.DeviceTensor.from_numpy(ctx, A, ["r", "c"])
    U, s, V = tenetgb.tensor_svd_thin(dA, ["r"], ["c"], "s")
    ref = np.linalg.svd(A.astype(np.complex128), compute_uv=False)
    assert np.abs(s.numpy() - ref).max() <= 1e-5 * ref.max()


def test_svd_rank_deficient_and_graded(ctx):
    import tenetgb

    rng = np.random.default_rng(7)
    m, n = 200, 120
    Uo, _ = np.linalg.qr(cgauss(rng, (m, n)))
    Vo, _ = np.linalg.qr(cgauss(rng, (n, n)))
    sv = np.logspace(0, -14, n)
    sv[-10:] = 0
    A = (Uo * sv) @ Vo.conj().T
    dA = tenetgb.DeviceTensor.from_numpy(ctx, A, ["r", "c"])
    U, s, V = tenetgb.tensor_svd_thin(dA, ["r"], ["c"], "s")
    out = s.numpy()
    assert np.abs(out - sv).max() <= 1e-12
    assert np.abs((U.numpy() * out) @ V.numpy() - A).max() <= 1e-12


@pytest.mark.parametrize("case", [
    ("ab,bc->ac", (30, 40), (40, 50)),
    ("abc,cd->abd", (20, 2, 30), (30, 25)),
    ("abc,dbe->acde", (6, 5, 7), (8, 5, 9)),
    ("ab,ab->ab", (10, 12), (10, 12)),
    ("abc,cb->ab", (16, 4, 8), (8, 4)),
    ("lsr,rtq->lstq", (16, 2, 16), (16, 2, 16)),
    ("xay,yaz->xz", (7, 3, 9), (9, 3, 11)),
])
def test_contract_matches_einsum(ctx, case):
    import tenetgb

    spec, sa, sb = case
    rng = np.random.default_rng(8)
    A, B = cgauss(rng, sa), cgauss(rng, sb)
    la, rest = spec.split(",")
    lb, lc = rest.split("->")
    shared = set(la) & set(lb)
    dims = [c for c in shared if c not in lc]
    ta = tenetgb.DeviceTensor.from_numpy(ctx, A, list(la))
    tb = tenetgb.DeviceTensor.from_numpy(ctx, B, list(lb))
    tc = tenetgb.binary_einsum(ta, tb, dims=dims, out_inds=list(lc))
    ref = np.einsum(spec, A, B)
    assert np.abs(tc.numpy() - ref).max() <= 1e-13 * max(1.0, np.abs(ref).max())


def test_hadamard_and_norm(ctx):
    import tenetgb

    rng = np.random.default_rng(9)
    A = cgauss(rng, (9, 2, 13))
    lam = np.abs(rng.standard_normal(13))
    ta = tenetgb.DeviceTensor.from_numpy(ctx, A, ["l", "o", "r"])
    ts = tenetgb.DeviceTensor.from_numpy(ctx, lam, ["r"])
    out = tenetgb.hadamard(ta, ts).numpy()
    np.testing.assert_array_equal(out, A * lam[None, None, :])
    assert abs(tenetgb.tensor_norm(ta) - np.linalg.norm(A)) <= 1e-14 * np.linalg.norm(A)


@pytest.mark.parametrize("precision", ["native", "mixed"])
def test_muscle_simple_update(ctx, precision):
    """Muscle.simple_update against the oracle's restatement: singular values kept and
    the reconstructed two-site tensor."""
    import tenetgb
    from oracle import tenet_oracle as O
    from tenetgb import workloads as W

    rng = np.random.default_rng(10)
    A = cgauss(rng, (12, 2, 20))
    B = cgauss(rng, (20, 2, 9))
    G = W.gate_tensor(W.haar_unitary(rng, 4))
    An_o, Bn_o, s_o, _ = O.simple_update_tensors(A, B, G, maxdim=10)
    ta = tenetgb.DeviceTensor.from_numpy(ctx, A, ["l", "pa", "m"])
    tb = tenetgb.DeviceTensor.from_numpy(ctx, B, ["m", "pb", "r"])
    tg = tenetgb.DeviceTensor.from_numpy(ctx, G, ["oa", "ob", "pa", "pb"])
    An, Bn = tenetgb.simple_update(ta, "pa", tb, "pb", "m", tg, "oa", "ob", maxdim=10, precision=precision)
    a, b = An.numpy(), Bn.numpy()
    assert a.shape == (12, 2, 10) and b.shape == (10, 2, 9)
    th = np.tensordot(a, b, axes=(2, 0))
    th_o = np.tensordot(An_o, Bn_o, axes=(2, 0))
    assert np.abs(th - th_o).max() <= 1e-12 * np.abs(th_o).max()


@pytest.mark.parametrize("prec,tol", [("mixed", 5e-6), ("tf32", 1e-3)])
@pytest.mark.parametrize("m,n,k", [(256, 256, 256), (130, 70, 90), (1000, 300, 520), (8, 1024, 64)])
@pytest.mark.parametrize("opa,opb", [("T", "N"), ("N", "N"), ("C", "T")])
def test_tensor_core_gemm_c32(ctx, prec, tol, m, n, k, opa, opb):
    """tcgen05 TF32 / 3xTF32 GEMM (complex via the real 4M block form) against FP64."""
    import ctypes as C

    import tenetgb

    rng = np.random.default_rng(11)
    ra, ca = (m, k) if opa == "N" else (k, m)
    rb, cb = (k, n) if opb == "N" else (n, k)
    A = cgauss(rng, (ra, ca), np.complex64)
    B = cgauss(rng, (rb, cb), np.complex64)

    def op(X, o):
        X = X.astype(np.complex128)
        return X if o == "N" else (X.T if o == "T" else X.conj().T)

    ref = op(A, opa) @ op(B, opb)
    dA = tenetgb.DeviceTensor.from_numpy(ctx, A)
    dB = tenetgb.DeviceTensor.from_numpy(ctx, B)
    dC = tenetgb.DeviceTensor(ctx, (m, n), np.complex64)
    one, zero = (C.c_double * 2)(1, 0), (C.c_double * 2)(0, 0)
    code = tenetgb.core.precision_code(prec)
    ctx.check(ctx.lib.tn_gemm(ctx.h, 2, code, opa.encode(), opb.encode(), m, n, k, one, C.c_void_p(dA.ptr), ra, 0,
                              C.c_void_p(dB.ptr), rb, 0, zero, C.c_void_p(dC.ptr), m, 0, 1))
    err = np.abs(dC.numpy() - ref).max() / (np.abs(op(A, opa)).max() * np.abs(op(B, opb)).max() * np.sqrt(k))
    assert err < tol, err


@pytest.mark.parametrize("prec", ["mixed", "tf32"])
def test_tensor_core_gemm_f32(ctx, prec):
    import ctypes as C

    import tenetgb

    rng = np.random.default_rng(12)
    m, n, k = 300, 200, 400
    A = rng.standard_normal((k, m)).astype(np.float32)
    B = rng.standard_normal((k, n)).astype(np.float32)
    ref = A.astype(np.float64).T @ B.astype(np.float64)
    dA = tenetgb.DeviceTensor.from_numpy(ctx, A)
    dB = tenetgb.DeviceTensor.from_numpy(ctx, B)
    dC = tenetgb.DeviceTensor(ctx, (m, n), np.float32)
    one, zero = (C.c_double * 2)(1, 0), (C.c_double * 2)(0, 0)
    ctx.check(ctx.lib.tn_gemm(ctx.h, 0, tenetgb.core.precision_code(prec), b"T", b"N", m, n, k, one, C.c_void_p(dA.ptr),
                              k, 0, C.c_void_p(dB.ptr), k, 0, zero, C.c_void_p(dC.ptr), m, 0, 1))
    err = np.abs(dC.numpy() - ref).max() / (np.abs(A).max() * np.abs(B).max() * np.sqrt(k))
    # measured on GB300: 3xTF32 ~1e-6 at K≈400 (the tensor pipe's FP32 accumulation is
    # coarser than FMA accumulation), single-pass TF32 ~2e-4
    assert err < (5e-6 if prec == "mixed" else 1e-3), err


def test_contract_c32_tensor_core(ctx):
    import tenetgb

    rng = np.random.default_rng(13)
    A, B = cgauss(rng, (16, 8, 32), np.complex64), cgauss(rng, (32, 8, 24), np.complex64)
    ta = tenetgb.DeviceTensor.from_numpy(ctx, A, list("abc"))
    tb = tenetgb.DeviceTensor.from_numpy(ctx, B, list("cbd"))
    tc = tenetgb.binary_einsum(ta, tb, out_inds=list("ad"), precision="mixed")
    ref = np.einsum("abc,cbd->ad", A.astype(np.complex128), B.astype(np.complex128))
    assert np.abs(tc.numpy() - ref).max() <= 1e-5 * np.abs(ref).max()


@pytest.mark.parametrize("dtype,tol", [(np.complex128, 1e-12), (np.complex64, 2e-5)])
def test_labelled_qr_and_svd_on_a_rank4_tensor(ctx, dtype, tol):
    """tn_tensor_qr_thin / tn_tensor_svd_thin (Muscle.tensor_qr_thin / tensor_svd_thin):
    the left labels are not leading in the tensor, so the library matricises by label;
    Q·R and U·diag(s)·V rebuild the tensor, Q and U are isometries, s matches LAPACK, and
    the truncated SVD keeps min(maxdim, k) values above the threshold with V compacted."""
    import tenetgb

    rng = np.random.default_rng(17)
    x = cgauss(rng, (6, 5, 7, 4)).astype(dtype)
    labels = ["a", "b", "c", "d"]
    t = tenetgb.DeviceTensor.from_numpy(ctx, x, labels)
    left = ["c", "a"]  # matrix rows: (c, a) → 42, columns: (b, d) → 20
    xm = np.transpose(x, (2, 0, 1, 3)).reshape(42, 20, order="F")
    Q, R = tenetgb.tensor_qr_thin(t, left, ind_virtual="v")
    assert Q.inds == ["c", "a", "v"] and R.inds == ["v", "b", "d"] and Q.shape == (7, 6, 20)
    q, r = Q.numpy().reshape(42, 20, order="F"), R.numpy().reshape(20, 20, order="F")
    assert np.abs(q @ r - xm).max() <= tol * np.abs(xm).max() * 10
    np.testing.assert_allclose(q.conj().T @ q, np.eye(20), atol=tol * 10)
    U, s, V = tenetgb.tensor_svd_thin(t, left, ind_s="s")
    s_ref = np.linalg.svd(xm.astype(np.complex128), compute_uv=False)
    assert np.abs(s.numpy() - s_ref).max() <= tol * s_ref[0] * 10
    u, v = U.numpy().reshape(42, 20, order="F"), V.numpy().reshape(20, 20, order="F")
    assert np.abs((u * s.numpy()) @ v - xm).max() <= tol * s_ref[0] * 10
    # truncation: maxdim 9, then |s| above the midpoint of s_5 and s_6 → keeps 6 values
    Ut, st, Vt = tenetgb.tensor_svd_thin(t, left, ind_s="s", maxdim=9, threshold=float(s_ref[5] + s_ref[6]) / 2)
    assert st.shape == (6,) and Ut.shape == (7, 6, 6) and Vt.shape == (6, 5, 4)
    ut, vt = Ut.numpy().reshape(42, 6, order="F"), Vt.numpy().reshape(6, 20, order="F")
    ref6 = (u[:, :6] * s.numpy()[:6]) @ v[:6, :]
    assert np.abs((ut * st.numpy()) @ vt - ref6).max() <= tol * s_ref[0] * 10
    with pytest.raises(ValueError):
        tenetgb.tensor_svd_thin(t, ["z"], ind_s="s")
    with pytest.raises(ValueError):
        tenetgb.tensor_qr_thin(t, ["a"], ind_virtual="b")


@pytest.mark.parametrize("k", [512, 4096])
def test_three_pass_tf32_is_fp32_grade(ctx, k):
    """3×TF32 (round-to-nearest split, corrections in their own accumulator) against the
    FP32 CUDA-core GEMM on the same ComplexF32 data.  Measured on GB300: the tensor pipe's
    FP32 accumulation of the hi·hi products truncates, so the error grows with K about
    linearly (2.4e-6 at K = 512, 1.9e-5 at K = 4096, against 5.7e-7 / 1.6e-6 for FMA
    accumulation) — within 16× of FP32, two orders better than one TF32 pass."""
    import ctypes as C

    import tenetgb

    rng = np.random.default_rng(14)
    m = n = 256
    A, B = cgauss(rng, (m, k), np.complex64), cgauss(rng, (k, n), np.complex64)
    ref = A.astype(np.complex128) @ B.astype(np.complex128)
    dA = tenetgb.DeviceTensor.from_numpy(ctx, A)
    dB = tenetgb.DeviceTensor.from_numpy(ctx, B)
    one, zero = (C.c_double * 2)(1, 0), (C.c_double * 2)(0, 0)
    errs = {}
    for prec in ("native", "mixed", "tf32"):
        dC = tenetgb.DeviceTensor(ctx, (m, n), np.complex64)
        ctx.check(ctx.lib.tn_gemm(ctx.h, 2, tenetgb.core.precision_code(prec), b"N", b"N", m, n, k, one,
                                  C.c_void_p(dA.ptr), m, 0, C.c_void_p(dB.ptr), k, 0, zero, C.c_void_p(dC.ptr), m, 0, 1))
        errs[prec] = np.linalg.norm(dC.numpy() - ref) / np.linalg.norm(ref)
    print(errs)
    assert errs["mixed"] <= 16.0 * errs["native"], errs
    assert errs["tf32"] > 10 * errs["mixed"], errs
