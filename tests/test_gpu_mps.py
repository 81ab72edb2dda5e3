"""GPU parity of the device-resident MPS operations (canonize!, compress!,
simple_update!, overlap, norm, amplitudes, ⟨O_i⟩, TEBD) against the CPU oracle and the
reference's own invariant tests (test/unit/mps.jl, test/unit/simple_update.jl), called
through the C ABI.  Gauge-dependent outputs are compared through gauge-invariant
quantities: contracted states, singular values, overlaps and expectation values."""

import numpy as np
import pytest

from oracle import tenet_oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import tenetgb

    return tenetgb.Context(0)


def jl(a, b, *shape):
    return np.arange(a, b + 1, dtype=np.float64).reshape(shape, order="F")


def fixture_arrays(first=None):
    return [jl(1, 16, 4, 4) if first is None else first, jl(1, 64, 4, 4, 4), jl(1, 64, 4, 4, 4), jl(1, 64, 4, 4, 4),
            jl(1, 16, 4, 4)]


def gpu_mps(ctx, arrays=None, sites=None, **kw):
    import tenetgb

    if arrays is not None:
        return tenetgb.MPS(arrays=arrays, order=("l", "r", "o"), ctx=ctx, **kw)
    return tenetgb.MPS(sites, ctx=ctx, **kw)


def state(psi):
    """contract(ψ) with Λ absorbed (the reference tests' hadamard + rmtensor!)."""
    import tenetgb

    sites = psi.sites()
    f = psi.form
    if isinstance(f, tenetgb.BondCanonical):
        lam = psi.lambda_()
        sites[f.a - 1] = sites[f.a - 1] * lam[None, None, :]
    v = sites[0]
    for A in sites[1:]:
        v = np.tensordot(v, A, axes=(v.ndim - 1, 0))
    return v.reshape(-1)


def close_state(a, b):
    return np.linalg.norm(a - b) <= np.sqrt(np.finfo(float).eps) * max(np.linalg.norm(a), np.linalg.norm(b))


def iso(psi, i, side):
    return O.isisometry(psi.site(i), 2 if side == "r" else 0)


def test_noncanonical_to_mixed(ctx):
    import tenetgb

    psi = gpu_mps(ctx, fixture_arrays())
    v0 = state(psi)
    psi.unsafe_setform_(tenetgb.NonCanonical())
    c = tenetgb.canonize(psi, 3)
    assert c.form == tenetgb.MixedCanonical(3)
    assert iso(c, 1, "r") and iso(c, 2, "r") and iso(c, 4, "l") and iso(c, 5, "l")
    assert not iso(c, 3, "l") and not iso(c, 3, "r")
    assert close_state(state(c), v0)
    c2 = tenetgb.canonize(psi, [2, 3])
    assert c2.form == tenetgb.MixedCanonical([2, 3])
    assert iso(c2, 1, "r") and iso(c2, 4, "l") and iso(c2, 5, "l")
    assert close_state(state(c2), v0)


@pytest.mark.parametrize("start", [5, [3, 4, 5], (4, 5), (2, 3)])
def test_to_mixed_from_various(ctx, start):
    import tenetgb

    psi = gpu_mps(ctx, fixture_arrays())
    v0 = state(psi)
    psi.canonize_(start)
    assert close_state(state(psi), v0)
    c = tenetgb.canonize(psi, 3)
    assert c.form == tenetgb.MixedCanonical(3)
    assert iso(c, 1, "r") and iso(c, 2, "r") and iso(c, 4, "l") and iso(c, 5, "l")
    assert close_state(state(c), v0)


@pytest.mark.parametrize("start", [None, 5, [3, 4, 5], (4, 5)])
def test_to_bond_canonical(ctx, start):
    import tenetgb

    psi = gpu_mps(ctx, fixture_arrays())
    v0 = state(psi)
    if start is None:
        psi.unsafe_setform_(tenetgb.NonCanonical())
    else:
        psi.canonize_(start)
    c = tenetgb.canonize(psi, (2, 3))
    assert c.form == tenetgb.BondCanonical(2, 3)
    assert iso(c, 1, "r") and not iso(c, 2, "l") and not iso(c, 3, "r")
    assert iso(c, 4, "l") and iso(c, 5, "l")
    assert close_state(state(c), v0)
    # Λ equals the oracle's Schmidt values at that bond
    p = O.mps_from_arrays(fixture_arrays(), order=("l", "r", "o"))
    O.canonize(p, (2, 3))
    lam = c.lambda_()
    ref = p.lam[2]
    assert np.abs(lam - ref).max() <= 1e-12 * ref.max()


def test_compress_single_and_all(ctx):
    import tenetgb

    for kw in (dict(maxdim=1), dict(threshold=0.1)):
        psi = gpu_mps(ctx, fixture_arrays(np.ones((4, 4))))
        v0 = state(psi)
        c = tenetgb.compress(psi, (1, 2), **kw)
        assert c.bondsizes()[0] == 1
        assert close_state(state(c), v0)
    psi = gpu_mps(ctx, fixture_arrays(np.ones((4, 4))))
    c = tenetgb.compress(psi, maxdim=1)
    assert all(b == 1 for b in c.bondsizes())


def test_bondsizes_truncate(ctx):
    import tenetgb
    from tenetgb import workloads as W

    psi = gpu_mps(ctx, sites=W.random_mps_arrays(8, 2, 128, seed=0))
    assert psi.bondsizes() == [2, 4, 8, 16, 8, 4, 2]
    tenetgb.truncate_(psi, maxdim=10)
    assert psi.maxbondsize() == 10
    # same Schmidt spectra as the oracle after truncation
    p = O.OMPS(W.random_mps_arrays(8, 2, 128, seed=0))
    O.compress(p, maxdim=10)
    assert psi.bondsizes() == p.bondsizes()
    assert abs(psi.norm() - O.norm(p)) <= 1e-12


def test_simple_update_known_answers(ctx):
    import tenetgb

    X = np.array([[0, 1], [1, 0]], dtype=np.complex128)
    psi = gpu_mps(ctx, sites=[np.array([1.0, 0.0]).reshape(1, 2, 1), np.array([0.0, 1.0]).reshape(1, 2, 1)])
    psi.simple_update_(X, [1])
    assert np.allclose(psi.site(1).reshape(-1), [0, 1])
    psi.simple_update_(X, [2])
    assert np.allclose(psi.site(2).reshape(-1), [1, 0])
    # CX on |11⟩ with gate indices [2, 1, 2', 1'] (test/unit/simple_update.jl:16-43)
    cx = np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]], dtype=np.complex128)
    G = np.transpose(cx.reshape(2, 2, 2, 2, order="F"), (1, 0, 3, 2))
    psi = gpu_mps(ctx, sites=[np.array([0.0, 1.0]).reshape(1, 2, 1), np.array([0.0, 1.0]).reshape(1, 2, 1)])
    tenetgb.simple_update_(psi, G, [1, 2])
    a, b = psi.site(1), psi.site(2)
    assert a.shape == (1, 2, 2)
    assert np.allclose(np.abs(a[0, :, 0]), [0, 1]) and np.allclose(np.abs(a[0, :, 1]), [0, 0])
    assert np.allclose(np.abs(b[0, :, 0]), [1, 0]) and np.allclose(np.abs(b[1, :, 0]), [0, 0])


def test_overlap_norm_amplitude_expectations(ctx):
    import tenetgb
    from tenetgb import workloads as W

    sites = W.random_mps_arrays(12, 2, 8, seed=11, orthogonalize=False)
    psi = gpu_mps(ctx, sites=sites)
    p = O.OMPS([s.copy() for s in sites])
    ov, ov_o = psi.overlap(psi), O.overlap(p, p)
    assert abs(ov - ov_o) <= 1e-12 * abs(ov_o)
    other = W.random_mps_arrays(12, 2, 5, seed=12, orthogonalize=False)
    q = gpu_mps(ctx, sites=other)
    x, x_o = psi.overlap(q), O.overlap(p, O.OMPS(other))
    assert abs(x - x_o) <= 1e-12 * np.sqrt(abs(ov_o) * abs(O.overlap(O.OMPS(other), O.OMPS(other))))
    for bits in ["010011010110", "+-ud01+-ud01"]:
        a, a_o = psi.amplitude(bits), O.amplitude(O.product_state_vectors(bits), p)
        assert abs(a - a_o) <= 1e-12 * np.sqrt(abs(ov_o))
    z, z_o = psi.local_expectations(W.pauli_z()), O.local_expectations(p, W.pauli_z())[0]
    assert np.abs(z - z_o).max() <= 1e-12
    n = tenetgb.norm(psi)
    assert abs(n**2 - ov_o.real) <= 1e-12 * ov_o.real
    tenetgb.normalize_(psi)
    assert abs(psi.norm() - 1) <= 1e-13


@pytest.mark.parametrize("serpentine", [True, False])
@pytest.mark.parametrize("precision", ["native", "mixed"])
def test_tebd_small_matches_oracle(ctx, precision, serpentine):
    """Brickwork TEBD with truncation (L=16, χ 4 → 16): overlaps and ⟨Z_i⟩ vs the oracle,
    with every layer swept left to right, and with the even layers swept right to left
    (the gates before the last of such a layer put S on their left site)."""
    from tenetgb import workloads as W

    sites = W.random_mps_arrays(16, 2, 4, seed=2)
    layers = W.tebd_layers(16, 6, serpentine=serpentine)
    psi = gpu_mps(ctx, sites=sites, max_bond=16, precision=precision)
    psi.evolve_brickwork_(layers, maxdim=16, threshold=1e-12)
    p = O.OMPS([s.copy() for s in sites])
    O.tebd(p, layers, maxdim=16, threshold=1e-12)
    assert psi.bondsizes() == p.bondsizes()
    ov, ov_o = psi.overlap(psi), O.overlap(p, p)
    assert abs(ov - ov_o) <= 1e-12 * abs(ov_o)
    z, z_o = psi.local_expectations(W.pauli_z()), O.local_expectations(p, W.pauli_z())[0]
    assert np.abs(z - z_o).max() <= 1e-11


def test_plain_small_config(ctx):
    """L=32, χ=64 Gaussian MPS (seed 1): left-canonize by QR sweep, ⟨ψ|ψ⟩ and ⟨ψ|Z₁₆|ψ⟩."""
    import tenetgb
    from tenetgb import workloads as W

    sites = W.plain_small_workload()
    psi = gpu_mps(ctx, sites=sites)
    psi.canonize_(32)
    p = O.OMPS([s.copy() for s in sites])
    O.canonize(p, 32)
    assert psi.bondsizes() == p.bondsizes()
    ov, ov_o = psi.overlap(psi), O.overlap(p, p)
    assert abs(ov - ov_o) <= 1e-12 * abs(ov_o)
    zpsi = psi.copy()
    zpsi.simple_update_(W.pauli_z(), [16])
    pz = p.copy()
    O.simple_update(pz, W.pauli_z(), [16])
    z, z_o = psi.overlap(zpsi), O.overlap(p, pz)
    assert abs(z - z_o) <= 1e-12 * abs(ov_o)
    assert abs(psi.norm() ** 2 - ov_o.real) <= 1e-12 * ov_o.real
    assert isinstance(psi.form, tenetgb.MixedCanonical)


@pytest.mark.parametrize("precision", ["native", "mixed"])
def test_batched_tebd_matches_oracle_per_instance(ctx, precision):
    """B=3 instances in lockstep: instance 0 is a product state written into χ=4 bonds
    (its θ spectra have exact zeros, so the cutoff keeps fewer values than for the
    random instances and the common bond is zero-padded).  Every instance must match its
    own oracle run."""
    import tenetgb
    from tenetgb import workloads as W

    L_, chi0 = 14, 4
    _, layers = W.tebd_workload(L=L_, chi0=chi0, n_layers=5)
    rand = [W.random_mps_arrays(L_, 2, chi0, seed=s) for s in (21, 22)]
    prod = [np.zeros_like(s) for s in rand[0]]
    for s in prod:
        s[0, 0, 0] = 1.0
    insts = [prod] + rand
    psi = tenetgb.MPS.batched(insts, ctx=ctx, max_bond=32, precision=precision)
    psi.evolve_brickwork_(layers, maxdim=32, threshold=1e-12)
    ov = psi.overlap(psi)
    z = psi.local_expectations(W.pauli_z())
    nrm = psi.norm()
    # ⟨Z_i⟩: 1e-11 in FP64; the mixed form is held to the 1e-10 of its accuracy target
    # (the product instance's spectra end in exact zeros right at the cutoff)
    z_tol = 1e-11 if precision == "native" else 1e-10
    for b, sites in enumerate(insts):
        p = O.OMPS([s.copy() for s in sites])
        O.tebd(p, layers, maxdim=32, threshold=1e-12)
        ov_o = O.overlap(p, p)
        assert abs(ov[b] - ov_o) <= 1e-12 * abs(ov_o), b
        z_o, _ = O.local_expectations(p, W.pauli_z())
        assert np.abs(z[b] - z_o).max() <= z_tol, b
        assert abs(nrm[b] ** 2 - ov_o.real) <= 1e-12 * ov_o.real
    # the product instance's true ranks are below the common (padded) bond dimension
    p0 = O.OMPS([s.copy() for s in insts[0]])
    O.tebd(p0, layers, maxdim=32, threshold=1e-12)
    pb, gb = p0.bondsizes(), psi.bondsizes()
    assert all(a <= b for a, b in zip(pb, gb)) and any(a < b for a, b in zip(pb, gb))


def test_batched_compress_and_amplitude(ctx):
    import tenetgb
    from tenetgb import workloads as W

    insts = [W.random_mps_arrays(10, 2, 16, seed=s, orthogonalize=False) for s in (31, 32, 33, 34)]
    psi = tenetgb.MPS.batched(insts, ctx=ctx)
    amp = psi.amplitude("0110100101")
    tenetgb.compress_(psi, maxdim=6)
    nrm = psi.norm()
    for b, sites in enumerate(insts):
        p = O.OMPS([s.copy() for s in sites])
        a_o = O.amplitude(O.product_state_vectors("0110100101"), p)
        assert abs(amp[b] - a_o) <= 1e-12 * np.sqrt(abs(O.overlap(p, p)))
        O.compress(p, maxdim=6)
        assert abs(nrm[b] - O.norm(p)) <= 1e-12 * O.norm(p)


@pytest.mark.parametrize("precision", ["native", "mixed"])
@pytest.mark.parametrize("chl,chr_", [(64, 64), (32, 64), (64, 32)])
def test_simple_update_absorb_modes(ctx, precision, chl, chr_):
    """Muscle.simple_update's absorb keyword: AbsorbEqually, AbsorbU and AbsorbV give the
    same truncated θ' = A'B'; AbsorbV leaves A' left-isometric, AbsorbU leaves B'
    right-isometric, AbsorbEqually splits S evenly (A'ᴴA' = B'B'ᴴ = diag S)."""
    import tenetgb
    from tenetgb import workloads as W

    rng = np.random.default_rng(chl + 2 * chr_)
    chm, d = 48, 2

    def cg(shape):
        return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) / np.sqrt(2)

    A = tenetgb.DeviceTensor.from_numpy(ctx, cg((chl, d, chm)), ["l", "a", "m"])
    B = tenetgb.DeviceTensor.from_numpy(ctx, cg((chm, d, chr_)), ["m", "b", "r"])
    G = tenetgb.DeviceTensor.from_numpy(ctx, W.gate_tensor(W.haar_unitary(rng, 4)), ["ao", "bo", "a", "b"])
    out = {}
    for absorb in ("equally", "u", "v"):
        An, Bn = tenetgb.simple_update(A, "a", B, "b", "m", G, "ao", "bo", maxdim=40, threshold=1e-12,
                                       precision=precision, absorb=absorb)
        a = An.numpy().reshape(chl * d, -1, order="F")
        b = Bn.numpy().reshape(-1, d * chr_, order="F")
        out[absorb] = (a, b)
    ref = out["equally"][0] @ out["equally"][1]
    for absorb, (a, b) in out.items():
        assert a.shape[1] == 40
        assert np.linalg.norm(a @ b - ref) <= 1e-12 * np.linalg.norm(ref), absorb
    a, _ = out["v"]
    assert np.abs(a.conj().T @ a - np.eye(40)).max() <= 1e-12
    _, b = out["u"]
    assert np.abs(b @ b.conj().T - np.eye(40)).max() <= 1e-12
    a, b = out["equally"]
    ga, gb = a.conj().T @ a, b @ b.conj().T
    assert np.abs(ga - gb).max() <= 1e-12 * np.abs(ga).max()
    with pytest.raises(ValueError):
        tenetgb.simple_update(A, "a", B, "b", "m", G, "ao", "bo", maxdim=40, absorb="both")
