"""Grouped (ragged) MPS batches (tn_group_*): canonize!(ψ, MixedCanonical(L)) →
compress!(ψ; maxdim) → norm(ψ) for instances of different lengths and bond dimensions in
one grouped sweep, checked per instance against the CPU oracle (the reference's
canonize.jl / compress.jl / norm.jl sequence) and against the per-instance device path
(tenetgb.MPS).  Compared through gauge-invariant quantities: the norm, the Schmidt values
Λ of the last bond, and the contracted state; FP64 tolerances as stated per check."""

import numpy as np
import pytest

from oracle import tenet_oracle as O

pytestmark = pytest.mark.gpu


def cgauss(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) / np.sqrt(2)


def instance(rng, L, chi, d=2):
    from tenetgb import workloads as W

    b = [1] + W.clamped_bonds(L, d, chi) + [1]
    return [cgauss(rng, (b[i], d, b[i + 1])) / np.sqrt(d * b[i]) for i in range(L)]


def contract(sites):
    v = sites[0]
    for A in sites[1:]:
        v = np.tensordot(v, A, axes=(v.ndim - 1, 0))
    return v.reshape(-1)


SHAPES = [(6, 4, 2), (9, 8, 4), (12, 16, 8), (5, 3, 1), (10, 16, 5), (8, 7, 3), (11, 12, 6), (9, 17, 8)]


@pytest.fixture(scope="module")
def data():
    rng = np.random.default_rng(21)
    return [instance(rng, L, chi) for L, chi, _ in SHAPES]


def test_group_matches_oracle_per_instance(data):
    from tenetgb.group import MPSGroup

    g = MPSGroup.from_arrays(data)
    maxdim = [md for _, _, md in SHAPES]
    norms = g.canonize_compress_norm(maxdim)
    for b, sites in enumerate(data):
        psi = O.OMPS([s.copy() for s in sites])
        O.canonize(psi, O.MixedCanonical(psi.L))
        O.compress(psi, maxdim=maxdim[b])
        ref_norm = O.norm(psi.copy())
        ref_lam = psi.lam[psi.L - 1]
        assert abs(norms[b] - ref_norm) <= 1e-12 * ref_norm
        lam = g.lambda_(b)
        assert lam.shape == ref_lam.shape
        np.testing.assert_allclose(lam, ref_lam, rtol=0, atol=1e-12 * ref_lam.max())
        bd = g.bond_dims(b)
        assert bd == psi.bondsizes()
        got = contract(g.sites(b))
        ref = O.contract_state(psi)
        assert np.linalg.norm(got - ref) <= 1e-11 * np.linalg.norm(ref)
        # sites 1..L−1 are left isometries after the sweep (Σ over (χl, d) of A*A = I)
        for A in g.sites(b)[:-1]:
            assert O.isisometry(A, 2)


def test_group_matches_per_instance_device_path(data):
    import tenetgb
    from tenetgb.group import MPSGroup

    g = MPSGroup.from_arrays(data)
    maxdim = [md for _, _, md in SHAPES]
    norms = g.canonize_compress_norm(maxdim)
    ctx = g.ctx
    for b, sites in enumerate(data):
        psi = tenetgb.MPS([s.copy() for s in sites], ctx=ctx)
        psi.canonize_(tenetgb.MixedCanonical(len(sites)))
        psi.compress_(maxdim=maxdim[b])
        n = psi.norm()
        assert abs(n - norms[b]) <= 1e-12 * n
        assert psi.bondsizes() == g.bond_dims(b)


def test_group_random_fill_and_population_shapes():
    from tenetgb import workloads as W
    from tenetgb.group import MPSGroup

    Ls, chis = W.batched_population(n=12, seed=5, Lmax=24, chimax=32)
    g = MPSGroup.random(Ls, chis, seed=3)
    norms = g.canonize_compress_norm([max(1, c // 2) for c in chis])
    for b in range(len(Ls)):
        bd = g.bond_dims(b)
        cl = W.clamped_bonds(Ls[b], 2, chis[b])
        assert bd == [min(x, max(1, chis[b] // 2)) for x in cl]
        assert np.isclose(np.linalg.norm(g.lambda_(b)), norms[b], rtol=1e-13)
        assert 0 < norms[b] < 10


def test_group_rejects_bad_maxdim(data):
    from tenetgb.group import MPSGroup

    g = MPSGroup.from_arrays(data[:2])
    with pytest.raises(ValueError):
        g.canonize_compress_norm([0, 3])


def test_group_refill_restores_the_creation_shape():
    from tenetgb import workloads as W
    from tenetgb.group import MPSGroup

    Ls, chis = [10, 14], [8, 12]
    g = MPSGroup.random(Ls, chis, seed=4)
    first = [g.sites(b) for b in range(2)]
    n1 = g.canonize_compress_norm([2, 3])
    g.ctx.check(g.lib.tn_group_fill_random(g.h, 4))
    for b in range(2):
        assert g.bond_dims(b) == W.clamped_bonds(Ls[b], 2, chis[b])
        for x, y in zip(g.sites(b), first[b]):
            np.testing.assert_array_equal(x, y)
    n2 = g.canonize_compress_norm([2, 3])
    np.testing.assert_allclose(n1, n2, rtol=1e-14)
