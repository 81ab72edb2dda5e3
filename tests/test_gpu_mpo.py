"""evolve!(ψ, MPO) on the device (direct contraction and zip-up, src/Operations/
evolve.jl:19-137) against the oracle restatement and the dense operator: states within
1e-12 of their norm, bond dimensions equal."""

import numpy as np
import pytest

from oracle import tenet_oracle as O

pytestmark = pytest.mark.gpu


def rand_sites(rng, bonds, d=2):
    return [(rng.standard_normal((bonds[i], d, bonds[i + 1])) + 1j * rng.standard_normal((bonds[i], d, bonds[i + 1])))
            / np.sqrt(2 * d * bonds[i]) for i in range(len(bonds) - 1)]


def rand_mpo(rng, L, d=2, w=3):
    ws = [1] + [w] * (L - 1) + [1]
    return [(rng.standard_normal((ws[i], d, d, ws[i + 1])) + 1j * rng.standard_normal((ws[i], d, d, ws[i + 1])))
            / np.sqrt(2 * d * w) for i in range(L)]


def state(psi):
    v = psi.site(1)
    for i in range(2, psi.nsites + 1):
        v = np.tensordot(v, psi.site(i), axes=(v.ndim - 1, 0))
    return v.reshape(-1)


@pytest.mark.parametrize("algorithm", ["direct", "zipup"])
def test_mpo_evolution_matches_oracle(algorithm):
    import tenetgb

    rng = np.random.default_rng(51)
    bonds = [1, 2, 4, 8, 8, 4, 2, 1]
    sites = rand_sites(rng, bonds)
    mpo = rand_mpo(rng, 7)
    psi = tenetgb.MPS([s.copy() for s in sites])
    ref = O.OMPS([s.copy() for s in sites])
    if algorithm == "direct":
        tenetgb.evolve_mpo_(psi, mpo)
        O.evolve_mpo_direct(ref, mpo)
        assert isinstance(psi.form, tenetgb.MixedCanonical) and psi.form.lo == 1 and psi.form.hi == 7
    else:
        tenetgb.evolve_mpo_(psi, mpo, algorithm="zipup", maxdim=10)
        O.evolve_mpo_zipup(ref, mpo, maxdim=10)
    assert psi.bondsizes() == ref.bondsizes()
    a, b = state(psi), O.contract_state(ref).reshape(-1)
    assert np.linalg.norm(a - b) <= 1e-12 * np.linalg.norm(b)


def test_mpo_direct_on_a_batch_of_instances():
    import tenetgb

    rng = np.random.default_rng(52)
    bonds = [1, 2, 4, 4, 2, 1]
    insts = [rand_sites(rng, bonds) for _ in range(3)]
    mpo = rand_mpo(rng, 5, w=2)
    psi = tenetgb.MPS.batched([[s.copy() for s in x] for x in insts])
    tenetgb.evolve_mpo_(psi, mpo)
    for b, x in enumerate(insts):
        ref = O.evolve_mpo_direct(O.OMPS([s.copy() for s in x]), mpo)
        got = psi.site(1, b)
        for i in range(2, 6):
            got = np.tensordot(got, psi.site(i, b), axes=(got.ndim - 1, 0))
        want = O.contract_state(ref).reshape(-1)
        assert np.linalg.norm(got.reshape(-1) - want) <= 1e-12 * np.linalg.norm(want)


def test_mpo_zipup_needs_a_truncation():
    import tenetgb

    rng = np.random.default_rng(53)
    psi = tenetgb.MPS(rand_sites(rng, [1, 2, 2, 1]))
    with pytest.raises(ValueError):
        tenetgb.evolve_mpo_(psi, rand_mpo(rng, 3), algorithm="zipup")
    with pytest.raises(ValueError):
        tenetgb.evolve_mpo_(psi, rand_mpo(rng, 2))


@pytest.mark.parametrize("precision", ["native", "mixed"])
def test_mpo_zipup_on_a_batch_of_instances(precision):
    """The zip-up on a batched MPS (evolve.jl:49-129 for every instance in lockstep): one
    instance is a product state written into the bonds, so its kept ranks are below the
    others' and its surplus is zero-padded; each instance must equal its own oracle run."""
    import tenetgb

    rng = np.random.default_rng(53)
    bonds = [1, 2, 4, 8, 8, 4, 2, 1]
    insts = [rand_sites(rng, bonds) for _ in range(2)]
    prod = [np.zeros_like(s) for s in insts[0]]
    for s in prod:
        s[0, 0, 0] = 1.0
    insts = [prod] + insts
    mpo = rand_mpo(rng, 7)
    psi = tenetgb.MPS.batched([[s.copy() for s in x] for x in insts], precision=precision)
    tenetgb.evolve_mpo_(psi, mpo, algorithm="zipup", maxdim=6, threshold=1e-12)
    for b, x in enumerate(insts):
        ref = O.OMPS([s.copy() for s in x])
        O.evolve_mpo_zipup(ref, mpo, maxdim=6, threshold=1e-12)
        v = psi.site(1, instance=b)
        for i in range(2, 8):
            v = np.tensordot(v, psi.site(i, instance=b), axes=(v.ndim - 1, 0))
        a, r = v.reshape(-1), O.contract_state(ref).reshape(-1)
        assert np.linalg.norm(a - r) <= 1e-12 * np.linalg.norm(r), b
        assert all(x <= y for x, y in zip(ref.bondsizes(), psi.bondsizes()))
