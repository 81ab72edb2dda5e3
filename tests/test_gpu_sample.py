"""sample(ψ, n) (src/Operations/sample.jl:20-72) and schmidt_values! /
entropy_vonneumann! (src/Operations/entropy.jl:25-67) on the device, checked against the
oracle with the same uniforms (identical outcomes), against the Born rule, and against
the oracle's Schmidt values (1e-12)."""

import numpy as np
import pytest

from oracle import tenet_oracle as O

pytestmark = pytest.mark.gpu


def random_sites(rng, bonds, d=2):
    return [(rng.standard_normal((bonds[i], d, bonds[i + 1])) + 1j * rng.standard_normal((bonds[i], d, bonds[i + 1])))
            / np.sqrt(2 * d * bonds[i]) for i in range(len(bonds) - 1)]


def test_samples_equal_oracle_with_same_uniforms():
    import tenetgb

    rng = np.random.default_rng(31)
    sites = random_sites(rng, [1, 2, 4, 8, 8, 8, 8, 4, 2, 1])
    psi = tenetgb.MPS([s.copy() for s in sites])
    u = rng.random((300, 9))
    got = np.array(tenetgb.sample(psi, 300, uniforms=u))
    ref = O.sample(O.OMPS([s.copy() for s in sites]), u)
    assert got.shape == ref.shape
    assert np.array_equal(got, ref)


def test_device_sampler_follows_the_born_rule():
    import tenetgb

    rng = np.random.default_rng(32)
    sites = random_sites(rng, [1, 2, 3, 2, 1])
    psi = tenetgb.MPS([s.copy() for s in sites])
    vec = O.contract_state(O.OMPS(sites)).reshape(-1)
    prob = np.abs(vec) ** 2 / np.sum(np.abs(vec) ** 2)
    n = 40000
    s = np.array(tenetgb.sample(psi, n, seed=7))
    freq = np.bincount(np.ravel_multi_index(tuple((s - 1).T), (2, 2, 2, 2)), minlength=16) / n
    assert np.all(np.abs(freq - prob) <= 5 * np.sqrt(prob * (1 - prob) / n) + 1e-12)


def test_sample_leaves_the_mps_unchanged():
    import tenetgb

    rng = np.random.default_rng(33)
    sites = random_sites(rng, [1, 2, 4, 4, 2, 1])
    psi = tenetgb.MPS([s.copy() for s in sites])
    psi.canonize_(tenetgb.MixedCanonical(3))
    before = [psi.site(i) for i in range(1, 6)]
    tenetgb.sample(psi, 10, seed=1)
    assert isinstance(psi.form, tenetgb.MixedCanonical) and psi.form.lo == 3
    for i in range(1, 6):
        np.testing.assert_array_equal(psi.site(i), before[i - 1])


def test_schmidt_values_and_entropy_match_oracle():
    import tenetgb

    rng = np.random.default_rng(34)
    sites = random_sites(rng, [1, 2, 4, 8, 6, 3, 1])
    phi = O.OMPS([s.copy() for s in sites])
    O.normalize(phi)
    psi = tenetgb.MPS([s.copy() for s in phi.sites])
    ent = tenetgb.entropy_vonneumann(psi)
    assert ent.shape == (5,)
    for i in range(1, 6):
        ref = O.OMPS([s.copy() for s in phi.sites])
        O.canonize(ref, O.BondCanonical(i, i + 1))
        lam = ref.lam[i]
        got = tenetgb.schmidt_values(psi, i)
        np.testing.assert_allclose(np.sort(got)[::-1], np.sort(lam)[::-1], atol=1e-12)
        assert abs(ent[i - 1] - float(-np.sum(lam**2 * 2 * np.log(lam)))) <= 1e-12
