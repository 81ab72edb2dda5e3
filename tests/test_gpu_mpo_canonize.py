"""canonize! / compress! on a device MPO (test/unit/mpo.jl) against the oracle: the
reference's constructor cases and canonical-form transitions on its integer fixtures,
with the isometry pattern of every form and the contracted operator unchanged."""

import numpy as np
import pytest

from oracle import tenet_oracle as O
from test_oracle_reference import MPO_TRANSITIONS, jl

pytestmark = pytest.mark.gpu


def fixture_arrays():
    # test/unit/mpo.jl:82-88
    return [jl((1, 64), 4, 4, 4)] + [jl((1, 256), 4, 4, 4, 4)] * 3 + [jl((1, 64), 4, 4, 4)]


def operator(H):
    """The contracted operator (fused physical index per site) with Λ absorbed when the
    form is bond-canonical."""
    import tenetgb

    sites = [s.copy() for s in H.mps.sites()]
    f = H.form
    if isinstance(f, tenetgb.BondCanonical):
        lam = H.lambda_()
        sites[f.a - 1] = sites[f.a - 1] * lam[None, None, :]
    v = sites[0]
    for A in sites[1:]:
        v = np.tensordot(v, A, axes=(v.ndim - 1, 0))
    return v.reshape(-1)


@pytest.mark.parametrize("arrays,order,bonds,phys", [
    ([np.ones((2, 3, 4)), 2 * np.ones((2, 2, 3, 4)), 3 * np.ones((2, 3, 4))], ("l", "r", "o", "i"), [2, 2],
     [(3, 4)] * 3),
    ([np.ones((4, 7, 1)), 2 * np.ones((4, 5, 6, 3)), 3 * np.ones((5, 8, 2))], ("l", "r", "o", "i"), [4, 5],
     [(7, 1), (6, 3), (8, 2)]),
    ([np.ones((4, 7, 1)), 2 * np.ones((5, 6, 4, 3)), 3 * np.ones((8, 5, 2))], ("r", "o", "l", "i"), [4, 5],
     [(7, 1), (6, 3), (8, 2)]),
])
def test_device_mpo_constructor(arrays, order, bonds, phys):
    import tenetgb

    if len({o * i for o, i in phys}) != 1:
        with pytest.raises(ValueError):
            tenetgb.MPO(arrays=arrays, order=order)
        return
    H = tenetgb.MPO(arrays=arrays, order=order)
    assert H.bondsizes() == bonds and H.phys == phys
    assert np.all(H.site(2) == 2)


@pytest.mark.parametrize("start,target,isos,not_isos", MPO_TRANSITIONS)
def test_device_mpo_canonize_transitions(start, target, isos, not_isos):
    import tenetgb

    H = tenetgb.MPO(arrays=fixture_arrays())
    ref = O.mpo_from_arrays(fixture_arrays())
    if start is None:
        H.mps.unsafe_setform_(tenetgb.NonCanonical())
        ref.form = O.NonCanonical()
    else:
        H.canonize_(start)
        O.canonize(ref, start)
    before = operator(H)
    c = tenetgb.mpo.canonize(H, target)
    rc = O.canonize(ref.copy(), target)
    assert c.bondsizes() == rc.bondsizes()
    for site, side in isos:
        assert O.isisometry(c.mps.site(site), 2 if side == "r" else 0, atol=1e-10), (site, side)
    for site, side in not_isos:
        assert not O.isisometry(c.mps.site(site), 2 if side == "r" else 0, atol=1e-10), (site, side)
    a, b = operator(c), O.contract_state(rc)
    assert np.linalg.norm(a - b) <= 1e-10 * np.linalg.norm(b)
    assert np.linalg.norm(a - before) <= 1e-10 * np.linalg.norm(before)


def test_device_mpo_compress_and_arrays_round_trip():
    import tenetgb

    rng = np.random.default_rng(80)
    ws = [1, 3, 5, 5, 3, 1]
    sites = [rng.standard_normal((ws[k], 2, 2, ws[k + 1])) + 1j * rng.standard_normal((ws[k], 2, 2, ws[k + 1]))
             for k in range(5)]
    H = tenetgb.MPO(sites)
    dense = O.mpo_dense(H.arrays())
    assert np.allclose(dense, O.mpo_dense(sites), atol=1e-12)
    c = tenetgb.mpo.compress(H, maxdim=2)
    assert max(c.bondsizes()) == 2
    ref = O.compress(O.OMPS([s.reshape(s.shape[0], 4, s.shape[3], order="F") for s in sites]), maxdim=2)
    assert c.bondsizes() == ref.bondsizes()
    a, b = operator(c), O.contract_state(ref)
    assert np.linalg.norm(a - b) <= 1e-10 * np.linalg.norm(b)
