"""Pins the CPU oracle against the reference's own invariant and known-answer tests.

Each test restates one testset of Tenet.jl's test suite (file:line given) on the same
deterministic integer fixtures, so the oracle's canonical-form, compression and
simple-update semantics follow the reference where it has been pinned.
"""

import numpy as np
import pytest

from oracle import tenet_oracle as O


def jl(arr_range, *shape):
    """Julia's ``collect(reshape(a:b, shape...))`` (column-major)."""
    return np.arange(arr_range[0], arr_range[1] + 1, dtype=np.float64).reshape(shape, order="F")


def fixture_mps(first=None):
    """test/unit/mps.jl:63-69 (default order (:l, :r, :o))."""
    arrays = [
        jl((1, 16), 4, 4) if first is None else first,
        jl((1, 64), 4, 4, 4),
        jl((1, 64), 4, 4, 4),
        jl((1, 64), 4, 4, 4),
        jl((1, 16), 4, 4),
    ]
    return O.mps_from_arrays(arrays, order=("l", "r", "o"))


def iso(psi, site, side):
    return O.isisometry(psi.site(site), 2 if side == "r" else 0)


def state_close(a, b):
    va, vb = O.contract_state(a), O.contract_state(b)
    return np.linalg.norm(va - vb) <= np.sqrt(np.finfo(float).eps) * max(np.linalg.norm(va), np.linalg.norm(vb))


def test_constructor_order():
    # test/unit/mps.jl:28-48: order [:r, :o, :l]
    a = np.ones((1, 2))
    b = 2 * np.ones((3, 2, 1))
    c = 3 * np.ones((2, 3))
    psi = O.mps_from_arrays([a, b, c], order=("r", "o", "l"))
    assert psi.bondsizes() == [1, 3]
    assert [s.shape[1] for s in psi.sites] == [2, 2, 2]


def test_noncanonical_to_mixed_single_site():
    # test/unit/mps.jl:62-90
    psi = fixture_mps()
    psi.form = O.NonCanonical()
    c = O.canonize(psi.copy(), 3)
    assert O.checkform(c)
    assert c.form == O.MixedCanonical(3)
    assert iso(c, 1, "r") and iso(c, 2, "r")
    assert not iso(c, 3, "l") and not iso(c, 3, "r")
    assert iso(c, 4, "l") and iso(c, 5, "l")
    assert state_close(c, psi)


def test_noncanonical_to_mixed_multi_site():
    # test/unit/mps.jl:92-119
    psi = fixture_mps()
    psi.form = O.NonCanonical()
    c = O.canonize(psi.copy(), [2, 3])
    assert c.form == O.MixedCanonical([2, 3]) and O.checkform(c)
    assert iso(c, 1, "r") and not iso(c, 2, "l") and not iso(c, 3, "r")
    assert iso(c, 4, "l") and iso(c, 5, "l")
    assert state_close(c, psi)


@pytest.mark.parametrize("start", [5, [3, 4, 5], [1, 2, 3, 4, 5]])
def test_mixed_to_mixed(start):
    # test/unit/mps.jl:121-208
    psi = fixture_mps()
    O.canonize(psi, start)
    c = O.canonize(psi.copy(), 3)
    assert c.form == O.MixedCanonical(3) and O.checkform(c)
    assert iso(c, 1, "r") and iso(c, 2, "r") and iso(c, 4, "l") and iso(c, 5, "l")
    assert not iso(c, 3, "l") and not iso(c, 3, "r")
    assert state_close(c, psi)


@pytest.mark.parametrize("start", [None, 5, [3, 4, 5]])
def test_to_bond_canonical(start):
    # test/unit/mps.jl:210-335
    psi = fixture_mps()
    if start is None:
        psi.form = O.NonCanonical()
    else:
        O.canonize(psi, start)
    c = O.canonize(psi.copy(), (2, 3))
    assert c.form == O.BondCanonical(2, 3) and O.checkform(c)
    assert set(c.lam) == {2}
    assert iso(c, 1, "r") and not iso(c, 2, "l") and not iso(c, 3, "r")
    assert iso(c, 4, "l") and iso(c, 5, "l")
    assert state_close(c, psi)


def test_mixed_to_bond_no_overlap():
    # test/unit/mps.jl:275-305
    psi = fixture_mps()
    O.canonize(psi, [3, 4, 5])
    c = O.canonize(psi.copy(), (1, 2))
    assert c.form == O.BondCanonical(1, 2) and O.checkform(c)
    assert not iso(c, 2, "r") and iso(c, 3, "l") and iso(c, 4, "l") and iso(c, 5, "l")
    assert state_close(c, psi)


def test_bond_to_bond_and_back_to_mixed():
    # test/unit/mps.jl:338-443
    psi = fixture_mps()
    O.canonize(psi, (4, 5))
    c = O.canonize(psi.copy(), (2, 3))
    assert c.form == O.BondCanonical(2, 3) and O.checkform(c)
    assert state_close(c, psi)
    for start, target in [((2, 3), 3), ((4, 5), 3)]:
        p = fixture_mps()
        O.canonize(p, start)
        c = O.canonize(p.copy(), target)
        assert c.form == O.MixedCanonical(3) and O.checkform(c)
        assert iso(c, 1, "r") and iso(c, 2, "r") and iso(c, 4, "l") and iso(c, 5, "l")
        assert state_close(c, p)


def test_compress_single_bond():
    # test/unit/mps.jl:465-495: rank-1 first site => compress to size 1 keeps the state
    for kw in (dict(maxdim=1), dict(threshold=0.1)):
        psi = fixture_mps(first=np.ones((4, 4)))
        c = O.compress(psi.copy(), (1, 2), **kw)
        assert c.bondsizes()[0] == 1
        assert state_close(c, psi)


def test_compress_all_bonds():
    # test/unit/mps.jl:497-522
    psi = fixture_mps(first=np.ones((4, 4)))
    c = O.compress(psi.copy(), maxdim=1)
    assert all(b == 1 for b in c.bondsizes())
    p2 = psi.copy()
    O.canonize(p2, (1, 2))
    threshold = p2.lam[1][1] * 1.1
    c = O.compress(psi.copy(), threshold=threshold)
    assert c.bondsizes()[0] == 1
    assert state_close(c, psi)


def test_bondsizes_and_truncate():
    # test/unit/mps.jl:524-531 (rand(MPS; n=8) → [2,4,8,16,8,4,2]; truncate!(maxdim=10))
    from tenetgb import workloads as W

    psi = O.OMPS(W.random_mps_arrays(8, 2, 128, seed=0))
    assert psi.bondsizes() == [2, 4, 8, 16, 8, 4, 2]
    O.compress(psi, maxdim=10)
    assert max(psi.bondsizes()) == 10


def test_simple_update_x():
    # test/unit/simple_update.jl:4-14 (applied to the MPS form of the product state)
    psi = O.mps_from_arrays([np.array([[1.0, 0.0]]), np.array([[0.0], [1.0]])], order=("r", "o", "l"))
    X = np.array([[0, 1], [1, 0]], dtype=float)
    O.simple_update(psi, X, [1])
    assert np.allclose(psi.site(1).reshape(-1), [0, 1])
    O.simple_update(psi, X, [2])
    assert np.allclose(psi.site(2).reshape(-1), [1, 0])


def test_simple_update_cx():
    # test/unit/simple_update.jl:16-43: CX on |11⟩, gate indices [2, 1, 2', 1']
    psi = O.mps_from_arrays([np.array([[0.0, 1.0]]), np.array([[0.0], [1.0]])], order=("r", "o", "l"))
    cx = np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]], dtype=float)
    g_jl = cx.reshape(2, 2, 2, 2, order="F")  # Julia reshape: axes (plug2, plug1, plug2', plug1')
    G = np.transpose(g_jl, (1, 0, 3, 2))  # → [plug1, plug2, plug1', plug2']
    O.simple_update(psi, G, [1, 2])
    a, b = psi.site(1), psi.site(2)  # (1, 2, χ), (χ, 2, 1)
    assert a.shape[2] == 2  # zero singular value kept
    assert np.allclose(np.abs(a[0, :, 0]), [0, 1]) and np.allclose(np.abs(a[0, :, 1]), [0, 0])
    assert np.allclose(np.abs(b[0, :, 0]), [1, 0]) and np.allclose(np.abs(b[1, :, 0]), [0, 0])


def test_overlap_norm_amplitude_consistency():
    from tenetgb import workloads as W

    psi = O.OMPS(W.random_mps_arrays(10, 2, 8, seed=11, orthogonalize=False))
    v = O.contract_state(psi)
    ov = O.overlap(psi, psi)
    assert abs(ov - np.vdot(v, v)) <= 1e-12 * abs(ov)
    n = O.norm(psi.copy())
    assert abs(n**2 - ov.real) <= 1e-12 * ov.real
    bits = "0110100101"
    amp = O.amplitude(O.product_state_vectors(bits), psi)
    idx = int(bits, 2)  # C-order flattening: site 1 is the most significant
    assert abs(amp - v[idx]) <= 1e-12 * abs(v).max()
    z, _ = O.local_expectations(psi, W.pauli_z())
    zs = []
    for i in range(10):
        pz = psi.copy()
        O.simple_update(pz, W.pauli_z(), [i + 1])
        zs.append(O.overlap(psi, pz) / ov)
    assert np.allclose(z, zs, rtol=1e-10, atol=1e-12)


def test_tebd_small_unitary_invariants():
    from tenetgb import workloads as W

    sites, layers = W.tebd_workload(L=12, chi0=4, n_layers=4)
    psi = O.OMPS(sites)
    O.tebd(psi, layers, maxdim=None, threshold=None)
    # no truncation: the evolution is exact and unitary
    assert abs(O.overlap(psi, psi) - 1) < 1e-12
    v0 = O.contract_state(O.OMPS(sites))
    # apply the same gates to the dense vector
    v = v0.reshape([2] * 12)
    for ly in layers:  # the gates of a layer commute: their order is immaterial here
        start, gates = ly[0], ly[1]
        for j, G in enumerate(gates):
            a = start + 2 * j - 1
            v = np.moveaxis(np.tensordot(G, v, axes=([2, 3], [a, a + 1])), [0, 1], [a, a + 1])
    assert np.allclose(O.contract_state(psi), v.reshape(-1), atol=1e-12)


def test_expectation_two_overlaps_matches_environment_sweep():
    """The serving queries' ⟨O_i⟩ (overlap(ψ, O_i ψ)/overlap(ψ, ψ), the reference's
    form) equals the left/right-environment evaluation for every site."""
    rng = np.random.default_rng(11)
    sites = []
    bonds = [1, 2, 4, 5, 3, 2, 1]
    for i in range(6):
        sites.append((rng.standard_normal((bonds[i], 2, bonds[i + 1])) +
                      1j * rng.standard_normal((bonds[i], 2, bonds[i + 1]))) / np.sqrt(2))
    psi = O.OMPS(sites)
    X = rng.standard_normal((2, 2)) + 1j * rng.standard_normal((2, 2))
    op = (X + X.conj().T) / 2
    ref, _ = O.local_expectations(psi, op)
    for i in range(1, 7):
        e = O.expectation(psi, i, op)
        assert abs(e - ref[i - 1]) <= 1e-13 * np.linalg.norm(op)
        assert abs(e.imag) <= 1e-13 * np.linalg.norm(op)  # Hermitian O


def test_sampler_follows_the_born_rule():
    """The oracle sampler (sample.jl:20-72 with explicit uniforms) reproduces |⟨bits|ψ⟩|²
    on a 4-site MPS: every bit string's frequency over 20000 draws lies within 5σ."""
    rng = np.random.default_rng(5)
    bonds = [1, 2, 3, 2, 1]
    sites = [(rng.standard_normal((bonds[i], 2, bonds[i + 1])) + 1j * rng.standard_normal((bonds[i], 2, bonds[i + 1])))
             for i in range(4)]
    psi = O.OMPS(sites)
    vec = O.contract_state(psi).reshape(-1)
    prob = np.abs(vec) ** 2 / np.sum(np.abs(vec) ** 2)  # C order: site 1 slowest
    n = 20000
    s = O.sample(psi, rng.random((n, 4)))
    idx = np.ravel_multi_index(tuple((s - 1).T), (2, 2, 2, 2))
    freq = np.bincount(idx, minlength=16) / n
    sigma = np.sqrt(prob * (1 - prob) / n)
    assert np.all(np.abs(freq - prob) <= 5 * sigma + 1e-12)


def _dense_mpo(mpo):
    """Operator matrix (outputs × inputs, site 1 slowest) of an MPO (w_l, o, s, w_r)."""
    t = mpo[0][0]  # (o, s, w)
    for W in mpo[1:]:
        t = np.tensordot(t, W, axes=(t.ndim - 1, 0))  # (..., o, s, w)
    t = t[..., 0]
    L = len(mpo)
    perm = [2 * i for i in range(L)] + [2 * i + 1 for i in range(L)]
    t = np.transpose(t, perm)
    n = int(np.prod(t.shape[:L]))
    return t.reshape(n, -1)


def _rand_mpo(rng, L, d=2, w=3):
    ws = [1] + [w] * (L - 1) + [1]
    return [(rng.standard_normal((ws[i], d, d, ws[i + 1])) + 1j * rng.standard_normal((ws[i], d, d, ws[i + 1])))
            / np.sqrt(2 * d * w) for i in range(L)]


def test_mpo_evolution_direct_and_zipup_match_dense():
    """evolve!(ψ, MPO) by the direct method (evolve.jl:19-46) equals the dense operator
    applied to the dense state; the zip-up (evolve.jl:49-129) without truncation equals it
    too, and with maxdim its bonds are capped."""
    rng = np.random.default_rng(41)
    L = 6
    bonds = [1, 2, 4, 4, 4, 2, 1]
    sites = [(rng.standard_normal((bonds[i], 2, bonds[i + 1])) + 1j * rng.standard_normal((bonds[i], 2, bonds[i + 1])))
             for i in range(L)]
    mpo = _rand_mpo(rng, L)
    ref = _dense_mpo(mpo) @ O.contract_state(O.OMPS(sites)).reshape(-1)
    d = O.evolve_mpo_direct(O.OMPS([s.copy() for s in sites]), mpo)
    assert d.bondsizes() == [bonds[i + 1] * 3 for i in range(L - 1)]
    np.testing.assert_allclose(O.contract_state(d).reshape(-1), ref, atol=1e-12 * np.linalg.norm(ref))
    z = O.evolve_mpo_zipup(O.OMPS([s.copy() for s in sites]), mpo, maxdim=1000)
    np.testing.assert_allclose(O.contract_state(z).reshape(-1), ref, atol=1e-12 * np.linalg.norm(ref))
    zt = O.evolve_mpo_zipup(O.OMPS([s.copy() for s in sites]), mpo, maxdim=3)
    assert max(zt.bondsizes()) <= 3


def known_answers():
    """The reference's own recorded DMRG answers (test/unit/dmrg.jl assertions and the
    examples/dmrg.ipynb outputs), extracted by tests/golden/extract_known_answers.py."""
    import json
    import os

    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_known_answers.json")
    with open(path) as f:
        return json.load(f)


# test/unit/dmrg.jl:5-39: n = 10, ising_1d_mpo(n, 1.0, 1.0), 10 sweeps, atol 1e-4 per site
DMRG_CASES = [(c["start"], c["method"].lower(), c["maxdim"] or 128, c["energy_per_site"])
              for c in known_answers()["dmrg_tests"]]


def dmrg_start(kind, n=10):
    """The starting states of test/unit/dmrg.jl: ProductState(fill([1, 0], n)) and the
    MPS of [I₂, δ…, I₂] with δ[1,1,1] = δ[2,2,2] = 1."""
    if kind == "product":
        return O.OMPS([np.array([1.0, 0.0], dtype=np.complex128).reshape(1, 2, 1) for _ in range(n)])
    delta = np.zeros((2, 2, 2), dtype=np.complex128)
    delta[0, 0, 0] = delta[1, 1, 1] = 1.0
    eye = np.eye(2, dtype=np.complex128)
    return O.mps_from_arrays([eye] + [delta] * (n - 2) + [eye])


@pytest.mark.parametrize("start,method,maxdim,energy", DMRG_CASES)
def test_dmrg_known_energies(start, method, maxdim, energy):
    n = 10
    H = O.ising_1d_mpo(n, 1.0, 1.0)
    psi, E = O.dmrg(dmrg_start(start, n), H, 10, method=method, maxdim=maxdim)
    # the reference's tolerance is 1e-4; the restated Lanczos reproduces the values to rounding
    assert abs(E / n - energy) < 1e-10
    assert O.checkform(psi)


def test_ising_mpo_matches_dense_hamiltonian():
    n = 6
    H = O.mpo_dense(O.ising_1d_mpo(n, 0.7, 1.3))
    X = np.array([[0, 1], [1, 0]], dtype=complex)
    Z = np.diag([1.0, -1.0]).astype(complex)

    def op(site_ops):
        m = np.eye(1)
        for i in range(n):
            m = np.kron(m, site_ops.get(i, np.eye(2)))
        return m

    ref = sum(-1.3 * op({i: Z, i + 1: Z}) for i in range(n - 1)) + sum(-0.7 * op({i: X}) for i in range(n))
    assert np.allclose(H, ref, atol=1e-14)


def test_lanczos_lm_exact_on_small_space():
    rng = np.random.default_rng(5)
    M = rng.standard_normal((2, 2)) + 1j * rng.standard_normal((2, 2))
    M = M + M.conj().T - 10 * np.eye(2)
    theta, x, _ = O.lanczos_lm(lambda v: M @ v, np.array([1.0, 0.3], dtype=complex))
    w = np.linalg.eigvalsh(M)
    assert abs(theta - w[np.argmax(abs(w))]) < 1e-12
    assert np.linalg.norm(M @ x - theta * x) < 1e-10


def test_heisenberg_mpo_matches_dense_hamiltonian():
    n, J, Jz, h = 5, 1.0, 0.7, 0.2
    H = O.mpo_dense(O.heisenberg_mpo(n, J, Jz, h))
    sp = np.array([[0.0, 1.0], [0.0, 0.0]])
    sm = sp.T.copy()
    sz = np.diag([0.5, -0.5])

    def op(site_ops):
        m = np.eye(1)
        for i in range(n):
            m = np.kron(m, site_ops.get(i, np.eye(2)))
        return m

    ref = sum(0.5 * J * (op({i: sp, i + 1: sm}) + op({i: sm, i + 1: sp})) + Jz * op({i: sz, i + 1: sz})
              for i in range(n - 1)) + sum(h * op({i: sz}) for i in range(n))
    assert np.allclose(H, ref, atol=1e-14)
    # and the oracle's DMRG reaches its ground state with a full bond
    psi0 = O.OMPS([np.array([1.0, 0.0] if i % 2 else [0.0, 1.0], dtype=np.complex128).reshape(1, 2, 1)
                   for i in range(n)])
    _, E = O.dmrg(psi0, O.heisenberg_mpo(n, J, Jz, h), 6, method="dmrg2", maxdim=8)
    w = np.linalg.eigvalsh(H)
    assert abs(E - w[np.argmax(np.abs(w))]) < 1e-9


# ---------------------------------------------------------------------------------
# MPO (test/unit/mpo.jl): canonize! on an MPO keeps (o, i) together on the physical side
# ---------------------------------------------------------------------------------
def fixture_mpo():
    """test/unit/mpo.jl:82-88 (default order (:l, :r, :o, :i))."""
    return O.mpo_from_arrays([jl((1, 64), 4, 4, 4)] + [jl((1, 256), 4, 4, 4, 4)] * 3 + [jl((1, 64), 4, 4, 4)])


@pytest.mark.parametrize("case,arrays,order,bonds,phys", [
    ("1", [np.ones((2, 3, 4)), 2 * np.ones((2, 2, 3, 4)), 3 * np.ones((2, 3, 4))], ("l", "r", "o", "i"), [2, 2],
     [(3, 4)] * 3),
    ("2", [np.ones((4, 7, 1)), 2 * np.ones((4, 5, 6, 3)), 3 * np.ones((5, 8, 2))], ("l", "r", "o", "i"), [4, 5],
     [(7, 1), (6, 3), (8, 2)]),
    ("3", [np.ones((4, 7, 1)), 2 * np.ones((5, 6, 4, 3)), 3 * np.ones((8, 5, 2))], ("r", "o", "l", "i"), [4, 5],
     [(7, 1), (6, 3), (8, 2)]),
])
def test_mpo_constructor(case, arrays, order, bonds, phys):
    # test/unit/mpo.jl:6-79: plug sizes (o, i) and bond sizes per case
    H = O.mpo_from_arrays(arrays, order=order)
    assert H.bondsizes() == bonds and H.phys == phys
    # the values sit where the reference puts them (site 2 is 2·ones)
    assert np.all(H.site(2) == 2)


# (start, target, isometries that must hold / must not hold): test/unit/mpo.jl:81-462
MPO_TRANSITIONS = [
    (None, 3, [(1, "r"), (2, "r"), (4, "l"), (5, "l")], [(3, "l"), (3, "r")]),
    (None, [2, 3], [(1, "r"), (4, "l"), (5, "l")], [(2, "l"), (3, "r")]),
    (5, 3, [(1, "r"), (2, "r"), (4, "l"), (5, "l")], [(3, "l"), (3, "r")]),
    ([3, 4, 5], 3, [(1, "r"), (2, "r"), (4, "l"), (5, "l")], [(3, "l"), (3, "r")]),
    ([1, 2, 3, 4, 5], [2, 3], [(1, "r"), (4, "l"), (5, "l")], [(2, "l"), (3, "r")]),
    (None, (2, 3), [(1, "r"), (4, "l"), (5, "l")], [(2, "l"), (3, "r")]),
    (5, (2, 3), [(1, "r"), (4, "l"), (5, "l")], [(2, "l"), (3, "r")]),
    ([3, 4, 5], (1, 2), [(3, "l"), (4, "l"), (5, "l")], [(2, "r")]),
    ((4, 5), (2, 3), [(1, "r"), (4, "l"), (5, "l")], []),
    ((2, 3), 3, [(1, "r"), (2, "r"), (4, "l"), (5, "l")], []),
    ((4, 5), 3, [(1, "r"), (2, "r"), (4, "l"), (5, "l")], []),
]


@pytest.mark.parametrize("start,target,isos,not_isos", MPO_TRANSITIONS)
def test_mpo_canonize_transitions(start, target, isos, not_isos):
    psi = fixture_mpo()
    if start is None:
        psi.form = O.NonCanonical()
    else:
        O.canonize(psi, start)
    c = O.canonize(psi.copy(), target)
    assert O.checkform(c)
    for site, side in isos:
        assert iso(c, site, side), (site, side)
    for site, side in not_isos:
        assert not iso(c, site, side), (site, side)
    assert state_close(c, psi)


def test_dmrg_known_answers_fixture_matches_the_reference_tests():
    cases = known_answers()["dmrg_tests"]
    assert [c["source"] for c in cases] == ["test/unit/dmrg.jl:13", "test/unit/dmrg.jl:23", "test/unit/dmrg.jl:32",
                                            "test/unit/dmrg.jl:38"]
    assert [(c["start"], c["method"], c["maxdim"]) for c in cases] == [
        ("product", "Dmrg1", None), ("delta", "Dmrg1", None), ("product", "Dmrg2", 1), ("product", "Dmrg2", 32)]


def test_dmrg_oracle_reproduces_the_notebook_first_calls():
    """examples/dmrg.ipynb cell 6: dmrg!(ψ, H, 1; Dmrg2, maxdim = 128) called repeatedly on
    the 100-site Ising chain from |0…0⟩.  The first two calls (bonds ≤ 16) are cheap; the
    oracle reproduces the printed energies to rounding."""
    ref = known_answers()["dmrg_notebook"]["dmrg2_product"]["energies_per_call"]
    n = 100
    psi = O.OMPS([np.array([1.0, 0.0], dtype=np.complex128).reshape(1, 2, 1) for _ in range(n)])
    H = O.ising_1d_mpo(n, 1.0, 1.0)
    for call in range(2):
        psi, E = O.dmrg(psi, H, 1, method="dmrg2", maxdim=128)
        assert abs(E - ref[call]) < 1e-11, (call, E, ref[call])


def test_mps_notebook_forms_and_bond_sizes():
    """examples/mps.ipynb (unseeded rand, so its printed forms and bond sizes are the
    knowns): canonize! → MixedCanonical(1); norm on MixedCanonical(all) moves the centre
    to site 1; simple_update! on sites (2, 3) leaves MixedCanonical([2, 3]); evolve! by a
    rand(MPO; n=3, maxdim=4) gives bonds 8, 8; compress!(maxdim=4) then gives 2, 2."""
    rng = np.random.default_rng(90)

    def r(*s):
        return rng.random(s) + 1j * rng.random(s)

    psi = O.mps_from_arrays([r(2, 2), r(2, 2, 2), r(2, 2)])
    assert psi.form == O.MixedCanonical([1, 2, 3])
    O.canonize(psi, O.MixedCanonical(1))
    assert psi.form == O.MixedCanonical(1)
    O.normalize(psi)
    assert abs(O.norm(psi) - 1.0) < 1e-14
    O.canonize(psi, O.MixedCanonical([1, 2, 3]))
    O.norm(psi)
    assert psi.form == O.MixedCanonical(1)
    O.simple_update(psi, r(2, 2, 2, 2), (2, 3))
    assert psi.form == O.MixedCanonical([2, 3])
    O.evolve_mpo_direct(psi, [r(1, 2, 2, 4), r(4, 2, 2, 4), r(4, 2, 2, 1)])
    assert psi.bondsizes() == [8, 8]
    O.compress(psi, maxdim=4)
    assert psi.bondsizes() == [2, 2]
