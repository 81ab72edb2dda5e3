"""dmrg!(ψ, H) on the device (src/Algorithms/DMRG.jl) against the reference's known
energies (test/unit/dmrg.jl), the oracle's per-half-sweep energies and the dense
Hamiltonian."""

import numpy as np
import pytest

from oracle import tenet_oracle as O

pytestmark = pytest.mark.gpu

# test/unit/dmrg.jl:5-39 (n = 10, h = J = 1, 10 sweeps; the reference checks atol 1e-4)
KNOWN = [
    ("product", 1, 128, -1.1902477482849715),
    ("delta", 1, 128, -1.2372129315563634),
    ("product", 2, 1, -1.1944098151375718),
    ("product", 2, 32, -1.2381489999654788),
]


def start_sites(kind, n=10):
    if kind == "product":
        return [np.array([1.0, 0.0], dtype=np.complex128).reshape(1, 2, 1) for _ in range(n)]
    delta = np.zeros((2, 2, 2), dtype=np.complex128)
    delta[0, 0, 0] = delta[1, 1, 1] = 1.0
    return O.mps_from_arrays([np.eye(2)] + [delta] * (n - 2) + [np.eye(2)]).sites


def rand_sites(rng, bonds, d=2):
    return [(rng.standard_normal((bonds[i], d, bonds[i + 1])) + 1j * rng.standard_normal((bonds[i], d, bonds[i + 1])))
            / np.sqrt(2 * d * bonds[i]) for i in range(len(bonds) - 1)]


def state(psi, instance=0):
    v = psi.site(1, instance)
    for i in range(2, psi.nsites + 1):
        v = np.tensordot(v, psi.site(i, instance), axes=(v.ndim - 1, 0))
    return v.reshape(-1)


@pytest.mark.parametrize("start,method,maxdim,energy", KNOWN)
def test_dmrg_reference_energies(start, method, maxdim, energy):
    import tenetgb

    n = 10
    H = tenetgb.ising_1d_mpo(n, 1.0, 1.0)
    psi = tenetgb.MPS([s.copy() for s in start_sites(start, n)])
    meth = tenetgb.Dmrg1 if method == 1 else tenetgb.Dmrg2
    phi, E = tenetgb.dmrg(psi, H, 10, method=meth, maxdim=maxdim)
    assert abs(E / n - energy) < 1e-10
    # the input is left alone (dmrg = dmrg!(copy(ψ), …)), the result ends MixedCanonical(1)
    assert psi.bondsizes() == [s.shape[2] for s in start_sites(start, n)][:-1]
    f = phi.form
    assert isinstance(f, tenetgb.MixedCanonical) and f.lo == f.hi == 1
    # the returned value is the last local eigenvalue (before truncation): it equals
    # ⟨ϕ|H|ϕ⟩ where nothing is truncated; otherwise ⟨ϕ|H|ϕ⟩ is the oracle's
    v = state(phi)
    Hd = O.mpo_dense(O.ising_1d_mpo(n, 1.0, 1.0))
    e_state = np.vdot(v, Hd @ v).real / np.vdot(v, v).real
    if method == 1 or maxdim >= 32:
        assert abs(e_state - E) < 1e-9
    else:
        ref, _ = O.dmrg(O.OMPS([s.copy() for s in start_sites(start, n)]), O.ising_1d_mpo(n, 1.0, 1.0), 10,
                        method="dmrg2", maxdim=maxdim)
        vr = O.contract_state(ref).reshape(-1)
        assert abs(e_state - np.vdot(vr, Hd @ vr).real / np.vdot(vr, vr).real) < 1e-9


@pytest.mark.parametrize("method", [1, 2])
def test_dmrg_half_sweeps_match_oracle(method):
    import tenetgb

    rng = np.random.default_rng(61)
    n = 8
    bonds = [1, 2, 4, 4, 4, 4, 4, 2, 1]
    sites = rand_sites(rng, bonds)
    H = tenetgb.ising_1d_mpo(n, 0.6, 1.1)
    psi = tenetgb.MPS([s.copy() for s in sites])
    meth = tenetgb.Dmrg1 if method == 1 else tenetgb.Dmrg2
    _, E, hist = tenetgb.dmrg_(psi, H, 3, method=meth, maxdim=6, history=True)
    ref_hist = []
    ref, Er = O.dmrg(O.OMPS([s.copy() for s in sites]), O.ising_1d_mpo(n, 0.6, 1.1), 3,
                     method="dmrg1" if method == 1 else "dmrg2", maxdim=6, history=ref_hist)
    assert np.allclose(hist, ref_hist, rtol=0, atol=1e-9)
    assert abs(E - Er) < 1e-9
    assert psi.bondsizes() == ref.bondsizes()
    # same state up to a global phase
    a, b = state(psi), O.contract_state(ref).reshape(-1)
    assert abs(abs(np.vdot(a, b)) - np.linalg.norm(a) * np.linalg.norm(b)) < 1e-8


def test_dmrg2_full_bond_reaches_exact_ground_state():
    import tenetgb

    n = 8
    H = tenetgb.ising_1d_mpo(n, 0.9, 1.0)
    psi = tenetgb.MPS(start_sites("product", n))
    _, E = tenetgb.dmrg_(psi, H, 8, method=tenetgb.Dmrg2, maxdim=16)
    exact = np.linalg.eigvalsh(O.mpo_dense(O.ising_1d_mpo(n, 0.9, 1.0)))[0]
    assert abs(E - exact) < 1e-9
    assert psi.bondsizes() == [2, 4, 8, 16, 8, 4, 2]


def test_dmrg_batched_field_scan_matches_oracle_per_instance():
    import tenetgb

    n = 10
    fields = [0.5, 1.0, 1.5]
    rng = np.random.default_rng(62)
    bonds = [1, 2, 4, 4, 4, 4, 4, 4, 4, 2, 1]
    insts = [rand_sites(rng, bonds) for _ in fields]
    psi = tenetgb.MPS.batched([[s.copy() for s in x] for x in insts])
    Hs = [tenetgb.ising_1d_mpo(n, h, 1.0) for h in fields]
    for method, name in ((tenetgb.Dmrg1, "dmrg1"), (tenetgb.Dmrg2, "dmrg2")):
        phi, E = tenetgb.dmrg(psi, Hs, 3, method=method, maxdim=8)
        assert E.shape == (3,)
        for b, h in enumerate(fields):
            _, Er = O.dmrg(O.OMPS([s.copy() for s in insts[b]]), O.ising_1d_mpo(n, h, 1.0), 3, method=name, maxdim=8)
            assert abs(E[b] - Er) < 1e-9, (name, b)


def test_dmrg_wide_mpo_bond_uses_gemm_path():
    """An Ising MPO embedded in bond dimension 9 (zero padding): the fibre contraction
    has 18 inputs per output and runs through the batched GEMM; the energies are those
    of the bond-3 MPO."""
    import tenetgb

    n = 6
    H3 = tenetgb.ising_1d_mpo(n, 0.8, 1.0)
    H9 = []
    for i, W in enumerate(H3):
        wl = 1 if i == 0 else 9
        wr = 1 if i == n - 1 else 9
        P = np.zeros((wl, 2, 2, wr), dtype=np.complex128)
        P[: W.shape[0], :, :, : W.shape[3]] = W
        H9.append(P)
    sites = start_sites("product", n)
    _, E3 = tenetgb.dmrg(tenetgb.MPS([s.copy() for s in sites]), H3, 4, method=tenetgb.Dmrg2, maxdim=8)
    _, E9 = tenetgb.dmrg(tenetgb.MPS([s.copy() for s in sites]), H9, 4, method=tenetgb.Dmrg2, maxdim=8)
    assert abs(E3 - E9) < 1e-10


def test_dmrg_argument_errors():
    import tenetgb

    psi = tenetgb.MPS(start_sites("product", 4))
    with pytest.raises(ValueError):
        tenetgb.dmrg(psi, tenetgb.ising_1d_mpo(5, 1.0, 1.0), 1)
    with pytest.raises(NotImplementedError):
        tenetgb.dmrg(psi, tenetgb.ising_1d_mpo(4, 1.0, 1.0), 1, ishermitian=False)
    with pytest.raises(ValueError, match="krylovdim"):
        tenetgb.dmrg(psi, tenetgb.ising_1d_mpo(4, 1.0, 1.0), 1, krylovdim=1)


def test_dmrg_mixed_precision_matches_native():
    """Mixed precision (FP32 Jacobi pre-pass, truncation-aware FP64 polish) on the DMRG
    pair splits: the Ising ground state's near-degenerate Schmidt values at the
    truncation boundary must not stall the polish; energies equal the FP64 run."""
    import tenetgb

    n, chi = 20, 64
    H = tenetgb.ising_1d_mpo(n, 1.0, 1.0)
    res = {}
    for prec in ("native", "mixed"):
        psi = tenetgb.MPS(start_sites("product", n), precision=prec)
        _, res[prec] = tenetgb.dmrg_(psi, H, 6, method=tenetgb.Dmrg2, maxdim=chi)
    assert abs(res["native"] - res["mixed"]) < 1e-9


def test_dmrg_ordered_phase_spectrum_below_fp64_range():
    """h = 0.5 (ordered phase): the Schmidt values of the pairs decay past 1e-300 once the
    bond saturates; the pair SVDs must converge and the sites stay isometries."""
    import tenetgb

    n, chi, h = 40, 64, 0.5
    psi = tenetgb.MPS(start_sites("product", n))
    _, E = tenetgb.dmrg_(psi, tenetgb.ising_1d_mpo(n, h, 1.0), 5, method=tenetgb.Dmrg2, maxdim=chi)
    _, Er = O.dmrg(O.OMPS(start_sites("product", n)), O.ising_1d_mpo(n, h, 1.0), 5, method="dmrg2", maxdim=chi)
    assert abs(E - Er) < 1e-9 * abs(Er)
    for i in range(2, n + 1):
        A = psi.site(i)
        m = A.reshape(A.shape[0], -1, order="F")
        assert np.linalg.norm(m @ m.conj().T - np.eye(A.shape[0])) < 1e-10, i


@pytest.mark.parametrize("method", [1, 2])
def test_dmrg_heisenberg_bond5_matches_oracle(method):
    """XXZ chain with a field (MPO bond 5: the fibre contractions take 10 inputs per
    output) from a Néel state (Dmrg2) or a random bond-4 MPS (Dmrg1)."""
    import tenetgb

    n = 8
    H = O.heisenberg_mpo(n, 1.0, 0.7, 0.2)
    if method == 2:
        sites = [np.array([1.0, 0.0] if i % 2 else [0.0, 1.0], dtype=np.complex128).reshape(1, 2, 1) for i in range(n)]
    else:
        sites = rand_sites(np.random.default_rng(63), [1, 2, 4, 4, 4, 4, 4, 2, 1])
    psi = tenetgb.MPS([s.copy() for s in sites])
    meth = tenetgb.Dmrg1 if method == 1 else tenetgb.Dmrg2
    _, E, hist = tenetgb.dmrg_(psi, H, 4, method=meth, maxdim=16, history=True)
    ref_hist = []
    _, Er = O.dmrg(O.OMPS([s.copy() for s in sites]), H, 4, method="dmrg1" if method == 1 else "dmrg2", maxdim=16,
                   history=ref_hist)
    assert np.allclose(hist, ref_hist, rtol=0, atol=1e-9)
    if method == 2:  # full bond: the extreme eigenvalue of H (which = :LM)
        w = np.linalg.eigvalsh(O.mpo_dense(H))
        assert abs(E - w[np.argmax(np.abs(w))]) < 1e-9


def _compare_with_oracle(sites, H, nsweeps, method, maxdim=16, krylovdim=3, maxiter=2):
    import tenetgb

    psi = tenetgb.MPS([s.copy() for s in sites])
    meth = tenetgb.Dmrg1 if method == 1 else tenetgb.Dmrg2
    _, E, hist = tenetgb.dmrg_(psi, H, nsweeps, method=meth, maxdim=maxdim, krylovdim=krylovdim, maxiter=maxiter,
                               history=True)
    ref_hist = []
    ref, Er = O.dmrg(O.OMPS([s.copy() for s in sites]), H, nsweeps, method="dmrg1" if method == 1 else "dmrg2",
                     maxdim=maxdim, krylovdim=krylovdim, maxiter=maxiter, history=ref_hist)
    assert np.allclose(hist, ref_hist, rtol=0, atol=1e-9)
    assert psi.bondsizes() == ref.bondsizes()
    return E


@pytest.mark.parametrize("L", [2, 3])
@pytest.mark.parametrize("method", [1, 2])
def test_dmrg_shortest_chains(L, method):
    """Every local update touches a boundary environment.  (An XXZ chain in a field: the
    transverse Ising spectrum is ± symmetric, and which = :LM would tie on it.)"""
    rng = np.random.default_rng(70 + L)
    bonds = [1] + [2] * (L - 1) + [1]
    _compare_with_oracle(rand_sites(rng, bonds), O.heisenberg_mpo(L, 1.0, 0.6, 0.3), 3, method)


@pytest.mark.parametrize("method", [1, 2])
def test_dmrg_spin1_d3(method):
    """d = 3 sites (spin-1 XXZ with anisotropy, MPO bond 5)."""
    rng = np.random.default_rng(72)
    n = 6
    bonds = [1, 3, 4, 4, 4, 3, 1]
    _compare_with_oracle(rand_sites(rng, bonds, d=3), O.spin1_xxz_mpo(n, 1.0, 0.8, 0.3), 3, method, maxdim=9)


def test_dmrg_larger_krylov_space():
    """krylovdim 6 and three Lanczos iterations (the wider orthogonalisation kernels and
    a restart from a longer basis)."""
    rng = np.random.default_rng(73)
    n = 8
    bonds = [1, 2, 4, 4, 4, 4, 4, 2, 1]
    _compare_with_oracle(rand_sites(rng, bonds), O.heisenberg_mpo(n, 1.0, 0.6, 0.1), 2, 2, maxdim=8, krylovdim=6,
                         maxiter=3)
