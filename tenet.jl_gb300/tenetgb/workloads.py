"""Seeded synthetic inputs for the five benchmark workloads.

No public dataset is involved: every input is generated here from
``numpy.random.default_rng(seed)`` so the CUDA path and the CPU oracle see identical
arrays.  Site tensors are returned as C-ordered numpy arrays with logical shape
(χ_left, d, χ_right); the host layer converts to the library's column-major layout.

Random MPS follow ``rand(MPS)`` (Tenet.jl src/Components/MPS.jl:113-165): bond i has
dimension min(χ, d^i, d^(L-i)) and every site is orthogonalised by an LQ
factorisation of its (χ_l) × (d·χ_r) matrix, which makes the state right-canonical
and normalised.  Entries are complex Gaussian (re + i·im)/√2 instead of the
reference's uniform reals.
"""

from __future__ import annotations

import numpy as np


def complex_gaussian(rng, shape, dtype=np.complex128):
    x = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) / np.sqrt(2.0)
    return x.astype(dtype)


def clamped_bonds(L, d, chi):
    """Bond i (between sites i and i+1, 1-based) = min(χ, d^i, d^(L-i))."""
    out = []
    for i in range(1, L):
        out.append(int(min(chi, d ** min(i, 60), d ** min(L - i, 60))))
    return out


def random_mps_arrays(L, d, chi, seed, orthogonalize=True, dtype=np.complex128):
    rng = np.random.default_rng(seed)
    bonds = [1] + clamped_bonds(L, d, chi) + [1]
    sites = []
    for i in range(L):
        cl, cr = bonds[i], bonds[i + 1]
        a = complex_gaussian(rng, (cl, d * cr), dtype)
        if orthogonalize:
            # LQ of a: a = l q with q having orthonormal rows (a^H = Q R, q = Q^H)
            q, _ = np.linalg.qr(a.conj().T, mode="reduced")
            a = q.conj().T
            k = a.shape[0]
            if k < cl:  # cannot happen with clamped bonds; keep the shape honest
                a = np.vstack([a, np.zeros((cl - k, d * cr), a.dtype)])
        sites.append(np.ascontiguousarray(a.reshape(cl, d, cr)))
    return sites


def haar_unitary(rng, n):
    """Haar-random n×n unitary: QR of a complex Gaussian with the phase fix
    Q · diag(R_ii / |R_ii|) (Mezzadri 2007)."""
    z = complex_gaussian(rng, (n, n))
    q, r = np.linalg.qr(z)
    ph = np.diagonal(r) / np.abs(np.diagonal(r))
    return q * ph[None, :]


def gate_tensor(u4):
    """4×4 unitary → gate array G[a, b, a', b'] (index order [plug i, plug i+1,
    plug i', plug i+1']) with U[(a,b), (a',b')] in C order."""
    return np.ascontiguousarray(u4.reshape(2, 2, 2, 2))


def tebd_layers(L, n_layers, seed_base=3, serpentine=False):
    """Brickwork layers: odd layers (1-based) act on bonds (1,2),(3,4),…; even layers
    on (2,3),(4,5),….  Layer ℓ (0-based) draws its gates from seed seed_base+ℓ.  With
    ``serpentine`` the even layers are applied right to left (layer tuples carry the
    direction), so each layer starts where the previous one left the orthogonality
    centre."""
    layers = []
    for ell in range(n_layers):
        rng = np.random.default_rng(seed_base + ell)
        start = 1 if ell % 2 == 0 else 2
        n_g = (L - start + 1) // 2
        gates = [gate_tensor(haar_unitary(rng, 4)) for _ in range(n_g)]
        layers.append((start, gates, serpentine and ell % 2 == 1))
    return layers


# -----------------------------------------------------------------------------
# the five workloads
# -----------------------------------------------------------------------------

TEBD = dict(L=64, d=2, chi0=16, chi_max=256, layers=10, cutoff=1e-12, seed=2)
PLAIN_SMALL = dict(L=32, d=2, chi=64, seed=1, z_site=16)


def tebd_workload(L=TEBD["L"], chi0=TEBD["chi0"], n_layers=TEBD["layers"], seed=TEBD["seed"]):
    """The TEBD workload: the seeded initial MPS and its brickwork layers, odd layers
    swept left to right and even layers right to left (serpentine)."""
    sites = random_mps_arrays(L, 2, chi0, seed)
    return sites, tebd_layers(L, n_layers, serpentine=True)


def plain_small_workload(L=32, chi=64, seed=1):
    """Config 'plain small': i.i.d. Gaussian sites (not orthogonalised)."""
    return random_mps_arrays(L, 2, chi, seed, orthogonalize=False)


def batched_workload(n=512, seed=5, L_range=(16, 128), chi_range=(16, 512)):
    """Many MPS of uneven length and bond dimension: L ~ U{16..128},
    χ = round(exp(U[ln16, ln512]))."""
    rng = np.random.default_rng(seed)
    specs = []
    for _ in range(n):
        L = int(rng.integers(L_range[0], L_range[1] + 1))
        chi = int(round(np.exp(rng.uniform(np.log(chi_range[0]), np.log(chi_range[1])))))
        specs.append((L, chi, int(rng.integers(0, 2**31 - 1))))
    return specs


def pauli_z():
    return np.array([[1, 0], [0, -1]], dtype=np.complex128)


# ----------------------------------------------------------------------------------
# query serving: device-resident pool + Poisson query trace
# ----------------------------------------------------------------------------------
SERVING_CHIS = (32, 64, 128, 256, 512, 1024)


def serving_pool(n_pairs=8, seed=6):
    """Pool of 2·n_pairs random MPS, d=2: L uniform in [8, 256], χ uniform in
    {32, …, 1024}, bonds clamped.  MPS come in pairs of equal L (χ drawn independently)
    so that overlap queries always have a partner.  Returns [(L, χ, seed)]."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_pairs):
        L = int(rng.integers(8, 257))
        ca, cb = (int(c) for c in rng.choice(SERVING_CHIS, 2))
        out.append((L, ca, 1000 * seed + 2 * k))
        out.append((L, cb, 1000 * seed + 2 * k + 1))
    return out


def serving_trace(pool_L, rate, n, seed=7, d=2):
    """n queries with exponential inter-arrival times at ``rate`` per second: 60 %
    amplitudes of uniform random bit strings on a uniform random pool MPS, 30 % ⟨O_i⟩
    with O = (X + X†)/2 (X complex Gaussian 2×2) at a uniform site, 10 % overlaps of the
    two MPS of a uniform random pair.  ``pool_L``: L of each pool entry (pairs adjacent).
    Returns [(t_arrival, kind, mps, arg)] with kind in {"amp", "exp", "ovl"}."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, n))
    t -= t[0]
    out = []
    npool = len(pool_L)
    for k in range(n):
        u = rng.random()
        if u < 0.6:
            m = int(rng.integers(npool))
            out.append((float(t[k]), "amp", m, rng.integers(0, d, pool_L[m])))
        elif u < 0.9:
            m = int(rng.integers(npool))
            X = complex_gaussian(rng, (d, d))
            out.append((float(t[k]), "exp", m, (int(rng.integers(1, pool_L[m] + 1)), (X + X.conj().T) / 2)))
        else:
            p = int(rng.integers(npool // 2))
            out.append((float(t[k]), "ovl", 2 * p, 2 * p + 1))
    return out


# ----------------------------------------------------------------------------------
# batched (ragged) population
# ----------------------------------------------------------------------------------
def batched_population(n=512, seed=5, Lmin=16, Lmax=128, chimin=16, chimax=512):
    """n independent MPS shapes: L uniform in [Lmin, Lmax], χ = round(exp(U[ln χmin,
    ln χmax])).  Returns (Ls, chis)."""
    rng = np.random.default_rng(seed)
    Ls = [int(x) for x in rng.integers(Lmin, Lmax + 1, n)]
    chis = [int(round(float(np.exp(u)))) for u in rng.uniform(np.log(chimin), np.log(chimax), n)]
    return Ls, chis
