"""CPU oracle: a numpy/scipy restatement of Tenet.jl's MPS hot path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product (the CUDA library and its host
mirror) imports this module; only ``tests/``, ``__graft_entry__.smoke()`` and the CPU
legs of ``bench.py`` use it, as the parity reference and as the timed CPU baseline.

What it restates (Tenet.jl v0.10.3, file:line relative to the project root):

* ``generic_canonize_site!``      src/Operations/canonize.jl:23-76   (QR / SVD gauge move)
* ``generic_bond_canonize_site!`` src/Operations/canonize.jl:78-116  (SVD, Λ kept apart)
* ``generic_mps_canonize!``       src/Operations/canonize.jl:121-252 (form transitions)
* ``generic_mps_compress!``       src/Operations/compress.jl:21-69   (maxdim, absolute threshold)
* ``generic_simple_update!``      src/Operations/simple_update.jl:20-92
* ``overlap``                     src/Operations/overlap.jl:22-50    (⟨b|a⟩ = Σ a·conj(b))
* ``norm`` / ``normalize!``       src/Operations/norm.jl:17-37, normalize.jl:15-37
* ``MPS(arrays; order)``          src/Components/MPS.jl:50-94
* ``rand(MPS)`` bond clamping     src/Components/MPS.jl:113-165
* ``ProductState(bitstr)``        src/Components/ProductState.jl:72-92
* ``checkform`` / ``isisometry``  src/Components/MPO.jl:41-83 (atol 1e-12)

The arithmetic itself lives in the un-vendored Muscle.jl (>= 0.3.9): ``binary_einsum``
(permute + BLAS gemm), ``tensor_qr_thin`` (LAPACK geqrf/ungqr), ``tensor_svd_thin``
(LAPACK gesdd) and ``simple_update`` (θ = A·B·op → thin SVD → keep ≤ maxdim → √S into
both sides).  Here those are numpy ``tensordot``/``einsum`` and scipy's LAPACK drivers.
Muscle choices invisible from Tenet's source are fixed as follows and documented:
no renormalisation after truncation; exact-zero singular values are kept up to
``maxdim`` (the CX known answer, test/unit/simple_update.jl:38-42, keeps a zero
singular value on bond 1-2); the optional absolute ``threshold`` of
``simple_update`` mirrors compress.jl:54-59 and always keeps at least one value.

Parity pinning: the reference ships no golden vectors for this path (and Julia is not
available to run it).  The oracle is pinned by the reference's own invariant and
known-answer tests, ported in tests/test_oracle_reference.py.  Results at the Muscle
boundary (raw Q, U, V) are gauge-dependent and are compared only through invariants.

Site layout: every site tensor is stored 3-D as (χ_left, d, χ_right), column-major
semantics kept by numpy index order; the open ends carry a size-1 bond.  This is
Tenet's ``(:l, :o, :r)`` order with the boundary 2-D tensors lifted to 3-D.
"""

from __future__ import annotations

import numpy as np
import scipy.linalg as sla

# ----------------------------------------------------------------------------------
# canonical forms (src/CanonicalForm.jl:10-87)
# ----------------------------------------------------------------------------------


class NonCanonical:
    def __eq__(self, other):
        return isinstance(other, NonCanonical)

    def __repr__(self):
        return "NonCanonical()"


class MixedCanonical:
    """Orthogonality centre = sites lo..hi (1-based, inclusive)."""

    def __init__(self, sites):
        if isinstance(sites, int):
            sites = [sites]
        self.sites = sorted(set(int(s) for s in sites))

    @property
    def lo(self):
        return self.sites[0]

    @property
    def hi(self):
        return self.sites[-1]

    def __eq__(self, other):
        return isinstance(other, MixedCanonical) and self.sites == other.sites

    def __repr__(self):
        return f"MixedCanonical({self.sites})"


class BondCanonical:
    """Orthogonality centre = bond (i, i+1); Λ stored at LambdaSite(bond)."""

    def __init__(self, a, b=None):
        if b is None:
            a, b = a
        self.a, self.b = min(a, b), max(a, b)

    def __eq__(self, other):
        return isinstance(other, BondCanonical) and (self.a, self.b) == (other.a, other.b)

    def __repr__(self):
        return f"BondCanonical({self.a}-{self.b})"


# ----------------------------------------------------------------------------------
# MPS container
# ----------------------------------------------------------------------------------


class OMPS:
    """Oracle MPS: site tensors (χl, d, χr), canonical form, Λ vectors by bond."""

    def __init__(self, sites, form=None):
        self.sites = [np.asarray(s) for s in sites]
        self.form = form if form is not None else MixedCanonical(range(1, len(sites) + 1))
        self.lam = {}  # bond index i (bond i-(i+1)) -> Λ vector

    @property
    def L(self):
        return len(self.sites)

    def copy(self):
        m = OMPS([s.copy() for s in self.sites], self.form)
        m.lam = {k: v.copy() for k, v in self.lam.items()}
        return m

    def bondsizes(self):
        return [self.sites[i].shape[2] for i in range(self.L - 1)]

    def site(self, i):
        return self.sites[i - 1]

    def set_site(self, i, t):
        self.sites[i - 1] = t


def mps_from_arrays(arrays, order=("l", "r", "o")):
    """``MPS(arrays; order)`` (src/Components/MPS.jl:50-94), lifted to 3-D sites."""
    order = tuple(order)
    assert sorted(order) == ["l", "o", "r"]
    L = len(arrays)
    out = []
    for i, a in enumerate(arrays):
        a = np.asarray(a)
        if i == 0:
            lo = tuple(x for x in order if x != "l")
            assert a.ndim == 2
            t = np.moveaxis(a, [lo.index("o"), lo.index("r")], [0, 1])[None, :, :]
        elif i == L - 1:
            lo = tuple(x for x in order if x != "r")
            assert a.ndim == 2
            t = np.moveaxis(a, [lo.index("l"), lo.index("o")], [0, 1])[:, :, None]
        else:
            assert a.ndim == 3
            t = np.moveaxis(a, [order.index("l"), order.index("o"), order.index("r")], [0, 1, 2])
        out.append(np.ascontiguousarray(t))
    return OMPS(out)


def mpo_from_arrays(arrays, order=("l", "r", "o", "i")):
    """``MPO(arrays; order)`` (src/Components/MPO.jl:85-125, default order (:l, :r, :o, :i))
    as an MPS whose physical index fuses (o, i) column-major (o fastest): canonize! and
    compress! on an MPO keep both plugs on the same side of every factorisation, so the
    fused MPS has the same gauge moves.  Returns the OMPS with ``phys`` = [(d_o, d_i)]."""
    order = tuple(order)
    assert sorted(order) == ["i", "l", "o", "r"]
    L = len(arrays)
    sites, phys = [], []
    for k, a in enumerate(arrays):
        a = np.asarray(a)
        own = tuple(x for x in order if not ((k == 0 and x == "l") or (k == L - 1 and x == "r")))
        assert a.ndim == len(own), f"site {k + 1}: expected {len(own)} dimensions"
        t = np.moveaxis(a, [own.index(x) for x in ("o", "i")] + [own.index(x) for x in ("l", "r") if x in own],
                        list(range(len(own))))
        # t: (o, i[, l][, r]) → (l, o, i, r) with size-1 open ends
        o, i = t.shape[0], t.shape[1]
        rest = t.shape[2:]
        l = rest[0] if "l" in own else 1
        r = rest[-1] if "r" in own else 1
        t = np.transpose(t.reshape(o, i, l, r), (2, 0, 1, 3))
        sites.append(np.ascontiguousarray(t.reshape(l, o * i, r, order="F")))
        phys.append((o, i))
    psi = OMPS(sites)
    psi.phys = phys
    return psi


# ----------------------------------------------------------------------------------
# Muscle-level primitives (restated)
# ----------------------------------------------------------------------------------


def qr_thin(m):
    """tensor_qr_thin on a matrix: LAPACK geqrf + ungqr, k = min(rows, cols)."""
    q, r = np.linalg.qr(m, mode="reduced")
    return q, r


def svd_thin(m, driver="gesdd"):
    """tensor_svd_thin on a matrix: LAPACK gesdd; s descending; m = U diag(s) Vh.
    ``driver="gesvd"`` selects LAPACK's QR-iteration SVD instead: the same
    decomposition with different rounding, which the full-size parity tests use to
    measure how far rounding alone moves a truncated TEBD run."""
    try:
        u, s, vh = sla.svd(m, full_matrices=False, lapack_driver=driver)
    except np.linalg.LinAlgError:
        u, s, vh = sla.svd(m, full_matrices=False, lapack_driver="gesvd")
    return u, s, vh


def isisometry(t, axis, atol=1e-12):
    """Muscle.isisometry(tensor, index): contracting all other indices with the
    conjugate gives the identity on ``axis``."""
    t = np.moveaxis(np.asarray(t), axis, -1)
    m = t.reshape(-1, t.shape[-1])
    g = m.conj().T @ m
    return bool(np.allclose(g, np.eye(g.shape[0]), atol=atol, rtol=0))


# ----------------------------------------------------------------------------------
# gauge moves (src/Operations/canonize.jl:23-116)
# ----------------------------------------------------------------------------------


def canonize_site(psi: OMPS, site: int, direction: str, method="qr"):
    """generic_canonize_site! (canonize.jl:23-76).  direction 'right' factorises site
    ``site`` across bond (site, site+1) and pushes R into site+1; 'left' factorises
    across bond (site-1, site) and pushes into site-1.  Size-1 bonds are skipped
    (canonize.jl:38)."""
    A = psi.site(site)
    if direction == "right":
        chi = A.shape[2]
        if chi == 1:
            return
        B = psi.site(site + 1)
        m = A.reshape(-1, chi, order="C")  # rows (χl, d), cols χr
        if method == "qr":
            q, r = qr_thin(m)
        else:
            u, s, vh = svd_thin(m)
            q, r = u, s[:, None] * vh
        k = q.shape[1]
        psi.set_site(site, q.reshape(A.shape[0], A.shape[1], k))
        psi.set_site(site + 1, np.tensordot(r, B, axes=(1, 0)))
    else:
        chi = A.shape[0]
        if chi == 1:
            return
        B = psi.site(site - 1)
        m = A.reshape(chi, -1).T  # rows (d, χr), cols χl
        if method == "qr":
            q, r = qr_thin(m)
        else:
            u, s, vh = svd_thin(m)
            q, r = u, s[:, None] * vh
        k = q.shape[1]
        psi.set_site(site, q.T.reshape(k, A.shape[1], A.shape[2]))
        psi.set_site(site - 1, np.tensordot(B, r.T, axes=(2, 0)))


def bond_canonize_site(psi: OMPS, site: int, bond_a: int):
    """generic_bond_canonize_site! (canonize.jl:78-116): thin SVD of ``site`` across
    bond (bond_a, bond_a+1); U stays, V is contracted into the neighbour, Λ kept."""
    assert bond_a not in psi.lam
    A = psi.site(site)
    if site == bond_a:  # factorise towards the right
        chi = A.shape[2]
        if chi == 1:
            return
        B = psi.site(site + 1)
        u, s, vh = svd_thin(A.reshape(-1, chi))
        k = s.size
        psi.set_site(site, u.reshape(A.shape[0], A.shape[1], k))
        psi.set_site(site + 1, np.tensordot(vh, B, axes=(1, 0)))
    else:  # site == bond_a + 1: factorise towards the left
        chi = A.shape[0]
        if chi == 1:
            return
        B = psi.site(site - 1)
        u, s, vh = svd_thin(A.reshape(chi, -1).T)
        k = s.size
        psi.set_site(site, u.T.reshape(k, A.shape[1], A.shape[2]))
        psi.set_site(site - 1, np.tensordot(B, vh.T, axes=(2, 0)))
    psi.lam[bond_a] = s


def hadamard_bond(t, lam, axis):
    """Muscle.hadamard(tensor, Λ) along one index (canonize.jl:198,209)."""
    shape = [1] * t.ndim
    shape[axis] = lam.size
    return t * lam.reshape(shape)


# ----------------------------------------------------------------------------------
# form transitions (src/Operations/canonize.jl:121-252)
# ----------------------------------------------------------------------------------


def canonize(psi: OMPS, new_form):
    """canonize!(ψ, form); ints and lists of ints mean MixedCanonical, tuples of two
    ints BondCanonical (canonize.jl:16-20)."""
    if isinstance(new_form, int) or isinstance(new_form, list):
        new_form = MixedCanonical(new_form)
    elif isinstance(new_form, tuple):
        new_form = BondCanonical(new_form)
    old = psi.form
    if isinstance(new_form, NonCanonical):
        psi.form = NonCanonical()
        return psi
    if isinstance(old, NonCanonical):
        psi.form = MixedCanonical(range(1, psi.L + 1))
        return canonize(psi, new_form)
    if isinstance(old, MixedCanonical) and isinstance(new_form, MixedCanonical):
        if old == new_form:
            return psi
        src_left, src_right = old.lo, old.hi
        dst_left, dst_right = new_form.lo - 1, new_form.hi + 1
        for i in range(src_left, dst_left + 1):  # canonize.jl:136-139
            canonize_site(psi, i, "right")
        for i in range(src_right, dst_right - 1, -1):  # canonize.jl:142-145
            canonize_site(psi, i, "left")
        psi.form = MixedCanonical(new_form.sites)
        return psi
    if isinstance(old, MixedCanonical) and isinstance(new_form, BondCanonical):
        old_min, old_max = old.lo, old.hi
        new_min, new_max = new_form.a, new_form.b
        if old_max <= new_min:
            canonize(psi, MixedCanonical(new_min))
            bond_canonize_site(psi, new_min, new_form.a)
        elif new_max <= old_min:
            canonize(psi, MixedCanonical(new_max))
            bond_canonize_site(psi, new_max, new_form.a)
        elif old_min <= new_min and new_max <= old_max:
            canonize(psi, MixedCanonical(new_min))
            bond_canonize_site(psi, new_min, new_form.a)
        else:
            raise ValueError(f"Cannot canonize from {old} to {new_form}")
        psi.form = new_form
        return psi
    if isinstance(old, BondCanonical) and isinstance(new_form, MixedCanonical):
        old_min, old_max = old.a, old.b
        new_min, new_max = new_form.lo, new_form.hi
        lam = psi.lam.pop(old.a)
        if old_max <= new_min:
            psi.set_site(old_max, hadamard_bond(psi.site(old_max), lam, 0))
            psi.form = MixedCanonical(old_max)
            canonize(psi, new_form)
        elif new_max <= old_min:
            psi.set_site(old_min, hadamard_bond(psi.site(old_min), lam, 2))
            psi.form = MixedCanonical(old_min)
            canonize(psi, new_form)
        else:
            raise ValueError(f"Cannot canonize from {old} to {new_form}")
        psi.form = new_form
        return psi
    if isinstance(old, BondCanonical) and isinstance(new_form, BondCanonical):
        if old == new_form:
            return psi
        old_min, old_max = old.a, old.b
        new_min, new_max = new_form.a, new_form.b
        if old_max <= new_min:
            canonize(psi, MixedCanonical(new_min))
            bond_canonize_site(psi, new_min, new_form.a)
        elif new_max <= old_min:
            canonize(psi, MixedCanonical(new_max))
            bond_canonize_site(psi, new_max, new_form.a)
        else:
            raise ValueError(f"Cannot canonize from {old} to {new_form}")
        psi.form = new_form
        return psi
    raise ValueError(f"Cannot canonize from {old} to {new_form}")


def checkform(psi: OMPS, atol=1e-12):
    """checkform (src/Components/MPO.jl:41-83)."""
    f = psi.form
    if isinstance(f, NonCanonical):
        return True
    left, right = (f.lo, f.hi) if isinstance(f, MixedCanonical) else (f.a, f.b)
    for i in range(1, psi.L + 1):
        if i < left and not isisometry(psi.site(i), 2, atol):
            raise ValueError(f"site {i} is not left-canonical")
        if i > right and not isisometry(psi.site(i), 0, atol):
            raise ValueError(f"site {i} is not right-canonical")
    return True


# ----------------------------------------------------------------------------------
# compress (src/Operations/compress.jl:21-69)
# ----------------------------------------------------------------------------------


def compress(psi: OMPS, bond=None, maxdim=None, threshold=None):
    if maxdim is None and threshold is None:
        raise ValueError("Either `maxdim` or `threshold` must be specified")
    if maxdim is not None and maxdim <= 0:
        raise ValueError("maxdim must be a positive integer")
    if threshold is not None and threshold <= 0:
        raise ValueError("Threshold must be positive")
    if bond is None:
        for i in range(1, psi.L):
            compress(psi, (i, i + 1), maxdim, threshold)
        return psi
    a, b = min(bond), max(bond)
    canonize(psi, BondCanonical(a, b))
    if a not in psi.lam:  # size-1 bond: nothing to truncate
        return psi
    s = psi.lam[a]
    keep = np.arange(s.size)
    if maxdim is not None:
        keep = keep[: min(maxdim, s.size)]
    if threshold is not None:
        keep = keep[np.abs(s[keep]) > threshold]
    psi.set_site(a, psi.site(a)[:, :, keep])
    psi.set_site(b, psi.site(b)[keep, :, :])
    psi.lam[a] = s[keep]
    return psi


# ----------------------------------------------------------------------------------
# simple update (src/Operations/simple_update.jl:20-92)
# ----------------------------------------------------------------------------------


def simple_update_tensors(A, B, G, maxdim=None, threshold=None, driver="gesdd"):
    """Muscle.simple_update with AbsorbEqually: θ[l,a,b,r] = Σ G[a,b,a',b'] A[l,a',m]
    B[m,b',r]; SVD over (l,a)|(b,r); keep ≤ maxdim (then |s| > threshold, ≥ 1 kept);
    A' = U√S, B' = √S Vh.  Returns (A', B', s_kept, s_full)."""
    chl, d1, _ = A.shape
    _, d2, chr_ = B.shape
    theta = np.tensordot(A, B, axes=(2, 0))  # l, a', b', r
    theta = np.einsum("abcd,lcdr->labr", G, theta, optimize=True)
    u, s, vh = svd_thin(theta.reshape(chl * d1, d2 * chr_), driver)
    k = s.size if maxdim is None else min(maxdim, s.size)
    if threshold is not None:
        k = max(1, int(np.count_nonzero(np.abs(s[:k]) > threshold)))
    sq = np.sqrt(s[:k])
    An = (u[:, :k] * sq[None, :]).reshape(chl, d1, k)
    Bn = (sq[:, None] * vh[:k, :]).reshape(k, d2, chr_)
    return An, Bn, s[:k], s


def simple_update(psi: OMPS, G, sites, maxdim=None, threshold=None, spectra=None, driver="gesdd"):
    """simple_update!(ψ::MPS, op) (simple_update.jl:82-92): move the centre onto the
    gate's sites, then apply; the 1-site shortcut is simple_update.jl:27-37.

    ``G`` is the gate array; for two sites its index order is
    [plug a, plug b, plug a', plug b'] with a < b adjacent, primed = input.
    ``spectra`` (a list) receives θ's full singular spectrum of a two-site gate."""
    sites = sorted(sites)
    canonize(psi, MixedCanonical(sites))
    if len(sites) == 1:
        i = sites[0]
        psi.set_site(i, np.einsum("ab,lbr->lar", G, psi.site(i)))
        return psi
    a, b = sites
    assert b == a + 1
    An, Bn, _, s_full = simple_update_tensors(psi.site(a), psi.site(b), G, maxdim, threshold, driver)
    if spectra is not None:
        spectra.append(s_full)
    psi.set_site(a, An)
    psi.set_site(b, Bn)
    return psi


# ----------------------------------------------------------------------------------
# overlap / norm (src/Operations/overlap.jl:22-50, norm.jl:17-37, normalize.jl:15-37)
# ----------------------------------------------------------------------------------


def overlap(a: OMPS, b: OMPS):
    """overlap(a::MPS, b::MPS) = ⟨b|a⟩ by a left-environment sweep (overlap.jl:36-50)."""
    if a.L != b.L:
        raise ValueError("nsites differ")
    env = np.ones((1, 1), dtype=np.result_type(a.sites[0], b.sites[0]))
    for A, B in zip(a.sites, b.sites):
        t = np.tensordot(env, A, axes=(0, 0))  # y, s, x'
        env = np.tensordot(t, B.conj(), axes=([0, 1], [0, 1]))  # x', y'
    return complex(env[0, 0])


def product_state_vectors(bits: str):
    """ProductState(bitstr) (ProductState.jl:72-92)."""
    table = {
        "0": [1.0, 0.0],
        "1": [0.0, 1.0],
        "+": [1 / np.sqrt(2), 1 / np.sqrt(2)],
        "-": [1 / np.sqrt(2), -1 / np.sqrt(2)],
        "u": [1 / np.sqrt(2), -1j / np.sqrt(2)],
        "↑": [1 / np.sqrt(2), -1j / np.sqrt(2)],
        "d": [-1 / np.sqrt(2), -1j / np.sqrt(2)],
        "↓": [-1 / np.sqrt(2), -1j / np.sqrt(2)],
    }
    out = []
    for c in bits:
        if c not in table:
            raise ValueError(f"invalid character: {c}")
        out.append(np.asarray(table[c], dtype=np.complex128))
    return out


def amplitude(vectors, psi: OMPS):
    """overlap(::ProductState, ::MPS) (overlap.jl:22-32): Σ ψ · v, v not conjugated."""
    env = np.ones((1,), dtype=np.complex128)
    for v, A in zip(vectors, psi.sites):
        M = np.tensordot(A, v, axes=(1, 0))  # l, r
        env = env @ M
    return complex(env[0])


def norm(psi: OMPS):
    """norm(ψ::MPS) (norm.jl:17-37); moves the centre like the reference."""
    f = psi.form
    if isinstance(f, NonCanonical):
        psi.form = MixedCanonical(range(1, psi.L + 1))
        return norm(psi)
    if isinstance(f, MixedCanonical):
        canonize(psi, MixedCanonical(f.lo))
        return float(np.linalg.norm(psi.site(f.lo)))
    return float(np.linalg.norm(psi.lam[f.a]))


def normalize(psi: OMPS):
    """normalize!(ψ::MPS) (normalize.jl:15-37)."""
    f = psi.form
    if isinstance(f, NonCanonical):
        psi.form = MixedCanonical(range(1, psi.L + 1))
        return normalize(psi)
    if isinstance(f, MixedCanonical):
        canonize(psi, MixedCanonical(f.lo))
        t = psi.site(f.lo)
        psi.set_site(f.lo, t / np.linalg.norm(t))
        return psi
    psi.lam[f.a] = psi.lam[f.a] / np.linalg.norm(psi.lam[f.a])
    return psi


def local_expectations(psi: OMPS, op):
    """⟨ψ|O_i|ψ⟩ / ⟨ψ|ψ⟩ for every site i with a left/right environment sweep.
    Equal to overlap(ψ, O_i ψ) / overlap(ψ, ψ) (the overlap.jl:36-50 convention) at a
    cost of ~3 overlaps instead of L."""
    L = psi.L
    lefts = [np.ones((1, 1), dtype=np.complex128)]
    for A in psi.sites[:-1]:
        t = np.tensordot(lefts[-1], A, axes=(0, 0))
        lefts.append(np.tensordot(t, A.conj(), axes=([0, 1], [0, 1])))
    rights = [np.ones((1, 1), dtype=np.complex128)]
    for A in psi.sites[:0:-1]:
        t = np.tensordot(A, rights[-1], axes=(2, 0))  # l, s, r'
        rights.append(np.tensordot(t, A.conj(), axes=([1, 2], [1, 2])))
    rights = rights[::-1]
    out = np.empty(L, dtype=np.complex128)
    nrm = None
    for i, A in enumerate(psi.sites):
        OA = np.einsum("ab,lbr->lar", op, A)
        t = np.tensordot(lefts[i], OA, axes=(0, 0))  # y, s, r
        t = np.tensordot(t, rights[i], axes=(2, 0))  # y, s, r'
        out[i] = np.tensordot(t, A.conj(), axes=([0, 1, 2], [0, 1, 2]))
        if nrm is None:
            t = np.tensordot(lefts[i], A, axes=(0, 0))
            t = np.tensordot(t, rights[i], axes=(2, 0))
            nrm = complex(np.tensordot(t, A.conj(), axes=([0, 1, 2], [0, 1, 2])))
    return out / nrm, nrm


def expectation(psi: OMPS, site: int, op):
    """⟨ψ|O_site|ψ⟩ / ⟨ψ|ψ⟩ computed the reference's way: overlap(ψ, O_site ψ) /
    overlap(ψ, ψ), two environment sweeps (overlap.jl:36-50); ``site`` is 1-based."""
    opsi = psi.copy()
    A = psi.site(site)
    opsi.set_site(site, np.einsum("ab,lbr->lar", op, A))
    return overlap(opsi, psi) / overlap(psi, psi)


def sample(psi: OMPS, uniforms):
    """sample(ψ, nsamples) (sample.jl:20-72) with explicit uniforms (nsamples × L in
    [0, 1)) in place of Julia's RNG: canonize a copy to MixedCanonical(1); for each site
    the marginals p_s = Σ_r |t[s, r]|² of the projected site t = proj · A_i, outcome by
    inverse CDF of u·Σp, proj ← t[s, :] / √p_s.  Returns 1-based outcomes."""
    phi = psi.copy()
    canonize(phi, MixedCanonical(1))
    u = np.asarray(uniforms, dtype=np.float64)
    out = np.zeros(u.shape, dtype=np.int64)
    for q in range(u.shape[0]):
        proj = np.ones((1,), dtype=np.complex128)
        for i, A in enumerate(phi.sites):
            t = np.tensordot(proj, A, axes=(0, 0))  # (d, χr)
            p = np.sum(np.abs(t) ** 2, axis=1)
            target = u[q, i] * p.sum()
            c = np.cumsum(p)
            ch = int(np.searchsorted(c, target, side="right"))
            ch = min(ch, len(p) - 1)
            while ch > 0 and p[ch] == 0.0:
                ch -= 1
            out[q, i] = ch + 1
            proj = t[ch] / np.sqrt(p[ch])
    return out


def evolve_mpo_direct(psi: OMPS, mpo):
    """evolve!(ψ::MPS, op::MPO) (evolve.jl:131-137): generic_evolve_mps_mpo_direct!
    (evolve.jl:19-46) — per site c = A·W over the physical index, the MPS and MPO bonds
    fused on both sides — then canonize!(ψ, MixedCanonical(all sites)).  MPO sites are
    (w_l, d_out, d_in, w_r)."""
    if len(mpo) != psi.L:
        raise ValueError("MPS and MPO must have the same number of sites")
    sites = []
    for A, W in zip(psi.sites, mpo):
        c = np.einsum("lsr,aosb->laorb", A, W)
        l, a, o, r, b = c.shape
        sites.append(c.reshape(l * a, o, r * b))
    psi.sites = sites
    psi.lam = {}
    psi.form = MixedCanonical(range(1, psi.L + 1))
    return psi


def _truncate(U, S, V, maxdim, threshold):
    keep = np.arange(S.size)
    if maxdim is not None:
        keep = keep[: min(maxdim, S.size)]
    if threshold is not None:
        keep = keep[np.abs(S[keep]) > threshold]
    return U[:, keep], S[keep], V[keep, :]


def evolve_mpo_zipup(psi: OMPS, mpo, maxdim=None, threshold=None):
    """generic_evolve_mps_mpo_zipup! (evolve.jl:49-129): C₁ = A₁·W₁ split by a thin SVD
    with the physical index on the U side, truncated (maxdim, then |s| > threshold),
    R = S·V carried right: R ← (R·A_i)·W_i, split with (left bond, physical) on the U
    side; the last site takes R·A_L·W_L.  The form is left as the reference leaves it."""
    if len(mpo) != psi.L:
        raise ValueError("MPS and MPO must have the same number of sites")
    if maxdim is None and threshold is None:
        raise ValueError("Either `maxdim` or `threhold` must be specified")
    L = psi.L
    sites = []
    # site 1: c[o, r, b] (A: 1 × s × r, W: 1 × o × s × b)
    c = np.einsum("lsr,aosb->orb", psi.sites[0], mpo[0])
    o, r, b = c.shape
    U, S, V = svd_thin(c.reshape(o, r * b))
    U, S, V = _truncate(U, S, V, maxdim, threshold)
    sites.append(U.reshape(1, o, -1))
    R = (S[:, None] * V).reshape(-1, r, b)  # (k, χ, w)
    for i in range(1, L - 1):
        A, W = psi.sites[i], mpo[i]
        t = np.einsum("kcw,csr,wosb->korb", R, A, W)
        k, o, r, b = t.shape
        U, S, V = svd_thin(t.reshape(k * o, r * b))
        U, S, V = _truncate(U, S, V, maxdim, threshold)
        sites.append(U.reshape(k, o, -1))
        R = (S[:, None] * V).reshape(-1, r, b)
    t = np.einsum("kcw,csr,wosb->kor", R, psi.sites[L - 1], mpo[L - 1])
    sites.append(t)
    psi.sites = sites
    psi.lam = {}
    return psi


def contract_state(psi: OMPS):
    """Full state vector (small L only): the ``contract(ψ)`` of the reference tests,
    with Λ absorbed when the MPS is bond-canonical."""
    sites = [s for s in psi.sites]
    if isinstance(psi.form, BondCanonical) and psi.form.a in psi.lam:
        a = psi.form.a
        sites[a - 1] = hadamard_bond(sites[a - 1], psi.lam[a], 2)
    v = sites[0]
    for A in sites[1:]:
        v = np.tensordot(v, A, axes=(v.ndim - 1, 0))
    return v.reshape(-1)


# ----------------------------------------------------------------------------------
# TEBD driver (brickwork of 2-site gates, each simple_update! + absolute cutoff)
# ----------------------------------------------------------------------------------


def tebd(psi: OMPS, layers, maxdim, threshold, spectra=None, driver="gesdd"):
    """Apply brickwork layers: (bond_start, [G...]) left→right, or (bond_start, [G...],
    reverse) right→left when reverse is true (gates listed left to right either way) —
    one simple_update! per gate, in that order.  ``spectra`` (a list) receives every
    gate's full θ spectrum, in order."""
    for ly in layers:
        start, gates = ly[0], ly[1]
        order = range(len(gates) - 1, -1, -1) if (len(ly) > 2 and ly[2]) else range(len(gates))
        for j in order:
            a = start + 2 * j
            simple_update(psi, gates[j], (a, a + 1), maxdim=maxdim, threshold=threshold, spectra=spectra,
                          driver=driver)
    return psi


def truncation_gap(s, maxdim, threshold):
    """Relative gap (σ_k − σ_{k+1}) / σ_k at a gate's cut, k the kept rank under the
    maxdim cap and the absolute threshold; +inf when nothing above the threshold is
    discarded (the cut then falls at the threshold, far below the kept values)."""
    k = s.size if maxdim is None else min(maxdim, s.size)
    if threshold is not None:
        k = max(1, int(np.count_nonzero(np.abs(s[:k]) > threshold)))
    if k >= s.size or s[k] <= (threshold or 0.0):
        return float("inf")
    return float((s[k - 1] - s[k]) / s[k - 1])


# ----------------------------------------------------------------------------------
# DMRG (src/Algorithms/DMRG.jl) with the Ising MPO (src/Models/Ising.jl)
# ----------------------------------------------------------------------------------


def ising_1d_mpo(L, h, J):
    """ising_1d_mpo(L, h, J) (src/Models/Ising.jl:12-31): H = -J Σ Z_i Z_{i+1} - h Σ X_i
    as a lower-triangular MPO with bond dimension 3 (start state 3, end state 1).  Sites
    are returned as (w_l, d_out, d_in, w_r) with the open ends lifted to size 1."""
    Id = np.eye(2)
    sx = np.array([[0.0, 1.0], [1.0, 0.0]])
    sz = np.array([[1.0, 0.0], [0.0, -1.0]])
    W = np.zeros((3, 2, 2, 3), dtype=np.complex128)  # (l, o, i, r)
    W[0, :, :, 0] = Id
    W[1, :, :, 0] = sz
    W[2, :, :, 0] = -h * sx
    W[2, :, :, 1] = -J * sz
    W[2, :, :, 2] = Id
    first = W[2:3].copy()  # W_1 = W[:, :, 3, :]
    last = W[:, :, :, 0:1].copy()  # W_n = W[:, :, :, 1]
    return [first] + [W.copy() for _ in range(L - 2)] + [last]


def heisenberg_mpo(L, J, Jz, h):
    """XXZ chain H = Σ J(S⁺S⁻ + S⁻S⁺)/2 + Jz SᶻSᶻ + h Σ Sᶻ as a bond-5 MPO in the layout of
    ising_1d_mpo (w_l, d_out, d_in, w_r): start state 4, end state 0.  Not a reference
    model: a second Hamiltonian (MPO bond 5) for the DMRG parity tests."""
    sp = np.array([[0.0, 1.0], [0.0, 0.0]])
    sm = sp.T.copy()
    sz = np.diag([0.5, -0.5])
    W = np.zeros((5, 2, 2, 5), dtype=np.complex128)
    W[0, :, :, 0] = np.eye(2)
    W[1, :, :, 0] = sp
    W[2, :, :, 0] = sm
    W[3, :, :, 0] = sz
    W[4, :, :, 0] = h * sz
    W[4, :, :, 1] = 0.5 * J * sm
    W[4, :, :, 2] = 0.5 * J * sp
    W[4, :, :, 3] = Jz * sz
    W[4, :, :, 4] = np.eye(2)
    return [W[4:5].copy()] + [W.copy() for _ in range(L - 2)] + [W[:, :, :, 0:1].copy()]


def spin1_xxz_mpo(L, J, Jz, D):
    """Spin-1 XXZ chain with single-ion anisotropy, H = Σ J(S⁺S⁻ + S⁻S⁺)/2 + Jz SᶻSᶻ +
    D Σ (Sᶻ)², bond-5 MPO, d = 3 (the layout of heisenberg_mpo).  Not a reference model: a
    d = 3 Hamiltonian for the DMRG parity tests."""
    r2 = np.sqrt(2.0)
    sp = np.array([[0.0, r2, 0.0], [0.0, 0.0, r2], [0.0, 0.0, 0.0]])
    sm = sp.T.copy()
    sz = np.diag([1.0, 0.0, -1.0])
    W = np.zeros((5, 3, 3, 5), dtype=np.complex128)
    W[0, :, :, 0] = np.eye(3)
    W[1, :, :, 0] = sp
    W[2, :, :, 0] = sm
    W[3, :, :, 0] = sz
    W[4, :, :, 0] = D * sz @ sz
    W[4, :, :, 1] = 0.5 * J * sm
    W[4, :, :, 2] = 0.5 * J * sp
    W[4, :, :, 3] = Jz * sz
    W[4, :, :, 4] = np.eye(3)
    return [W[4:5].copy()] + [W.copy() for _ in range(L - 2)] + [W[:, :, :, 0:1].copy()]


def mpo_dense(mpo):
    """The MPO as a dense 2^L × 2^L matrix (small L only): H[o…, i…]."""
    M = mpo[0][0]  # (o, i, r)
    for W in mpo[1:]:
        # M[(O), (I), a] · W[a, o, i, b] → M[(O o), (I i), b]
        t = np.einsum("OIa,aoib->OoIib", M, W)
        O, o, I, i, b = t.shape
        M = t.reshape(O * o, I * i, b)
    return M[:, :, 0]


def lanczos_lm(apply, x0, krylovdim=3, maxiter=2, tol=1e-12):
    """KrylovKit.eigsolve(f, x0, 1, :LM; ishermitian=true, krylovdim, maxiter) (KrylovKit
    0.9.5–0.10, src/eigsolve/lanczos.jl; a dependency absent from the reference tree)
    restated in exact-arithmetic terms:

    * the Lanczos factorisation grows from x0/‖x0‖ until it holds ``krylovdim`` vectors or
      the residual norm β drops to ``tol`` (an invariant subspace);
    * the tridiagonal Rayleigh quotient is diagonalised and its eigenpairs sorted by
      descending |θ| (``which = :LM``, a stable sort of the ascending spectrum);
    * the leading Ritz pair is converged when |β·u_K| ≤ tol; otherwise, unless the
      iteration count reached ``maxiter``, the factorisation is shrunk to
      keep = ⌊(3·krylovdim + 2·converged)/5⌋ = 1 vector (the Ritz vector, with the
      residual as the next basis direction) and grown again.

    Full re-orthogonalisation replaces KrylovKit's local one; in exact arithmetic both
    give the same factorisation.  Returns (θ, Ritz vector (unit norm), matvecs)."""
    shape = x0.shape
    v = x0.reshape(-1) / np.linalg.norm(x0)
    V = [v]
    alpha, beta = [], []
    w = apply(v.reshape(shape)).reshape(-1)
    nops = 1
    a = np.vdot(v, w).real
    r = w - a * v
    r -= V[0] * np.vdot(V[0], r)
    alpha.append(a)
    b = np.linalg.norm(r)
    it = 1
    while True:
        K = len(V)
        if K == krylovdim or b <= tol:
            if K == 1:
                theta, U = np.array([alpha[0]]), np.ones((1, 1))
                f = np.array([b])
            else:
                T = np.diag(alpha) + np.diag(beta, 1) + np.diag(beta, -1)
                theta, U = np.linalg.eigh(T)  # ascending
                p = sorted(range(K), key=lambda j: -abs(theta[j]))  # stable
                theta, U = theta[p], U[:, p]
                f = U[K - 1, :] * b
            converged = abs(f[0]) <= tol
            if converged or (K == krylovdim and it == maxiter) or (b <= tol):
                x = sum(U[j, 0] * V[j] for j in range(K))
                return float(theta[0]), x.reshape(shape), nops
        if K < krylovdim:
            vn = r / b
            V.append(vn)
            beta.append(b)
            w = apply(vn.reshape(shape)).reshape(-1)
            nops += 1
            a = np.vdot(vn, w).real
            r = w - a * vn - b * V[-2]
            for _ in range(2):
                for q in V:
                    r = r - q * np.vdot(q, r)
            alpha.append(a)
            b = np.linalg.norm(r)
        else:
            # thick restart with one kept vector: [u₁ | r̂], T = [[θ₁, |f₁|], …]
            u = sum(U[j, 0] * V[j] for j in range(K))
            rhat = (np.sign(f[0]) if f[0] != 0 else 1.0) * r / b
            V = [u, rhat]
            alpha = [float(theta[0])]
            beta = [abs(f[0])]
            w = apply(rhat.reshape(shape)).reshape(-1)
            nops += 1
            a = np.vdot(rhat, w).real
            r = w - a * rhat - beta[0] * u
            for _ in range(2):
                for q in V:
                    r = r - q * np.vdot(q, r)
            alpha.append(a)
            b = np.linalg.norm(r)
            it += 1


def _env_left(Lenv, A, W):
    """Left environment update: L'[b, v, b'] = Σ L[a, w, a'] A[a, s, b] W[w, o, s, v]
    conj(A[a', o, b']) — the binary_einsum chain of DMRG.jl:106-115."""
    t = np.tensordot(Lenv, A, axes=(0, 0))  # [w, a', s, b]
    t = np.tensordot(t, W, axes=([0, 2], [0, 2]))  # [a', b, o, v]
    return np.tensordot(t, A.conj(), axes=([0, 2], [0, 1]))  # [b, v, b']


def _env_right(Renv, A, W):
    """Right environment update: R'[a, w, a'] = Σ A[a, s, b] W[w, o, s, v] conj(A[a', o, b'])
    R[b, v, b'] (DMRG.jl:69-79)."""
    t = np.tensordot(A, Renv, axes=(2, 0))  # [a, s, v, b']
    t = np.tensordot(t, W, axes=([1, 2], [2, 3]))  # [a, b', w, o]
    return np.tensordot(t, A.conj(), axes=([3, 1], [1, 2]))  # [a, w, a']


def _heff1(Lenv, W, Renv):
    def apply(x):
        t = np.tensordot(Lenv, x, axes=(0, 0))  # [w, a', s, b]
        t = np.tensordot(t, W, axes=([0, 2], [0, 2]))  # [a', b, o, v]
        return np.tensordot(t, Renv, axes=([1, 3], [0, 1]))  # [a', o, b']
    return apply


def _heff2(Lenv, W1, W2, Renv):
    def apply(x):
        t = np.tensordot(Lenv, x, axes=(0, 0))  # [w, a', s1, s2, c]
        t = np.tensordot(t, W1, axes=([0, 2], [0, 2]))  # [a', s2, c, o1, v]
        t = np.tensordot(t, W2, axes=([4, 1], [0, 2]))  # [a', c, o1, o2, u]
        t = np.tensordot(t, Renv, axes=([1, 4], [0, 1]))  # [a', o1, o2, c']
        return t
    return apply


class _Stop(Exception):
    pass


def dmrg(psi: OMPS, mpo, nsweeps=4, method="dmrg1", maxdim=128, krylovdim=3, maxiter=2, tol=1e-12,
         history=None, limit=None, timing=None):
    """dmrg!(ψ, H; method) (src/Algorithms/DMRG.jl:45-461) on a copy of ψ.

    Dmrg1 (DMRG.jl:45-210): right environments from canonize!(ψ, i), i = n-1…1; each sweep
    optimises sites 2…n left→right then n-1…1 right→left, moving the centre with a QR
    gauge move before the environment update and replacing the site by the Ritz vector.
    Dmrg2 (DMRG.jl:212-459): the pair (i-1, i) [left→right, centre i] or (i, i+1)
    [right→left, centre i] is optimised as one tensor θ, split by a thin SVD, the leading
    min(maxdim, k) values kept and normalised, and S absorbed towards the sweep direction.
    Returns (ψ, energy of the last eigensolve).  ``history`` (a list) receives the energy
    after each half sweep.  ``limit`` stops after that many local updates (a bounded CPU
    sample; ``timing``, a dict, then receives the environment set-up time and the number
    and time of the updates done)."""
    import time as _time

    t_start = _time.perf_counter()
    psi = psi.copy()
    n = psi.L
    one = np.ones((1, 1, 1), dtype=np.complex128)
    envL = {0: one}
    envR = {n: one}
    for i in range(n - 1, 0, -1):
        canonize(psi, MixedCanonical(i))
        envR[i] = _env_right(envR[i + 1], psi.site(i + 1), mpo[i])
    energy = 0.0
    t_env = _time.perf_counter() - t_start
    done = [0]
    lanczos = lanczos_lm

    def lanczos_lm_counted(*a):  # noqa: ANN001
        if limit is not None and done[0] >= limit:
            raise _Stop
        done[0] += 1
        return lanczos(*a)

    try:
        return _dmrg_sweeps(psi, mpo, nsweeps, method, maxdim, krylovdim, maxiter, tol, history, envL, envR,
                            lanczos_lm_counted)
    except _Stop:
        return psi, energy
    finally:
        if timing is not None:
            timing.update({"env_s": t_env, "updates": done[0], "updates_s": _time.perf_counter() - t_start - t_env})


def _dmrg_sweeps(psi, mpo, nsweeps, method, maxdim, krylovdim, maxiter, tol, history, envL, envR, lanczos_lm):
    n = psi.L
    energy = 0.0
    if method == "dmrg1":
        for _ in range(nsweeps):
            for i in range(2, n + 1):
                canonize(psi, MixedCanonical(i))
                envL[i - 1] = _env_left(envL[i - 2], psi.site(i - 1), mpo[i - 2])
                energy, y, _ = lanczos_lm(_heff1(envL[i - 1], mpo[i - 1], envR[i]), psi.site(i), krylovdim, maxiter,
                                          tol)
                psi.set_site(i, y)
            if history is not None:
                history.append(energy)
            for i in range(n - 1, 0, -1):
                canonize(psi, MixedCanonical(i))
                envR[i] = _env_right(envR[i + 1], psi.site(i + 1), mpo[i])
                energy, y, _ = lanczos_lm(_heff1(envL[i - 1], mpo[i - 1], envR[i]), psi.site(i), krylovdim, maxiter,
                                          tol)
                psi.set_site(i, y)
            if history is not None:
                history.append(energy)
        return psi, energy
    if method != "dmrg2":
        raise ValueError(f"unknown DMRG method {method!r}")

    def split(y, absorb_right):
        a, s1, s2, c = y.shape
        U, S, Vh = svd_thin(y.reshape(a * s1, s2 * c))
        keep = min(maxdim, S.size)
        U, S, Vh = U[:, :keep], S[:keep], Vh[:keep]
        S = S / np.linalg.norm(S)
        if absorb_right:
            Vh = S[:, None] * Vh
        else:
            U = U * S[None, :]
        return U.reshape(a, s1, keep), Vh.reshape(keep, s2, c)

    for _ in range(nsweeps):
        for i in range(2, n + 1):
            canonize(psi, MixedCanonical(i))
            if i > 2:
                envL[i - 2] = _env_left(envL[i - 3], psi.site(i - 2), mpo[i - 3])
            theta = np.tensordot(psi.site(i - 1), psi.site(i), axes=(2, 0))
            energy, y, _ = lanczos_lm(_heff2(envL[i - 2], mpo[i - 2], mpo[i - 1], envR[i]), theta, krylovdim, maxiter,
                                      tol)
            A, B = split(y, True)
            psi.set_site(i - 1, A)
            psi.set_site(i, B)
            psi.form = MixedCanonical(i)
        if history is not None:
            history.append(energy)
        for i in range(n - 1, 0, -1):
            canonize(psi, MixedCanonical(i))
            if i < n - 1:
                envR[i + 1] = _env_right(envR[i + 2], psi.site(i + 2), mpo[i + 1])
            theta = np.tensordot(psi.site(i), psi.site(i + 1), axes=(2, 0))
            energy, y, _ = lanczos_lm(_heff2(envL[i - 1], mpo[i - 1], mpo[i], envR[i + 1]), theta, krylovdim, maxiter,
                                      tol)
            A, B = split(y, False)
            psi.set_site(i, A)
            psi.set_site(i + 1, B)
            psi.form = MixedCanonical(i)
        if history is not None:
            history.append(energy)
    return psi, energy
