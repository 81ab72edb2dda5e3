"""Device-resident MPS with Tenet's MPS API (src/Components/MPS.jl, src/Operations/*).

Julia's in-place ``f!`` maps to ``f_`` here (``canonize_``, ``compress_``,
``simple_update_``, ``normalize_``); the non-mutating forms copy first, as Tenet's
``canonize(tn, …) = canonize!(copy(tn), …)`` does (src/Operations/canonize.jl:13).

The sites stay in HBM inside a native ``tn_mps`` handle; the canonical-form trait
(src/CanonicalForm.jl) is tracked in native code and mirrored by the form classes below.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .core import Context, default_context, precision_code


class NonCanonical:
    def __eq__(self, o):
        return isinstance(o, NonCanonical)

    def __repr__(self):
        return "NonCanonical()"


class MixedCanonical:
    """MixedCanonical(orthog_center): sites lo..hi (1-based)."""

    def __init__(self, sites):
        if isinstance(sites, (int, np.integer)):
            sites = [int(sites)]
        self.sites = sorted(set(int(s) for s in sites))

    @property
    def lo(self):
        return self.sites[0]

    @property
    def hi(self):
        return self.sites[-1]

    def __eq__(self, o):
        return isinstance(o, MixedCanonical) and (o.lo, o.hi) == (self.lo, self.hi)

    def __repr__(self):
        return f"MixedCanonical({self.sites})"


class BondCanonical:
    """BondCanonical(bond"a-b") with b = a + 1; Λ stored at LambdaSite(bond)."""

    def __init__(self, a, b=None):
        if b is None:
            a, b = a
        self.a, self.b = min(a, b), max(a, b)

    def __eq__(self, o):
        return isinstance(o, BondCanonical) and (o.a, o.b) == (self.a, self.b)

    def __repr__(self):
        return f"BondCanonical({self.a}-{self.b})"


def _as_form(f):
    if isinstance(f, (NonCanonical, MixedCanonical, BondCanonical)):
        return f
    if isinstance(f, (int, np.integer, list)):
        return MixedCanonical(f)
    if isinstance(f, tuple) and len(f) == 2:
        return BondCanonical(f)
    raise ValueError(f"not a canonical form: {f!r}")


def _sites_from_arrays(arrays, order=("l", "r", "o")):
    """MPS(arrays; order) (src/Components/MPS.jl:50-94) → 3-D (χl, d, χr) sites."""
    order = tuple(order)
    if sorted(order) != ["l", "o", "r"]:
        raise ValueError("order must be a permutation of (:l, :r, :o)")
    n = len(arrays)
    if n < 2:
        raise ValueError("an MPS needs at least 2 sites")
    out = []
    for i, a in enumerate(arrays):
        a = np.asarray(a)
        if i == 0:
            lo = tuple(x for x in order if x != "l")
            if a.ndim != 2:
                raise ValueError("First array must have 2 dimensions")
            t = np.moveaxis(a, [lo.index("o"), lo.index("r")], [0, 1])[None]
        elif i == n - 1:
            lo = tuple(x for x in order if x != "r")
            if a.ndim != 2:
                raise ValueError("Last array must have 2 dimensions")
            t = np.moveaxis(a, [lo.index("l"), lo.index("o")], [0, 1])[:, :, None]
        else:
            if a.ndim != 3:
                raise ValueError("All arrays must have 3 dimensions")
            t = np.moveaxis(a, [order.index("l"), order.index("o"), order.index("r")], [0, 1, 2])
        out.append(t.astype(np.complex128))
    return out


class MPS:
    """MatrixProductState on one GB300.  ``sites`` are (χl, d, χr) arrays (C-ordered
    numpy accepted; any memory order is fine).

    ``MPS.batched([sites_0, sites_1, …])`` holds B instances with equal bond dimensions
    that every operation advances in lockstep (one batched launch per kernel); values
    that are scalars for one MPS (overlap, norm, amplitude) become length-B arrays."""

    def __init__(self, sites=None, *, arrays=None, order=("l", "r", "o"), ctx: Context | None = None,
                 max_bond=0, precision="native", _handle=None, _instances=None):
        self.ctx = ctx or default_context()
        self.lib = self.ctx.lib
        if _handle is not None:
            self.h = _handle
            return
        if arrays is not None:
            sites = _sites_from_arrays(arrays, order)
        instances = _instances if _instances is not None else [sites]
        instances = [[np.asarray(s, dtype=np.complex128) for s in inst] for inst in instances]
        sites = instances[0]
        L_ = len(sites)
        d = sites[0].shape[1]
        bonds = [s.shape[2] for s in sites[:-1]]
        for inst in instances:
            if len(inst) != L_ or [s.shape for s in inst] != [s.shape for s in sites]:
                raise ValueError("batched MPS instances must have identical shapes")
        for i in range(L_ - 1):
            if sites[i].shape[2] != sites[i + 1].shape[0]:
                raise ValueError(f"bond {i + 1}-{i + 2}: dims differ")
        if any(s.ndim != 3 or s.shape[1] != d for s in sites):
            raise ValueError("every site must be a (χl, d, χr) array with the same physical dimension d")
        if sites[0].shape[0] != 1 or sites[-1].shape[2] != 1:
            raise ValueError("open boundary: end sites must have a size-1 outer bond")
        h = C.c_void_p()
        b = (C.c_int64 * (L_ - 1))(*bonds)
        self.ctx.check(self.lib.tn_mps_create_batched(self.ctx.h, len(instances), L_, d, b, int(max_bond),
                                                      precision_code(precision), C.byref(h)))
        self.h = h
        for bi, inst in enumerate(instances):
            fs = [np.asfortranarray(s) for s in inst]
            ptrs = (C.c_void_p * L_)(*[f.ctypes.data for f in fs])
            self.ctx.check(self.lib.tn_mps_set_instance_sites(self.h, bi, ptrs))
        self._L, self._d = L_, d

    @classmethod
    def batched(cls, instances, **kw):
        return cls(_instances=list(instances), **kw)

    @property
    def batch(self):
        v = C.c_int32()
        self._chk(self.lib.tn_mps_batch_size(self.h, C.byref(v)))
        return v.value

    def _one(self, arr):
        return arr[0] if self.batch == 1 else arr

    # -- bookkeeping -----------------------------------------------------------
    def __del__(self):
        if L.shutting_down():
            return
        try:
            if getattr(self, "h", None):
                self.lib.tn_mps_destroy(self.h)
                self.h = None
        except Exception:
            pass

    def _chk(self, st):
        self.ctx.check(st)

    @property
    def nsites(self):
        return len(self.bondsizes()) + 1

    def bondsizes(self):
        n = self._L - 1
        out = (C.c_int64 * n)()
        self._chk(self.lib.tn_mps_bond_dims(self.h, out))
        return list(out)

    def maxbondsize(self):
        return max(self.bondsizes())

    @property
    def form(self):
        k, lo, hi = C.c_int32(), C.c_int32(), C.c_int32()
        self._chk(self.lib.tn_mps_form(self.h, C.byref(k), C.byref(lo), C.byref(hi)))
        if k.value == L.TN_FORM_NONCANONICAL:
            return NonCanonical()
        if k.value == L.TN_FORM_MIXED:
            return MixedCanonical(list(range(lo.value, hi.value + 1)))
        return BondCanonical(lo.value, hi.value)

    def unsafe_setform_(self, form):
        form = _as_form(form)
        if isinstance(form, NonCanonical):
            self._chk(self.lib.tn_mps_set_form(self.h, L.TN_FORM_NONCANONICAL, 0, 0))
        elif isinstance(form, MixedCanonical):
            self._chk(self.lib.tn_mps_set_form(self.h, L.TN_FORM_MIXED, form.lo, form.hi))
        else:
            raise ValueError("only NonCanonical / MixedCanonical can be set without computation")
        return self

    def set_precision(self, precision):
        self._chk(self.lib.tn_mps_set_precision(self.h, precision_code(precision)))

    def copy(self):
        h = C.c_void_p()
        self._chk(self.lib.tn_mps_copy(self.h, C.byref(h)))
        m = MPS(ctx=self.ctx, _handle=h)
        m._L, m._d = self._L, self._d
        return m

    def save(self, path):
        """Dump all instances, the form and Λ to a raw file (tn_mps_save)."""
        self._chk(self.lib.tn_mps_save(self.h, str(path).encode()))

    @classmethod
    def load(cls, path, ctx=None, max_bond=0):
        """An MPS dumped by ``save`` back on the device (tn_mps_load)."""
        ctx = ctx or default_context()
        h = C.c_void_p()
        ctx.check(ctx.lib.tn_mps_load(ctx.h, str(path).encode(), int(max_bond), C.byref(h)))
        m = MPS(ctx=ctx, _handle=h)
        Lc, dc = C.c_int32(), C.c_int32()
        ctx.check(ctx.lib.tn_mps_shape(h, C.byref(Lc), C.byref(dc), None))
        m._L, m._d = Lc.value, dc.value
        return m

    def site(self, i, instance=0, out=None):
        """Site tensor i (1-based) as a (χl, d, χr) numpy array.  ``out``: a flat complex128
        buffer of at least χl·d·χr elements (e.g. page-locked host memory) to copy into;
        the returned array is then a column-major view of it."""
        b = [1] + self.bondsizes() + [1]
        shape = (b[i - 1], self._d, b[i])
        size = int(np.prod(shape))
        if out is None:
            buf = np.empty(size, dtype=np.complex128)
        else:
            if out.dtype != np.complex128 or out.ndim != 1 or out.size < size or not out.flags.c_contiguous:
                raise ValueError("out must be a contiguous 1-D complex128 buffer large enough for the site")
            buf = out[:size]
        self._chk(self.lib.tn_mps_get_instance_site(self.h, instance, i, buf.ctypes.data_as(C.c_void_p)))
        return buf.reshape(shape, order="F")

    def sites(self, instance=0, out=None):
        """All site tensors of one instance, copied in one call; ``out``: a list of flat
        complex128 buffers (one per site, e.g. page-locked) to copy into."""
        b = [1] + self.bondsizes() + [1]
        shapes = [(b[i - 1], self._d, b[i]) for i in range(1, self._L + 1)]
        bufs = []
        for k, shp in enumerate(shapes):
            size = int(np.prod(shp))
            if out is None:
                bufs.append(np.empty(size, dtype=np.complex128))
            else:
                o = out[k]
                if o.dtype != np.complex128 or o.ndim != 1 or o.size < size or not o.flags.c_contiguous:
                    raise ValueError("each out buffer must be a contiguous 1-D complex128 array large enough")
                bufs.append(o[:size])
        ptrs = (C.c_void_p * self._L)(*[x.ctypes.data for x in bufs])
        self._chk(self.lib.tn_mps_get_instance_sites(self.h, instance, ptrs))
        return [x.reshape(shp, order="F") for x, shp in zip(bufs, shapes)]

    def lambda_(self):
        """Λ at the bond-canonical centre (LambdaSite(bond)); (B, χ) when batched."""
        n = C.c_int64()
        self._chk(self.lib.tn_mps_get_lambda(self.h, None, C.byref(n)))
        out = np.empty((self.batch, n.value), dtype=np.float64)
        self._chk(self.lib.tn_mps_get_lambda(self.h, out.ctypes.data_as(C.POINTER(C.c_double)), C.byref(n)))
        return self._one(out)

    # -- Tenet operations --------------------------------------------------------
    def canonize_(self, form):
        """canonize!(ψ, form)."""
        form = _as_form(form)
        if isinstance(form, NonCanonical):
            return self.unsafe_setform_(form)
        if isinstance(form, MixedCanonical):
            self._chk(self.lib.tn_mps_canonize_mixed(self.h, form.lo, form.hi))
        else:
            self._chk(self.lib.tn_mps_canonize_bond(self.h, form.a))
        return self

    def compress_(self, bond=None, maxdim=None, threshold=None):
        """compress!(ψ[, bond]; maxdim, threshold) ≡ truncate! (compress.jl:18-69)."""
        if maxdim is None and threshold is None:
            raise ValueError("Either `maxdim` or `threshold` must be specified")
        if maxdim is not None and maxdim <= 0:
            raise ValueError("maxdim must be a positive integer")
        if threshold is not None and threshold <= 0:
            raise ValueError("Threshold must be positive")
        a = 0 if bond is None else min(bond)
        self._chk(self.lib.tn_mps_compress(self.h, a, -1 if maxdim is None else int(maxdim),
                                           -1.0 if threshold is None else float(threshold)))
        return self

    truncate_ = compress_

    def simple_update_(self, op, sites, maxdim=None, threshold=None):
        """simple_update!(ψ, op; maxdim) on the given 1-based sites; a 2-site op has
        index order [plug a, plug b, plug a', plug b'] (a < b adjacent)."""
        sites = sorted(int(s) for s in np.atleast_1d(sites))
        op = np.asfortranarray(np.asarray(op, dtype=np.complex128))
        if len(sites) not in (1, 2):
            raise ValueError("Operator must act on one or two sites")
        if len(sites) == 2 and sites[1] != sites[0] + 1:
            raise ValueError("2-site gates must act on adjacent sites")
        # the library reads d^(2·nsites) entries from the host array
        if op.size != self._d ** (2 * len(sites)):
            raise ValueError(f"a {len(sites)}-site operator on sites of dimension {self._d} has "
                             f"{self._d ** (2 * len(sites))} entries, got shape {op.shape}")
        self._chk(self.lib.tn_mps_simple_update(self.h, len(sites), sites[0], op.ctypes.data_as(C.c_void_p),
                                                -1 if maxdim is None else int(maxdim),
                                                -1.0 if threshold is None else float(threshold)))
        return self

    def evolve_(self, op, sites):
        """evolve!(ψ, gate) → simple_update! without keyword arguments (evolve.jl:140-143)."""
        return self.simple_update_(op, sites)

    def evolve_brickwork_(self, layers, maxdim=None, threshold=None):
        """Apply brickwork layers in one library call.  A layer is (start_bond, [G, …]) —
        gates on bonds start, start+2, … applied left to right — or (start_bond, [G, …],
        reverse) with reverse true for right to left (the gates still listed left to
        right)."""
        starts = (C.c_int32 * len(layers))(*[int(ly[0]) for ly in layers])
        counts = (C.c_int32 * len(layers))(*[len(ly[1]) for ly in layers])
        rev = (C.c_int32 * len(layers))(*[int(bool(ly[2])) if len(ly) > 2 else 0 for ly in layers])
        flat = [np.asfortranarray(np.asarray(G, dtype=np.complex128)).reshape(-1, order="F") for ly in layers
                for G in ly[1]]
        for G in flat:  # the library reads d⁴ entries per gate
            if G.size != self._d ** 4:
                raise ValueError(f"a two-site gate on sites of dimension {self._d} has {self._d ** 4} entries, "
                                 f"got {G.size}")
        buf = np.ascontiguousarray(np.concatenate(flat)) if flat else np.zeros(1, np.complex128)
        self._chk(self.lib.tn_mps_evolve_layers(self.h, len(layers), starts, counts, rev,
                                                buf.ctypes.data_as(C.c_void_p),
                                                -1 if maxdim is None else int(maxdim),
                                                -1.0 if threshold is None else float(threshold)))
        return self

    def norm(self):
        """norm(ψ) (norm.jl:17-37); moves the orthogonality centre like the reference."""
        v = np.empty(self.batch, dtype=np.float64)
        self._chk(self.lib.tn_mps_norm(self.h, v.ctypes.data_as(C.POINTER(C.c_double))))
        return float(v[0]) if self.batch == 1 else v

    def normalize_(self):
        self._chk(self.lib.tn_mps_normalize(self.h))
        return self

    def overlap(self, other: "MPS"):
        """overlap(self, other) = ⟨other|self⟩ (overlap.jl:36-50)."""
        out = np.empty(2 * self.batch, dtype=np.float64)
        self._chk(self.lib.tn_mps_overlap(self.h, other.h, out.ctypes.data_as(C.POINTER(C.c_double))))
        v = out[0::2] + 1j * out[1::2]
        return complex(v[0]) if self.batch == 1 else v

    def amplitude(self, bits):
        """overlap(ProductState(bits), ψ) (overlap.jl:22-32); ``bits`` is a string of
        0/1/+/-/u/d or a list of length-d vectors."""
        if isinstance(bits, str):
            vecs = _product_vectors(bits)
        else:
            vecs = [np.asarray(v, dtype=np.complex128) for v in bits]
        if len(vecs) != self._L or any(x.shape != (self._d,) for x in vecs):
            raise ValueError(f"a product state of {self._L} vectors of length {self._d} is needed")
        v = np.ascontiguousarray(np.stack(vecs))
        out = np.empty(2 * self.batch, dtype=np.float64)
        self._chk(self.lib.tn_mps_amplitude(self.h, v.ctypes.data_as(C.c_void_p), out.ctypes.data_as(C.POINTER(C.c_double))))
        a = out[0::2] + 1j * out[1::2]
        return complex(a[0]) if self.batch == 1 else a

    def local_expectations(self, op):
        """⟨ψ|O_i|ψ⟩/⟨ψ|ψ⟩ for every site i."""
        o = np.asfortranarray(np.asarray(op, dtype=np.complex128))
        if o.shape != (self._d, self._d):
            raise ValueError(f"a one-site operator is {self._d}×{self._d}, got shape {o.shape}")
        out = np.empty(2 * self._L * self.batch, dtype=np.float64)
        self._chk(self.lib.tn_mps_local_expectations(self.h, o.ctypes.data_as(C.c_void_p),
                                                     out.ctypes.data_as(C.POINTER(C.c_double))))
        z = (out[0::2] + 1j * out[1::2]).reshape(self.batch, self._L)
        return z[0] if self.batch == 1 else z


def _product_vectors(bits):
    s = 1 / np.sqrt(2)
    table = {"0": [1, 0], "1": [0, 1], "+": [s, s], "-": [s, -s], "u": [s, -1j * s], "↑": [s, -1j * s],
             "d": [-s, -1j * s], "↓": [-s, -1j * s]}
    out = []
    for c in bits:
        if c not in table:
            raise ValueError(f"invalid character: {c}")
        out.append(np.asarray(table[c], dtype=np.complex128))
    return out


# module-level Tenet-style functions -------------------------------------------------
def canonize_(psi, form):
    return psi.canonize_(form)


def canonize(psi, form):
    return psi.copy().canonize_(form)


def compress_(psi, bond=None, **kw):
    return psi.compress_(bond, **kw)


def compress(psi, bond=None, **kw):
    return psi.copy().compress_(bond, **kw)


truncate_ = compress_
truncate = compress


def simple_update_(psi, op, sites, **kw):
    return psi.simple_update_(op, sites, **kw)


def evolve_(psi, op, sites):
    return psi.evolve_(op, sites)


def overlap(a, b):
    return a.overlap(b)


def norm(psi):
    return psi.norm()


def normalize_(psi):
    return psi.normalize_()


def normalize(psi):
    return psi.copy().normalize_()


# ----------------------------------------------------------------------------------
# sampling and Schmidt values (src/Operations/sample.jl:20-72, entropy.jl:25-67)
# ----------------------------------------------------------------------------------
def sample(psi, nsamples=1, seed=None, uniforms=None, instance=0):
    """sample(ψ, nsamples): ``nsamples`` bit strings as lists of 1-based outcomes, drawn
    on the device site by site from the marginals of ψ (moved to MixedCanonical(1) on a
    copy, as the reference does).  ``uniforms`` (nsamples × L in [0, 1)) replaces the
    reference's RNG; by default they come from numpy's default_rng(seed)."""
    L = psi.nsites
    if uniforms is None:
        uniforms = np.random.default_rng(seed).random((nsamples, L))
    u = np.ascontiguousarray(uniforms, dtype=np.float64)
    if u.shape != (nsamples, L):
        raise ValueError(f"uniforms must have shape ({nsamples}, {L})")
    out = np.zeros((nsamples, L), np.int32)
    tmp = psi.copy()
    tmp._chk(tmp.lib.tn_mps_sample(tmp.h, int(instance), int(nsamples), u.ctypes.data_as(C.POINTER(C.c_double)),
                                   out.ctypes.data_as(C.POINTER(C.c_int32))))
    return [list(map(int, row)) for row in out]


def schmidt_values_(psi, bond):
    """schmidt_values!(ψ, bond): canonize!(ψ, BondCanonical(bond)), then Λ."""
    a, b = (bond, bond + 1) if isinstance(bond, (int, np.integer)) else tuple(sorted(bond))
    psi.canonize_(BondCanonical(a, b))
    return psi.lambda_()


def schmidt_values(psi, bond):
    return schmidt_values_(psi.copy(), bond)


def entropy_vonneumann_(psi, bond=None):
    """entropy_vonneumann!(ψ[, bond]) = −Σ x² · 2 log(x) over the Schmidt values, per
    bond 1..L−1 when no bond is given (entropy.jl:25-35); the MPS should be normalised."""
    if bond is not None:
        x = np.asarray(schmidt_values_(psi, bond), dtype=np.float64)
        with np.errstate(divide="ignore", invalid="ignore"):
            return float(-np.sum(x**2 * 2 * np.log(x)))
    return np.array([entropy_vonneumann_(psi, i) for i in range(1, psi.nsites)])


def entropy_vonneumann(psi, bond=None):
    return entropy_vonneumann_(psi.copy(), bond)


# ----------------------------------------------------------------------------------
# MPO × MPS evolution (src/Operations/evolve.jl:19-137)
# ----------------------------------------------------------------------------------
def evolve_mpo_(psi, mpo, algorithm="direct", maxdim=None, threshold=None):
    """evolve!(ψ, op::MPO): ``mpo`` is a list of site arrays (w_l, d_out, d_in, w_r) (2-D
    or 3-D boundary sites are lifted).  ``algorithm`` "direct" (the reference's
    evolve!(::MPS, ::MPO): exact, bonds multiply, MixedCanonical(all)) or "zipup"
    (generic_evolve_mps_mpo_zipup!, truncated to maxdim / threshold)."""
    L = psi.nsites
    if len(mpo) != L:
        raise ValueError("MPS and MPO must have the same number of sites")
    arrs = []
    for i, W in enumerate(mpo):
        W = np.asarray(W, dtype=np.complex128)
        if W.ndim == 3:
            W = W[None] if i == 0 else W[..., None]
        if W.ndim == 2:
            W = W[None, :, :, None]
        if W.ndim != 4 or W.shape[1] != psi._d or W.shape[2] != psi._d:
            raise ValueError(f"MPO site {i + 1}: expected (w_l, {psi._d}, {psi._d}, w_r), got {W.shape}")
        # the library reads w_{i-1}·d·d·w_i entries per site, w_0 = w_L = 1
        w_left = 1 if i == 0 else arrs[-1].shape[3]
        if W.shape[0] != w_left or (i == L - 1 and W.shape[3] != 1):
            raise ValueError(f"MPO site {i + 1}: virtual dimensions {W.shape[0]}, {W.shape[3]} do not chain "
                             f"(left neighbour {w_left}, open ends 1)")
        arrs.append(np.asfortranarray(W))
    wb = (C.c_int64 * max(1, L - 1))(*[a.shape[3] for a in arrs[:-1]])
    ptrs = (C.c_void_p * L)(*[a.ctypes.data for a in arrs])
    alg = {"direct": 0, "zipup": 1}[algorithm]
    psi._chk(psi.lib.tn_mps_evolve_mpo(psi.h, ptrs, wb, alg, int(maxdim or 0), float(threshold or 0.0)))
    return psi


def evolve_mpo(psi, mpo, **kw):
    return evolve_mpo_(psi.copy(), mpo, **kw)
