"""Device-resident MPO with Tenet's MPO API for the gauge path (src/Components/MPO.jl,
src/Operations/canonize.jl, compress.jl): ``canonize!`` / ``compress!`` on an MPO keep its
two plugs (o, i) together on the physical side of every factorisation, so an MPO is held
as an MPS whose physical index fuses (o, i) column-major (o fastest) and every gauge move
is the MPS's.  ``arrays()`` returns the (w_l, d_out, d_in, w_r) site arrays that
``evolve_mpo_`` and ``dmrg_`` take."""

from __future__ import annotations

import numpy as np

from .core import Context
from .mps import MPS


def _mpo_sites(arrays, order):
    """MPO(arrays; order) (MPO.jl:85-125) → (χl, d_o, d_i, χr) sites."""
    order = tuple(order)
    if sorted(order) != ["i", "l", "o", "r"]:
        raise ValueError("order must be a permutation of (:l, :r, :o, :i)")
    n = len(arrays)
    if n < 2:
        raise ValueError("an MPO needs at least 2 sites")
    out = []
    for k, a in enumerate(arrays):
        a = np.asarray(a)
        own = tuple(x for x in order if not ((k == 0 and x == "l") or (k == n - 1 and x == "r")))
        if a.ndim != len(own):
            raise ValueError(f"site {k + 1}: expected {len(own)} dimensions, got {a.ndim}")
        src = [own.index(x) for x in ("o", "i")] + [own.index(x) for x in ("l", "r") if x in own]
        t = np.moveaxis(a, src, list(range(len(own))))
        o, i = t.shape[0], t.shape[1]
        l = t.shape[2] if "l" in own else 1
        r = t.shape[-1] if "r" in own else 1
        out.append(np.transpose(t.reshape(o, i, l, r), (2, 0, 1, 3)).astype(np.complex128))
    return out


class MPO:
    """MatrixProductOperator on one GB300 for canonize! / compress! / truncate!.  ``sites``
    are (χl, d_out, d_in, χr) arrays; ``arrays=`` with ``order`` follows Tenet's
    ``MPO(arrays; order)`` (default (:l, :r, :o, :i))."""

    def __init__(self, sites=None, *, arrays=None, order=("l", "r", "o", "i"), ctx: Context | None = None,
                 max_bond=0, precision="native", _mps=None, _phys=None):
        if _mps is not None:
            self.mps, self.phys = _mps, list(_phys)
            return
        if arrays is not None:
            sites = _mpo_sites(arrays, order)
        sites = [np.asarray(s, dtype=np.complex128) for s in sites]
        if any(s.ndim != 4 for s in sites):
            raise ValueError("MPO sites must be (χl, d_out, d_in, χr) arrays")
        self.phys = [(s.shape[1], s.shape[2]) for s in sites]
        if len(set(o * i for o, i in self.phys)) != 1:
            raise ValueError("every site needs the same d_out·d_in")
        fused = [s.reshape(s.shape[0], s.shape[1] * s.shape[2], s.shape[3], order="F") for s in sites]
        self.mps = MPS(fused, ctx=ctx, max_bond=max_bond, precision=precision)

    # -- views ---------------------------------------------------------------------
    @property
    def nsites(self):
        return self.mps.nsites

    def bondsizes(self):
        return self.mps.bondsizes()

    @property
    def form(self):
        return self.mps.form

    def site(self, i):
        """Site i (1-based) as a (χl, d_out, d_in, χr) array."""
        f = self.mps.site(i)
        o, ii = self.phys[i - 1]
        return f.reshape(f.shape[0], o, ii, f.shape[2], order="F")

    def sites(self):
        return [self.site(i) for i in range(1, self.nsites + 1)]

    def arrays(self):
        """The (w_l, d_out, d_in, w_r) site arrays (for evolve_mpo_ / dmrg_)."""
        return self.sites()

    def copy(self):
        return MPO(_mps=self.mps.copy(), _phys=self.phys)

    # -- Tenet operations ----------------------------------------------------------
    def canonize_(self, form):
        """canonize!(H, form): MixedCanonical / BondCanonical as for an MPS."""
        self.mps.canonize_(form)
        return self

    def compress_(self, bond=None, maxdim=None, threshold=None):
        """compress!(H; maxdim, threshold) on one bond or all of them."""
        self.mps.compress_(bond=bond, maxdim=maxdim, threshold=threshold)
        return self

    def lambda_(self):
        return self.mps.lambda_()


def canonize(H, form):
    return H.copy().canonize_(form)


def compress(H, bond=None, **kw):
    return H.copy().compress_(bond=bond, **kw)
