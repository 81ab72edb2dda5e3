"""Grouped (ragged) MPS batches: the host face of tn_group_* (include/tenet_gb300.h).

``MPSGroup`` holds B independent MPS of different lengths and bond dimensions on the
device.  ``canonize_compress_norm(maxdim)`` runs, for every instance, the reference's
canonize!(ψ, MixedCanonical(L)) → compress!(ψ; maxdim) → norm(ψ)
(src/Operations/canonize.jl:121-252, compress.jl:21-69, norm.jl:31-34) as grouped
launches: each step of the three sweeps is one launch per kernel over all instances.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .core import default_context
from .workloads import clamped_bonds


class MPSGroup:
    def __init__(self, Ls, bonds, d=2, ctx=None):
        """``bonds[b]``: the L_b − 1 inner bond dimensions of instance b."""
        self.ctx = ctx or default_context()
        self.lib = self.ctx.lib
        self.L = [int(x) for x in Ls]
        self.d = int(d)
        flat = [int(x) for bl in bonds for x in bl]
        h = C.c_void_p()
        self.ctx.check(self.lib.tn_group_create(self.ctx.h, len(self.L), (C.c_int32 * len(self.L))(*self.L), self.d,
                                                (C.c_int64 * max(1, len(flat)))(*flat), C.byref(h)))
        self.h = h

    @classmethod
    def random(cls, Ls, chis, d=2, seed=0, ctx=None):
        """Gaussian MPS generated on the device (entries of variance 1/(d χ_{i-1})), bonds
        clamped like rand(MPS) (src/Components/MPS.jl:122-152)."""
        g = cls(Ls, [clamped_bonds(L, d, chi) for L, chi in zip(Ls, chis)], d=d, ctx=ctx)
        g.ctx.check(g.lib.tn_group_fill_random(g.h, int(seed)))
        return g

    @classmethod
    def from_arrays(cls, instances, ctx=None):
        """``instances[b]``: list of site arrays (χl, d, χr)."""
        Ls = [len(s) for s in instances]
        bonds = [[a.shape[2] for a in s[:-1]] for s in instances]
        g = cls(Ls, bonds, d=instances[0][0].shape[1], ctx=ctx)
        for b, sites in enumerate(instances):
            for i, a in enumerate(sites):
                a = np.asfortranarray(np.asarray(a, np.complex128))
                g.ctx.check(g.lib.tn_group_set_site(g.h, b, i + 1, a.ctypes.data))
        return g

    @property
    def B(self):
        return len(self.L)

    def bond_dims(self, b):
        out = (C.c_int64 * max(1, self.L[b] - 1))()
        self.ctx.check(self.lib.tn_group_bond_dims(self.h, b, out))
        return list(out)[: self.L[b] - 1]

    def sites(self, b):
        bd = [1] + self.bond_dims(b) + [1]
        out = []
        for i in range(self.L[b]):
            a = np.empty((bd[i], self.d, bd[i + 1]), np.complex128, order="F")
            self.ctx.check(self.lib.tn_group_get_site(self.h, b, i + 1, a.ctypes.data))
            out.append(np.ascontiguousarray(a))
        return out

    def canonize_compress_norm(self, maxdim):
        """maxdim: one int or one per instance.  Returns norm(ψ_b) for every b."""
        md = np.broadcast_to(np.asarray(maxdim, dtype=np.int64), (self.B,)).copy()
        out = np.zeros(self.B)
        self.ctx.check(self.lib.tn_group_canonize_compress_norm(
            self.h, md.ctypes.data_as(C.POINTER(C.c_int64)), out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def lambda_(self, b):
        n = C.c_int64()
        self.ctx.check(self.lib.tn_group_lambda(self.h, b, None, C.byref(n)))
        out = np.zeros(n.value)
        self.ctx.check(self.lib.tn_group_lambda(self.h, b, out.ctypes.data_as(C.POINTER(C.c_double)), C.byref(n)))
        return out

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value and not _lib.shutting_down():
            self.lib.tn_group_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
