"""DMRG ground-state search on a device MPS (Tenet.jl src/Algorithms/DMRG.jl) and the Ising
MPO of src/Models/Ising.jl.

``dmrg_(ψ, H, nsweeps; method=Dmrg1())`` runs in place in native code (tn_mps_dmrg) and
returns ``(ψ, energy)`` like the reference's ``dmrg!``; ``dmrg`` works on a copy.  A
batched MPS (``MPS.batched``) runs every instance in lockstep; ``H`` is then one MPO for
all of them or a list of B MPOs (for instance a scan over the field h), and the energies
come back as a length-B array."""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L


class Dmrg1:
    """1-site DMRG (DMRG.jl:45-210): bond dimensions stay as they are."""

    code = 1


class Dmrg2:
    """2-site DMRG (DMRG.jl:212-459): bonds grow up to ``maxdim``."""

    code = 2


def ising_1d_mpo(L_, h, J):
    """ising_1d_mpo(L, h, J) (src/Models/Ising.jl:12-31): H = -J Σ Z_i Z_{i+1} - h Σ X_i,
    sites as (w_l, d_out, d_in, w_r) complex arrays with size-1 open ends."""
    if L_ < 2:
        raise ValueError("the Ising chain needs at least 2 sites")
    Id = np.eye(2)
    sx = np.array([[0.0, 1.0], [1.0, 0.0]])
    sz = np.array([[1.0, 0.0], [0.0, -1.0]])
    W = np.zeros((3, 2, 2, 3), dtype=np.complex128)
    W[0, :, :, 0] = Id
    W[1, :, :, 0] = sz
    W[2, :, :, 0] = -h * sx
    W[2, :, :, 1] = -J * sz
    W[2, :, :, 2] = Id
    return [W[2:3].copy()] + [W.copy() for _ in range(L_ - 2)] + [W[:, :, :, 0:1].copy()]


def _lift(mpo, n, d=None):
    if len(mpo) != n:
        raise ValueError("MPS and MPO must have the same number of sites")
    out = []
    for i, W in enumerate(mpo):
        W = np.asarray(W, dtype=np.complex128)
        if W.ndim == 3:
            W = W[None] if i == 0 else W[..., None]
        if W.ndim == 2:
            W = W[None, :, :, None]
        if W.ndim != 4:
            raise ValueError("MPO sites must be (w_l, d_out, d_in, w_r) arrays")
        if d is not None and (W.shape[1] != d or W.shape[2] != d):
            raise ValueError(f"MPO site {i + 1}: physical dimensions {W.shape[1:3]} differ from the MPS's d = {d}")
        out.append(np.asfortranarray(W))
    return out


def dmrg_(psi, H, nsweeps=4, *, method=Dmrg1, maxdim=128, ishermitian=True, krylovdim=3, maxiter=2, tol=1e-12,
          history=False):
    """dmrg!(ψ, H, nsweeps; method, maxdim, ishermitian, krylovdim, maxiter).  Returns
    (ψ, energy) — energy a float, or a length-B array for a batched MPS — and with
    ``history=True`` also the energies after every half sweep, shape (2·nsweeps, B)."""
    if not ishermitian:
        raise NotImplementedError("only Hermitian Hamiltonians (ishermitian=true, the reference's default)")
    code = method.code if hasattr(method, "code") else {"dmrg1": 1, "dmrg2": 2}[str(method).lower()]
    n, B = psi.nsites, psi.batch
    mpos = H if (len(H) and isinstance(H[0], (list, tuple))) else [H]
    if len(mpos) not in (1, B):
        raise ValueError("give one MPO or one per instance")
    lifted = [_lift(m, n, psi._d) for m in mpos]
    bonds = [a.shape[3] for a in lifted[0][:-1]]
    for m in lifted:
        if [a.shape[3] for a in m[:-1]] != bonds:
            raise ValueError("all MPOs must share their bond dimensions")
        for i, a in enumerate(m):
            if a.shape[0] != (1 if i == 0 else bonds[i - 1]) or a.shape[3] != (1 if i == n - 1 else bonds[i]):
                raise ValueError(f"MPO site {i + 1}: bond dimensions do not chain")
    ptrs = (C.c_void_p * (n * len(lifted)))(*[a.ctypes.data for m in lifted for a in m])
    wb = (C.c_int64 * max(1, n - 1))(*bonds)
    energy = np.zeros(B, dtype=np.float64)
    hist = np.zeros((max(1, 2 * nsweeps), B), dtype=np.float64)
    psi._chk(psi.lib.tn_mps_dmrg(psi.h, ptrs, wb, len(lifted), code, int(nsweeps), int(maxdim or 0), int(krylovdim),
                                 int(maxiter), float(tol), energy.ctypes.data_as(L._pdbl),
                                 hist.ctypes.data_as(L._pdbl) if history else None))
    e = energy[0] if B == 1 else energy
    if history:
        h = hist[: 2 * nsweeps]
        return psi, e, (h[:, 0] if B == 1 else h)
    return psi, e


def dmrg(psi, H, nsweeps=4, **kw):
    """dmrg(ψ, H, …) = dmrg!(copy(ψ), H, …) (DMRG.jl:41)."""
    return dmrg_(psi.copy(), H, nsweeps, **kw)


def last_stats(ctx=None):
    """Device time (ms) of the last DMRG run per phase — gauge moves, environments,
    eigensolves, pair splits — and the number of local updates (tn_dmrg_last_stats)."""
    from .core import default_context

    ctx = ctx or default_context()
    ms = np.zeros(4, dtype=np.float64)
    n = (C.c_int64 * 2)()
    ctx.check(ctx.lib.tn_dmrg_last_stats(ctx.h, ms.ctypes.data_as(L._pdbl), n))
    return {"canonize_ms": ms[0], "environments_ms": ms[1], "eigsolve_ms": ms[2], "split_ms": ms[3],
            "updates": n[0], "svd_sweeps": n[1]}
