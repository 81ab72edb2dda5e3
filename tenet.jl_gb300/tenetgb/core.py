"""Context, device tensors and the Muscle-level operations on GB300.

Tenet.jl never computes: it calls Muscle.jl on labelled ``Tensor`` values.  This module
is the Python mirror of those calls, backed by libtenetgb.so:

=========================  ===============================================  ==================
Muscle / Tenet call        reference call site                              here
=========================  ===============================================  ==================
binary_einsum(a, b; dims)  src/Operations/canonize.jl:44,47,61,100          binary_einsum
tensor_qr_thin             src/Operations/canonize.jl:58                     tensor_qr_thin
tensor_svd_thin            src/Operations/canonize.jl:41,97                  tensor_svd_thin
hadamard                   src/Operations/canonize.jl:198,209                hadamard
simple_update              src/Operations/simple_update.jl:53-64             simple_update
LinearAlgebra.norm         src/Operations/norm.jl:27,33                      norm
=========================  ===============================================  ==================

A :class:`DeviceTensor` is a dense column-major (Julia-layout) device array with one
label per mode — the GB300 counterpart of ``Tangles.Tensor{T,N,GB300Array}``.
"""

from __future__ import annotations

import ctypes as C
import itertools

import numpy as np

from . import _lib as L

_DT = {
    np.dtype(np.complex128): L.TN_C64,
    np.dtype(np.complex64): L.TN_C32,
    np.dtype(np.float64): L.TN_F64,
    np.dtype(np.float32): L.TN_F32,
}
_PREC = {"native": L.TN_PREC_NATIVE, "fp64": L.TN_PREC_NATIVE, "fp32": L.TN_PREC_NATIVE, "mixed": L.TN_PREC_MIXED,
         "3xtf32": L.TN_PREC_MIXED, "tf32": L.TN_PREC_TF32, "split_bf16": L.TN_PREC_SPLIT_BF16}


def precision_code(p):
    if isinstance(p, int):
        return p
    try:
        return _PREC[p]
    except KeyError:
        raise ValueError(f"unknown precision {p!r}; use 'native', 'mixed' or 'split_bf16'") from None


class Context:
    """One library context = one device + one stream (tn_create)."""

    def __init__(self, device=0):
        self.lib = L.load()
        h = C.c_void_p()
        st = self.lib.tn_create(C.byref(h), int(device))
        L.check(st, None)
        self.h = h
        self.device = device

    def close(self):
        if getattr(self, "h", None):
            self.lib.tn_destroy(self.h)
            self.h = None

    def __del__(self):
        if L.shutting_down():
            return
        try:
            self.close()
        except Exception:
            pass

    def check(self, st):
        L.check(st, self.h)

    def sync(self):
        self.check(self.lib.tn_sync(self.h))

    def set_stream(self, stream_handle):
        self.check(self.lib.tn_set_stream(self.h, C.c_void_p(stream_handle)))

    @property
    def stream(self):
        return self.lib.tn_get_stream(self.h)

    def alloc(self, nbytes):
        p = C.c_void_p()
        self.check(self.lib.tn_alloc(self.h, C.c_size_t(max(int(nbytes), 1)), C.byref(p)))
        return p.value

    def free(self, ptr):
        if ptr:
            self.check(self.lib.tn_free(self.h, C.c_void_p(ptr)))

    def h2d(self, dst, arr):
        arr = np.asarray(arr)
        self.check(self.lib.tn_memcpy_h2d(self.h, C.c_void_p(dst), arr.ctypes.data_as(C.c_void_p), arr.nbytes))

    def d2h(self, arr, src):
        self.check(self.lib.tn_memcpy_d2h(self.h, arr.ctypes.data_as(C.c_void_p), C.c_void_p(src), arr.nbytes))

    def set_hbm_budget(self, nbytes):
        self.check(self.lib.tn_set_hbm_budget(self.h, C.c_size_t(int(nbytes))))

    def hbm_in_use(self):
        v = C.c_size_t()
        self.check(self.lib.tn_hbm_in_use(self.h, C.byref(v)))
        return v.value

    def set_autotune(self, enable=True):
        """Time candidate launch configurations on the first call of each new shape and
        keep the fastest (per context)."""
        self.check(self.lib.tn_set_autotune(self.h, int(bool(enable))))

    def tuning(self):
        """The autotuner's table as text (one "key v1 v2" line per shape)."""
        n = C.c_size_t()
        self.check(self.lib.tn_tuning_dump(self.h, None, 0, C.byref(n)))
        buf = C.create_string_buffer(n.value)
        self.check(self.lib.tn_tuning_dump(self.h, buf, n.value, None))
        return buf.value.decode()

    def load_tuning(self, text):
        self.check(self.lib.tn_tuning_load(self.h, text.encode()))

    def save_tuning(self, path):
        with open(path, "w") as f:
            f.write(self.tuning())

    def launches(self):
        v = C.c_int64()
        self.check(self.lib.tn_kernel_launches(self.h, C.byref(v)))
        return v.value

    def set_split_slices(self, slices):
        """Digit planes per operand of the split-BF16 C64 GEMMs (2…8, default 8)."""
        self.check(self.lib.tn_set_split_slices(self.h, int(slices)))

    PROFILE_CLASSES = ("jacobi_fp32", "jacobi_fp64", "gemm_fp64", "gemm_split_bf16", "split_prep", "qr",
                       "jacobi_coop")

    def profile(self, enable=True):
        """Time the hot-path phases by CUDA events on the context stream (resets the totals)."""
        self.check(self.lib.tn_profile_enable(self.h, int(bool(enable))))

    def profile_read(self):
        """{class: {launches, ms, flops, bytes}} since profiling was enabled."""
        out = {}
        for i, name in enumerate(self.PROFILE_CLASSES):
            n, ms, fl, by = C.c_int64(), C.c_double(), C.c_double(), C.c_double()
            self.check(self.lib.tn_profile_read(self.h, i, C.byref(n), C.byref(ms), C.byref(fl), C.byref(by)))
            out[name] = {"launches": n.value, "ms": ms.value, "flops": fl.value, "bytes": by.value}
        return out

    def refine_stats(self, reset=False):
        """Cumulative counts of the truncated mixed SVD: calls, refinement iterations,
        near-degenerate pairs finished by the FP64 Jacobi of the marked columns, and calls
        that needed full FP64 sweeps."""
        t = (C.c_int64 * 4)()
        self.check(self.lib.tn_svd_refine_stats(self.h, t, int(bool(reset))))
        return {"calls": t[0], "iterations": t[1], "marked_pairs": t[2], "full_fp64_sweeps": t[3]}

    def last_refine(self):
        """The last truncated mixed SVD's refinement: per iteration (largest step, largest
        |I − VᴴV|, largest ‖E‖_F, marked pairs) and the outcome ("converged", "diverged",
        "out_of_iterations")."""
        tr = (C.c_float * 32)()
        it, oc = C.c_int32(), C.c_int32()
        self.check(self.lib.tn_svd_last_refine(self.h, tr, C.byref(it), C.byref(oc)))
        rows = [tuple(tr[4 * k + q] for q in range(4)) for k in range(min(it.value, 8))]
        return rows, ("converged", "diverged", "out_of_iterations")[oc.value]

    def pipe_peak(self, which):
        """Measured FMA rate of the CUDA cores in TFLOP/s: which = "fp32" or "fp64"."""
        v = C.c_double()
        self.check(self.lib.tn_pipe_peak(self.h, {"fp32": 0, "fp64": 1}[which], C.byref(v)))
        return v.value


_default_ctx = None


def default_context():
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


class DeviceTensor:
    """Dense column-major device tensor with mode labels."""

    def __init__(self, ctx, shape, dtype, inds=None, ptr=None):
        self.ctx = ctx
        self.shape = tuple(int(s) for s in shape)
        self.dtype = np.dtype(dtype)
        if self.dtype not in _DT:
            raise ValueError(f"unsupported dtype {dtype}")
        self.inds = list(inds) if inds is not None else [f"_{i}" for i in range(len(self.shape))]
        if len(self.inds) != len(self.shape):
            raise ValueError("one label per mode")
        self.owned = ptr is None
        self.ptr = ctx.alloc(self.nbytes) if ptr is None else ptr

    @property
    def size(self):
        return int(np.prod(self.shape, dtype=np.int64)) if self.shape else 1

    @property
    def nbytes(self):
        return self.size * self.dtype.itemsize

    @property
    def code(self):
        return _DT[self.dtype]

    def __del__(self):
        if L.shutting_down():
            return
        try:
            if self.owned and self.ptr:
                self.ctx.free(self.ptr)
                self.ptr = None
        except Exception:
            pass

    @classmethod
    def from_numpy(cls, ctx, array, inds=None):
        a = np.asfortranarray(array)
        t = cls(ctx, a.shape, a.dtype, inds)
        ctx.h2d(t.ptr, a.reshape(-1, order="F") if a.ndim else a.reshape(1))
        return t

    def numpy(self):
        out = np.empty(self.size, dtype=self.dtype)
        self.ctx.d2h(out, self.ptr)
        return out.reshape(self.shape, order="F")

    def dim(self, ind):
        return self.shape[self.inds.index(ind)]


def _modes(labels_a, labels_b, labels_c):
    ids = {}
    counter = itertools.count()
    for lab in itertools.chain(labels_a, labels_b, labels_c):
        if lab not in ids:
            ids[lab] = next(counter)
    return ids


def _desc(t, ids, inds=None):
    d = L.tn_tensor()
    inds = t.inds if inds is None else inds
    d.rank = len(inds)
    for i, lab in enumerate(inds):
        d.modes[i] = ids[lab]
        d.dims[i] = t.shape[i] if t is not None else 0
    d.data = t.ptr if t is not None else None
    return d


def binary_einsum(a: DeviceTensor, b: DeviceTensor, dims=None, out_inds=None, precision="native"):
    """Muscle.binary_einsum(a, b; dims): contract the labels in ``dims`` (default: every
    shared label); shared labels not in ``dims`` are kept (Hadamard / batch modes).
    Output labels: a's kept labels, then b's (shared-kept labels once)."""
    shared = [i for i in a.inds if i in b.inds]
    dims = shared if dims is None else list(dims)
    for i in dims:
        if i not in shared:
            raise ValueError(f"contracted index {i!r} is not shared")
    if out_inds is None:
        out_inds = [i for i in a.inds if i not in dims] + [i for i in b.inds if i not in dims and i not in a.inds]
    ids = _modes(a.inds, b.inds, out_inds)
    shape = []
    for lab in out_inds:
        shape.append(a.dim(lab) if lab in a.inds else b.dim(lab))
    if a.dtype != b.dtype:
        raise ValueError("operands must share a dtype")
    c = DeviceTensor(a.ctx, shape, a.dtype, out_inds)
    da, db = _desc(a, ids), _desc(b, ids)
    dc = L.tn_tensor()
    dc.rank = len(out_inds)
    for i, lab in enumerate(out_inds):
        dc.modes[i] = ids[lab]
    dc.data = c.ptr
    a.ctx.check(a.ctx.lib.tn_contract(a.ctx.h, a.code, precision_code(precision), C.byref(da), C.byref(db), C.byref(dc)))
    return c


def permute(t: DeviceTensor, new_inds, conj=False):
    """permutedims to the label order ``new_inds`` (K1)."""
    perm = [t.inds.index(i) for i in new_inds]
    out = DeviceTensor(t.ctx, [t.shape[p] for p in perm], t.dtype, list(new_inds))
    dims = (C.c_int64 * len(t.shape))(*t.shape)
    pr = (C.c_int32 * len(perm))(*perm)
    t.ctx.check(t.ctx.lib.tn_permute(t.ctx.h, t.code, len(perm), dims, None, pr, C.c_void_p(t.ptr), C.c_void_p(out.ptr), int(conj)))
    return out


def _as_matrix(t, row_inds, col_inds):
    order = list(row_inds) + list(col_inds)
    if sorted(map(str, order)) != sorted(map(str, t.inds)) or len(order) != len(t.inds):
        raise ValueError("row and column labels must partition the tensor's labels")
    mt = t if order == t.inds else permute(t, order)
    m = int(np.prod([t.dim(i) for i in row_inds], dtype=np.int64)) if row_inds else 1
    n = int(np.prod([t.dim(i) for i in col_inds], dtype=np.int64)) if col_inds else 1
    return mt, m, n


def _labelled_modes(A, left, new_label):
    """Integer modes for A's labels (by position) plus one for the new label."""
    ids = {lab: k for k, lab in enumerate(A.inds)}
    if new_label in ids:
        raise ValueError(f"label {new_label!r} is already an index of the tensor")
    ids[new_label] = len(ids)
    for lab in left:
        if lab not in ids or lab == new_label:
            raise ValueError(f"label {lab!r} is not an index of the tensor")
    return ids


def tensor_qr_thin(A: DeviceTensor, inds_q, inds_r=None, ind_virtual="_qr", precision="native"):
    """Muscle.tensor_qr_thin (tn_tensor_qr_thin): Q carries (inds_q…, ind_virtual),
    R (ind_virtual, inds_r…); inds_r defaults to A's other labels in A's order."""
    inds_q = list(inds_q)
    rest = [i for i in A.inds if i not in inds_q]
    if inds_r is not None and sorted(map(str, inds_r)) != sorted(map(str, rest)):
        raise ValueError("inds_q and inds_r must partition the tensor's labels")
    ids = _labelled_modes(A, inds_q, ind_virtual)
    m = int(np.prod([A.dim(i) for i in inds_q], dtype=np.int64)) if inds_q else 1
    n = int(np.prod([A.dim(i) for i in rest], dtype=np.int64)) if rest else 1
    k = min(m, n)
    Q = DeviceTensor(A.ctx, [A.dim(i) for i in inds_q] + [k], A.dtype, inds_q + [ind_virtual])
    R = DeviceTensor(A.ctx, [k] + [A.dim(i) for i in rest], A.dtype, [ind_virtual] + rest)
    qm = (C.c_int32 * max(1, len(inds_q)))(*[ids[i] for i in inds_q])
    da, dq, dr = _desc(A, ids), _desc(Q, ids), _desc(R, ids)
    A.ctx.check(A.ctx.lib.tn_tensor_qr_thin(A.ctx.h, A.code, precision_code(precision), C.byref(da), len(inds_q), qm,
                                            ids[ind_virtual], C.byref(dq), C.byref(dr)))
    if inds_r is not None and list(inds_r) != rest:
        R = permute(R, [ind_virtual] + list(inds_r))
    return Q, R


def tensor_svd_thin(A: DeviceTensor, inds_u, inds_v=None, ind_s="_svd", precision="native", maxdim=None,
                    threshold=None):
    """Muscle.tensor_svd_thin (tn_tensor_svd_thin): U (inds_u…, ind_s), s (ind_s) real
    FP64 descending, V (ind_s, inds_v…) with A = U·diag(s)·V.  ``maxdim`` / ``threshold``
    truncate like compress! (keep ≤ maxdim, then |s| > threshold, at least one)."""
    inds_u = list(inds_u)
    rest = [i for i in A.inds if i not in inds_u]
    if inds_v is not None and sorted(map(str, inds_v)) != sorted(map(str, rest)):
        raise ValueError("inds_u and inds_v must partition the tensor's labels")
    ids = _labelled_modes(A, inds_u, ind_s)
    m = int(np.prod([A.dim(i) for i in inds_u], dtype=np.int64)) if inds_u else 1
    n = int(np.prod([A.dim(i) for i in rest], dtype=np.int64)) if rest else 1
    k = min(m, n)
    U = DeviceTensor(A.ctx, [A.dim(i) for i in inds_u] + [k], A.dtype, inds_u + [ind_s])
    s = DeviceTensor(A.ctx, [k], np.float64, [ind_s])
    V = DeviceTensor(A.ctx, [k] + [A.dim(i) for i in rest], A.dtype, [ind_s] + rest)
    um = (C.c_int32 * max(1, len(inds_u)))(*[ids[i] for i in inds_u])
    du, dv = _desc(U, ids), _desc(V, ids)
    da = _desc(A, ids)
    r = C.c_int64()
    A.ctx.check(A.ctx.lib.tn_tensor_svd_thin(A.ctx.h, A.code, precision_code(precision), C.byref(da), len(inds_u), um,
                                             ids[ind_s], -1 if maxdim is None else int(maxdim),
                                             -1.0 if threshold is None else float(threshold), C.byref(du),
                                             C.c_void_p(s.ptr), C.byref(dv), C.byref(r)))
    kr = r.value
    U.shape = tuple(du.dims[i] for i in range(du.rank))
    V.shape = tuple(dv.dims[i] for i in range(dv.rank))
    s.shape = (kr,)
    if inds_v is not None and list(inds_v) != rest:
        V = permute(V, [ind_s] + list(inds_v))
    return U, s, V


def hadamard(t: DeviceTensor, s: DeviceTensor):
    """Muscle.hadamard(t, s): multiply t by the real vector s along s's label."""
    if len(s.inds) != 1 or s.dtype != np.float64:
        raise ValueError("s must be a real FP64 vector")
    axis = t.inds.index(s.inds[0])
    out = DeviceTensor(t.ctx, t.shape, t.dtype, t.inds)
    dims = (C.c_int64 * len(t.shape))(*t.shape)
    t.ctx.check(t.ctx.lib.tn_hadamard(t.ctx.h, t.code, len(t.shape), dims, axis, C.c_void_p(t.ptr), C.c_void_p(s.ptr), C.c_void_p(out.ptr)))
    return out


def norm(t: DeviceTensor):
    v = C.c_double()
    t.ctx.check(t.ctx.lib.tn_norm2(t.ctx.h, t.code, t.size, C.c_void_p(t.ptr), C.byref(v)))
    return v.value


def scale(t: DeviceTensor, s):
    """t ← s·t in place (real s)."""
    t.ctx.check(t.ctx.lib.tn_scale(t.ctx.h, t.code, t.size, C.c_void_p(t.ptr), float(s)))
    return t


_ABSORB = {"equally": 0, "v": 1, "u": 2}


def simple_update(A: DeviceTensor, ia, B: DeviceTensor, ib, bond, op: DeviceTensor, oa, ob, maxdim=None,
                  threshold=None, precision="native", absorb="equally"):
    """Muscle.simple_update(A, ia, B, ib, bond, op, oa, ob; maxdim, absorb): ``absorb`` is
    "equally" (AbsorbEqually, A' = U√S, B' = √S Vh), "u" (AbsorbU: A' = U·S, B' = Vh) or
    "v" (AbsorbV: A' = U, B' = S·Vh).

    ``ia``/``ib`` are A's and B's physical labels, ``oa``/``ob`` the gate's output labels
    matching them; the gate's input labels are ``ia``/``ib``.  Returns (A', B') with A'
    labelled (A's other labels, oa→ia, bond) and B' (bond, ib, B's other labels)."""
    la = [i for i in A.inds if i not in (ia, bond)]
    lb = [i for i in B.inds if i not in (ib, bond)]
    if len(la) > 1 or len(lb) > 1:
        raise ValueError("A and B must each carry one virtual label besides the bond")
    Am = permute(A, la + [ia, bond]) if A.inds != la + [ia, bond] else A
    Bm = permute(B, [bond, ib] + lb) if B.inds != [bond, ib] + lb else B
    G = permute(op, [oa, ob, ia, ib]) if op.inds != [oa, ob, ia, ib] else op
    chl = Am.shape[0] if la else 1
    d1, chm = A.dim(ia), A.dim(bond)
    d2 = B.dim(ib)
    chr_ = Bm.shape[2] if lb else 1
    kmax = min(chl * d1, d2 * chr_)
    An = DeviceTensor(A.ctx, ([chl] if la else []) + [d1, kmax], A.dtype, la + [ia, bond])
    Bn = DeviceTensor(A.ctx, [kmax, d2] + ([chr_] if lb else []), A.dtype, [bond, ib] + lb)
    r = C.c_int64()
    if absorb not in _ABSORB:
        raise ValueError(f"absorb must be one of {sorted(_ABSORB)}")
    A.ctx.check(
        A.ctx.lib.tn_simple_update_absorb(A.ctx.h, L.TN_C64, precision_code(precision), chl, d1, chm, d2, chr_,
                                          C.c_void_p(Am.ptr), C.c_void_p(Bm.ptr), C.c_void_p(G.ptr),
                                          -1 if maxdim is None else int(maxdim),
                                          -1.0 if threshold is None else float(threshold), _ABSORB[absorb],
                                          C.c_void_p(An.ptr), C.c_void_p(Bn.ptr), None, C.byref(r))
    )
    k = r.value
    An.shape = tuple(([chl] if la else []) + [d1, k])
    Bn.shape = tuple([k, d2] + ([chr_] if lb else []))
    return An, Bn
