"""Generic tensor networks contracted to a scalar (Tangles' ``contract(tn)``).

Tenet reaches ``Tangles.contract(tn)`` for whole-network contractions (e.g.
src/Operations/overlap.jl:12 and every ``contract(ψc) ≈ contract(ψ)`` test); Tangles
asks EinExprs.jl for a pairwise path and runs it as a chain of ``binary_einsum`` calls.
Here the path comes from a greedy planner written for this project (same spirit as
EinExprs' greedy: repeatedly contract the pair that shrinks the network most, with a cap
on intermediate sizes) and every step is one ``tn_contract`` on the GPU (permute + GEMM,
on the tcgen05 tensor pipe for ComplexF32 in the 3×TF32 / TF32 modes).
"""

from __future__ import annotations

import math
import time
from dataclasses import dataclass, field

import numpy as np

from .core import Context, DeviceTensor, binary_einsum, default_context, scale
from .core import norm as tensor_norm


@dataclass
class Network:
    """Tensors with integer/string labels; every label appears in at most two tensors
    (open labels appear once)."""

    arrays: list = field(default_factory=list)
    labels: list = field(default_factory=list)
    dims: dict = field(default_factory=dict)

    def add(self, array, labels):
        array = np.asarray(array)
        if array.ndim != len(labels):
            raise ValueError("one label per mode")
        for lab, n in zip(labels, array.shape):
            if self.dims.setdefault(lab, n) != n:
                raise ValueError(f"label {lab!r}: dimension mismatch")
        self.arrays.append(array)
        self.labels.append(list(labels))

    def open_labels(self):
        count = {}
        for labs in self.labels:
            for lab in labs:
                count[lab] = count.get(lab, 0) + 1
        return [lab for lab, c in count.items() if c == 1]


def lattice_2d(nx=8, ny=8, bond=8, seed=4, dtype=np.complex64):
    """Closed nx×ny square lattice, open boundary: corners rank 2, edges rank 3, bulk
    rank 4, every bond of dimension ``bond``; entries complex Gaussian × 1/√(bond^rank)."""
    rng = np.random.default_rng(seed)
    net = Network()
    for x in range(nx):
        for y in range(ny):
            labs = []
            if x > 0:
                labs.append(("h", x - 1, y))
            if x < nx - 1:
                labs.append(("h", x, y))
            if y > 0:
                labs.append(("v", x, y - 1))
            if y < ny - 1:
                labs.append(("v", x, y))
            shape = (bond,) * len(labs)
            a = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) / np.sqrt(2.0)
            a = a / np.sqrt(float(bond) ** len(labs))
            net.add(a.astype(dtype), labs)
    return net


def _size(labels, dims):
    return math.prod(dims[lab] for lab in labels) if labels else 1


def _out(la, lb, counts):
    shared = set(la) & set(lb)
    return [x for x in la if x not in shared or counts[x] > 2] + [x for x in lb if x not in la]


def greedy_path(labels_list, dims, max_size=2**28, strategy="region"):
    """Pairwise path as a list of (i, j) over SSA ids (inputs 0..n-1, each contraction
    appends a new id).

    ``strategy="region"`` (default): grow one intermediate from the smallest tensor,
    each step absorbing the neighbour that gives the smallest result (ties: the larger
    contracted extent).  On lattices this sweeps a boundary across the network (8×8,
    bond 8: peak 2^27 elements, 2.6 TFLOP).
    ``strategy="pairwise"``: at each step contract, among all pairs sharing a label, the
    one minimising size(out) − size(a) − size(b), within ``max_size``.
    Disconnected remainders are joined by outer products."""
    live = {i: list(l) for i, l in enumerate(labels_list)}
    counts = {}
    for labs in labels_list:
        for lab in labs:
            counts[lab] = counts.get(lab, 0) + 1
    nxt = len(labels_list)
    path = []

    def commit(a, b, out):
        nonlocal nxt
        for x in set(live[a]) & set(live[b]):
            if x not in out:
                counts[x] -= 2
        del live[a], live[b]
        live[nxt] = out
        path.append((a, b))
        nxt += 1
        return nxt - 1

    if strategy == "region":
        cur = min(live, key=lambda i: (_size(live[i], dims), i))
        while len(live) > 1:
            lc = live[cur]
            best = None
            for b in sorted(live):
                if b == cur or not (set(live[b]) & set(lc)):
                    continue
                out = _out(lc, live[b], counts)
                so = _size(out, dims)
                k = _size([x for x in set(lc) & set(live[b]) if x not in out], dims)
                key = (so, -k, b)
                if best is None or key < best[0]:
                    best = (key, b, out)
            if best is None:  # disconnected: outer product with the smallest remaining
                b = min((i for i in live if i != cur), key=lambda i: (_size(live[i], dims), i))
                out = _out(lc, live[b], counts)
            else:
                _, b, out = best
            if _size(out, dims) > max_size:
                raise ValueError(f"intermediate of {_size(out, dims)} elements exceeds {max_size}")
            cur = commit(cur, b, out)
        return path

    while len(live) > 1:
        best = None
        by_label = {}
        for i in sorted(live):
            for lab in live[i]:
                by_label.setdefault(lab, []).append(i)
        cand = set()
        for owners in by_label.values():
            for p in range(len(owners)):
                for q in range(p + 1, len(owners)):
                    cand.add((owners[p], owners[q]))
        for a, b in cand:
            out = _out(live[a], live[b], counts)
            so = _size(out, dims)
            if so > max_size:
                continue
            key = (so - _size(live[a], dims) - _size(live[b], dims), so, a, b)
            if best is None or key < best[0]:
                best = (key, a, b, out)
        if best is None:
            if cand:
                raise ValueError(f"no contraction keeps intermediates within {max_size} elements")
            a, b = sorted(live)[:2]
            out = _out(live[a], live[b], counts)
        else:
            _, a, b, out = best
        commit(a, b, out)
    return path


def path_flops(labels_list, dims, path):
    """Complex-algorithmic flops (8 per complex MAC) per step and the peak intermediate."""
    live = {i: list(l) for i, l in enumerate(labels_list)}
    counts = {}
    for labs in labels_list:
        for lab in labs:
            counts[lab] = counts.get(lab, 0) + 1
    nxt = len(labels_list)
    steps = []
    peak = 0
    for a, b in path:
        la, lb = live.pop(a), live.pop(b)
        shared = set(la) & set(lb)
        out = [x for x in la if x not in shared or counts[x] > 2] + [x for x in lb if x not in la]
        contracted = [x for x in shared if x not in out]
        k = _size(contracted, dims)
        so = _size(out, dims)
        steps.append({"out": so, "k": k, "flops": 8 * so * k})
        peak = max(peak, so)
        for x in contracted:
            counts[x] -= 2
        live[nxt] = out
        nxt += 1
    return steps, peak


def contract(net: Network, path=None, precision="mixed", dtype=None, ctx: Context | None = None,
             max_size=2**28, timing=False, rescale=True):
    """Contract ``net`` to a scalar on the GPU along ``path`` (greedy by default).

    ``dtype`` overrides the storage type (e.g. complex128 for the FP64 run).  With
    ``rescale`` every intermediate is divided by its norm (an FP64 reduction) and the log
    of the scale is carried in FP64: a closed 8×8 network of unit-norm tensors has a
    value near 1e-51, below the FP32 range, so unscaled FP32 intermediates underflow.
    Returns the scalar (complex128), or (scalar, stats) with ``timing``."""
    ctx = ctx or default_context()
    if path is None:
        path = greedy_path(net.labels, net.dims, max_size)
    dt = np.dtype(dtype) if dtype is not None else net.arrays[0].dtype
    live = {}
    for i, (a, labs) in enumerate(zip(net.arrays, net.labels)):
        live[i] = DeviceTensor.from_numpy(ctx, np.asarray(a, dtype=dt), labs)
    counts = {}
    for labs in net.labels:
        for lab in labs:
            counts[lab] = counts.get(lab, 0) + 1
    nxt = len(net.arrays)
    log_scale = 0.0
    t0 = time.perf_counter()
    for a, b in path:
        ta, tb = live.pop(a), live.pop(b)
        shared = set(ta.inds) & set(tb.inds)
        out = [x for x in ta.inds if x not in shared or counts[x] > 2] + [x for x in tb.inds if x not in ta.inds]
        contracted = [x for x in shared if x not in out]
        for x in contracted:
            counts[x] -= 2
        res = binary_einsum(ta, tb, dims=contracted, out_inds=out, precision=precision)
        if rescale:
            nrm = tensor_norm(res)
            if nrm > 0 and np.isfinite(nrm):
                scale(res, 1.0 / nrm)
                log_scale += math.log(nrm)
        live[nxt] = res
        del ta, tb
        nxt += 1
    (res,) = live.values()
    val = res.numpy().astype(np.complex128)
    val = complex(val.reshape(-1)[0]) if res.size == 1 else val
    val = val * math.exp(log_scale) if log_scale > -700 else complex(np.float64(val) * np.exp(np.float64(log_scale)))
    if not timing:
        return val
    ctx.sync()
    return val, {"seconds": time.perf_counter() - t0, "steps": len(path)}
