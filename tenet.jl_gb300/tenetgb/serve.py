"""Python face of the query server (tn_serve_* in include/tenet_gb300.h).

A ``Server`` keeps a pool of MPS on the device and answers the reference's per-state
queries with continuous batching:

* ``amplitude(id, bits)``     ⟨bits|ψ⟩ = overlap(ProductState(bits), ψ)  (src/Operations/overlap.jl:22-32)
* ``expectation(id, site, O)`` ⟨ψ|O_site|ψ⟩ / ⟨ψ|ψ⟩                        (src/Operations/overlap.jl:36-50)
* ``overlap(a, b)``            ⟨ψ_b|ψ_a⟩                                  (src/Operations/overlap.jl:36-50)

Each ``submit_*`` returns a ticket at once; ``wait(ticket)`` returns the value and the
latency.  Queries submitted from several threads are batched together by the server's
worker thread.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib


def _check(status):
    if status == _lib.TN_OK:
        return
    msg = _lib.load().tn_serve_last_error().decode(errors="replace")
    if status == _lib.TN_EINVAL:
        raise ValueError(msg)
    if status == _lib.TN_ENOMEM:
        raise MemoryError(msg)
    if status == _lib.TN_ETIMEOUT:
        raise _lib.DeviceTimeoutError(msg)
    raise _lib.TenetGBError(f"status {status}: {msg}")


def product_vectors(bits, d=2):
    """L×d complex product-state vectors of a bit string (site-major), the ``ProductState``
    of the reference."""
    bits = np.asarray(bits, dtype=np.int64)
    v = np.zeros((bits.size, d), np.complex128)
    v[np.arange(bits.size), bits] = 1.0
    return v


STAT_KEYS = ("completed", "short_jobs", "overlap_jobs", "max_batch", "deferred", "pool_bytes", "pending",
             "in_flight")


class Server:
    def __init__(self, device=0, hbm_budget=0, work_bytes=1 << 30, max_batch=64, precision="native"):
        """precision "native" (FP64) or "mixed" (FP32 amplitude and overlap sweeps)."""
        self.lib = _lib.load()
        h = C.c_void_p()
        prec = {"native": _lib.TN_PREC_NATIVE, "fp64": _lib.TN_PREC_NATIVE, "mixed": _lib.TN_PREC_MIXED}[precision]
        _check(self.lib.tn_serve_create(device, int(hbm_budget), int(work_bytes), int(max_batch), prec, C.byref(h)))
        self.precision = precision
        self.h = h
        self._shape = {}

    # ---- pool ----
    def add_mps(self, arrays):
        """Sites as numpy arrays (χl, d, χr) (2-D boundary sites (d, χr) / (χl, d) are
        accepted); returns the pool id."""
        sites = []
        for i, a in enumerate(arrays):
            a = np.asarray(a, dtype=np.complex128)
            if a.ndim == 2:
                a = a[None, :, :] if i == 0 else a[:, :, None]
            sites.append(np.asfortranarray(a))
        L, d = len(sites), sites[0].shape[1]
        bonds = (C.c_int64 * max(1, L - 1))(*[s.shape[2] for s in sites[:-1]])
        ptrs = (C.c_void_p * L)(*[s.ctypes.data for s in sites])
        out = C.c_int32()
        _check(self.lib.tn_serve_add_mps(self.h, L, d, bonds, ptrs, C.byref(out)))
        self._shape[out.value] = (L, d)
        return out.value

    def add_random_mps(self, L, chi, d=2, seed=0):
        out = C.c_int32()
        _check(self.lib.tn_serve_add_random_mps(self.h, int(L), int(d), int(chi), int(seed), C.byref(out)))
        self._shape[out.value] = (int(L), int(d))
        return out.value

    def remove_mps(self, mid):
        _check(self.lib.tn_serve_remove_mps(self.h, int(mid)))
        self._shape.pop(mid, None)

    def info(self, mid):
        L, d = C.c_int32(), C.c_int32()
        n2 = C.c_double()
        _check(self.lib.tn_serve_mps_info(self.h, int(mid), C.byref(L), C.byref(d), None, C.byref(n2)))
        bonds = (C.c_int64 * max(1, L.value - 1))()
        _check(self.lib.tn_serve_mps_info(self.h, int(mid), C.byref(L), C.byref(d), bonds, None))
        return {"L": L.value, "d": d.value, "bonds": list(bonds)[: L.value - 1], "norm2": n2.value}

    def sites(self, mid):
        """The pool MPS's site tensors as numpy arrays (χl, d, χr)."""
        inf = self.info(mid)
        b = [1] + inf["bonds"] + [1]
        out = []
        for i in range(inf["L"]):
            a = np.empty((b[i], inf["d"], b[i + 1]), np.complex128, order="F")
            _check(self.lib.tn_serve_get_site(self.h, int(mid), i + 1, a.ctypes.data))
            out.append(np.ascontiguousarray(a))
        return out

    # ---- queries ----
    def _submit(self, kind, mid, mid_b=-1, site=0, data=None):
        keep = None
        q = _lib.tn_query(kind, int(mid), int(mid_b), int(site), None)
        if data is not None:
            keep = np.asfortranarray(np.asarray(data, dtype=np.complex128))
            q.data = keep.ctypes.data
        t = C.c_int64()
        _check(self.lib.tn_serve_submit(self.h, C.byref(q), C.byref(t)))  # copies data before returning
        return t.value

    def submit_amplitude(self, mid, bits=None, vectors=None):
        if vectors is None:
            # an unknown id is rejected by the server (ValueError), as for the other queries
            vectors = product_vectors(bits, self._shape.get(mid, (0, 2))[1])
        # site-major L×d: row i holds site i's vector
        return self._submit(_lib.TN_Q_AMPLITUDE, mid, data=np.ascontiguousarray(vectors).reshape(-1))

    def submit_expectation(self, mid, site, op):
        """``site`` is 1-based, as in the reference."""
        return self._submit(_lib.TN_Q_EXPECTATION, mid, site=site, data=np.asarray(op))

    def submit_overlap(self, mid_ket, mid_bra):
        return self._submit(_lib.TN_Q_OVERLAP, mid_ket, mid_b=mid_bra)

    def wait(self, ticket, timeout=600.0):
        v = (C.c_double * 2)()
        lat = C.c_double()
        _check(self.lib.tn_serve_wait(self.h, int(ticket), float(timeout), v, C.byref(lat)))
        return complex(v[0], v[1]), lat.value

    def amplitude(self, mid, bits):
        return self.wait(self.submit_amplitude(mid, bits))[0]

    def expectation(self, mid, site, op):
        return self.wait(self.submit_expectation(mid, site, op))[0]

    def overlap(self, mid_ket, mid_bra):
        return self.wait(self.submit_overlap(mid_ket, mid_bra))[0]

    def stats(self):
        s = (C.c_int64 * 8)()
        _check(self.lib.tn_serve_stats(self.h, s))
        return dict(zip(STAT_KEYS, list(s)))

    def close(self):
        if self.h is not None and self.h.value and not _lib.shutting_down():
            self.lib.tn_serve_destroy(self.h)
        self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
