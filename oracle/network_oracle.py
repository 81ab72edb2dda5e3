"""CPU oracle for whole-network contraction (Tangles' ``contract(tn)``).

TEST INFRASTRUCTURE ONLY (tests/, smoke, bench's CPU leg).  Contracts a network along a
given pairwise path with numpy ``tensordot`` in complex128 — the arithmetic the
reference reaches through Tangles → EinExprs → Muscle.binary_einsum (permute + BLAS
gemm).  The path itself is not pinned to EinExprs (neither package is available here);
only the scalar is compared, which is path-independent up to rounding.
"""

import numpy as np


def contract_along(arrays, labels, path, dtype=np.complex128):
    live = {i: (np.asarray(a, dtype=dtype), list(l)) for i, (a, l) in enumerate(zip(arrays, labels))}
    counts = {}
    for labs in labels:
        for lab in labs:
            counts[lab] = counts.get(lab, 0) + 1
    nxt = len(arrays)
    for a, b in path:
        (ta, la), (tb, lb) = live.pop(a), live.pop(b)
        shared = set(la) & set(lb)
        out = [x for x in la if x not in shared or counts[x] > 2] + [x for x in lb if x not in la]
        contracted = [x for x in shared if x not in out]
        kept_shared = [x for x in shared if x in out]
        for x in contracted:
            counts[x] -= 2
        if kept_shared:
            letters = {}
            for x in la + lb:
                letters.setdefault(x, chr(ord("a") + len(letters)) if len(letters) < 26 else chr(ord("A") + len(letters) - 26))
            spec = "".join(letters[x] for x in la) + "," + "".join(letters[x] for x in lb) + "->" + "".join(letters[x] for x in out)
            res = np.einsum(spec, ta, tb)
        else:
            ia = [la.index(x) for x in contracted]
            ib = [lb.index(x) for x in contracted]
            res = np.tensordot(ta, tb, axes=(ia, ib))
            cur = [x for x in la if x not in contracted] + [x for x in lb if x not in contracted]
            res = np.transpose(res, [cur.index(x) for x in out]) if out else res
        live[nxt] = (res, out)
        nxt += 1
    ((res, _),) = live.values()
    return res
