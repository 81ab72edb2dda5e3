"""Whole-network contraction (Tangles' ``contract(tn)``, used at
src/Operations/overlap.jl:12 and by the reference tests' ``contract(ψ)``): the greedy
planner on CPU, and GPU parity of every precision mode against the complex128 oracle
along the same path."""

import math

import numpy as np
import pytest

from oracle import network_oracle as NO


def test_region_path_on_lattice_is_valid_and_bounded():
    from tenetgb import network as N

    net = N.lattice_2d(8, 8, 8)
    path = N.greedy_path(net.labels, net.dims)
    assert len(path) == len(net.arrays) - 1
    steps, peak = N.path_flops(net.labels, net.dims, path)
    assert peak <= 2**28
    assert 1e12 < sum(s["flops"] for s in steps) < 1e13


@pytest.mark.parametrize("strategy", ["region", "pairwise"])
def test_paths_agree_with_einsum_on_small_lattice(strategy):
    from tenetgb import network as N

    net = N.lattice_2d(3, 4, 3, seed=9, dtype=np.complex128)
    path = N.greedy_path(net.labels, net.dims, strategy=strategy)
    val = NO.contract_along(net.arrays, net.labels, path)
    letters = {}
    for labs in net.labels:
        for lab in labs:
            letters.setdefault(lab, chr(ord("a") + len(letters)) if len(letters) < 26 else chr(ord("A") + len(letters) - 26))
    spec = ",".join("".join(letters[x] for x in labs) for labs in net.labels) + "->"
    ref = np.einsum(spec, *net.arrays, optimize=True)
    assert abs(val - ref) <= 1e-12 * max(1.0, abs(ref))


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(4, 4, 4), (5, 5, 4), (6, 6, 3)])
@pytest.mark.parametrize("mode,dtype,tol", [
    ("native", np.complex128, 1e-12),
    ("native", np.complex64, 1e-5),
    ("mixed", np.complex64, 2e-5),
    ("tf32", np.complex64, 1e-2),
])
def test_gpu_lattice_contraction(shape, mode, dtype, tol):
    import tenetgb
    from tenetgb import network as N

    ctx = tenetgb.Context(0)
    net = N.lattice_2d(*shape, seed=4)
    path = N.greedy_path(net.labels, net.dims)
    ref = NO.contract_along(net.arrays, net.labels, path)
    val = N.contract(net, path, precision=mode, dtype=dtype, ctx=ctx)
    # scale: product of the tensors' norms bounds |ref|; compare relative to it
    scale = math.prod(float(np.linalg.norm(a)) for a in net.arrays)
    assert abs(val - ref) <= tol * max(abs(ref), 1e-3 * scale)


def test_mpo_dimension_checks_without_a_device():
    """The MPO argument of dmrg! / evolve! is validated on the host before any device
    work (the library reads (w_l, d, d, w_r) elements per site)."""
    import pytest

    import tenetgb

    class FakeMPS:
        _d = 2
        nsites = 3
        batch = 1

    W = [np.zeros((1, 3, 3, 2)), np.zeros((2, 3, 3, 2)), np.zeros((2, 3, 3, 1))]
    with pytest.raises(ValueError, match="physical dimensions"):
        tenetgb.dmrg_(FakeMPS(), W, 1)
    with pytest.raises(ValueError, match="same number of sites"):
        tenetgb.dmrg_(FakeMPS(), W[:2], 1)
