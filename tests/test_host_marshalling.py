"""CPU checks of the host layer's argument marshalling for the layer evolution entry
(no GPU: the library call is replaced by a recorder): layer starts, gate counts, the
per-layer direction (two-element layers are left to right), the gates flattened in
column-major order layer after layer, and the truncation arguments."""

import ctypes as C

import numpy as np


class Recorder:
    def __init__(self):
        self.calls = []

    def tn_mps_evolve_layers(self, h, n, starts, counts, rev, buf, maxdim, thr):
        total = sum(counts[i] for i in range(n))
        p = C.cast(buf, C.POINTER(C.c_double))
        flat = np.array([p[i] for i in range(2 * 16 * total)])
        self.calls.append(dict(n=n, starts=[starts[i] for i in range(n)], counts=[counts[i] for i in range(n)],
                               rev=[rev[i] for i in range(n)], gates=flat[0::2] + 1j * flat[1::2], maxdim=maxdim,
                               thr=thr))
        return 0


def fake_mps(lib, L=10, d=2):
    """A host-side MPS object whose library calls go to ``lib`` (no device)."""
    from tenetgb.mps import MPS

    m = MPS.__new__(MPS)
    m.lib = lib
    m.h = None
    m._chk = lambda st: None
    m._L, m._d = L, d
    return m


def test_layers_marshalled():
    from tenetgb.mps import MPS

    rng = np.random.default_rng(0)
    g = [rng.standard_normal((2, 2, 2, 2)) + 1j * rng.standard_normal((2, 2, 2, 2)) for _ in range(5)]
    m = fake_mps(Recorder())
    m.evolve_brickwork_([(1, g[:3]), (2, g[3:], True)], maxdim=64, threshold=1e-12)
    c = m.lib.calls[0]
    assert c["n"] == 2 and c["starts"] == [1, 2] and c["counts"] == [3, 2] and c["rev"] == [0, 1]
    want = np.concatenate([G.reshape(-1, order="F") for G in g])
    assert np.array_equal(c["gates"], want)
    assert c["maxdim"] == 64 and c["thr"] == 1e-12
    m.evolve_brickwork_([(1, g[:1], False)])
    c = m.lib.calls[1]
    assert c["rev"] == [0] and c["maxdim"] == -1 and c["thr"] == -1.0


def test_serpentine_workload_directions():
    from tenetgb import workloads as W

    layers = W.tebd_layers(10, 4, serpentine=True)
    assert [ly[2] for ly in layers] == [False, True, False, True]
    assert [ly[0] for ly in layers] == [1, 2, 1, 2] and [len(ly[1]) for ly in layers] == [5, 4, 5, 4]
    assert all(not ly[2] for ly in W.tebd_layers(10, 4))


class Refuser:
    """Any library call is a failure: the host checks must stop bad arrays first."""

    def __getattr__(self, name):
        raise AssertionError(f"{name} reached the library with a malformed host array")


def test_host_arrays_checked_before_the_library_reads_them():
    """The library reads d^(2·nsites) gate entries, d⁴ per brickwork gate, L×d product
    vectors and a d×d operator from host memory; wrong shapes are ValueErrors (Tenet's
    @argcheck) instead of out-of-bounds host reads."""
    import pytest

    m = fake_mps(Refuser(), L=4, d=2)
    with pytest.raises(ValueError):
        m.simple_update_(np.eye(3), [1])
    with pytest.raises(ValueError):
        m.simple_update_(np.eye(2), [1, 2])
    with pytest.raises(ValueError):
        m.simple_update_(np.eye(4), [1, 2, 3])
    with pytest.raises(ValueError):
        m.evolve_brickwork_([(1, [np.eye(2)])])
    with pytest.raises(ValueError):
        m.amplitude("010")
    with pytest.raises(ValueError):
        m.amplitude([np.ones(3)] * 4)
    with pytest.raises(ValueError):
        m.local_expectations(np.eye(4))


class BondsOnly(Refuser):
    """Answers the bond-dimension query of an L-site MPS; any other call is a failure."""

    def __init__(self, L):
        self.L = L

    def tn_mps_bond_dims(self, h, out):
        for i in range(self.L - 1):
            out[i] = 2
        return 0


def test_mpo_sizes_must_chain_before_the_library_reads_them():
    import pytest

    from tenetgb.mps import evolve_mpo_

    m = fake_mps(BondsOnly(3), L=3, d=2)

    def site(wl, wr, d=2):
        return np.zeros((wl, d, d, wr), np.complex128)

    with pytest.raises(ValueError):  # middle site's left dimension differs from its neighbour's right one
        evolve_mpo_(m, [site(1, 3), site(2, 3), site(3, 1)])
    with pytest.raises(ValueError):  # open ends must be 1
        evolve_mpo_(m, [site(1, 3), site(3, 3), site(3, 2)])
    with pytest.raises(ValueError):  # physical dimension
        evolve_mpo_(m, [site(1, 3), site(3, 3, d=3), site(3, 1)])
    with pytest.raises(ValueError):  # one site per MPS site
        evolve_mpo_(m, [site(1, 3), site(3, 1)])
