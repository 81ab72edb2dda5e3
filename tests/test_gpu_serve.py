"""The query server (tn_serve_*): amplitude, ⟨O_i⟩ and overlap queries on a
device-resident MPS pool, checked against the CPU oracle (the reference's
overlap(ProductState, ψ), overlap(ψ, O_i ψ)/overlap(ψ, ψ) and overlap(ψ, ϕ) of
src/Operations/overlap.jl:22-50), alone and in a concurrent mix.

Tolerances (FP64 throughout): a result agrees with the oracle to 1e-12 of its natural
scale — ‖ψ‖ for an amplitude, ‖O‖ for ⟨O_i⟩, ‖ψ_a‖‖ψ_b‖ for an overlap — and a result
computed inside a batch agrees with the same query computed alone to 1e-13 of that
scale (the batched arithmetic is the same per query; in practice the values are
bitwise equal)."""

import threading

import numpy as np
import pytest

from oracle import tenet_oracle as O

pytestmark = pytest.mark.gpu


def cgauss(rng, shape):
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) / np.sqrt(2)


def hermitian(rng, d=2):
    X = cgauss(rng, (d, d))
    return (X + X.conj().T) / 2


@pytest.fixture(scope="module")
def pool():
    from tenetgb import serve
    from tenetgb import workloads as W

    srv = serve.Server(work_bytes=256 << 20, max_batch=32)
    ids = {
        "a": srv.add_random_mps(10, 8, seed=1),
        "b": srv.add_random_mps(10, 16, seed=2),
        "c": srv.add_random_mps(13, 32, seed=3),
        "d": srv.add_random_mps(13, 12, seed=4),
        "h": srv.add_mps(W.random_mps_arrays(9, 2, 16, seed=5, orthogonalize=False)),
    }
    omps = {k: O.OMPS(srv.sites(v)) for k, v in ids.items()}
    yield srv, ids, omps
    srv.close()


def make_queries(ids, omps, seed=0, n_amp=4, n_exp=3):
    rng = np.random.default_rng(seed)
    qs = []
    for k, mid in ids.items():
        L = omps[k].L
        for _ in range(n_amp):
            qs.append(("amp", k, rng.integers(0, 2, L)))
        for _ in range(n_exp):
            qs.append(("exp", k, (int(rng.integers(1, L + 1)), hermitian(rng))))
    qs += [("ovl", "a", "b"), ("ovl", "b", "a"), ("ovl", "c", "d"), ("ovl", "d", "c"), ("ovl", "c", "c")]
    return qs


def scale(q, omps):
    n = {k: np.sqrt(abs(O.overlap(m, m))) for k, m in omps.items()}
    if q[0] == "amp":
        return n[q[1]]
    if q[0] == "exp":
        return np.linalg.norm(q[2][1])
    return n[q[1]] * n[q[2]]


def oracle_value(q, omps):
    if q[0] == "amp":
        vecs = [np.eye(2, dtype=np.complex128)[b] for b in q[2]]
        return O.amplitude(vecs, omps[q[1]])
    if q[0] == "exp":
        return O.expectation(omps[q[1]], q[2][0], q[2][1])
    return O.overlap(omps[q[1]], omps[q[2]])


def submit(srv, ids, q):
    if q[0] == "amp":
        return srv.submit_amplitude(ids[q[1]], bits=q[2])
    if q[0] == "exp":
        return srv.submit_expectation(ids[q[1]], q[2][0], q[2][1])
    return srv.submit_overlap(ids[q[1]], ids[q[2]])


def test_pool_norms_match_oracle(pool):
    srv, ids, omps = pool
    for k, mid in ids.items():
        ref = O.overlap(omps[k], omps[k]).real
        assert abs(srv.info(mid)["norm2"] - ref) <= 1e-12 * ref


def test_queries_alone_match_oracle(pool):
    srv, ids, omps = pool
    for q in make_queries(ids, omps, seed=1):
        val, lat = srv.wait(submit(srv, ids, q))
        ref = oracle_value(q, omps)
        assert abs(val - ref) <= 1e-12 * scale(q, omps), (q[0], q[1], val, ref)
        assert lat > 0


def test_mix_equals_alone(pool):
    """Every query submitted alone, then all of them (each twice) from four threads at
    once: the batched results equal the lone ones, and batching did happen."""
    srv, ids, omps = pool
    qs = make_queries(ids, omps, seed=2, n_amp=6, n_exp=4)
    alone = [srv.wait(submit(srv, ids, q))[0] for q in qs]
    before = srv.stats()
    order = list(range(len(qs))) * 2
    np.random.default_rng(3).shuffle(order)
    tickets = [None] * len(order)
    go = threading.Event()

    def client(part):
        go.wait()
        for pos in part:
            tickets[pos] = submit(srv, ids, qs[order[pos]])

    threads = [threading.Thread(target=client, args=(range(t, len(order), 4),)) for t in range(4)]
    for th in threads:
        th.start()
    go.set()
    for th in threads:
        th.join()
    mixed = [srv.wait(t)[0] for t in tickets]
    for pos, qi in enumerate(order):
        q = qs[qi]
        assert abs(mixed[pos] - alone[qi]) <= 1e-13 * scale(q, omps), (q[0], mixed[pos], alone[qi])
        assert abs(mixed[pos] - oracle_value(q, omps)) <= 1e-12 * scale(q, omps)
    after = srv.stats()
    assert after["completed"] - before["completed"] == len(order)
    assert after["max_batch"] > 1


def test_admission_waits_for_workspace():
    """An overlap at χ=64 needs 256 KiB of workspace, so a 1 MiB arena runs at most four
    at once: a burst of 24 is admitted in pieces as jobs return their blocks, and every
    result is still right."""
    from tenetgb import serve

    with serve.Server(work_bytes=1 << 20, max_batch=64) as srv:
        a = srv.add_random_mps(14, 64, seed=9)
        b = srv.add_random_mps(14, 64, seed=10)
        pa, pb = O.OMPS(srv.sites(a)), O.OMPS(srv.sites(b))
        ref_ab, ref_ba = O.overlap(pa, pb), O.overlap(pb, pa)
        ts = [(srv.submit_overlap(a, b), ref_ab) if k % 2 == 0 else (srv.submit_overlap(b, a), ref_ba)
              for k in range(24)]
        vals = [(srv.wait(t)[0], ref) for t, ref in ts]
        st = srv.stats()
        assert st["deferred"] > 0
        scale = np.sqrt(abs(O.overlap(pa, pa)) * abs(O.overlap(pb, pb)))
        for v, ref in vals:
            assert abs(v - ref) <= 1e-12 * scale


def test_errors_and_budget():
    from tenetgb import serve

    with serve.Server(hbm_budget=64 << 20, work_bytes=2 << 20) as srv:
        a = srv.add_random_mps(8, 8, seed=1)
        b = srv.add_random_mps(9, 8, seed=2)
        with pytest.raises(ValueError):
            srv.submit_amplitude(99, bits=[0] * 8)
        with pytest.raises(ValueError):
            srv.submit_expectation(a, 9, np.eye(2))
        with pytest.raises(ValueError):
            srv.submit_overlap(a, b)  # lengths differ
        with pytest.raises(MemoryError):
            srv.add_random_mps(64, 512, seed=3)  # ≈ 0.5 GB > the 64 MiB budget
        big = srv.add_random_mps(12, 64, seed=4)
        # an expectation query at χ=64 needs 2·64·2·64·16 B = 256 KiB: fits in 2 MiB
        assert np.isfinite(abs(srv.expectation(big, 6, np.eye(2))))
        srv.remove_mps(big)
        with pytest.raises(ValueError):
            srv.submit_amplitude(big, bits=[0] * 12)
        st = srv.stats()
        assert st["pending"] == 0 and st["in_flight"] == 0


def test_query_larger_than_workspace_is_refused():
    from tenetgb import serve

    with serve.Server(work_bytes=1 << 20) as srv:
        a = srv.add_random_mps(16, 256, seed=5)
        b = srv.add_random_mps(16, 256, seed=6)
        with pytest.raises(MemoryError):  # an overlap at χ=256 needs 4 MiB of workspace
            srv.submit_overlap(a, b)
        assert abs(srv.expectation(a, 8, np.eye(2)) - 1.0) <= 1e-12  # needs a few KiB
        assert np.isfinite(abs(srv.amplitude(a, [1] * 16)))


def test_remove_while_queries_run():
    """Removing an MPS with queries in flight waits for them; queries still waiting
    fail with ValueError; nothing else is disturbed."""
    from tenetgb import serve

    rng = np.random.default_rng(6)
    with serve.Server(work_bytes=64 << 20) as srv:
        keep = srv.add_random_mps(12, 32, seed=7)
        gone = srv.add_random_mps(12, 32, seed=8)
        ts = []
        for _ in range(30):
            ts.append(("gone", srv.submit_amplitude(gone, bits=rng.integers(0, 2, 12))))
            ts.append(("keep", srv.submit_overlap(keep, keep)))
        srv.remove_mps(gone)
        ok = failed = 0
        for who, t in ts:
            try:
                v, _ = srv.wait(t)
                ok += 1
                if who == "keep":
                    assert abs(v - srv.info(keep)["norm2"]) <= 1e-12 * abs(v)
            except ValueError:
                assert who == "gone"
                failed += 1
        assert ok + failed == len(ts)


def test_mixed_precision_server_within_fp32_tolerance(pool):
    """A mixed server (FP32 amplitude chains and overlap sweeps, FP64 ⟨O_i⟩) agrees with
    the oracle to 1e-5 of each value's scale (FP32 products over ≤ 13 sites), and its
    batched results equal its lone results exactly."""
    from tenetgb import serve

    _, _, omps = pool
    with serve.Server(work_bytes=256 << 20, precision="mixed") as srv:
        ids = {k: srv.add_mps(m.sites) for k, m in omps.items()}
        qs = make_queries(ids, omps, seed=5, n_amp=3, n_exp=2)
        alone = [srv.wait(submit(srv, ids, q))[0] for q in qs]
        tickets = [submit(srv, ids, q) for q in qs]
        mixed = [srv.wait(t)[0] for t in tickets]
        for q, a, m in zip(qs, alone, mixed):
            ref = oracle_value(q, omps)
            tol = 1e-12 if q[0] == "exp" else 1e-5
            assert abs(a - ref) <= tol * scale(q, omps), (q[0], a, ref)
            assert a == m
