"""bench.py's replica path (one process per GPU, no data-path collective) on CPU: two
gloo ranks take each timing's maximum over the ranks and report the whole-job
throughput, as torchrun runs it on N GPUs."""

import multiprocessing as mp
import os
import socket
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2",
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=2)
    ws, r, local = bench.dist_env()
    local_times = [1.0 + rank, 3.0 - rank, 0.5]
    t = bench.max_over_ranks(local_times, ws)
    dist.barrier()
    dist.destroy_process_group()
    q.put((r, ws, local, t, bench.replica_throughput(ws, 16, 3, t[0])))


def test_two_gloo_ranks_reduce_to_the_slowest():
    with socket.socket() as sck:
        sck.bind(("127.0.0.1", 0))
        port = sck.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict((r, (ws, local, t, v)) for r, ws, local, t, v in (q.get(timeout=120) for _ in range(2)))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in (0, 1):
        ws, local, t, v = got[r]
        assert ws == 2 and local == r
        assert t == [2.0, 3.0, 0.5]  # each timing's maximum over the ranks
        assert abs(v - 2 * 16 * 3 / 2.0) < 1e-12


def test_one_rank_is_the_identity():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks([1.5, 2.5], 1) == [1.5, 2.5]
    assert bench.replica_throughput(1, 16, 3, 2.0) == 24.0
