"""bench.py's multi-process form: one replica per rank, the slowest rank's
times (max over ranks) and whole-job rates; world_size 2 over gloo on the
CPU, as torchrun would launch it (rendezvous on 127.0.0.1)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist

    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        assert bench.dist_info() == (rank, rank, world)
        # rank r is slower on the first value, faster on the second
        got = bench.max_over_ranks([10.0 + rank, 5.0 - rank], dist)
        q.put((rank, got))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_replica_rate_world_2():
    torch = pytest.importorskip("torch")
    import bench

    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = dict(q.get(timeout=10) for _ in range(2))
    assert res[0] == res[1] == [11.0, 5.0]
    # two replicas of 1M units each, the slowest taking 11 ms
    assert bench.replica_rate(1_000_000, 11.0, 2) == pytest.approx(2e6 / 11e-3 / 1e6)
    assert bench.replica_rate(5, 0.0, 2) == 0.0


def test_one_process_needs_no_collective():
    pytest.importorskip("torch")
    import bench

    assert bench.max_over_ranks([3.0, 4.5]) == [3.0, 4.5]


def test_search_kernel_bytes_follow_the_oracle_counts():
    """The search kernel's algorithmic bytes use the oracle's node-record count
    when given (32 B each), else three records per search."""
    import bench

    m = 100_000
    sched = bench.reinsertion_schedule(2 * m - 1)
    searched = sum(s for _, s in sched)
    lower = bench.kernel_byte_models(m, 1_000_000, 10_000, m)["k_find"]
    counted = bench.kernel_byte_models(m, 1_000_000, 10_000, m, search_nodes=searched * 46)["k_find"]
    assert lower == searched * (4 + 16) + searched * 3 * 32
    assert counted == searched * (4 + 16) + searched * 46 * 32
