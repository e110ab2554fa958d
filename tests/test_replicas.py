"""The N > 1 path of bench.py (independent replicas, one GPU each): two gloo
ranks on the CPU share the barrier and the maximum of their timings, and the
whole-job rate is all ranks' units over the slowest rank's time."""
import importlib.util
import os
import socket

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_for_replicas", os.path.join(REPO, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench = _bench()
        bench.sync_ranks(dist)
        seconds = 1.5 + rank  # rank 1 is the slower replica
        slowest = bench.max_over_ranks(seconds, dist)
        out.put((rank, slowest, bench.replica_rate(100, slowest, world)))
        bench.sync_ranks(dist)
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas_share_the_slowest_time():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    q = mp.Queue()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [2.5, 2.5]
    assert all(abs(r[2] - 2 * 100 / 2.5) < 1e-12 for r in res)


def test_single_rank_needs_no_process_group():
    bench = _bench()
    assert bench.max_over_ranks(3.0, None) == 3.0
    assert bench.replica_rate(10, 2.0, 1) == 5.0
