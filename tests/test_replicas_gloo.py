"""The N > 1 path of bench.py on CPU: two ranks over gloo (127.0.0.1) set up
their process group through bench.dist_setup and combine replica results with
bench.aggregate: units are summed over ranks, time is the maximum over ranks
(whole-job throughput of independent replicas; no data-path collective)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

torch = pytest.importorskip("torch")
mp = pytest.importorskip("torch.multiprocessing")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "KZ_BENCH_BACKEND": "gloo"})
    sys.path.insert(0, ROOT)
    import bench
    r, w, dist = bench.dist_setup(world)
    assert (r, w) == (rank, world) and dist is not None
    # replica k traced (k + 1) * 1e6 path bounces in (k + 2) seconds
    units, secs = bench.aggregate((rank + 1) * 1e6, float(rank + 2), dist)
    dist.barrier()
    out.put((rank, units, secs))
    dist.destroy_process_group()


def test_two_replicas_aggregate_over_gloo():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(k, world, port, q)) for k in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, units, secs in res:
        assert units == pytest.approx(3e6)   # sum over ranks
        assert secs == pytest.approx(3.0)    # max over ranks
    assert [r for r, _, _ in res] == [0, 1]


def test_single_process_needs_no_group(monkeypatch):
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    sys.path.insert(0, ROOT)
    import bench
    assert bench.dist_setup(1) == (0, 1, None)
    assert bench.aggregate(5.0, 2.0, None) == (5.0, 2.0)
