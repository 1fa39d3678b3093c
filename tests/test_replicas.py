"""The multi-GPU arm of the benchmark runs independent replicas (the step does not shard on
this one-GPU-per-box pool): each rank advances its own copy of the workload, and the job's
rate is every rank's cells over the slowest rank's time.  That reduction runs here as two
gloo ranks on the CPU."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, ws, port, ms_of_rank, out):
    import torch.distributed as tdist
    sys.path.insert(0, ROOT)
    import bench
    tdist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=ws)
    try:
        value, ms = bench.aggregate_rate(ms_of_rank[rank], cells=256 ** 3, steps=20, ws=ws, device="cpu")
        out.put((rank, value, ms))
    finally:
        tdist.destroy_process_group()


def test_replica_rate_uses_the_slowest_rank_and_every_ranks_cells():
    torch = pytest.importorskip("torch")
    import socket
    mp = torch.multiprocessing.get_context("spawn")
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ws = 2
    ms_of_rank = [231.0, 244.5]
    q = mp.Queue()
    procs = [mp.Process(target=_worker, args=(r, ws, port, ms_of_rank, q)) for r in range(ws)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in range(ws))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    expect = ws * 256 ** 3 * 20 / (max(ms_of_rank) / 1e3)
    for rank, value, ms in got:
        assert ms == max(ms_of_rank)
        assert value == pytest.approx(expect, rel=1e-12)


def test_single_rank_rate_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    value, ms = bench.aggregate_rate(11.5, cells=1000, steps=4, ws=1, device="cpu")
    assert ms == 11.5 and value == pytest.approx(1000 * 4 / 11.5e-3)
