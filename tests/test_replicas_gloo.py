"""The multi-GPU path of bench.py is replicas only: one independent grid per
rank, a barrier around the timed region, the slowest rank's time, and the
whole-job MLUPS summed over ranks.  This checks that host logic with two
gloo ranks on the CPU (no GPU, no collective on the data path)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
dist = pytest.importorskip("torch.distributed")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    bench.barrier(world)
    ms = bench.max_over_ranks(10.0 + 5.0 * rank, world, torch.device("cpu"))
    out.put((rank, ms, bench.replica_mlups(1000, 20, ms, world)))
    bench.barrier(world)
    dist.destroy_process_group()


def test_two_replicas_gloo():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # every rank sees the slowest rank's time; value counts both replicas' work
    assert [r[1] for r in res] == [15.0, 15.0]
    assert res[0][2] == pytest.approx(2 * 1000 * 20 / 0.015 / 1e6)


def test_single_rank_is_identity():
    import bench
    assert bench.max_over_ranks(3.5, 1, torch.device("cpu")) == 3.5
    assert bench.replica_mlups(2407500, 2000, 340.0, 1) == pytest.approx(2407500 * 2000 / 0.34 / 1e6)
