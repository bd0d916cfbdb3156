"""Multi-GPU form of the benchmark: replicas only (every rank evaluates its own copy of the
workload; no collective on the data path).  The cross-rank bookkeeping -- the maximum of the
ranks' timings and the whole-job throughput -- checked with two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r: 0.10 + 0.05 r ms for the FP32 step, 1.0 + 0.1 r for FP64, 0.2 - 0.01 r end to end
        mine = [0.10 + 0.05 * rank, 1.0 + 0.1 * rank, 0.2 - 0.01 * rank]
        got = bench.max_over_ranks(mine, world, "cpu")
        out.put((rank, got, bench.replica_throughput(4096, world, got[0])))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_throughput_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    world, port = 2, _free_port()
    out = mp.Queue()
    procs = [mp.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    results = sorted(out.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, got, value in results:
        assert got == pytest.approx([0.15, 1.1, 0.2])
        assert value == pytest.approx(4096 * 2 / 0.15e-3)


def test_single_rank_is_the_identity():
    pytest.importorskip("torch")
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks([0.3, 2.0], 1, "cpu") == [0.3, 2.0]
    assert bench.replica_throughput(100, 1, 0.5) == pytest.approx(2e5)
