"""The multi-GPU path of bench.py is replicas only: every rank steps its own copy
of the workload and the whole-job figure is all ranks' particles over the
slowest rank's time.  Checked here with two gloo ranks on the CPU (no GPU), plus
the reference arm's rule that only rank 0 works under torchrun."""
import os
import socket
import sys

import pytest

from .conftest import ROOT

sys.path.insert(0, str(ROOT))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    value, slowest = bench.job_throughput(1000, 10, 0.1 * (rank + 1), world, device="cpu")
    out.put((rank, value, slowest))
    dist.barrier()
    dist.destroy_process_group()


def test_whole_job_throughput_over_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, value, slowest in res:
        assert slowest == pytest.approx(0.2)
        assert value == pytest.approx(2 * 1000 * 10 / 0.2)


def test_single_rank_is_its_own_job():
    import bench

    assert bench.job_throughput(1000, 10, 0.5, 1) == (20000.0, 0.5)


def test_reference_arm_only_on_rank_zero(monkeypatch):
    import bench

    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    assert bench.run_reference(None) is None
