"""The multi-process (N > 1) path of bench.py on CPU: `gloo`, world size 2.
Every rank runs an independent replica; the job time is the slowest rank's and
the whole-job throughput counts every rank's evaluations.  The reference arm
runs on rank 0 only."""
import os
import sys

import pytest

torch = pytest.importorskip("torch")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    local_ms = 1000.0 * (rank + 1)  # rank 1 is the slow one
    rate, ms = bench.replica_throughput(local_ms, steps=4, world=world, dist=dist, device="cpu")
    out.put((rank, rate, ms))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_throughput_takes_the_slowest_rank():
    import socket
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, rate, ms in got:
        assert ms == pytest.approx(2000.0)
        assert rate == pytest.approx(2 * 4 / 2.0)


def test_single_process_throughput():
    sys.path.insert(0, ROOT)
    import bench
    rate, ms = bench.replica_throughput(500.0, steps=5, world=1)
    assert ms == 500.0 and rate == pytest.approx(10.0)


def test_reference_arm_is_rank0_only(capsys):
    sys.path.insert(0, ROOT)
    import bench

    class A:
        gpus, steps, warmup = 2, 1, 1
    bench.run_reference(A(), rank=1, world=2)
    assert capsys.readouterr().out == ""


def test_cpu_figures_scale_to_the_workload():
    """The CPU baseline scales the largest sampled sub-grid linearly in nodes to
    the benchmarked workload and reports the fitted cost exponent beside it."""
    sys.path.insert(0, ROOT)
    import bench
    # cost ~ n^2: 1 s at 1,000 nodes, 4 s at 2,000 nodes
    cb = bench._cpu_figures([(1000, 1.0), (2000, 4.0)], n_full=20000, passes=1)
    assert cb["cost_exponent"] == pytest.approx(2.0)
    assert cb["value"] == pytest.approx(1.0 / (4.0 * 10.0))          # linear in nodes from the largest sample
    assert cb["value_power_law"] == pytest.approx(1.0 / (4.0 * 100.0))
    assert cb["sample_evals_per_s"] == pytest.approx(0.25) and cb["sample_nodes"] == 2000
    assert cb["unit"] == "evals/s" and cb["kind"] == "port"
