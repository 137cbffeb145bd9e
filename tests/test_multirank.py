"""The benchmark's N > 1 path on CPU: ranks are independent replicas, and the
whole-job figure is every rank's points over the slowest rank's time. Two
`gloo` ranks (127.0.0.1) all-reduce different step times; both must see the
maximum, and the reference arm does its work on rank 0 only."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = 100.0 + 25.0 * rank  # rank 1 is the slow one
    got = bench.max_over_ranks(ms, world, "cpu")
    dist.barrier()
    dist.destroy_process_group()
    with open(os.path.join(out_dir, f"r{rank}"), "w") as f:
        f.write(repr(got))


def test_max_over_ranks_gloo_world_2(tmp_path):
    import torch.multiprocessing as mp
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world,
                       start_method="spawn", join=True)
    vals = [float(open(tmp_path / f"r{r}").read()) for r in range(world)]
    assert vals == [125.0, 125.0]


def test_replica_value_and_single_rank():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(42.5, 1) == 42.5
    # 60,800 points on each of 2 ranks, slowest rank 1.0 s per step
    assert bench.replica_value(60800, 2, 1000.0) == pytest.approx(121600.0)


def test_reference_arm_runs_on_rank_0_only(capsys):
    sys.path.insert(0, ROOT)
    import bench

    class Args:
        config = 2
        ref_sample = 1
        warmup = 0
        steps = 1

    assert bench.run_reference(Args(), 1, 2) is None
    assert capsys.readouterr().out == ""
