"""The multi-process side of bench.py on CPU (gloo, world size 2): one process
per GPU, replicas only.  The whole-job time of a step is the maximum over the
ranks, and under a multi-rank launch the reference arm runs on rank 0 alone."""
import json
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    mine = [10.0 + rank, 5.0 - rank]          # this rank's step times (ms)
    got = bench.max_over_ranks(torch, mine, device="cpu")
    dist.barrier()
    dist.destroy_process_group()
    with open(os.path.join(out, f"r{rank}.json"), "w") as f:
        json.dump(got, f)


def test_step_time_is_max_over_ranks(tmp_path):
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    for r in range(world):
        with open(tmp_path / f"r{r}.json") as f:
            assert json.load(f) == [11.0, 5.0]


def test_reference_arm_runs_on_rank0_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    called = []
    monkeypatch.setattr(bench, "cpu_baseline_run", lambda *a, **k: called.append(a) or (1.0, 1))

    class Args:
        steps, warmup, ref_images, gpus = 1, 0, 1, 2
    bench.run_reference(Args())
    assert not called and capsys.readouterr().out == ""
