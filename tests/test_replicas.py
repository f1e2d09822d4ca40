"""The multi-GPU path of bench.py: independent replicas (one system per
rank, no collective on the data path), the step time reduced as the maximum
over ranks, rank 0 alone printing; the reference arm runs on rank 0 only.
Two gloo ranks on the CPU stand in for the GPUs."""
import json
import os
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _rank_main(rank, world, port, out):
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    import bench
    got = bench.max_over_ranks(1.5 + rank, world)
    dist.barrier()
    dist.destroy_process_group()
    Path(out, f"r{rank}.json").write_text(json.dumps({"rank": rank, "max": got}))


def test_max_over_ranks_on_two_gloo_ranks(tmp_path):
    port = 29500 + os.getpid() % 1000
    mp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    res = [json.loads(Path(tmp_path, f"r{r}.json").read_text()) for r in range(2)]
    assert [r["max"] for r in res] == [2.5, 2.5]


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks(3.25, 1) == 3.25


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, str(ROOT))
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--levels", "3"])
    bench.run_reference(bench.parse())
    assert capsys.readouterr().out == ""  # rank 1 exits without work or output
