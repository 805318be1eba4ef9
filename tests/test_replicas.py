"""The multi-GPU form of the benchmark (replicas only: every rank runs its own
sessions on its own seeded scenes, no data-path collective) on CPU: two gloo
ranks reduce their timings to the slowest rank's, the whole-job rate counts
both ranks' frames over that time, and the ranks' seeds differ."""
from __future__ import annotations

import json
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out_dir: str) -> None:
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    res = {"max_ms": bench.rank_max(40.0 + 10.0 * rank), "seeds": bench.replica_seeds(rank)}
    dist.barrier()
    dist.destroy_process_group()
    Path(out_dir, f"rank{rank}.json").write_text(json.dumps(res))


def test_two_gloo_replicas(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    import bench

    world, port = 2, _free_port()
    mp.start_processes(_rank_main, args=(world, port, str(tmp_path)), nprocs=world, start_method="spawn", join=True)
    res = [json.loads((tmp_path / f"rank{r}.json").read_text()) for r in range(world)]
    assert [r["max_ms"] for r in res] == [50.0, 50.0]
    seeds = [r["seeds"] for r in res]
    for key in ("scene", "served", "batched"):
        assert seeds[0][key] != seeds[1][key]
    # 100 frames per rank over the slowest rank's 50 ms: 4000 frames/s for the job
    assert bench.whole_job_rate(world, 100, res[0]["max_ms"] * 1e-3) == pytest.approx(4000.0)
    assert bench.rank_max(7.0) == 7.0  # no process group: the value itself
