"""The N > 1 path of bench.py on the CPU: replicas over world_size-2 gloo ranks.

One scene does not shard (every pass would need a halo exchange), so
``bench.py --gpus N`` runs N independent replicas and reports the whole job:
every rank's particle-updates over the slowest rank's time.  The aggregation
is bench.whole_job_rate; here two gloo ranks with unequal times check it.
"""
from __future__ import annotations

import datetime
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, times_ms, out_dir: str) -> None:
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=60))
    import bench

    rate, ms = bench.whole_job_rate(1000 * 240, times_ms[rank], dist, device="cpu")
    dist.barrier()
    dist.destroy_process_group()
    Path(out_dir, f"rank{rank}.txt").write_text(f"{rate!r} {ms!r}")


@pytest.mark.timeout(120)
def test_whole_job_rate_over_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp

    times = (400.0, 500.0)
    mp.spawn(_rank, args=(2, _free_port(), times, str(tmp_path)), nprocs=2, join=True)
    for rank in range(2):
        rate, ms = (float(x) for x in (tmp_path / f"rank{rank}.txt").read_text().split())
        assert ms == 500.0                              # the slowest rank's time, on every rank
        assert rate == pytest.approx(2 * 1000 * 240 / 0.5)  # both replicas' updates over it


def test_whole_job_rate_one_process():
    sys.path.insert(0, str(ROOT))
    import bench

    rate, ms = bench.whole_job_rate(1000 * 240, 500.0)
    assert ms == 500.0 and rate == pytest.approx(1000 * 240 / 0.5)
