"""The multi-rank path of bench.py on the CPU: two gloo ranks (world size 2, 127.0.0.1)
reduce their timings with max_over_ranks and report the whole-job rate of weak scaling
(every rank solves its own pair, no collective on the data path)."""
import json
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import torch
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    w, r, local = bench.rank_info()
    ms = 5.0 + 2.0 * r                      # rank 1 is the slow one
    ms_max = bench.max_over_ranks(ms, w, torch.device("cpu"))
    dist.barrier()
    rate = bench.whole_job_rate(w, 254016, ms_max)
    Path(out_dir, f"rank{r}.json").write_text(json.dumps({"world": w, "rank": r, "local": local, "ms_max": ms_max,
                                                          "rate": rate}))
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest(tmp_path):
    torch = pytest.importorskip("torch")
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    torch.multiprocessing.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    got = [json.loads((tmp_path / f"rank{r}.json").read_text()) for r in range(2)]
    for r, g in enumerate(got):
        assert g["world"] == 2 and g["rank"] == r and g["local"] == r
        assert g["ms_max"] == 7.0                       # every rank sees the slowest rank's time
        assert g["rate"] == pytest.approx(2 * 254016 / 7e-3)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks(3.5, 1, None) == 3.5
    assert bench.whole_job_rate(1, 1000, 2.0) == pytest.approx(5e5)
