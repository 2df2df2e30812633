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


def _band_main(rank, world, port, out_dir):
    """One rank of the row-band split: its band of the queue (dic_split_rows), solved by the
    CPU oracle on a small pair, gathered to rank 0 over gloo and concatenated there."""
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import numpy as np
    import torch.distributed as dist
    import fasticgn_gb300 as dic
    from fasticgn_gb300 import speckle
    from oracle import oracle as O
    dist.init_process_group("gloo", rank=rank, world_size=world)
    pr = speckle.pair_affine(seed=3, width=160, height=144)
    q = dic.grid_queue(160, 144, 10, 5)
    starts = dic.split_rows(q, world)
    band = q[starts[rank]:starts[rank + 1]]
    pois = O.make_pois(band["x"], band["y"])
    O.run_pair(pr.ref.astype(np.float32), pr.tar.astype(np.float32), pois, 10, threads=1)
    parts = [None] * world
    dist.all_gather_object(parts, (int(starts[rank]), pois.tobytes()))
    if rank == 0:
        joined = b"".join(b for _, b in sorted(parts))
        whole = O.make_pois(q["x"], q["y"])
        O.run_pair(pr.ref.astype(np.float32), pr.tar.astype(np.float32), whole, 10, threads=1)
        Path(out_dir, "split.json").write_text(json.dumps({
            "starts": starts.tolist(), "n": len(q), "same": joined == whole.tobytes(),
            "band_rows": [sorted(set(q["y"][starts[k]:starts[k + 1]].tolist())) for k in range(world)]}))
    dist.barrier()
    dist.destroy_process_group()


def test_row_band_split_over_two_gloo_ranks(tmp_path):
    """The multi-GPU pair path's partition and concatenation, on the CPU: two gloo ranks take
    contiguous row bands of one queue (no row split between ranks, near-equal halves), solve
    them independently and the concatenation equals the single-process result byte for byte."""
    torch = pytest.importorskip("torch")
    import socket
    sys.path.insert(0, str(ROOT))
    from oracle import oracle as O
    O.lib()
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    torch.multiprocessing.spawn(_band_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    got = json.loads((tmp_path / "split.json").read_text())
    assert got["same"]
    s0, s1, s2 = got["starts"]
    assert s0 == 0 and s2 == got["n"] and abs(s1 - got["n"] / 2) <= 30      # 30 POIs per row
    assert not set(got["band_rows"][0]) & set(got["band_rows"][1])


def test_split_rows_partition_rules():
    """dic_split_rows on the CPU (no device is touched): boundaries at row starts, monotonic,
    covering the queue, for several part counts; an unsorted or single-row queue too."""
    sys.path.insert(0, str(ROOT))
    import numpy as np
    import fasticgn_gb300 as dic
    q = dic.grid_queue(300, 200, 7, 4)
    for parts in (1, 2, 3, 4, 8, 64):
        st = dic.split_rows(q, parts)
        assert st[0] == 0 and st[-1] == len(q) and np.all(np.diff(st) >= 0)
        for c in st[1:-1]:
            assert c in (0, len(q)) or q["y"][c] != q["y"][c - 1]
    one_row = dic.make_queue(np.arange(10, 50, 2), np.full(20, 30.0))
    assert dic.split_rows(one_row, 4).tolist() == [0, 20, 20, 20, 20]
    with pytest.raises(ValueError):
        dic.split_rows(q, 0)
