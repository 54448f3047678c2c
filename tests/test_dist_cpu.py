"""The multi-rank path of bench.py on CPU: world size 2 over gloo (replicas of the
projection workload; the batch sharded by a host-side partition with no data exchange)."""
import os
import socket
import sys

import pytest

from conftest import ROOT

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, ws, port, out_path):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    w, r, _ = bench.dist_env()
    dist = bench.init_dist(w)
    m = bench.max_over_ranks(dist, 1.5 + r)
    bench.barrier(dist)
    mine = bench.shard(256, r, w)
    counts = torch.tensor([len(mine)], dtype=torch.float64)
    dist.all_reduce(counts)
    with open(f"{out_path}.{rank}", "w") as f:
        f.write(f"{m} {int(counts.item())} {min(mine)} {','.join(map(str, mine[:3]))}\n")
    dist.destroy_process_group()


def test_two_ranks_over_gloo(tmp_path):
    mp = torch.multiprocessing.get_context("spawn")
    port = _free_port()
    out = str(tmp_path / "rank")
    procs = [mp.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    lines = [open(f"{out}.{r}").read().split() for r in range(2)]
    assert all(float(l[0]) == 2.5 for l in lines)         # max over ranks
    assert all(int(l[1]) == 256 for l in lines)            # the shards cover the batch once
    assert lines[0][3] == "0,2,4" and lines[1][3] == "1,3,5"


def test_shard_partitions_without_overlap():
    sys.path.insert(0, ROOT)
    import bench
    for ws in (1, 2, 3, 8):
        parts = [bench.shard(37, r, ws) for r in range(ws)]
        flat = sorted(k for p in parts for k in p)
        assert flat == list(range(37))
