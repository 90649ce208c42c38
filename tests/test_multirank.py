"""Several GPUs run disjoint replica sets (replicas only): the host-side
bookkeeping that crosses ranks (mcx/shard.py), checked on CPU with gloo and
world size 2 -- the replica shards, the slowest-rank time, and the
law-of-total-variance combination of every rank's po.dat rows against the
oracle's restatement of the reference's average_replicas.py."""
import json
import os
import socket
import sys

import numpy as np
import pytest

from oracle import replicas as OR

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "mclics-backend_gb300"))

from mcx import shard  # noqa: E402  (pure host code: no GPU, no library load)


def _rows(n, seed=5, pear=False):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        S = float(rng.uniform(0.2, 0.8))
        r = [1.1, S, float(rng.uniform(1e-5, 1e-3)), -9 * S + float(rng.normal(0, 0.1)), float(rng.uniform(1e-4, 1e-2))]
        if pear:
            r.append(float(rng.uniform(0, 0.5)))
        out.append(r)
    return out


def test_shard_partitions_every_replica_once():
    for n in range(0, 23):
        for world in range(1, 6):
            parts = [shard.shard(n, world, r) for r in range(world)]
            flat = [i for p in parts for i in p]
            assert flat == list(range(n))
            sizes = [len(p) for p in parts]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard.shard(4, 2, 2)


@pytest.mark.parametrize("pear", [False, True])
def test_combine_rows_matches_oracle(pear):
    rows = _rows(9, pear=pear)
    np.testing.assert_allclose(shard.combine_rows(rows), OR.combine([[r] for r in rows])[0], rtol=1e-13)
    bad = [list(r) for r in rows]
    bad[3][0] += 0.01
    with pytest.raises(ValueError):
        shard.combine_rows(bad)


def test_po_row_matches_oracle():
    st = [40, 22.0, 12.5, -200.0, 1001.0]
    assert shard.po_row(1.05, st, 0.3) == pytest.approx(OR.po_row(1.05, st, 0.3))
    with pytest.raises(ValueError):
        shard.po_row(1.0, [0, 0, 0, 0, 0])


def _worker(rank, world, port, rows, out_dir):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = [rows[i] for i in shard.shard(len(rows), world, rank)]
        res = {"combined": shard.combine_across_ranks(mine), "slowest": shard.max_over_ranks(10.0 + rank)}
        with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
            json.dump(res, f)
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_ranks_gloo(tmp_path):
    import torch.multiprocessing as tmp
    rows = _rows(7)
    tmp.spawn(_worker, args=(2, _free_port(), rows, str(tmp_path)), nprocs=2, join=True)
    want = OR.combine([[r] for r in rows])[0]
    for rank in range(2):
        res = json.load(open(tmp_path / f"rank{rank}.json"))
        np.testing.assert_allclose(res["combined"], want, rtol=1e-13)
        assert res["slowest"] == 11.0
