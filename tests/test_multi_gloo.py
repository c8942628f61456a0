"""World-size-2 tests of the multi-GPU host logic on CPU (gloo backend):
sharding by longest-processing-time, max-over-ranks timing, and the gather
of per-rank results.  Each rank runs its shard through the oracle here (no
GPU in this container); on GPUs the shard goes through the C ABI."""
import os
import socket

import numpy as np
import pytest

from tweakseq_gb300 import multi
from tweakseq_gb300 import workloads as W


def test_lpt_shards_cover_and_balance():
    rng = np.random.default_rng(0)
    cells = rng.integers(1, 10_000_000, 5000)
    shards = multi.lpt_shards(cells, 4)
    allidx = np.concatenate(shards)
    assert len(allidx) == len(cells) and len(np.unique(allidx)) == len(cells)
    loads = [int(cells[s].sum()) for s in shards]
    # LPT: the spread is at most the largest item.
    assert max(loads) - min(loads) <= cells.max()
    assert multi.lpt_shards(cells, 1)[0].tolist() == list(range(len(cells)))
    # Deterministic: every rank computes the same split.
    again = multi.lpt_shards(cells, 4)
    assert all(np.array_equal(a, b) for a, b in zip(shards, again))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_path):
    import torch.distributed as dist

    from oracle import oracle as O

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ps = W.uneven_pairs(n_pairs=400, seed=21)
        cells = ps.a_len.astype(np.int64) * ps.b_len
        shard = multi.lpt_shards(cells, world)[rank]
        sub = ps.subset(shard)
        res = O.batch(sub.seqs, sub.a_off, sub.a_len, sub.b_off, sub.b_len, mode=O.MODE_SCORE, nthreads=2)
        table = multi.gather_table(res, shard, len(ps))
        slowest = multi.max_over_ranks(float(rank + 1))
        if rank == 0:
            np.save(out_path, table)
            with open(out_path + ".max", "w") as f:
                f.write(str(slowest))
        else:
            assert table is None
    finally:
        dist.destroy_process_group()


def test_two_ranks_shard_gather_and_time(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    from oracle import oracle as O

    O.build()
    out = str(tmp_path / "gathered.npy")
    port = _free_port()
    mp.spawn(_rank_main, args=(2, port, out), nprocs=2, join=True)
    gathered = np.load(out)
    ps = W.uneven_pairs(n_pairs=400, seed=21)
    want = O.batch(ps.seqs, ps.a_off, ps.a_len, ps.b_off, ps.b_len, mode=O.MODE_SCORE)
    assert np.array_equal(gathered["score"], want["score"])
    assert float(open(out + ".max").read()) == 2.0


def test_single_process_fallbacks():
    rows = np.zeros(3, dtype=[("score", np.int32)])
    rows["score"] = [7, 8, 9]
    out = multi.gather_table(rows, np.array([2, 0, 1]), 3)
    assert out["score"].tolist() == [8, 9, 7]
    assert multi.max_over_ranks(1.5) == 1.5
