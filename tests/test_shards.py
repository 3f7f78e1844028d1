"""Row-range shards and their k-way merge (distributed/build_shards.py, coordinator.py:27-37).

CPU only: the shards' local searches are the oracle (the reference's CPU algorithm), so a merge
over any split of the rows must equal the oracle over all rows, bit for bit. The multi-rank path
runs as two gloo processes on 127.0.0.1, with a failure injected on the host (a rank whose local
search raises).
"""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from oracle import oracle as O
from vecsearch_gb300 import datasets as D
from vecsearch_gb300.shards import ShardedIndex, merge_shard_lists, shard_bounds


class OracleShard:
    """A CPU stand-in for one rank's GpuBruteForceIndex (same add / search / len interface)."""

    def __init__(self, dim, metric, fail=False):
        self.dim, self.metric, self.fail = dim, metric, fail
        self.x = np.zeros((0, dim), np.float32)

    def add(self, x):
        self.x = np.concatenate([self.x, np.asarray(x, np.float32)])

    def __len__(self):
        return len(self.x)

    def search(self, q, k, method="auto", filter=None):
        if self.fail:
            raise RuntimeError("injected shard failure")
        allowed = None if filter is None else np.asarray(filter, dtype=bool)
        ids, dists = O.search(self.x, q, k, self.metric, allowed=allowed)
        return O.ids_to_int64(ids), dists


def _full(x, q, k, metric, allowed=None):
    ids, dists = O.search(x, q, k, metric, allowed=allowed)
    return O.ids_to_int64(ids), dists


def test_bounds():
    assert shard_bounds(10, 3).tolist() == [0, 3, 6, 10]
    assert shard_bounds(2, 4).tolist() == [0, 0, 1, 1, 2]
    with pytest.raises(ValueError):
        shard_bounds(5, 0)


@pytest.mark.parametrize("metric", ["ip", "l2"])
@pytest.mark.parametrize("shards", [1, 3, 7])
def test_merge_equals_unsharded(metric, shards):
    x = D.portable(3000, 40, 5, normalize=metric == "ip")
    q = D.portable(9, 40, 6, normalize=metric == "ip")
    b = shard_bounds(len(x), shards)
    lists = []
    for s in range(shards):
        lo, hi = int(b[s]), int(b[s + 1])
        ids, dists = _full(x[lo:hi], q, 10, metric)
        lists.append((np.where(ids >= 0, ids + lo, -1), dists))
    got_i, got_d = merge_shard_lists(lists, 10)
    want_i, want_d = _full(x, q, 10, metric)
    np.testing.assert_array_equal(got_i, want_i)
    np.testing.assert_array_equal(got_d.view(np.uint32), want_d.view(np.uint32))


def test_merge_ties_padding_and_failures():
    # equal distances across shards go to the lower id; pads sort last; None shards are skipped
    a = (np.array([[7, -1]]), np.array([[0.5, np.inf]], np.float32))
    b = (np.array([[3, 9]]), np.array([[0.5, 0.7]], np.float32))
    i, d = merge_shard_lists([a, None, b], 4)
    assert i.tolist() == [[3, 7, 9, -1]]
    assert d[0, :3].tolist() == [0.5, 0.5, np.float32(0.7)] and np.isinf(d[0, 3])
    i, d = merge_shard_lists([a], 0)
    assert i.shape == (1, 0)
    with pytest.raises(RuntimeError, match="all shards failed"):
        merge_shard_lists([None, None], 3)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        x = D.portable(2500, 24, 11)
        q = D.portable(6, 24, 12)
        mask = D.portable_mask(len(x), 0.3, seed=13)
        idx = ShardedIndex(24, "l2", local=OracleShard(24, "l2"))
        idx.add(x)
        plain = idx.search(q, 12)
        filt = idx.search(q, 12, filter=mask)
        # add_local with the total found by an all-reduce
        idx2 = ShardedIndex(24, "l2", local=OracleShard(24, "l2", fail=(rank == 1)))
        b = shard_bounds(len(x), world)
        idx2.add_local(x[b[rank]:b[rank + 1]], int(b[rank]))
        partial = idx2.search(q, 12)
        idx3 = ShardedIndex(24, "l2", local=OracleShard(24, "l2", fail=(rank == 1)), strict=True)
        idx3.add(x)
        try:
            idx3.search(q, 5)
            strict = "no error"
        except RuntimeError as e:
            strict = str(e)
        np.savez(os.path.join(out_dir, f"r{rank}.npz"), pi=plain[0], pd=plain[1], fi=filt[0], fd=filt[1],
                 xi=partial[0], xd=partial[1], total=len(idx2), failed=np.array(idx2.failed), strict=strict)
    finally:
        dist.destroy_process_group()


def test_two_rank_gloo(tmp_path):
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    x = D.portable(2500, 24, 11)
    q = D.portable(6, 24, 12)
    mask = D.portable_mask(len(x), 0.3, seed=13)
    want_i, want_d = _full(x, q, 12, "l2")
    fw_i, fw_d = _full(x, q, 12, "l2", allowed=mask.astype(bool))
    b = shard_bounds(len(x), world)
    r0_i, r0_d = _full(x[:b[1]], q, 12, "l2")
    for r in range(world):
        z = np.load(tmp_path / f"r{r}.npz")
        np.testing.assert_array_equal(z["pi"], want_i)
        np.testing.assert_array_equal(z["pd"].view(np.uint32), want_d.view(np.uint32))
        np.testing.assert_array_equal(z["fi"], fw_i)
        np.testing.assert_array_equal(z["fd"].view(np.uint32), fw_d.view(np.uint32))
        # rank 1 failed: the answer is rank 0's shard alone, and both ranks know it
        np.testing.assert_array_equal(z["xi"], r0_i)
        assert int(z["total"]) == len(x)
        assert z["failed"].tolist() == [False, True]
        assert str(z["strict"]) == ("shards [1] failed" if r == 0 else "injected shard failure")
