"""Row-range shards of one exact index, one per rank, and the k-way merge of their results.

The reference splits a base into contiguous row ranges (distributed/build_shards.py:18-29); each
shard worker adds its range's first row to its local ids (distributed/shard_worker.py:35); the
coordinator merges the shards' sorted (dist, id) lists and skips shards that failed, so a partial
answer beats none (distributed/coordinator.py:27-37).

Here a rank is one process with one GPU holding one range in its own :class:`GpuBruteForceIndex`.
A search runs on every rank at once; the one exchange is an all-gather of each rank's nq x k
(dist, id) lists and a status flag (nq * k * 12 bytes + 8 per rank), after which every rank
merges the live shards' lists by (dist, id) on the host. Shards partition the rows, so the
per-rank work is fixed as ranks are added (weak scaling at a fixed rows-per-rank).
"""
import numpy as np

__all__ = ["shard_bounds", "merge_shard_lists", "ShardedIndex"]


def shard_bounds(n, shards):
    """Row bounds of `shards` contiguous ranges over n rows (build_shards.py:18-20)."""
    if shards < 1:
        raise ValueError("shards must be >= 1")
    return np.linspace(0, n, shards + 1, dtype=np.int64)


def merge_shard_lists(lists, k):
    """Merge per-shard results into the global top-k.

    lists: one entry per shard, either None (the shard failed; it is skipped as the reference's
    coordinator skips it) or (ids int64 [nq, ks], dists float32 [nq, ks]) with GLOBAL ids, -1 and
    +inf marking missing entries. Returns (ids int64 [nq, k], dists float32 [nq, k]) ordered by
    (dist, id) - the order of heapq.merge over (dist, id) tuples - padded with -1 / +inf.
    Raises RuntimeError when every shard failed ("all shards failed", coordinator.py:35-36).
    """
    live = [e for e in lists if e is not None]
    if not live:
        raise RuntimeError("all shards failed")
    k = int(k)
    ids = np.concatenate([np.asarray(i, dtype=np.int64).reshape(np.shape(i)[0], -1) for i, _ in live], axis=1)
    dists = np.concatenate([np.asarray(d, dtype=np.float32).reshape(np.shape(d)[0], -1) for _, d in live], axis=1)
    nq = ids.shape[0]
    out_i = np.full((nq, k), -1, dtype=np.int64)
    out_d = np.full((nq, k), np.inf, dtype=np.float32)
    if ids.shape[1] == 0 or k == 0:
        return out_i, out_d
    # Missing entries (-1) sort after every real row at the same distance (+inf).
    id_key = np.where(ids < 0, np.iinfo(np.int64).max, ids)
    order = np.lexsort((id_key, dists), axis=-1)
    take = min(k, ids.shape[1])
    sel = order[:, :take]
    out_i[:, :take] = np.take_along_axis(ids, sel, axis=1)
    out_d[:, :take] = np.take_along_axis(dists, sel, axis=1)
    out_i[~np.isfinite(out_d)] = -1
    return out_i, out_d


class ShardedIndex:
    """One contiguous row range per rank of a torch.distributed group; search merges all ranks.

    ``add(x)`` takes the FULL base on every rank and keeps rows [lo, hi) of this rank, or
    ``add_local(rows, offset)`` takes this rank's rows directly. ``search(queries, k, method,
    filter)`` must be called by every rank with the same queries and k; ``filter`` is a global
    mask (length = total rows) or per-query masks (nq x total rows). Each rank returns the merged
    global result. A rank whose local search raised still joins the gather with a failed flag
    and no lists, and its shard is skipped (``failed`` lists the flags of the last search); with
    ``strict=True`` every rank raises instead. ``local`` may be any object with the
    GpuBruteForceIndex ``add`` / ``search`` / ``len`` interface; by default it is one.
    """

    def __init__(self, dim, metric="l2", group=None, device=None, local=None, strict=False):
        import torch.distributed as dist
        self._dist = dist
        self._group = group
        self.rank = dist.get_rank(group)
        self.world = dist.get_world_size(group)
        if local is None:
            from . import GpuBruteForceIndex
            import torch
            local = GpuBruteForceIndex(dim, metric, device=torch.cuda.current_device() if device is None else device)
        self.local = local
        self.dim = dim
        self.metric = metric
        self.strict = strict
        self.offset = 0
        self.total = 0
        self.failed = [False] * self.world

    def _device(self):
        import torch
        if self._dist.get_backend(self._group) == "nccl":
            return torch.device("cuda", torch.cuda.current_device())
        return torch.device("cpu")

    def add(self, x):
        """Keep this rank's range of the full base x (the same x on every rank)."""
        b = shard_bounds(len(x), self.world)
        lo, hi = int(b[self.rank]), int(b[self.rank + 1])
        self.add_local(np.asarray(x)[lo:hi], lo, total=len(x))

    def add_local(self, rows, offset, total=None):
        """This rank's rows, whose first row has global id `offset`; `total` = rows over all ranks."""
        self.offset = int(offset)
        self.local.add(rows)
        if total is None:
            import torch
            t = torch.tensor([len(self.local)], dtype=torch.int64, device=self._device())
            self._dist.all_reduce(t, group=self._group)
            total = int(t.item())
        self.total = int(total)

    def __len__(self):
        return self.total

    def _local_filter(self, filter):
        if filter is None:
            return None
        f = np.asarray(filter)
        n = len(self.local)
        if f.shape[-1] != self.total:
            raise ValueError(f"filter must have {self.total} columns (one per row over all shards)")
        return f[..., self.offset:self.offset + n]

    def search(self, queries, k=10, method="auto", filter=None):
        import torch
        q = np.asarray(queries, dtype=np.float32)
        if q.ndim == 1:
            q = q.reshape(1, -1)
        nq, k = q.shape[0], int(k)
        status, error = 0, None
        try:
            ids, dists = self.local.search(q, k, method=method, filter=self._local_filter(filter))
            ids = np.where(ids >= 0, ids + self.offset, -1)
        except Exception as e:  # still joins the gather below, so the other ranks do not wait
            status, error = 1, e
            ids = np.full((nq, k), -1, dtype=np.int64)
            dists = np.full((nq, k), np.inf, dtype=np.float32)
        dev = self._device()
        ti = torch.from_numpy(np.ascontiguousarray(ids, dtype=np.int64)).to(dev)
        td = torch.from_numpy(np.ascontiguousarray(dists, dtype=np.float32)).to(dev)
        ts = torch.tensor([status], dtype=torch.int64, device=dev)
        gi = [torch.empty_like(ti) for _ in range(self.world)]
        gd = [torch.empty_like(td) for _ in range(self.world)]
        gs = [torch.empty_like(ts) for _ in range(self.world)]
        self._dist.all_gather(gs, ts, group=self._group)
        self._dist.all_gather(gi, ti, group=self._group)
        self._dist.all_gather(gd, td, group=self._group)
        failed = [int(s.item()) != 0 for s in gs]
        if self.strict and any(failed):
            if error is not None:
                raise error
            raise RuntimeError(f"shards {[r for r, f in enumerate(failed) if f]} failed")
        lists = [None if failed[r] else (gi[r].cpu().numpy(), gd[r].cpu().numpy()) for r in range(self.world)]
        self.failed = failed
        return merge_shard_lists(lists, k)
