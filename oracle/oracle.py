"""TEST INFRASTRUCTURE ONLY: Python access to the CPU oracle.

Used by tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg, as
the checker or the timed baseline - never by the product path.

* :func:`search` - the C restatement of the reference's
  ``BruteForceIndex::search_batch`` (src/brute_force.cpp:116-170) and of
  ``HNSWIndex::search_exact`` (src/hnsw.cpp:336-354) when a byte mask is given.
* :class:`Reference` - the reference's own CPU classes, compiled from its
  sources into ``oracle/_ref/`` (present only where the reference tree was).
* :func:`fp64_topk` - a float64 numpy oracle, top-k by (dist, id).
* :func:`check_ids` - the near-tie parity rule against the float64 oracle.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
NONE = 0xFFFFFFFF

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")

_lib = None


def _oracle_lib():
    global _lib
    if _lib is None:
        from oracle.build_ref import build_oracle
        lib = ctypes.CDLL(build_oracle())
        lib.vso_search.restype = ctypes.c_int
        lib.vso_search.argtypes = [_f32p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_int, _f32p,
                                   ctypes.c_size_t, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_int,
                                   _u32p, _f32p]
        lib.vso_pair_distances.restype = None
        lib.vso_pair_distances.argtypes = [_f32p, ctypes.c_size_t, ctypes.c_int, _f32p, ctypes.c_size_t,
                                           _u32p, ctypes.c_size_t, _f32p]
        _lib = lib
    return _lib


def _metric_code(metric):
    if metric == "l2":
        return 0
    if metric in ("ip", "cosine"):
        return 1
    raise ValueError(metric)


def search(x, q, k, metric="ip", num_threads=1, allowed=None):
    """Oracle top-k: (ids uint32 [nq,k] with 0xFFFFFFFF for missing, dists float32 [nq,k])."""
    x = np.ascontiguousarray(x, np.float32)
    q = np.ascontiguousarray(q, np.float32)
    nq, d = q.shape
    ids = np.empty((nq, k), np.uint32)
    dists = np.empty((nq, k), np.float32)
    mask_ptr = None
    if allowed is not None:
        allowed = np.ascontiguousarray(allowed, np.uint8)
        mask_ptr = allowed.ctypes.data
    rc = _oracle_lib().vso_search(x, x.shape[0], d, _metric_code(metric), q, nq, k, mask_ptr,
                                  num_threads, ids, dists)
    if rc != 0:
        raise MemoryError("oracle search failed")
    return ids, dists


def pair_distances(x, q, ids, metric="ip"):
    """Oracle distance for each (query, id) pair; +inf for missing ids."""
    x = np.ascontiguousarray(x, np.float32)
    q = np.ascontiguousarray(q, np.float32)
    ids = np.ascontiguousarray(ids, np.uint32)
    out = np.empty(ids.shape, np.float32)
    _oracle_lib().vso_pair_distances(x, x.shape[1], _metric_code(metric), q, q.shape[0], ids,
                                     ids.shape[1], out)
    return out


def ids_to_int64(ids):
    """uint32 ids with 0xFFFFFFFF for missing -> int64 with -1 (python/bindings.cpp:50-56)."""
    out = ids.astype(np.int64)
    out[ids == NONE] = -1
    return out


def fp64_distances(x, q, metric="ip", rows=None):
    """float64 distances [nq, n] (or [nq, len(rows)] for a row subset)."""
    x64 = np.asarray(x if rows is None else x[rows], np.float64)
    q64 = np.asarray(q, np.float64)
    if metric == "l2":
        d = (q64 * q64).sum(1)[:, None] + (x64 * x64).sum(1)[None, :] - 2.0 * (q64 @ x64.T)
        return np.maximum(d, 0.0)
    return 1.0 - q64 @ x64.T


def fp64_topk(x, q, k, metric="ip", allowed=None, chunk=65536):
    """float64 top-k by (dist, id) with int64 ids (-1 missing) and the float64 distances."""
    n = x.shape[0]
    nq = q.shape[0]
    best_d = np.full((nq, 0), np.inf)
    best_i = np.zeros((nq, 0), np.int64)
    for c0 in range(0, n, chunk):
        rows = np.arange(c0, min(n, c0 + chunk))
        if allowed is not None:
            rows = rows[np.asarray(allowed[c0:c0 + chunk]) != 0]
            if rows.size == 0:
                continue
        d = fp64_distances(x, q, metric, rows)
        ri = np.broadcast_to(rows, (nq, rows.size))
        kk = max(4 * k, k + 16)
        if rows.size > kk:
            # Preselect the kk smallest of the chunk per query (linear time); every row left out is
            # at or above the largest kept value, so when that value lies above the k-th smallest
            # kept one no row that ties the k-th is lost. Otherwise the whole chunk is sorted.
            part = np.argpartition(d, kk - 1, axis=1)[:, :kk]
            pd = np.take_along_axis(d, part, 1)
            kth = np.partition(pd, k - 1, axis=1)[:, k - 1]
            if np.all(pd.max(1) > kth):
                d, ri = pd, np.take_along_axis(ri, part, 1)
        cat_d = np.concatenate([best_d, d], 1)
        cat_i = np.concatenate([best_i, ri], 1)
        order = np.lexsort((cat_i, cat_d), axis=1)[:, :k]
        best_d = np.take_along_axis(cat_d, order, 1)
        best_i = np.take_along_axis(cat_i, order, 1)
    if best_d.shape[1] < k:
        pad = k - best_d.shape[1]
        best_d = np.concatenate([best_d, np.full((nq, pad), np.inf)], 1)
        best_i = np.concatenate([best_i, np.full((nq, pad), -1, np.int64)], 1)
    return best_i, best_d


def check_ids(got_ids, want_ids, x, q, metric="ip", rel=1e-6, abs_floor=0.0, rel_order=1e-5):
    """Parity rule: two top-k id lists may differ only at near-ties.

    An id in one list but not the other (a different top-k set) is allowed only at the k-th
    boundary: its float64 distance and the one it replaces lie within ``rel`` (relative, plus
    ``abs_floor``) of each other or of the k-th float64 distance of ``want``. Two ids that are in
    both lists but in swapped places (the same set, another order) are allowed when their float64
    distances lie within ``rel_order`` relative: FP32 sums in different orders (the reference's
    AVX2 loop, the GPU's lane split) can order such rows either way. Returns the number of
    tolerated disagreements; raises AssertionError on a real mismatch.
    """
    got_ids = np.asarray(got_ids, np.int64)
    want_ids = np.asarray(want_ids, np.int64)
    assert got_ids.shape == want_ids.shape, (got_ids.shape, want_ids.shape)
    tolerated = 0
    bad = np.nonzero((got_ids != want_ids).any(1))[0]
    for qi in bad:
        g, w = got_ids[qi], want_ids[qi]
        assert ((g >= 0) == (w >= 0)).all(), f"query {qi}: missing-result pattern differs"
        ids = np.union1d(g[g >= 0], w[w >= 0])
        d = dict(zip(ids.tolist(), fp64_distances(x, q[qi:qi + 1], metric, ids)[0].tolist()))
        kth = d[int(w[w >= 0][-1])]
        tol = rel * abs(kth) + abs_floor
        tol_order = rel_order * abs(kth) + abs_floor
        gs, ws = set(g.tolist()), set(w.tolist())
        for a, b in zip(g, w):
            if a == b:
                continue
            da, db = d[int(a)], d[int(b)]
            if int(a) in ws and int(b) in gs:  # the same rows, another order
                assert abs(da - db) <= tol_order, (
                    f"query {qi}: ids {a} (d64={da!r}) and {b} (d64={db!r}) swapped, tol={tol_order!r}")
            else:  # a different row at the k-th boundary
                assert abs(da - db) <= tol or (abs(da - kth) <= tol and abs(db - kth) <= tol), (
                    f"query {qi}: id {a} (d64={da!r}) vs {b} (d64={db!r}), k-th d64={kth!r}, tol={tol!r}")
            tolerated += 1
    return tolerated


class Reference:
    """The reference's own CPU classes (oracle/_ref/libvsref.so), or unavailable."""

    def __init__(self, path=None):
        path = path or os.path.join(HERE, "_ref", "libvsref.so")
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        lib = ctypes.CDLL(path)
        lib.vsref_bf_create.restype = ctypes.c_void_p
        lib.vsref_bf_create.argtypes = [ctypes.c_size_t, ctypes.c_int]
        lib.vsref_bf_destroy.argtypes = [ctypes.c_void_p]
        lib.vsref_bf_add.argtypes = [ctypes.c_void_p, _f32p, ctypes.c_size_t]
        lib.vsref_bf_search_batch.argtypes = [ctypes.c_void_p, _f32p, ctypes.c_size_t, ctypes.c_size_t,
                                              _u32p, _f32p, ctypes.c_int]
        lib.vsref_bf_search_one.restype = ctypes.c_size_t
        lib.vsref_bf_search_one.argtypes = [ctypes.c_void_p, _f32p, ctypes.c_size_t, _u32p, _f32p]
        lib.vsref_hnsw_create.restype = ctypes.c_void_p
        lib.vsref_hnsw_create.argtypes = [ctypes.c_size_t, ctypes.c_size_t, ctypes.c_int]
        lib.vsref_hnsw_destroy.argtypes = [ctypes.c_void_p]
        lib.vsref_hnsw_add.restype = ctypes.c_int
        lib.vsref_hnsw_add.argtypes = [ctypes.c_void_p, _f32p, ctypes.c_size_t, ctypes.c_int]
        lib.vsref_hnsw_search.argtypes = [ctypes.c_void_p, _f32p, ctypes.c_size_t, ctypes.c_size_t,
                                          ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t, _u32p, _f32p,
                                          ctypes.c_int]
        lib.vsref_hnsw_save.restype = ctypes.c_int
        lib.vsref_hnsw_save.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
        self.lib = lib

    def hnsw_save(self, x, path, metric="l2", num_threads=1):
        """HNSWIndex(dim, n, metric).add(x).save(path): the reference's own index file."""
        x = np.ascontiguousarray(x, np.float32)
        h = self.lib.vsref_hnsw_create(x.shape[1], x.shape[0], _metric_code(metric))
        try:
            if self.lib.vsref_hnsw_add(h, x, x.shape[0], num_threads) != 0:
                raise RuntimeError("reference HNSW add failed")
            if self.lib.vsref_hnsw_save(h, str(path).encode()) != 0:
                raise RuntimeError("reference HNSW save failed")
        finally:
            self.lib.vsref_hnsw_destroy(h)

    def bf_search(self, x, q, k, metric="ip", num_threads=1):
        """BruteForceIndex(dim, metric).add(x).search_batch(q, k): uint32 ids, float32 dists."""
        x = np.ascontiguousarray(x, np.float32)
        q = np.ascontiguousarray(q, np.float32)
        h = self.lib.vsref_bf_create(x.shape[1], _metric_code(metric))
        try:
            self.lib.vsref_bf_add(h, x, x.shape[0])
            ids = np.empty((q.shape[0], k), np.uint32)
            dists = np.empty((q.shape[0], k), np.float32)
            self.lib.vsref_bf_search_batch(h, q, q.shape[0], k, ids, dists, num_threads)
            return ids, dists
        finally:
            self.lib.vsref_bf_destroy(h)

    def bf_search_one(self, x, q, k, metric="ip"):
        """Single-query BruteForceIndex::search for each row of q (heap path)."""
        x = np.ascontiguousarray(x, np.float32)
        q = np.ascontiguousarray(q, np.float32)
        h = self.lib.vsref_bf_create(x.shape[1], _metric_code(metric))
        try:
            self.lib.vsref_bf_add(h, x, x.shape[0])
            ids = np.full((q.shape[0], k), NONE, np.uint32)
            dists = np.full((q.shape[0], k), np.inf, np.float32)
            for i in range(q.shape[0]):
                ri = np.empty(k, np.uint32)
                rd = np.empty(k, np.float32)
                m = self.lib.vsref_bf_search_one(h, np.ascontiguousarray(q[i]), k, ri, rd)
                ids[i, :m] = ri[:m]
                dists[i, :m] = rd[:m]
            return ids, dists
        finally:
            self.lib.vsref_bf_destroy(h)

    def hnsw_exact(self, x, q, k, allowed, exact_below, metric="l2", num_threads=1):
        """HNSWIndex.search(q, k, filter=allowed, exact_below=...) through the reference."""
        x = np.ascontiguousarray(x, np.float32)
        q = np.ascontiguousarray(q, np.float32)
        allowed = np.ascontiguousarray(allowed, np.uint8)
        h = self.lib.vsref_hnsw_create(x.shape[1], x.shape[0], _metric_code(metric))
        try:
            if self.lib.vsref_hnsw_add(h, x, x.shape[0], num_threads) != 0:
                raise RuntimeError("reference HNSW add failed")
            ids = np.empty((q.shape[0], k), np.uint32)
            dists = np.empty((q.shape[0], k), np.float32)
            self.lib.vsref_hnsw_search(h, q, q.shape[0], k, 64, allowed.ctypes.data, exact_below, ids,
                                       dists, num_threads)
            return ids, dists
        finally:
            self.lib.vsref_hnsw_destroy(h)
