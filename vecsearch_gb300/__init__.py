"""vecsearch_gb300 - GB300-native exact k-NN behind vecsearch's exact-search API.

Drop-in names (python/vecsearch/__init__.py and python/bindings.cpp of vecsearch):

* :class:`GpuBruteForceIndex` - ``(dim, metric="l2", device=0)``, ``add(x)``,
  ``search(queries, k=10, method="auto", filter=None)`` -> ``(ids int64, dists float32)``,
  ``dim``, ``len()``; the same argument coercion, errors and -1 / +inf padding as the
  reference's bindings (bindings.cpp:151-189). ``filter`` is new: None, a 1-D bool/uint8
  mask of length ``len(index)`` shared by all queries, or a 2-D (nq, len(index)) mask with
  one row per query.
* :func:`cuda_available`, :func:`normalize`, :func:`recall_at_k`.
* :class:`HNSWExactRoute` - the HNSW index's ``exact_below`` switch on the GPU.
* :func:`pybind_module` - the same GpuBruteForceIndex and cuda_available as a compiled pybind11
  module (``_vecsearch_gb300``), the form the reference's own bindings take.
"""
import ctypes
import operator

import numpy as np

from . import _native
from .datasets import pack_bits

__all__ = ["GpuBruteForceIndex", "HNSWExactRoute", "Server", "cuda_available", "normalize", "recall_at_k",
           "hnsw_file_info", "insert_candidates", "DeviceTimeoutError", "pybind_module"]
__version__ = "0.1.0"

DeviceTimeoutError = _native.DeviceTimeoutError


def cuda_available() -> bool:
    """True if the library is built and the CUDA runtime sees a GPU (cuda_available(),
    gpu_brute_force.cu:334-341; False without the build, as bindings.cpp:191-197 returns in a
    build without CUDA). The index itself raises ImportError without the library."""
    try:
        l = _native.lib()
    except ImportError:
        return False
    return bool(l.vsg_cuda_available())


def pybind_module():
    """The pybind11 front end, module ``_vecsearch_gb300`` (GpuBruteForceIndex with the reference's
    constructor, add, search, dim and len; cuda_available), or None where it was not built
    (pybind11's headers absent). It calls the same library as this package."""
    import importlib.machinery
    import importlib.util
    import os
    from . import build as _build
    path = _build.pybind_module_path()
    if not os.path.exists(path):
        return None
    _native.lib()  # the library first: the module links against the same file
    loader = importlib.machinery.ExtensionFileLoader("_vecsearch_gb300", path)
    spec = importlib.util.spec_from_file_location("_vecsearch_gb300", path, loader=loader)
    mod = importlib.util.module_from_spec(spec)
    loader.exec_module(mod)
    return mod


def normalize(x: np.ndarray) -> np.ndarray:
    """L2-normalize rows so inner product == cosine similarity (vecsearch/__init__.py:15-18)."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    return x / np.maximum(np.linalg.norm(x, axis=1, keepdims=True), 1e-12)


def recall_at_k(found: np.ndarray, truth: np.ndarray, k: int = 10) -> float:
    """Fraction of the true top-k found in the returned top-k (vecsearch/__init__.py:21-24)."""
    hits = sum(len(set(f[:k]) & set(t[:k])) for f, t in zip(found, truth))
    return hits / (len(found) * k)


def hnsw_file_info(path):
    """(dim, rows, metric) from the header of a saved HNSWIndex file (src/hnsw.cpp:368-389)."""
    dim, rows, metric = ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_uint32()
    _native.check(_native.lib().vsg_hnsw_file_info(str(path).encode(), ctypes.byref(dim), ctypes.byref(rows),
                                                   ctypes.byref(metric)))
    return dim.value, rows.value, ("l2" if metric.value == _native.METRIC_L2 else "ip")


def _parse_metric(metric):
    if metric == "l2":
        return _native.METRIC_L2
    if metric in ("ip", "cosine"):
        return _native.METRIC_IP
    raise ValueError("metric must be 'l2', 'ip' or 'cosine' (cosine expects normalized vectors)")


def _as_f32(a):
    """py::array_t<float, c_style | forcecast> (bindings.cpp:17)."""
    return np.ascontiguousarray(a, dtype=np.float32)


def _as_k(k):
    """k as pybind converts it to size_t (bindings.cpp:167, :79): an integer (or anything with
    __index__) that is not negative; anything else is a TypeError."""
    try:
        v = operator.index(k)
    except TypeError:
        raise TypeError(f"k must be a non-negative integer, got {k!r}") from None
    if v < 0:
        raise TypeError(f"k must be a non-negative integer, got {k!r}")
    return v


def _as_mask_u8(a):
    """py::array_t<uint8_t, c_style | forcecast> (bindings.cpp:18): a mask of any numeric type is
    cast to uint8 first (0.5 -> 0, 256 -> 0), then a nonzero byte allows its row."""
    a = np.asarray(a)
    if a.dtype == np.bool_ or a.dtype == np.uint8:
        return a
    with np.errstate(all="ignore"):  # the same unchecked cast numpy's forcecast makes
        return a.astype(np.uint8)


def _check_2d(a, dim):
    if a.ndim != 2 or a.shape[1] != dim:
        raise ValueError(f"expected array of shape (n, {dim})")


def _ids_to_int64(ids):
    out = ids.astype(np.int64)
    out[ids == _native.NONE] = -1
    return out


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


def insert_candidates(x, k, metric="l2", batch=1024, device=0):
    """Exact neighbour candidates for building an HNSW graph in insertion order: row i's list is
    the k nearest of rows 0 .. i-1 by (dist, id) (the nodes HNSWIndex::insert, src/hnsw.cpp:247-309,
    searches when it inserts node i), padded with -1 / +inf while i < k. Returns
    (ids int64 [n, k], dists float32 [n, k]). Batches of `batch` rows are searched against the rows
    before them and against their own earlier rows on the GPU, then merged."""
    x = _as_f32(x)
    if x.ndim != 2:
        raise ValueError("expected a 2-D array of rows")
    n, dim = x.shape
    k = operator.index(k)
    if k < 0:
        raise TypeError("k must be a non-negative integer")
    ids = np.empty((n, k), dtype=np.uint32)
    dists = np.empty((n, k), dtype=np.float32)
    if n and k:
        _native.check(_native.lib().vsg_insert_candidates(_ptr(x), n, dim, _parse_metric(metric), int(device), k,
                                                          int(batch), _ptr(ids), _ptr(dists)))
    return _ids_to_int64(ids), dists


class GpuBruteForceIndex:
    """Exact k-NN on one GB300 (vecsearch.GpuBruteForceIndex, gpu_brute_force.h:25-50)."""

    kNone = _native.NONE
    kMaxK = _native.MAX_K

    def __init__(self, dim, metric="l2", device=0):
        lib = _native.lib()
        self._h = ctypes.c_void_p()
        _native.check(lib.vsg_create(int(dim), _parse_metric(metric), int(device), ctypes.byref(self._h)))
        self._dim = int(dim)
        self._metric = metric

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            _native.lib().vsg_destroy(h)
            self._h = None

    @property
    def dim(self):
        return self._dim

    @property
    def metric(self):
        return "l2" if _native.lib().vsg_metric(self._h) == _native.METRIC_L2 else "ip"

    def __len__(self):
        return int(_native.lib().vsg_size(self._h))

    @classmethod
    def from_hnsw_file(cls, path, device=0):
        """A device index holding the vectors of a saved HNSWIndex (HNSWIndex.save's file)."""
        dim, _, metric = hnsw_file_info(path)
        idx = cls(dim, metric, device=device)
        idx.add_hnsw_file(path)
        return idx

    def add_hnsw_file(self, path):
        """Append the vectors of a saved HNSWIndex (same dim and metric); returns the rows added."""
        added = ctypes.c_size_t(0)
        _native.check(_native.lib().vsg_add_hnsw_file(self._h, str(path).encode(), ctypes.byref(added)))
        return added.value

    def add(self, x):
        """Append rows (bindings.cpp:157-164); ids continue from len(self)."""
        x = _as_f32(x)
        _check_2d(x, self._dim)
        _native.check(_native.lib().vsg_add(self._h, _ptr(x), x.shape[0]))

    def _mask_words(self, filter, nq):
        """(words, per_query, ld) for the C ABI, with as_mask's validation (bindings.cpp:28-36)."""
        n = len(self)
        f = _as_mask_u8(filter)
        if f.ndim == 1 and f.shape[0] == n:
            return np.ascontiguousarray(pack_bits(f)), 0, 0
        if f.ndim == 2 and f.shape == (nq, n):
            w = np.ascontiguousarray(pack_bits(f))
            return w, 1, w.shape[1]
        raise ValueError(f"filter must be a 1-D bool array of length {n} or a 2-D array of shape ({nq}, {n})")

    def search(self, queries, k=10, method="auto", filter=None):
        """Exact top-k (bindings.cpp:165-186); returns (ids[int64, nq x k], dists[float32, nq x k])."""
        if method not in _native.METHODS:
            raise ValueError("method must be 'auto', 'naive', 'skinny', 'tiled', 'bf16', 'tc_exact' or 'fp8'")
        q = _as_f32(queries)
        if q.ndim == 1:
            q = q.reshape(1, q.shape[0])
        _check_2d(q, self._dim)
        k = _as_k(k)
        nq = q.shape[0]
        ids = np.empty((nq, k), np.uint32)
        dists = np.empty((nq, k), np.float32)
        lib = _native.lib()
        if filter is None:
            rc = lib.vsg_search(self._h, _ptr(q), nq, k, _ptr(ids), _ptr(dists), _native.METHODS[method])
        else:
            words, per_query, ld = self._mask_words(filter, nq)
            rc = lib.vsg_search_filtered(self._h, _ptr(q), nq, k, _ptr(words), per_query, ld, _ptr(ids),
                                         _ptr(dists), _native.METHODS[method])
        _native.check(rc)
        return _ids_to_int64(ids), dists

    # ---- device-resident form (for serving and benchmarks) ------------------------------------
    def search_device(self, q_ptr, ldq, nq, k, out_ids_ptr, out_dists_ptr, stream=0, mask_ptr=0,
                      per_query=False, mask_ld=0, method="auto"):
        """Queue a search on device buffers (raw pointers, e.g. torch ``data_ptr()``); no sync."""
        _native.check(_native.lib().vsg_search_device(
            self._h, ctypes.c_void_p(q_ptr), ldq, nq, k, ctypes.c_void_p(mask_ptr or None), int(per_query),
            mask_ld, ctypes.c_void_p(out_ids_ptr), ctypes.c_void_p(out_dists_ptr), _native.METHODS[method],
            ctypes.c_void_p(stream or None)))

    def search_host_ptr(self, q_ptr, nq, k, out_ids_ptr, out_dists_ptr, method="auto"):
        """search() on raw host pointers (e.g. pinned buffers), blocking; no numpy conversion."""
        _native.check(_native.lib().vsg_search(self._h, ctypes.c_void_p(q_ptr), nq, k,
                                               ctypes.c_void_p(out_ids_ptr), ctypes.c_void_p(out_dists_ptr),
                                               _native.METHODS[method]))

    def sync(self):
        """Wait for queued device work; raises if a kernel reported a failure."""
        _native.check(_native.lib().vsg_sync(self._h))

    def set_tunable(self, name, value):
        """Set a named tunable (e.g. "gather_max_fraction"); see include/vsg.h."""
        _native.check(_native.lib().vsg_set_tunable(self._h, name.encode(), float(value)))

    def get_tunable(self, name):
        v = ctypes.c_double()
        _native.check(_native.lib().vsg_get_tunable(self._h, name.encode(), ctypes.byref(v)))
        return v.value

    def autotune(self, batches=(1, 8, 32, 64, 128, 512, 2048), k=10, method="auto", queries=None):
        """Time candidate schedules per batch size and keep the fastest; returns the table.
        queries: a sample of real queries to time with (else queries near the index's rows)."""
        b = (ctypes.c_size_t * len(batches))(*[int(v) for v in batches])
        if queries is None:
            _native.check(_native.lib().vsg_autotune(self._h, b, len(batches), int(k), _native.METHODS[method]))
        else:
            qs = _as_f32(queries)
            _check_2d(qs, self._dim)
            _native.check(_native.lib().vsg_autotune_with_queries(self._h, _ptr(qs), qs.shape[0], b, len(batches),
                                                                  int(k), _native.METHODS[method]))
        return self.tuning(method)

    def tuning(self, method="auto"):
        """The tuned table. Exact methods: [{"batch", "kernel", "split"} (+ "shortlist": first-pass k'
        of the certified path)]; bf16: [{"batch", "sample" (rows sampled, 0 = none)}]."""
        cnt = ctypes.c_size_t(64)
        bt = (ctypes.c_uint32 * 64)()
        ch = (ctypes.c_uint32 * 64)()
        sp = (ctypes.c_double * 64)()
        kp = (ctypes.c_uint32 * 64)()
        _native.check(_native.lib().vsg_autotune_table(self._h, _native.METHODS[method], ctypes.byref(cnt), bt, ch,
                                                       sp, kp))
        n = min(cnt.value, 64)
        if method == "bf16":
            return [{"batch": bt[i], "sample": int(ch[i])} for i in range(n)]
        names = {0: "skinny", 1: "tiled", 2: "tc_exact"}
        return [dict({"batch": bt[i], "kernel": names[ch[i]], "split": sp[i]},
                     **({"shortlist": int(kp[i])} if ch[i] == 2 else {})) for i in range(n)]

    def save_tuning(self, path):
        _native.check(_native.lib().vsg_autotune_save(self._h, str(path).encode()))

    def load_tuning(self, path):
        _native.check(_native.lib().vsg_autotune_load(self._h, str(path).encode()))

    def kernel_launches(self):
        """Kernels this index has launched since it was created (searches and conversions)."""
        v = ctypes.c_uint64()
        _native.check(_native.lib().vsg_kernel_launches(self._h, ctypes.byref(v)))
        return v.value

    def tc_exact_stats(self):
        """(queries searched by the certified exact path, queries its shortlist pass could not
        certify, queries it ran in the scan kernel) since the index was created; the last two are
        the same queries. Waits for the index's queued work."""
        q, s2, f = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        _native.check(_native.lib().vsg_tc_exact_stats(self._h, ctypes.byref(q), ctypes.byref(s2), ctypes.byref(f)))
        return q.value, s2.value, f.value

    def tiled_stats(self):
        """(queries searched by the tiled FP32 kernel, queries its certificate could not prove and
        the scan kernel answered) since the index was created. Waits for the index's queued work."""
        q, f = ctypes.c_uint64(), ctypes.c_uint64()
        _native.check(_native.lib().vsg_tiled_stats(self._h, ctypes.byref(q), ctypes.byref(f)))
        return q.value, f.value

    def profile(self, enable=True):
        """Start (or stop) recording CUDA-event times of the scan and merge kernels."""
        _native.check(_native.lib().vsg_profile_enable(self._h, int(enable)))

    def profile_read(self):
        """(scan_ms_total, merge_ms_total, searches) since the last read; clears the record."""
        a, b, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_size_t()
        _native.check(_native.lib().vsg_profile_read(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(n)))
        return a.value, b.value, n.value


class Server:
    """Continuous-batching exact search over a GpuBruteForceIndex: the certified tensor-core path
    (BF16 shortlist, exact FP32 rerank, a proof per query, the FP32 scan for queries it cannot
    prove), so every result equals ``index.search(..., method="skinny")`` bit for bit.

    ``submit(queries, k, filter=None)`` queues a request and returns a ticket; ``wait(ticket)``
    returns ``(ids int64 [nq, k], dists float32 [nq, k], latency_ms)``. Requests arriving while
    others run are batched into the next free slot; results do not depend on the batch.
    ``filter`` is None or a 1-D bool/uint8 mask over the index rows, shared by the request's queries.
    """

    def __init__(self, index, max_batch=1024, max_k=100, slots=2):
        self._h = ctypes.c_void_p()
        self.index = index
        _native.check(_native.lib().vsg_server_create(index._h, int(max_batch), int(max_k), int(slots),
                                                      ctypes.byref(self._h)))
        self._pending = {}

    def submit(self, queries, k=10, filter=None, filter_words=None):
        """Queue a request; ``filter_words`` may pass an already packed mask (datasets.pack_bits)."""
        q = _as_f32(queries)
        if q.ndim == 1:
            q = q.reshape(1, q.shape[0])
        _check_2d(q, self.index.dim)
        nq = q.shape[0]
        ids = np.empty((nq, int(k)), np.uint32)
        dists = np.empty((nq, int(k)), np.float32)
        words = None
        if filter_words is not None:
            words = np.ascontiguousarray(filter_words, np.uint32)
            if words.ndim != 1 or words.shape[0] != (len(self.index) + 31) // 32:
                raise ValueError("filter_words must hold ceil(len(index) / 32) uint32 words")
        elif filter is not None:
            f = _as_mask_u8(filter)
            if f.ndim != 1 or f.shape[0] != len(self.index):
                raise ValueError(f"filter must be a 1-D bool array of length {len(self.index)}")
            words = np.ascontiguousarray(pack_bits(f))
        t = ctypes.c_uint64()
        _native.check(_native.lib().vsg_server_submit(self._h, _ptr(q), nq, int(k),
                                                      _ptr(words) if words is not None else None,
                                                      _ptr(ids), _ptr(dists), ctypes.byref(t)))
        self._pending[t.value] = (q, words, ids, dists)  # kept alive until wait()
        return t.value

    def wait(self, ticket, timeout=0.0):
        lat = ctypes.c_double()
        rc = _native.lib().vsg_server_wait(self._h, ctypes.c_uint64(ticket), float(timeout), ctypes.byref(lat))
        q, words, ids, dists = self._pending.pop(ticket)
        _native.check(rc)
        return _ids_to_int64(ids), dists, lat.value

    def stats(self):
        """Micro-batches, queries, requests, slots, and the queries the certificate could not prove
        (answered by the FP32 scan inside the same graph)."""
        v = [ctypes.c_uint64() for _ in range(4)]
        _native.check(_native.lib().vsg_server_stats(self._h, *[ctypes.byref(x) for x in v]))
        u = ctypes.c_uint64()
        _native.check(_native.lib().vsg_server_uncertified(self._h, ctypes.byref(u)))
        return dict(zip(("batches", "queries", "requests", "slots", "uncertified"), [x.value for x in v] + [u.value]))

    def close(self):
        if self._h:
            _native.lib().vsg_server_destroy(self._h)
            self._h = None

    def __del__(self):
        if getattr(self, "_h", None):
            self.close()


class HNSWExactRoute:
    """The HNSW index's exact_below switch (hnsw.cpp:322-334) with the exact scan on the GPU.

    Wraps any object with the reference's ``HNSWIndex.search`` signature (the graph) and a
    :class:`GpuBruteForceIndex` holding the same rows. ``search(queries, k, ef, num_threads,
    filter, exact_below)`` behaves like ``HNSWIndex.search`` (bindings.cpp:77-111): with a filter
    that allows no row the result is all -1 / +inf; with 0 < allowed <= exact_below it is the
    exact filtered scan (search_exact, hnsw.cpp:336-354) computed on the GPU; otherwise the
    wrapped graph search answers. ``graph`` may be None when only the exact route is used.
    The GPU index returns at most 128 neighbours (GpuBruteForceIndex.kMaxK); a larger k is left
    to the wrapped HNSWIndex.search, which then runs its own exact scan (or, without a graph,
    is a ValueError).
    """

    def __init__(self, gpu_index, graph=None):
        self.gpu = gpu_index
        self.graph = graph

    def search(self, queries, k=10, ef=64, num_threads=1, filter=None, exact_below=0):
        q = _as_f32(queries)
        if q.ndim == 1:
            q = q.reshape(1, q.shape[0])
        _check_2d(q, self.gpu.dim)
        nq = q.shape[0]
        k = _as_k(k)
        handled = ctypes.c_int(0)
        ids = np.empty((nq, k), np.uint32)
        dists = np.empty((nq, k), np.float32)
        if filter is not None and k > _native.MAX_K and self.graph is None:
            raise ValueError(f"k must be at most {_native.MAX_K} on the GPU route without a graph")
        if filter is not None and k <= _native.MAX_K:
            mask = _as_mask_u8(filter)
            if mask.ndim != 1 or mask.shape[0] != len(self.gpu):
                raise ValueError(f"filter must be a 1-D bool array of length {len(self.gpu)}")
            mask = np.ascontiguousarray(mask != 0, dtype=np.uint8)
            _native.check(_native.lib().vsg_hnsw_exact_below(
                self.gpu._h, _ptr(q), nq, k, _ptr(mask), mask.shape[0], int(exact_below), _ptr(ids), _ptr(dists),
                ctypes.byref(handled)))
        if handled.value:
            return _ids_to_int64(ids), dists
        if self.graph is None:
            raise NotImplementedError("the graph search is not part of the GPU route; pass graph=HNSWIndex")
        return self.graph.search(queries, k=k, ef=ef, num_threads=num_threads, filter=filter,
                                 exact_below=exact_below)
