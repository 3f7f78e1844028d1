"""A GPU-backed shard worker for vecsearch's gRPC ``Searcher`` service.

The reference's worker (distributed/shard_worker.py:18-40) serves one shard: it loads the shard's
HNSW file, answers ``Search`` with that index's top k (local ids + the shard's offset, missing
entries dropped, distances ascending, ``timings_ms = {"shard_<id>": ms}``) and ``Info`` with
(num_vectors, dim, num_shards = 1). The coordinator (distributed/coordinator.py:27-41) scatters each
query to every worker and merges their lists by (distance, id).

Here the shard's rows live in a :class:`GpuBruteForceIndex` (loaded straight from the same
``VSHNSW01`` file, or from any array), so every answer is the shard's exact top k. A worker receives
one query per call; a batcher thread gathers the calls that arrive together into one GPU search
(up to ``max_batch`` queries; while the previous batch held several calls it also waits up to
``max_wait_ms`` for company, so a lone caller is not delayed), runs it with the
largest k among them, and hands each call the first k of its row. Exact lists are ordered by
(distance, id), so the first k of a top-K list is the top k: batching never changes an answer.

The wire format is search.proto's (package ``vecsearch``, service ``Searcher``; reference
distributed/search.proto:1-27). The few messages are encoded and decoded here directly in
proto3's binary form, so neither protoc nor generated modules are needed; grpcio carries the
bytes through generic method handlers. ``python -m vecsearch_gb300.shard_worker --manifest M
--shard-id I --port P`` mirrors the reference worker's command line.
"""
import argparse
import json
import os
import queue
import struct
import threading
import time

import numpy as np

__all__ = ["encode_search_request", "decode_search_request", "encode_search_response",
           "decode_search_response", "encode_info_response", "decode_info_response",
           "ShardSearcher", "serve", "pin_cpus", "parse_args", "SERVICE"]

SERVICE = "vecsearch.Searcher"

# ---- proto3 binary encoding of search.proto's messages ----
_VARINT, _I64, _LEN, _I32 = 0, 1, 2, 5


def _varint(v):
    v &= (1 << 64) - 1  # negative int32 / int64 values go out as 10-byte two's complement
    out = bytearray()
    while True:
        b = v & 0x7F
        v >>= 7
        if v:
            out.append(b | 0x80)
        else:
            out.append(b)
            return bytes(out)


def _read_varint(buf, pos):
    v, shift = 0, 0
    while True:
        if pos >= len(buf):
            raise ValueError("truncated varint")
        b = buf[pos]
        pos += 1
        v |= (b & 0x7F) << shift
        if not b & 0x80:
            return v, pos
        shift += 7
        if shift > 63:
            raise ValueError("varint too long")


def _signed(v, bits):
    v &= (1 << bits) - 1
    return v - (1 << bits) if v >> (bits - 1) else v


def _key(field, wire):
    return _varint((field << 3) | wire)


def _fields(buf):
    """(field number, wire type, value) for each field of a message; LEN values are bytes."""
    pos, n = 0, len(buf)
    while pos < n:
        key, pos = _read_varint(buf, pos)
        field, wire = key >> 3, key & 7
        if wire == _VARINT:
            v, pos = _read_varint(buf, pos)
        elif wire == _I64:
            v, pos = bytes(buf[pos:pos + 8]), pos + 8
        elif wire == _I32:
            v, pos = bytes(buf[pos:pos + 4]), pos + 4
        elif wire == _LEN:
            ln, pos = _read_varint(buf, pos)
            v, pos = bytes(buf[pos:pos + ln]), pos + ln
        else:
            raise ValueError(f"unsupported wire type {wire}")
        if pos > n:
            raise ValueError("truncated message")
        yield field, wire, v


def encode_search_request(query, k, ef=0):
    """SearchRequest{query = little-endian float32 bytes, k, ef}."""
    q = np.ascontiguousarray(query, dtype="<f4").tobytes()
    out = bytearray()
    if q:
        out += _key(1, _LEN) + _varint(len(q)) + q
    if k:
        out += _key(2, _VARINT) + _varint(int(k))
    if ef:
        out += _key(3, _VARINT) + _varint(int(ef))
    return bytes(out)


def decode_search_request(buf):
    """-> (query float32 array, k, ef); absent fields are proto3 defaults."""
    q, k, ef = b"", 0, 0
    for f, w, v in _fields(buf):
        if f == 1 and w == _LEN:
            q = v
        elif f == 2 and w == _VARINT:
            k = _signed(v, 32)
        elif f == 3 and w == _VARINT:
            ef = _signed(v, 32)
    if len(q) % 4:
        raise ValueError("query bytes are not a whole number of float32")
    return np.frombuffer(q, dtype="<f4").astype(np.float32), k, ef


def encode_search_response(ids, distances, timings_ms=None):
    """SearchResponse{ids (packed int64), distances (packed float), timings_ms map}."""
    out = bytearray()
    ids = [int(i) for i in ids]
    if ids:
        body = b"".join(_varint(i) for i in ids)
        out += _key(1, _LEN) + _varint(len(body)) + body
    d = np.ascontiguousarray(distances, dtype="<f4").tobytes()
    if d:
        out += _key(2, _LEN) + _varint(len(d)) + d
    for name, ms in (timings_ms or {}).items():
        kb = str(name).encode()
        entry = _key(1, _LEN) + _varint(len(kb)) + kb + _key(2, _I64) + struct.pack("<d", float(ms))
        out += _key(3, _LEN) + _varint(len(entry)) + entry
    return bytes(out)


def decode_search_response(buf):
    """-> (ids list of int, distances list of float, timings dict); packed or unpacked fields."""
    ids, dists, timings = [], [], {}
    for f, w, v in _fields(buf):
        if f == 1 and w == _LEN:
            pos = 0
            while pos < len(v):
                x, pos = _read_varint(v, pos)
                ids.append(_signed(x, 64))
        elif f == 1 and w == _VARINT:
            ids.append(_signed(v, 64))
        elif f == 2 and w == _LEN:
            dists.extend(struct.unpack(f"<{len(v) // 4}f", v))
        elif f == 2 and w == _I32:
            dists.append(struct.unpack("<f", v)[0])
        elif f == 3 and w == _LEN:
            key, val = "", 0.0
            for f2, w2, v2 in _fields(v):
                if f2 == 1 and w2 == _LEN:
                    key = v2.decode()
                elif f2 == 2 and w2 == _I64:
                    val = struct.unpack("<d", v2)[0]
            timings[key] = val
    return ids, dists, timings


def encode_info_response(num_vectors, dim, num_shards):
    out = bytearray()
    for field, v in ((1, num_vectors), (2, dim), (3, num_shards)):
        if v:
            out += _key(field, _VARINT) + _varint(int(v))
    return bytes(out)


def decode_info_response(buf):
    r = {"num_vectors": 0, "dim": 0, "num_shards": 0}
    names = {1: ("num_vectors", 64), 2: ("dim", 32), 3: ("num_shards", 32)}
    for f, w, v in _fields(buf):
        if f in names and w == _VARINT:
            r[names[f][0]] = _signed(v, names[f][1])
    return r


# ---- the worker ----
class SearchError(ValueError):
    """A request the worker rejects (the gRPC layer answers INVALID_ARGUMENT)."""


class ShardSearcher:
    """One shard behind the Searcher methods, on raw request / response bytes.

    ``index``: a GpuBruteForceIndex (or any object with its ``search(queries, k, method)``,
    ``dim`` and ``len``) holding the shard's rows; ``offset``: global id of its first row.
    Calls from many threads are batched by one worker thread (see the module docstring);
    ``max_batch=1`` searches each call on its own, ``wait_always=True`` waits up to
    ``max_wait_ms`` for company before every batch.
    """

    def __init__(self, index, offset=0, shard_id=0, method="auto", max_batch=256, max_wait_ms=0.2,
                 wait_always=False):
        self.index = index
        self.offset = int(offset)
        self.shard_id = int(shard_id)
        self.method = method
        self.max_batch = max(1, int(max_batch))
        self.max_wait = max(0.0, float(max_wait_ms)) / 1e3
        self.wait_always = bool(wait_always)  # wait for company even after a lone call
        self.dim = int(index.dim)
        self._q = queue.Queue()
        self._stop = threading.Event()
        self._thread = threading.Thread(target=self._loop, name=f"shard{shard_id}-batcher", daemon=True)
        self._thread.start()
        self.batches = 0  # searches run (a batch of calls each)
        self.calls = 0

    def close(self):
        self._stop.set()
        self._q.put(None)
        self._thread.join()

    def _loop(self):
        last = 1  # calls in the previous batch
        while not self._stop.is_set():
            first = self._q.get()
            if first is None:
                break
            group = [first]
            # Wait for company only under load (the previous batch had several calls): a lone
            # caller is searched at once.
            deadline = time.perf_counter() + (self.max_wait if (last > 1 or self.wait_always) else 0.0)
            while len(group) < self.max_batch:
                left = deadline - time.perf_counter()
                try:
                    item = self._q.get_nowait() if left <= 0 else self._q.get(timeout=left)
                except queue.Empty:
                    break
                if item is None:
                    self._stop.set()
                    break
                group.append(item)
            last = len(group)
            self._run(group)

    def _run(self, group):
        kmax = max(item[1] for item in group)
        try:
            qs = np.stack([item[0] for item in group])
            ids, dists = self.index.search(qs, kmax, method=self.method)
            for j, item in enumerate(group):
                item[2]["result"] = (ids[j, :item[1]], dists[j, :item[1]])
        except Exception as e:  # every waiting call gets the error
            for item in group:
                item[2]["error"] = e
        finally:
            self.batches += 1
            self.calls += len(group)
            for item in group:
                item[2]["done"].set()

    def search(self, request):
        """Search RPC body: SearchRequest bytes -> SearchResponse bytes."""
        t = time.perf_counter()
        q, k, _ef = decode_search_request(request)  # ef is an HNSW knob: the search is exact
        if q.shape[0] != self.dim:
            raise SearchError(f"expected dim {self.dim}, got {q.shape[0]}")
        if k <= 0:
            return encode_search_response([], [], {f"shard_{self.shard_id}": (time.perf_counter() - t) * 1e3})
        if k > 128:
            raise SearchError("k must be at most 128")
        slot = {"done": threading.Event()}
        self._q.put((q, int(k), slot))
        slot["done"].wait()
        if "error" in slot:
            raise slot["error"]
        ids, d = slot["result"]
        keep = ids >= 0
        return encode_search_response((ids[keep] + self.offset).tolist(), d[keep].tolist(),
                                      {f"shard_{self.shard_id}": (time.perf_counter() - t) * 1e3})

    def info(self, request=b""):
        """Info RPC body: InfoResponse bytes (num_vectors, dim, num_shards = 1)."""
        return encode_info_response(len(self.index), self.dim, 1)


def serve(searcher, port, threads=8, host="[::]"):
    """Starts a gRPC server with the Searcher service on `port`; returns (server, bound port)."""
    import grpc
    from concurrent import futures

    def call(fn):
        def handler(request, ctx):
            try:
                return fn(request)
            except SearchError as e:
                ctx.abort(grpc.StatusCode.INVALID_ARGUMENT, str(e))
            except Exception as e:  # noqa: BLE001
                ctx.abort(grpc.StatusCode.INTERNAL, f"{type(e).__name__}: {e}")
        return grpc.unary_unary_rpc_method_handler(handler)  # raw bytes in and out

    server = grpc.server(futures.ThreadPoolExecutor(max_workers=threads), options=[("grpc.so_reuseport", 0)])
    server.add_generic_rpc_handlers((grpc.method_handlers_generic_handler(
        SERVICE, {"Search": call(searcher.search), "Info": call(searcher.info)}),))
    try:
        bound = server.add_insecure_port(f"{host}:{port}")
    except RuntimeError:
        bound = 0
    if bound == 0:  # a port clash fails here rather than sharing it (shard_worker.py:55)
        server.stop(0)
        raise RuntimeError(f"could not bind {host}:{port}")
    server.start()
    return server, bound


def pin_cpus(cpus):
    """--cpus of the reference worker (distributed/shard_worker.py:48-51): pin this process to
    the listed CPUs, e.g. "2,3" (Linux; a no-op where affinity cannot be set or nothing is listed)."""
    if cpus and hasattr(os, "sched_setaffinity"):
        os.sched_setaffinity(0, {int(c) for c in cpus.split(",")})


def parse_args(argv=None):
    ap = argparse.ArgumentParser(description="GPU shard worker for the vecsearch Searcher service")
    ap.add_argument("--manifest", required=True)
    ap.add_argument("--shard-id", type=int, required=True)
    ap.add_argument("--port", type=int, required=True)
    ap.add_argument("--threads", type=int, default=8, help="gRPC handler threads")
    ap.add_argument("--cpus", default="", help="pin to CPUs, e.g. '2,3' (Linux)")
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--method", default="auto", choices=["auto", "skinny", "tiled", "tc_exact"])
    ap.add_argument("--max-batch", type=int, default=256)
    ap.add_argument("--max-wait-ms", type=float, default=0.2)
    return ap.parse_args(argv)


def main(argv=None):
    a = parse_args(argv)
    pin_cpus(a.cpus)
    from . import GpuBruteForceIndex
    shard = json.load(open(a.manifest))["shards"][a.shard_id]
    path = os.path.join(os.path.dirname(os.path.abspath(a.manifest)), shard["file"])
    t = time.time()
    idx = GpuBruteForceIndex.from_hnsw_file(path, device=a.device)
    print(f"[shard {a.shard_id}] loaded {len(idx):,} vectors in {time.time() - t:.1f}s", flush=True)
    searcher = ShardSearcher(idx, shard["offset"], a.shard_id, a.method, a.max_batch, a.max_wait_ms)
    server, port = serve(searcher, a.port, a.threads)
    print(f"[shard {a.shard_id}] serving on :{port}", flush=True)
    server.wait_for_termination()
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
