"""The GPU shard worker's wire format, batching and gRPC service, on CPU.

The codec is pinned against protobuf's own encoder over search.proto's messages (reference
distributed/search.proto:1-27), rebuilt here from descriptors; the worker runs over a NumPy exact
index with the GpuBruteForceIndex interface, so that batching and the service can be checked
without a GPU. The GPU index behind the same worker is tested in test_gpu_shard_worker.py.
"""
import heapq
import threading

import numpy as np
import pytest

from vecsearch_gb300 import shard_worker as W


class NumpyExact:
    """Exact top k by (distance, id) over rows, the GpuBruteForceIndex search interface."""

    def __init__(self, x, metric="ip"):
        self.x = np.asarray(x, np.float32)
        self.metric = metric
        self.calls = []

    @property
    def dim(self):
        return self.x.shape[1]

    def __len__(self):
        return len(self.x)

    def search(self, q, k, method="auto"):
        q = np.atleast_2d(np.asarray(q, np.float32))
        self.calls.append(len(q))
        if self.metric == "ip":
            d = 1.0 - q @ self.x.T
        else:
            d = ((q[:, None, :] - self.x[None]) ** 2).sum(-1)
        order = np.lexsort((np.broadcast_to(np.arange(len(self.x)), d.shape), d), axis=-1)[:, :k]
        ids = np.full((len(q), k), -1, np.int64)
        dists = np.full((len(q), k), np.inf, np.float32)
        ids[:, :order.shape[1]] = order
        dists[:, :order.shape[1]] = np.take_along_axis(d, order, axis=1)
        return ids, dists


def _proto_classes():
    """search.proto's messages from descriptors (no protoc in this environment)."""
    pytest.importorskip("google.protobuf")
    from google.protobuf import descriptor_pb2, descriptor_pool, message_factory
    F = descriptor_pb2.FieldDescriptorProto
    fd = descriptor_pb2.FileDescriptorProto(name="search_test.proto", package="vecsearch", syntax="proto3")

    def msg(name, fields, nested=()):
        m = fd.message_type.add(name=name)
        for n, num, typ, label in fields:
            f = m.field.add(name=n, number=num, type=typ, label=label)
            if typ == F.TYPE_MESSAGE:
                f.type_name = f".vecsearch.{name}.TimingsMsEntry"
        for nm, nf in nested:
            e = m.nested_type.add(name=nm)
            e.options.map_entry = True
            for n, num, typ in nf:
                e.field.add(name=n, number=num, type=typ, label=F.LABEL_OPTIONAL)
        return m

    opt, rep = F.LABEL_OPTIONAL, F.LABEL_REPEATED
    msg("SearchRequest", [("query", 1, F.TYPE_BYTES, opt), ("k", 2, F.TYPE_INT32, opt), ("ef", 3, F.TYPE_INT32, opt)])
    msg("SearchResponse", [("ids", 1, F.TYPE_INT64, rep), ("distances", 2, F.TYPE_FLOAT, rep),
                           ("timings_ms", 3, F.TYPE_MESSAGE, rep)],
        nested=[("TimingsMsEntry", [("key", 1, F.TYPE_STRING), ("value", 2, F.TYPE_DOUBLE)])])
    msg("InfoResponse", [("num_vectors", 1, F.TYPE_INT64, opt), ("dim", 2, F.TYPE_INT32, opt),
                         ("num_shards", 3, F.TYPE_INT32, opt)])
    pool = descriptor_pool.DescriptorPool()
    pool.Add(fd)
    get = lambda n: message_factory.GetMessageClass(pool.FindMessageTypeByName(f"vecsearch.{n}"))
    return get("SearchRequest"), get("SearchResponse"), get("InfoResponse")


def test_codec_matches_protobuf():
    Req, Resp, Info = _proto_classes()
    q = np.random.default_rng(0).standard_normal(37).astype(np.float32)
    r = Req()
    r.ParseFromString(W.encode_search_request(q, 10, 64))
    assert r.k == 10 and r.ef == 64 and np.frombuffer(r.query, "<f4").tolist() == q.tolist()
    dq, k, ef = W.decode_search_request(Req(query=q.tobytes(), k=7, ef=-3).SerializeToString())
    assert k == 7 and ef == -3 and dq.tolist() == q.tolist()
    assert W.decode_search_request(b"") [1:] == (0, 0)

    ids = [0, 5, 2**40, 123456789]
    dists = [0.0, 0.25, 1.5, -2.0]
    timings = {"shard_0": 1.25, "coordinator_total": 3.5}
    m = Resp()
    m.ParseFromString(W.encode_search_response(ids, dists, timings))
    assert list(m.ids) == ids and list(m.distances) == dists and dict(m.timings_ms) == timings
    m2 = Resp(ids=ids, distances=dists)
    m2.timings_ms.update(timings)
    assert W.decode_search_response(m2.SerializeToString()) == (ids, dists, timings)
    assert W.decode_search_response(b"") == ([], [], {})

    i = Info()
    i.ParseFromString(W.encode_info_response(3_000_000, 384, 1))
    assert (i.num_vectors, i.dim, i.num_shards) == (3_000_000, 384, 1)
    assert W.decode_info_response(Info(num_vectors=5, dim=8, num_shards=2).SerializeToString()) == \
        {"num_vectors": 5, "dim": 8, "num_shards": 2}


def test_codec_rejects_malformed():
    with pytest.raises(ValueError):
        W.decode_search_request(b"\x0a\x05ab")  # length past the end
    with pytest.raises(ValueError):
        W.decode_search_request(b"\x0a\x03abc")  # 3 bytes: not float32s
    with pytest.raises(ValueError):
        W.decode_search_response(b"\x08")  # truncated varint


def _data(n=3000, d=24, nq=40, seed=5):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((n, d)).astype(np.float32)
    x /= np.linalg.norm(x, axis=1, keepdims=True)
    q = rng.standard_normal((nq, d)).astype(np.float32)
    return x, q


def test_searcher_batches_concurrent_calls():
    x, q = _data()
    idx = NumpyExact(x)
    s = W.ShardSearcher(idx, offset=1000, shard_id=3, max_batch=64, max_wait_ms=20.0, wait_always=True)
    ks = [1 + (i * 7) % 30 for i in range(len(q))]
    out = [None] * len(q)
    barrier = threading.Barrier(len(q))

    def call(i):
        barrier.wait()
        out[i] = W.decode_search_response(s.search(W.encode_search_request(q[i], ks[i], 64)))

    ts = [threading.Thread(target=call, args=(i,)) for i in range(len(q))]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    s.close()
    ref_i, ref_d = NumpyExact(x).search(q, 30)
    for i, (ids, dists, timings) in enumerate(out):
        assert ids == (ref_i[i, :ks[i]] + 1000).tolist()
        np.testing.assert_array_equal(np.float32(dists), ref_d[i, :ks[i]])
        assert set(timings) == {"shard_3"}
    assert s.calls == len(q) and s.batches < len(q)  # calls were served together
    assert max(idx.calls) > 1


def test_searcher_errors_and_short_shards():
    x, q = _data(n=5)
    s = W.ShardSearcher(NumpyExact(x), offset=7, max_batch=1)
    with pytest.raises(W.SearchError):
        s.search(W.encode_search_request(q[0][:5], 3))  # wrong dim
    with pytest.raises(W.SearchError):
        s.search(W.encode_search_request(q[0], 129))
    ids, dists, _ = W.decode_search_response(s.search(W.encode_search_request(q[0], 10)))
    assert sorted(ids) == list(range(7, 12)) and len(dists) == 5  # missing entries are dropped
    assert W.decode_search_response(s.search(W.encode_search_request(q[0], 0)))[0] == []
    assert W.decode_info_response(s.info()) == {"num_vectors": 5, "dim": 24, "num_shards": 1}
    s.close()


def test_grpc_service_and_coordinator_merge():
    grpc = pytest.importorskip("grpc")
    x, q = _data(n=4000, nq=12)
    bounds = [0, 1500, 4000]
    searchers, servers, chans = [], [], []
    for sid in range(2):
        lo, hi = bounds[sid], bounds[sid + 1]
        s = W.ShardSearcher(NumpyExact(x[lo:hi]), offset=lo, shard_id=sid)
        srv, port = W.serve(s, 0, threads=4, host="127.0.0.1")
        assert port > 0
        searchers.append(s)
        servers.append(srv)
        chans.append(grpc.insecure_channel(f"127.0.0.1:{port}"))
    try:
        search = [c.unary_unary(f"/{W.SERVICE}/Search") for c in chans]
        info = [c.unary_unary(f"/{W.SERVICE}/Info") for c in chans]
        assert [W.decode_info_response(f(b""))["num_vectors"] for f in info] == [1500, 2500]
        ref_i, ref_d = NumpyExact(x).search(q, 10)
        for i in range(len(q)):
            lists = []
            for f in search:
                ids, dists, _ = W.decode_search_response(f(W.encode_search_request(q[i], 10, 64), timeout=10))
                lists.append(list(zip(dists, ids)))
            top = heapq.nsmallest(10, heapq.merge(*lists))  # the reference coordinator's merge
            assert [t[1] for t in top] == ref_i[i].tolist()
        with pytest.raises(grpc.RpcError) as e:
            search[0](W.encode_search_request(q[0][:3], 10), timeout=10)
        assert e.value.code() == grpc.StatusCode.INVALID_ARGUMENT
    finally:
        for c in chans:
            c.close()
        for srv in servers:
            srv.stop(0)
        for s in searchers:
            s.close()


def test_lone_caller_is_not_delayed():
    # The batching window applies only after a batch of several calls: a lone caller is searched
    # at once even with a long window.
    import time
    x, q = _data(n=200)
    s = W.ShardSearcher(NumpyExact(x), max_batch=64, max_wait_ms=200.0)
    t = time.perf_counter()
    for i in range(5):
        s.search(W.encode_search_request(q[i], 5))
    assert time.perf_counter() - t < 0.5  # five 200 ms windows would take 1 s
    assert s.batches == 5
    s.close()


def test_command_line_mirrors_the_reference_worker():
    # distributed/shard_worker.py:44-51: the same flags (plus the GPU's own), --cpus pins the process.
    import os
    a = W.parse_args(["--manifest", "m.json", "--shard-id", "2", "--port", "5001", "--threads", "3",
                      "--cpus", "0"])
    assert (a.manifest, a.shard_id, a.port, a.threads, a.cpus) == ("m.json", 2, 5001, 3, "0")
    assert W.parse_args(["--manifest", "m", "--shard-id", "0", "--port", "1"]).cpus == ""
    if not hasattr(os, "sched_getaffinity"):
        pytest.skip("no CPU affinity on this platform")
    before = os.sched_getaffinity(0)
    one = min(before)
    try:
        W.pin_cpus(str(one))
        assert os.sched_getaffinity(0) == {one}
        W.pin_cpus("")  # nothing listed: unchanged
        assert os.sched_getaffinity(0) == {one}
    finally:
        os.sched_setaffinity(0, before)


def test_port_clash_fails_instead_of_sharing():
    pytest.importorskip("grpc")
    x, _ = _data(n=50)
    s = W.ShardSearcher(NumpyExact(x))
    srv, port = W.serve(s, 0, threads=2, host="127.0.0.1")
    try:
        with pytest.raises(RuntimeError):
            W.serve(s, port, threads=2, host="127.0.0.1")
    finally:
        srv.stop(0)
        s.close()
