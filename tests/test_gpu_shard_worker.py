"""GPU: the shard worker over a device index (no gRPC here: the GPU image lacks grpcio, so the
Searcher method bodies run on raw request bytes, as the gRPC handlers call them).

A shard loaded straight from a saved HNSW file answers with its exact top k plus the shard's
offset; calls that arrive together are searched as one batch with the same answers.
"""
import threading

import numpy as np
import pytest

from tests.conftest import GOLDEN
from tests.golden.make_golden import HNSW_FILE, hnsw_file_rows

pytestmark = pytest.mark.gpu


def test_worker_on_hnsw_file_shard(gpu_ready):
    vsg = gpu_ready
    from vecsearch_gb300 import shard_worker as W
    from oracle import oracle as O
    idx = vsg.GpuBruteForceIndex.from_hnsw_file(f"{GOLDEN}/{HNSW_FILE['name']}")
    x = hnsw_file_rows()
    s = W.ShardSearcher(idx, offset=500, shard_id=2, max_batch=1)
    q = x[:8] + 0.01
    for i in range(len(q)):
        ids, dists, timings = W.decode_search_response(s.search(W.encode_search_request(q[i], 10, 64)))
        want_i, want_d = O.search(x, q[i:i + 1], 10, "l2")
        assert ids == (O.ids_to_int64(want_i)[0] + 500).tolist()
        np.testing.assert_allclose(dists, want_d[0], rtol=1e-5, atol=2e-6)
        assert "shard_2" in timings
    assert W.decode_info_response(s.info()) == {"num_vectors": 150, "dim": 13, "num_shards": 1}
    s.close()


@pytest.mark.parametrize("method", ["auto", "tc_exact"])
def test_worker_batches_on_gpu(gpu_ready, method):
    vsg = gpu_ready
    from vecsearch_gb300 import datasets as D
    from vecsearch_gb300 import shard_worker as W
    x, _ = D.portable_clustered(50_000, 96, 64, 0.35, seed=300, centroid_seed=301, unit=True)
    q, _ = D.portable_clustered(160, 96, 64, 0.35, seed=302, centroid_seed=301, unit=True)
    idx = vsg.GpuBruteForceIndex(96, "cosine")
    idx.add(x)
    s = W.ShardSearcher(idx, offset=10_000, shard_id=0, method=method, max_batch=128, max_wait_ms=50.0,
                        wait_always=True)
    ks = [1 + (i * 5) % 32 for i in range(len(q))]
    out = [None] * len(q)
    barrier = threading.Barrier(len(q))

    def call(i):
        barrier.wait()
        out[i] = W.decode_search_response(s.search(W.encode_search_request(q[i], ks[i])))

    ts = [threading.Thread(target=call, args=(i,)) for i in range(len(q))]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    s.close()
    assert s.batches < len(q)
    ref_i, ref_d = idx.search(q, 32, method="skinny")
    for i, (ids, dists, _) in enumerate(out):
        got_d = np.float32(dists)
        if method == "tc_exact":  # bit for bit the scan kernel's answer
            assert ids == (ref_i[i, :ks[i]] + 10_000).tolist()
            np.testing.assert_array_equal(got_d.view(np.uint32), ref_d[i, :ks[i]].view(np.uint32))
        else:  # auto may take the tiled kernel for some batch sizes: the FP32 parity rule
            from oracle import oracle as O
            O.check_ids(np.array([ids]) - 10_000, ref_i[i:i + 1, :ks[i]], x, q[i:i + 1], "ip", rel=1e-6)
            np.testing.assert_allclose(got_d, ref_d[i, :ks[i]], rtol=1e-5, atol=2e-6)
