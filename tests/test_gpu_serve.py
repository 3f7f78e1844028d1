"""GPU: the continuous-batching server (persistent BF16 shortlist kernel in CUDA graphs).

A request's result must equal the index's own BF16 shortlist search for unfiltered requests
(bitwise: the same shortlist and the same exact rerank) and the exact filtered search for
filtered ones (parity rule of test_gpu_parity.py), and must be the same alone and inside a
burst of other requests.
"""
import threading

import numpy as np
import pytest

from oracle import oracle as O
from tests.test_gpu_parity import assert_parity

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def served(gpu_ready):
    vsg = gpu_ready
    from vecsearch_gb300 import datasets as D
    x, _ = D.portable_clustered(60_000, 128, 64, 0.35, seed=90, centroid_seed=91)
    q, _ = D.portable_clustered(600, 128, 64, 0.35, seed=92, centroid_seed=91)
    groups = D.zipf_groups(len(x), 200, 1.1, seed=93)
    idx = vsg.GpuBruteForceIndex(128, "cosine")
    idx.add(x)
    srv = vsg.Server(idx, max_batch=256, max_k=20, slots=2)
    yield vsg, idx, srv, x, q, groups
    srv.close()


def _requests(q, groups, rng, n):
    reqs, pos = [], 0
    for _ in range(n):
        m = int(np.exp(rng.uniform(0, np.log(32))))  # 1..32 queries, log-uniform
        m = min(m, len(q) - pos) or 1
        k = int(rng.choice([10, 20]))
        filt = (groups == int(rng.integers(0, 40))) if rng.random() < 0.3 else None
        reqs.append((q[pos:pos + m], k, filt))
        pos = (pos + m) % (len(q) - 32)
    return reqs


def test_server_matches_index_paths(served):
    vsg, idx, srv, x, q, groups = served
    rng = np.random.default_rng(5)
    reqs = _requests(q, groups, rng, 40)
    tickets = [srv.submit(r, k, f) for r, k, f in reqs]
    for (r, k, f), t in zip(reqs, tickets):
        ids, dists, lat = srv.wait(t, timeout=30)
        assert ids.shape == (len(r), k) and lat > 0
        if f is None:
            bi, bd = idx.search(r, k, method="bf16")
            np.testing.assert_array_equal(ids, bi)
            np.testing.assert_array_equal(dists.view(np.uint32), bd.view(np.uint32))
        else:
            wi, wd = O.search(x, r, k, "ip", num_threads=4, allowed=f.astype(np.uint8))
            assert_parity(ids, dists, wi, wd, x, r, "ip")
    st = srv.stats()
    assert st["requests"] >= 40 and st["batches"] >= 1 and st["slots"] >= 1


def test_alone_equals_in_the_mix(served):
    vsg, idx, srv, x, q, groups = served
    rng = np.random.default_rng(6)
    probe = (q[100:117], 10, groups == 3)
    alone = srv.wait(srv.submit(*probe), timeout=30)
    others = _requests(q, groups, rng, 60)
    barrier = threading.Barrier(3)
    out = {}

    def flood(part):
        barrier.wait()
        ts = [srv.submit(r, k, f) for r, k, f in part]
        out[id(part)] = [srv.wait(t, timeout=60) for t in ts]

    threads = [threading.Thread(target=flood, args=(others[i::2],)) for i in range(2)]
    for th in threads:
        th.start()
    barrier.wait()
    mixed = srv.wait(srv.submit(*probe), timeout=60)
    for th in threads:
        th.join()
    np.testing.assert_array_equal(mixed[0], alone[0])
    np.testing.assert_array_equal(mixed[1].view(np.uint32), alone[1].view(np.uint32))


def test_server_rejects_bad_requests(served):
    vsg, idx, srv, x, q, groups = served
    with pytest.raises(ValueError):
        srv.submit(q[:300], 10)  # more queries than a slot holds
    with pytest.raises(ValueError):
        srv.submit(q[:3], 21)  # k above max_k
    with pytest.raises(ValueError):
        srv.submit(q[:3], 10, np.ones(5, bool))
