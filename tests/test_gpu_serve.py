"""GPU: the continuous-batching server (certified tensor-core path in CUDA graphs).

Every served result must equal the index's FP32 scan kernel (method skinny) bit for bit, filtered
or not, and the oracle (the reference's CPU search restated) within the parity rule of
test_gpu_parity.py; and it must be the same alone and inside a burst of other requests.
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
    srv = vsg.Server(idx, max_batch=256, max_k=100, slots=2)
    yield vsg, idx, srv, x, q, groups
    srv.close()


def _requests(q, groups, rng, n):
    reqs, pos = [], 0
    for _ in range(n):
        m = int(np.exp(rng.uniform(0, np.log(32))))  # 1..32 queries, log-uniform
        m = min(m, len(q) - pos) or 1
        k = int(rng.choice([10, 20, 100]))
        filt = (groups == int(rng.integers(0, 40))) if rng.random() < 0.3 else None
        reqs.append((q[pos:pos + m], k, filt))
        pos = (pos + m) % (len(q) - 32)
    return reqs


def _same(got, want):
    np.testing.assert_array_equal(got[0], want[0])
    np.testing.assert_array_equal(got[1].view(np.uint32), want[1].view(np.uint32))


def test_server_is_exact(served):
    vsg, idx, srv, x, q, groups = served
    rng = np.random.default_rng(5)
    reqs = _requests(q, groups, rng, 40)
    tickets = [srv.submit(r, k, f) for r, k, f in reqs]
    for (r, k, f), t in zip(reqs, tickets):
        ids, dists, lat = srv.wait(t, timeout=30)
        assert ids.shape == (len(r), k) and lat > 0
        _same((ids, dists), idx.search(r, k, method="skinny", filter=f))
        wi, wd = O.search(x, r, k, "ip", num_threads=4, allowed=None if f is None else f.astype(np.uint8))
        assert_parity(ids, dists, wi, wd, x, r, "ip")
    st = srv.stats()
    assert st["requests"] >= 40 and st["batches"] >= 1 and st["slots"] >= 1
    assert st["uncertified"] < st["queries"] // 10  # the certificate holds for most queries


def test_server_falls_back_when_it_cannot_prove(gpu_ready):
    # Rows 1e-4 apart around a few centres: distances closer than the bf16 error bound, so most
    # queries are not certified and run in the FP32 scan inside the slot's graph, filtered or
    # not; results still equal the scan's bit for bit.
    vsg = gpu_ready
    from vecsearch_gb300 import datasets as D
    centres = D.portable(50, 64, 210, normalize=True)
    x = vsg.normalize(np.repeat(centres, 400, axis=0) + 1e-4 * D.portable(20_000, 64, 211))
    q = vsg.normalize(centres[:40] + 1e-3 * D.portable(40, 64, 212))
    idx = vsg.GpuBruteForceIndex(64, "cosine")
    idx.add(x)
    mask = np.zeros(len(x), bool)
    mask[::3] = True
    srv = vsg.Server(idx, max_batch=64, max_k=100, slots=2)
    try:
        reqs = [(q[:17], 10, None), (q[17:40], 100, mask), (q[5:6], 33, None), (q[20:36], 10, mask)]
        tickets = [srv.submit(r, k, f) for r, k, f in reqs]
        for (r, k, f), t in zip(reqs, tickets):
            ids, dists, _ = srv.wait(t, timeout=30)
            _same((ids, dists), idx.search(r, k, method="skinny", filter=f))
        assert srv.stats()["uncertified"] > 0  # the fallback ran
    finally:
        srv.close()


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
        srv.submit(q[:3], 101)  # k above max_k
    with pytest.raises(ValueError):
        srv.submit(q[:3], 10, np.ones(5, bool))
