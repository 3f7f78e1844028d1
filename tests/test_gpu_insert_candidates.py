"""GPU: exact neighbour candidates for an HNSW build in insertion order (insert_candidates).

Row i's list must be the exact k nearest of rows 0 .. i-1 (the nodes the reference's
HNSWIndex::insert, src/hnsw.cpp:247-309, searches when it inserts node i): against the oracle
(the reference's CPU search restated, over the prefix) by the parity rule, and bit for bit against
one masked GPU search over the same prefix, across batch boundaries.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.test_gpu_parity import assert_parity

pytestmark = pytest.mark.gpu


def _prefix_mask(n, i):
    m = np.zeros(n, bool)
    m[:i] = True
    return m


@pytest.mark.parametrize("metric,d,k,batch", [("l2", 37, 10, 256), ("ip", 128, 100, 300), ("l2", 64, 128, 1000),
                                              ("ip", 16, 5, 1)])
def test_candidates_match_prefix_search(gpu_ready, metric, d, k, batch):
    vsg = gpu_ready
    from vecsearch_gb300 import datasets as D
    n = 1200 if batch > 1 else 150
    x = D.portable(n, d, 500 + d, normalize=metric == "ip")
    ids, dists = vsg.insert_candidates(x, k, metric=metric, batch=batch)
    assert ids.shape == (n, k) and dists.shape == (n, k)
    for i in range(n):
        have = min(i, k)
        assert (ids[i, :have] >= 0).all() and (ids[i, have:] == -1).all() and np.isinf(dists[i, have:]).all()
        assert (ids[i, :have] < i).all()
    # against the oracle over each row's prefix (rows with at least one earlier row)
    rows = list(range(1, n, max(1, n // 97)))
    for i in rows:
        wi, wd = O.search(x[:i], x[i:i + 1], k, metric, num_threads=2)
        assert_parity(ids[i:i + 1], dists[i:i + 1], wi, wd, x[:i], x[i:i + 1], metric)
    # bit for bit against one masked search of the full index over the same prefix
    full = vsg.GpuBruteForceIndex(d, metric)
    full.add(x)
    for i in rows[::7] + [n - 1]:
        gi, gd = full.search(x[i:i + 1], k, method="skinny", filter=_prefix_mask(n, i))
        np.testing.assert_array_equal(ids[i], gi[0])
        np.testing.assert_array_equal(dists[i].view(np.uint32), gd[0].view(np.uint32))


def test_candidates_arguments(gpu_ready):
    vsg = gpu_ready
    x = np.ones((4, 8), np.float32)
    ids, dists = vsg.insert_candidates(x, 0)
    assert ids.shape == (4, 0)
    with pytest.raises(ValueError):
        vsg.insert_candidates(x, 129)
    with pytest.raises(ValueError):
        vsg.insert_candidates(x, 3, metric="hamming")
    ids, dists = vsg.insert_candidates(x, 3)  # equal rows: ties to the lower id
    assert ids.tolist() == [[-1, -1, -1], [0, -1, -1], [0, 1, -1], [0, 1, 2]]
    assert (dists[1:, 0] == 0).all()
