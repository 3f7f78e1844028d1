"""GPU: the CUDA path against the reference's outputs (golden fixtures) and the oracle.

The reference's own test cases run through both front ends: the ctypes package and the pybind11
module (the form of the reference's bindings), which call the same library.

Parity rule (stated with every check): ids equal the reference's, except at near-ties,
where both disagreeing rows' float64 distances lie within 1e-6 (relative) of each other
or of the k-th float64 distance; distances equal the reference's within
rtol 1e-5 + atol 2e-6 (FP32 sums in a different order).
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.conftest import load_golden
from tests.golden.make_golden import CASES

pytestmark = pytest.mark.gpu

RTOL, ATOL, REL_TIE = 1e-5, 2e-6, 1e-6
METHODS = ["naive", "skinny", "tiled", "auto"]
BF_CASES = [c["name"] for c in CASES if not c["name"].startswith("filter")]


def assert_parity(ids, dists, want_i, want_d, x, q, metric):
    want64 = O.ids_to_int64(want_i)
    assert ids.shape == want64.shape and ids.dtype == np.int64 and dists.dtype == np.float32
    np.testing.assert_allclose(dists, want_d, rtol=RTOL, atol=ATOL)
    O.check_ids(ids, want64, x, q, metric, rel=REL_TIE)
    fin = np.isfinite(dists)
    assert np.all(np.diff(np.where(fin, dists, np.finfo(np.float32).max), axis=1) >= 0)
    assert ((ids >= 0) == fin).all()


@pytest.fixture(params=["ctypes", "pybind"])
def front(gpu_ready, request):
    """The index class of either front end: the ctypes package or the pybind11 module."""
    vsg = gpu_ready
    if request.param == "ctypes":
        return vsg.GpuBruteForceIndex
    mod = vsg.pybind_module()
    if mod is None:
        pytest.skip("the pybind11 front end was not built (no pybind11 headers)")
    return mod.GpuBruteForceIndex


@pytest.mark.parametrize("name", BF_CASES)
def test_golden(front, name):
    want_i, want_d, x, q, k, metric, _ = load_golden(name)
    idx = front(x.shape[1], metric)
    idx.add(x)
    ids, dists = idx.search(q, k)
    assert_parity(ids, dists, want_i, want_d, x, q, metric)


@pytest.mark.parametrize("metric", ["l2", "ip"])
@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("d", [37, 128])
@pytest.mark.parametrize("nq", [1, 5, 300])
def test_matches_cpu(front, metric, method, d, nq):
    # tests/python/test_gpu.py:17-33, with two adds so the device buffer grows.
    want_i, want_d, x, q, k, _, _ = load_golden(f"gpu_cpu_d{d}_{metric}")
    gpu = front(d, metric)
    gpu.add(x[:1000])
    gpu.add(x[1000:])
    assert len(gpu) == 3000 and gpu.dim == d
    ids, dists = gpu.search(q[:nq], k, method=method)
    assert_parity(ids, dists, want_i[:nq], want_d[:nq], x, q[:nq], metric)


@pytest.mark.parametrize("k", [1, 16, 17, 100, 128])
def test_k_buckets(front, k):
    # tests/python/test_gpu.py:36-45 (there: recall > 0.99; here: the parity rule)
    want_i, want_d, x, q, _, metric, _ = load_golden("kbuckets")
    gpu = front(64)
    gpu.add(x)
    ids, dists = gpu.search(q, k)
    assert_parity(ids, dists, want_i[:, :k], want_d[:, :k], x, q, metric)


def test_many_queries_and_chunks(front):
    # tests/python/test_gpu.py:48-57: 5000 queries over 70000 rows.
    want_i, want_d, x, q, k, metric, _ = load_golden("chunks")
    gpu = front(16)
    gpu.add(x)
    ids, dists = gpu.search(q, k)
    assert_parity(ids, dists, want_i, want_d, x, q, metric)


def test_missing_results_and_limits(front):
    # tests/python/test_gpu.py:60-70
    gpu = front(8)
    ids, dists = gpu.search(np.zeros((2, 8), np.float32), 5)  # empty index
    assert (ids == -1).all() and np.isinf(dists).all()
    from vecsearch_gb300 import datasets as D
    gpu.add(D.portable(3, 8, 7))
    ids, dists = gpu.search(np.zeros(8, np.float32), 5)
    assert (ids[0, :3] >= 0).all() and (ids[0, 3:] == -1).all() and np.isinf(dists[0, 3:]).all()
    with pytest.raises(ValueError):
        gpu.search(np.zeros(8, np.float32), 129)
    with pytest.raises(ValueError):
        gpu.search(np.zeros(8, np.float32), 5, method="fast")
    with pytest.raises(ValueError):
        gpu.search(np.zeros((2, 9), np.float32), 5)
    ids, dists = gpu.search(np.zeros((0, 8), np.float32), 5)
    assert ids.shape == (0, 5)
    ids, dists = gpu.search(np.zeros((2, 8), np.float32), 0)
    assert ids.shape == (2, 0)


def test_padding_known_answers(gpu_ready):
    # tests/cpp/test_brute_force.cpp:9-20 and :45-65
    vsg = gpu_ready
    for name in ("line", "pad", "clamp"):
        want_i, want_d, x, q, k, metric, _ = load_golden(name)
        gpu = vsg.GpuBruteForceIndex(x.shape[1], metric)
        gpu.add(x)
        ids, dists = gpu.search(q, k)
        np.testing.assert_array_equal(ids, O.ids_to_int64(want_i))
        np.testing.assert_allclose(dists, want_d, rtol=RTOL, atol=ATOL)


@pytest.mark.parametrize("method", ["skinny", "tiled"])
def test_batch_invariance_bitwise(gpu_ready, method):
    # Within one kernel a query's result does not depend on the batch it is searched in: each
    # kernel sums a (query, row) pair in an order fixed by the dims alone.
    vsg = gpu_ready
    _, _, x, q, k, metric, _ = load_golden("gpu_cpu_d128_ip")
    gpu = vsg.GpuBruteForceIndex(128, metric)
    gpu.add(x)
    all_i, all_d = gpu.search(q, k, method=method)
    for sl in (slice(0, 1), slice(7, 9), slice(100, 105), slice(37, 300)):
        i, d = gpu.search(q[sl], k, method=method)
        np.testing.assert_array_equal(i, all_i[sl])
        np.testing.assert_array_equal(d.view(np.uint32), all_d[sl].view(np.uint32))
    # across kernels (method "auto" picks by batch size) the sums agree within the FP32 tolerance
    other = gpu.search(q, k, method="tiled" if method == "skinny" else "skinny")
    np.testing.assert_allclose(other[1], all_d, rtol=RTOL, atol=ATOL)
    O.check_ids(other[0], all_i, x, q, metric, rel=REL_TIE)


def test_concurrent_callers_get_their_own_results(gpu_ready):
    # Host threads searching one index at once, with different methods, k, batch sizes and
    # filters: the index serialises its calls (one mutex per index, as the reference's
    # GpuBruteForceIndex does, src/gpu_brute_force.cu:351,430), so each call returns what it
    # returns alone, bit for bit.
    import threading
    vsg = gpu_ready
    from vecsearch_gb300 import datasets as D
    x = D.portable(30_000, 96, 300, normalize=True)
    q = D.portable(200, 96, 301, normalize=True)
    gpu = vsg.GpuBruteForceIndex(96, "cosine")
    gpu.add(x)
    mask = np.zeros(len(x), bool)
    mask[::3] = True
    calls = [(q[:1], 10, "auto", None), (q[:37], 5, "skinny", None), (q, 10, "tc_exact", None),
             (q[:150], 17, "tiled", None), (q[:64], 10, "auto", mask), (q[3:133], 10, "skinny", mask)]
    want = [gpu.search(qq, k, method=m, filter=f) for qq, k, m, f in calls]
    got = [[] for _ in calls]
    errors = []
    barrier = threading.Barrier(len(calls), timeout=120)

    def run(j):
        try:
            qq, k, m, f = calls[j]
            barrier.wait()
            for _ in range(4):
                got[j].append(gpu.search(qq, k, method=m, filter=f))
        except Exception as e:  # reported below, on the main thread
            errors.append(e)

    threads = [threading.Thread(target=run, args=(j,)) for j in range(len(calls))]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=600)
    assert not any(t.is_alive() for t in threads)
    assert not errors, errors
    for j, (wi, wd) in enumerate(want):
        assert len(got[j]) == 4
        for gi, gd in got[j]:
            np.testing.assert_array_equal(gi, wi)
            np.testing.assert_array_equal(gd.view(np.uint32), wd.view(np.uint32))


def test_duplicate_rows_tie_to_lower_id(gpu_ready):
    # Equal distances go to the lower id (brute_force.cpp:152-169 merge order).
    vsg = gpu_ready
    from vecsearch_gb300 import datasets as D
    base = D.portable(200, 24, 12)
    x = np.concatenate([base, base, base])  # every row three times
    q = D.portable(9, 24, 13)
    gpu = vsg.GpuBruteForceIndex(24, "l2")
    gpu.add(x)
    ids, dists = gpu.search(q, 12)
    oi, od = O.search(x, q, 12, "l2")
    np.testing.assert_array_equal(ids % 200, O.ids_to_int64(oi) % 200)
    for row_i, row_d in zip(ids, dists):
        for a in range(0, 12, 3):
            assert (row_d[a] == row_d[a:a + 3]).all() and list(row_i[a:a + 3]) == sorted(row_i[a:a + 3])


# Config-shape fixtures: the reference's outputs for 100k x 384 rows from a 256-cluster mixture.
#   c1          unit rows, 1,000 queries, IP, k = 10 (config 1: batch sizes 1 and 128)
#   c1_k100     the same base, 256 queries, k = 100
#   c2_l2_100k  unnormalised rows of the same mixture, 256 queries, L2, k = 10
# Every method runs each case at batch 1 and batch 128 over the queries in order. Method auto
# takes the scan kernel at batch 1 on an index this small and the certified tensor-core path
# (tc_exact) at batch 128; tc_exact runs the certified path at both.
CONFIG_CASES = {"c1": 1000, "c1_k100": 256, "c2_l2_100k": 256}
CONFIG_METHODS = ["auto", "tc_exact", "skinny", "tiled"]


@pytest.fixture(scope="module")
def config_indexes(gpu_ready):
    vsg = gpu_ready
    out = {}
    for name in CONFIG_CASES:
        want_i, want_d, x, q, k, metric, _ = load_golden(name)
        gpu = vsg.GpuBruteForceIndex(384, metric)
        gpu.add(x)
        out[name] = (want_i, want_d, x, q, k, metric, gpu)
    yield out
    out.clear()


@pytest.mark.parametrize("batch", [1, 128])
@pytest.mark.parametrize("method", CONFIG_METHODS)
@pytest.mark.parametrize("name", list(CONFIG_CASES))
def test_config_cases_against_reference(config_indexes, name, method, batch):
    want_i, want_d, x, q, k, metric, gpu = config_indexes[name]
    nq = len(q) if batch > 1 or name == "c1" else 64  # batch 1: every c1 query, 64 of the others
    q0 = gpu.tc_exact_stats()[0]
    parts = [gpu.search(q[s:min(s + batch, nq)], k, method=method) for s in range(0, nq, batch)]
    ids = np.concatenate([p[0] for p in parts])
    dists = np.concatenate([p[1] for p in parts])
    assert_parity(ids, dists, want_i[:nq], want_d[:nq], x, q[:nq], metric)
    certified = gpu.tc_exact_stats()[0] - q0
    if method == "tc_exact":
        assert certified == nq  # the certified path answered (its unproven queries via the scan)
    elif method == "auto" and batch == 128:  # batches of 128 (not a shorter last one) on this index
        assert certified == sum(len(p[0]) for p in parts if len(p[0]) >= 128)


def test_c1_config_against_fp64(config_indexes):
    # Config 1: the GPU's ids against the FP64 oracle (recall 1.0 up to the near-tie rule).
    _, _, x, q, k, metric, gpu = config_indexes["c1"]
    gi, _ = O.fp64_topk(x, q, k, metric)
    ids, _ = gpu.search(q, k)
    O.check_ids(ids, gi, x, q, metric, rel=REL_TIE)
