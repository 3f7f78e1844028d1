"""GPU: filtered exact search and the HNSW exact_below route against the reference and the oracle.

Restates tests/cpp/test_filter.cpp:72-121 and tests/python/test_bindings.py:76-91 for the GPU route,
with the parity rule of test_gpu_parity.py.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.conftest import load_golden
from tests.test_gpu_parity import assert_parity

pytestmark = pytest.mark.gpu


MODES = {"gather": 1.0, "masked_full_scan": 0.0}  # gather_max_fraction forcing each filter mode


@pytest.mark.parametrize("mode", sorted(MODES))
@pytest.mark.parametrize("name", ["filter_exact", "filter_third"])
def test_hnsw_exact_below_matches_reference(gpu_ready, name, mode):
    vsg = gpu_ready
    want_i, want_d, x, q, k, metric, extra = load_golden(name)
    gpu = vsg.GpuBruteForceIndex(x.shape[1], metric)
    gpu.add(x)
    gpu.set_tunable("gather_max_fraction", MODES[mode])
    route = vsg.HNSWExactRoute(gpu)
    mask = extra["mask"].astype(bool)
    ids, dists = route.search(q, k=k, filter=mask, exact_below=extra["exact_below"])
    assert_parity(ids, dists, want_i, want_d, x, q, metric)
    assert mask[ids[ids >= 0]].all()  # only allowed ids (test_filter.cpp:72-80)
    # same through the plain filtered search
    ids2, dists2 = gpu.search(q, k, filter=mask)
    np.testing.assert_array_equal(ids2, ids)


def test_exact_below_routing_rules(gpu_ready):
    vsg = gpu_ready
    from vecsearch_gb300 import datasets as D
    x, q = D.portable(5000, 32, 30), D.portable(20, 32, 31)
    gpu = vsg.GpuBruteForceIndex(32)
    gpu.add(x)

    class Graph:  # stands in for the HNSW graph search; records that it was asked
        calls = 0

        def search(self, *a, **kw):
            Graph.calls += 1
            return "graph"

    route = vsg.HNSWExactRoute(gpu, graph=Graph())
    empty = np.zeros(5000, bool)  # test_filter.cpp:110-113: no allowed id -> nothing
    ids, d = route.search(q, k=10, filter=empty, exact_below=100)
    assert (ids == -1).all() and np.isinf(d).all()
    few = np.zeros(5000, bool)
    few[[7, 4000]] = True  # test_filter.cpp:115-121: fewer allowed than k
    ids, d = route.search(q, k=10, filter=few, exact_below=100)
    assert set(ids[:, :2].ravel()) <= {7, 4000} and (ids[:, 2:] == -1).all()
    many = np.ones(5000, bool)
    assert route.search(q, k=10, filter=many, exact_below=100) == "graph"  # 5000 > exact_below
    assert route.search(q, k=10) == "graph"  # no filter -> graph
    assert Graph.calls == 2
    with pytest.raises(ValueError):
        route.search(q, filter=np.ones(5, bool), exact_below=10)  # bindings.cpp:28-36


def test_allow_all_equals_unfiltered(gpu_ready):
    # test_filter.cpp:99-108
    vsg = gpu_ready
    _, _, x, q, k, metric, _ = load_golden("gpu_cpu_d128_ip")
    gpu = vsg.GpuBruteForceIndex(128, metric)
    gpu.add(x)
    # filters run in the streaming scan kernel; the same kernel unfiltered is bit-identical
    a = gpu.search(q, k, method="skinny")
    b = gpu.search(q, k, filter=np.ones(len(x), np.uint8))
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    # the large-batch tiled kernel sums in another order: equal within the FP32 tolerance
    t = gpu.search(q, k, method="tiled")
    np.testing.assert_allclose(t[1], b[1], rtol=1e-5, atol=2e-6)
    O.check_ids(t[0], b[0], x, q, metric)


@pytest.mark.parametrize("mode", sorted(MODES))
@pytest.mark.parametrize("metric", ["ip", "l2"])
def test_per_query_group_masks(gpu_ready, metric, mode):
    # Config 3 shape at small size: Zipf group labels, each query filtered to one group.
    vsg = gpu_ready
    from vecsearch_gb300 import datasets as D
    x, _ = D.portable_clustered(40000, 96, 64, 0.35, seed=5, centroid_seed=6, unit=metric == "ip")
    q, _ = D.portable_clustered(70, 96, 64, 0.35, seed=7, centroid_seed=6, unit=metric == "ip")
    groups = D.zipf_groups(len(x), 200, 1.1, seed=9)
    qg = np.arange(70) % 200  # includes big and tiny groups; some have fewer rows than k
    masks = np.stack([groups == g for g in qg])
    gpu = vsg.GpuBruteForceIndex(96, metric)
    gpu.add(x)
    gpu.set_tunable("gather_max_fraction", MODES[mode])
    ids, dists = gpu.search(q, 10, filter=masks)
    for i in range(len(q)):
        wi, wd = O.search(x, q[i:i + 1], 10, metric, num_threads=2, allowed=masks[i].astype(np.uint8))
        assert_parity(ids[i:i + 1], dists[i:i + 1], wi, wd, x, q[i:i + 1], metric)
    with pytest.raises(ValueError):
        gpu.search(q, 10, filter=masks[:5])  # wrong number of rows


def test_filter_modes_agree_bitwise_and_shared_mask(gpu_ready):
    # Both filter modes compute the same per-pair arithmetic: results are bit-identical.
    vsg = gpu_ready
    from vecsearch_gb300 import datasets as D
    x, _ = D.portable_clustered(50000, 128, 32, 0.35, seed=15, centroid_seed=16)
    q, _ = D.portable_clustered(40, 128, 32, 0.35, seed=17, centroid_seed=16)
    gpu = vsg.GpuBruteForceIndex(128, "cosine")
    gpu.add(x)
    for frac in (0.001, 0.05, 0.5, 0.97):
        mask = D.portable_mask(len(x), frac, seed=int(frac * 1000) + 1).astype(bool)
        out = {}
        for mode, v in MODES.items():
            gpu.set_tunable("gather_max_fraction", v)
            out[mode] = gpu.search(q, 17, filter=mask)
        np.testing.assert_array_equal(out["gather"][0], out["masked_full_scan"][0])
        np.testing.assert_array_equal(out["gather"][1].view(np.uint32), out["masked_full_scan"][1].view(np.uint32))
        wi, wd = O.search(x, q, 17, "ip", num_threads=4, allowed=mask.astype(np.uint8))
        assert_parity(out["gather"][0], out["gather"][1], wi, wd, x, q, "ip")
    with pytest.raises(ValueError):
        gpu.set_tunable("gather_max_fraction", 2.0)
    with pytest.raises(ValueError):
        gpu.set_tunable("no_such_knob", 1.0)


def test_device_masks_per_query(gpu_ready):
    # Device-resident per-query masks through vsg_search_device.
    import torch
    vsg = gpu_ready
    from vecsearch_gb300 import datasets as D
    x = D.portable(20000, 64, 41, normalize=True)
    q = D.portable(12, 64, 42, normalize=True)
    groups = D.zipf_groups(len(x), 50, 1.1, seed=4)
    words = D.group_masks(groups, np.arange(12) % 50)
    gpu = vsg.GpuBruteForceIndex(64, "cosine")
    gpu.add(x)
    qd, wd = torch.from_numpy(q).cuda(), torch.from_numpy(words.view(np.int32)).cuda()
    oi = torch.empty((12, 10), dtype=torch.int32, device="cuda")
    od = torch.empty((12, 10), dtype=torch.float32, device="cuda")
    gpu.search_device(qd.data_ptr(), 64, 12, 10, oi.data_ptr(), od.data_ptr(),
                      stream=torch.cuda.current_stream().cuda_stream, mask_ptr=wd.data_ptr(), per_query=True,
                      mask_ld=words.shape[1])
    gpu.sync()
    torch.cuda.synchronize()
    hi, hd = gpu.search(q, 10, filter=np.stack([groups == g for g in np.arange(12) % 50]))
    np.testing.assert_array_equal(oi.cpu().numpy().astype(np.int64), hi)
    np.testing.assert_array_equal(od.cpu().numpy(), hd)
