"""GPU: the certified exact path (method "tc_exact") equals the streaming scan kernel bit for bit.

The shortlist comes from the BF16 tensor-core pass; the rerank kernel certifies each query with a
bound on the bf16 rounding error, and uncertified queries run again in the scan kernel. Whatever
the mix, the result must be the scan kernel's (method "skinny"), ids and distance bits.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _clustered(n, nq, d, clusters, unit, seed):
    from vecsearch_gb300 import datasets as D
    x, _ = D.portable_clustered(n, d, clusters, 0.35, seed=seed, centroid_seed=seed + 1, unit=unit)
    q, _ = D.portable_clustered(nq, d, clusters, 0.35, seed=seed + 2, centroid_seed=seed + 1, unit=unit)
    return x, q


def _same(a, b):
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1].view(np.uint32), b[1].view(np.uint32))


@pytest.mark.parametrize("metric,unit", [("ip", True), ("l2", False)])
def test_tc_exact_equals_scan(gpu_ready, metric, unit):
    vsg = gpu_ready
    x, q = _clustered(120_000, 300, 384, 128, unit, 200)
    gpu = vsg.GpuBruteForceIndex(384, metric)
    gpu.add(x)
    q0, s0, f0 = gpu.tc_exact_stats()
    _same(gpu.search(q, 10, method="tc_exact"), gpu.search(q, 10, method="skinny"))
    q1, s1, f1 = gpu.tc_exact_stats()
    assert q1 - q0 == 300
    assert s1 - s0 < 30 and f1 - f0 <= s1 - s0  # the certificate holds for most queries


@pytest.mark.parametrize("metric,unit", [("cosine", True), ("l2", False)])
def test_tc_exact_any_margin_is_exact(gpu_ready, metric, unit):
    # The margin only decides how many rows each query keeps: the smallest (1.0) leaves more
    # queries to the later stages, a large one keeps k' rows; the results never change.
    vsg = gpu_ready
    x, q = _clustered(60_000, 256, 128, 64, unit, 205)
    gpu = vsg.GpuBruteForceIndex(128, metric)
    gpu.add(x)
    assert gpu.get_tunable("cert_margin") == pytest.approx(1.3)
    want = gpu.search(q, 10, method="skinny")
    retried = {}
    for m in (1.0, 1.3, 3.0):
        gpu.set_tunable("cert_margin", m)
        q0, s0, _ = gpu.tc_exact_stats()
        _same(gpu.search(q, 10, method="tc_exact"), want)
        q1, s1, _ = gpu.tc_exact_stats()
        assert q1 - q0 == 256
        retried[m] = s1 - s0
    assert retried[1.0] >= retried[3.0]
    with pytest.raises(ValueError):
        gpu.set_tunable("cert_margin", 0.5)


def test_tc_exact_falls_back_when_it_cannot_prove(gpu_ready):
    # Rows 1e-4 apart around a few centres: distances closer than the bf16 error bound, so most
    # queries are not certified and run in the scan kernel; the results must not change.
    vsg = gpu_ready
    from vecsearch_gb300 import datasets as D
    centres = D.portable(50, 64, 210, normalize=True)
    x = vsg.normalize(np.repeat(centres, 400, axis=0) + 1e-4 * D.portable(20_000, 64, 211))
    q = vsg.normalize(centres[:40] + 1e-3 * D.portable(40, 64, 212))
    gpu = vsg.GpuBruteForceIndex(64, "cosine")
    gpu.add(x)
    q0, s0, f0 = gpu.tc_exact_stats()
    _same(gpu.search(q, 10, method="tc_exact"), gpu.search(q, 10, method="skinny"))
    q1, s1, f1 = gpu.tc_exact_stats()
    assert q1 - q0 == 40 and s1 - s0 > 0 and f1 - f0 > 0  # both later stages ran


def test_fallback_split_any_value_is_exact(gpu_ready):
    # Half of a 300-query batch sits where the bf16 bound cannot separate rows, so many queries
    # are left to the scan kernel. Its row splits follow fallback_split_queries (0: as for the
    # whole batch); the results never change.
    vsg = gpu_ready
    from vecsearch_gb300 import datasets as D
    centres = D.portable(50, 64, 210, normalize=True)
    x = vsg.normalize(np.repeat(centres, 400, axis=0) + 1e-4 * D.portable(20_000, 64, 211))
    near = centres[np.arange(150) % 50] + 1e-3 * D.portable(150, 64, 213)
    q = vsg.normalize(np.concatenate([near, D.portable(150, 64, 214)]).astype(np.float32))
    gpu = vsg.GpuBruteForceIndex(64, "cosine")
    gpu.add(x)
    assert gpu.get_tunable("fallback_split_queries") == 128
    want = gpu.search(q, 10, method="skinny")
    for v in (128, 0, 1, 8, 20_000):
        gpu.set_tunable("fallback_split_queries", v)
        q0, _, f0 = gpu.tc_exact_stats()
        _same(gpu.search(q, 10, method="tc_exact"), want)
        q1, _, f1 = gpu.tc_exact_stats()
        assert q1 - q0 == 300 and f1 - f0 > 0
    with pytest.raises(ValueError):
        gpu.set_tunable("fallback_split_queries", -1)


@pytest.mark.parametrize("n,d,nq,k", [(90, 37, 5, 10), (5000, 40, 131, 17), (30_000, 128, 200, 100),
                                      (300, 200, 1, 120)])
def test_tc_exact_shapes(gpu_ready, n, d, nq, k):
    vsg = gpu_ready
    from vecsearch_gb300 import datasets as D
    x = D.portable(n, d, 220 + n, normalize=True)
    q = D.portable(nq, d, 230 + n, normalize=True)
    gpu = vsg.GpuBruteForceIndex(d, "cosine")
    gpu.add(x)
    _same(gpu.search(q, k, method="tc_exact"), gpu.search(q, k, method="skinny"))


def test_tc_exact_duplicates_tie_to_lower_id(gpu_ready):
    vsg = gpu_ready
    from vecsearch_gb300 import datasets as D
    base = D.portable(3000, 96, 240, normalize=True)
    x = np.concatenate([base, base[:500], base[:500]])  # exact duplicates at higher ids
    q = base[:64] * 0.999
    gpu = vsg.GpuBruteForceIndex(96, "cosine")
    gpu.add(x)
    got = gpu.search(q, 10, method="tc_exact")
    _same(got, gpu.search(q, 10, method="skinny"))
    assert (got[0][:, 0] == np.arange(64)).all()


def test_auto_routes_large_batches(gpu_ready):
    vsg = gpu_ready
    x, q = _clustered(60_000, 256, 128, 64, True, 250)
    gpu = vsg.GpuBruteForceIndex(128, "cosine")
    gpu.add(x)
    assert gpu.get_tunable("tc_exact_min_batch") == 128
    q0 = gpu.tc_exact_stats()[0]
    _same(gpu.search(q, 10), gpu.search(q, 10, method="skinny"))  # auto: 256 >= 128, k <= 32
    assert gpu.tc_exact_stats()[0] - q0 == 256
    _same(gpu.search(q, 64), gpu.search(q, 64, method="skinny"))  # every k <= 128 unfiltered
    q1 = gpu.tc_exact_stats()[0]
    assert q1 - q0 == 512
    gpu.search(q[:64], 10)  # below the threshold: FP32 kernels
    gpu.search(q[:64], 100)
    # Filtered: the certified path when (batch x largest allowed fraction) >= 0.35, from 8 queries,
    # and for every filtered batch from half the threshold (64 queries).
    few = np.zeros(len(x), bool)
    few[::100] = True  # 1 % allowed
    gpu.search(q[:32], 10, filter=few)  # 32 x 0.01 < 0.35: the gather scan
    wide = np.ones(len(x), bool)
    gpu.search(q[:4], 10, filter=wide)  # fewer than 8 queries: the scan kernel
    assert gpu.tc_exact_stats()[0] == q1
    _same(gpu.search(q[:48], 10, filter=few), gpu.search(q[:48], 10, method="skinny", filter=few))
    assert gpu.tc_exact_stats()[0] == q1 + 48  # 48 x 0.01 >= 0.35
    _same(gpu.search(q[:16], 10, filter=wide), gpu.search(q[:16], 10, method="skinny", filter=wide))
    assert gpu.tc_exact_stats()[0] == q1 + 64  # a wide filter from 8 queries
    _same(gpu.search(q, 10, filter=few), gpu.search(q, 10, method="skinny", filter=few))
    assert gpu.tc_exact_stats()[0] == q1 + 320  # from 64 queries any filter


def test_tc_exact_filtered(gpu_ready):
    # A shared mask and per-query masks (Zipf groups: from a handful of rows, fewer than k, to
    # many): the certified path equals the filtered scan bit for bit.
    vsg = gpu_ready
    from vecsearch_gb300 import datasets as D
    x, q = _clustered(80_000, 300, 128, 64, True, 260)
    gpu = vsg.GpuBruteForceIndex(128, "cosine")
    gpu.add(x)
    shared = D.portable_mask(len(x), 0.3, seed=261)
    _same(gpu.search(q, 10, method="tc_exact", filter=shared), gpu.search(q, 10, method="skinny", filter=shared))
    groups = D.zipf_groups(len(x), 2000, 1.1, seed=262)
    pick = np.array([0, 1, 5, 50, 500, 1999])[np.arange(300) % 6]  # common to rare groups
    per_query = groups[None, :] == pick[:, None]
    assert per_query.sum(1).min() < 10
    _same(gpu.search(q, 10, method="tc_exact", filter=per_query),
          gpu.search(q, 10, method="skinny", filter=per_query))
    # auto: a large batch with a wide mask takes the certified path
    q0 = gpu.tc_exact_stats()[0]
    _same(gpu.search(q, 10, filter=shared), gpu.search(q, 10, method="skinny", filter=shared))
    assert gpu.tc_exact_stats()[0] - q0 == 300


def test_bf16_filtered(gpu_ready):
    vsg = gpu_ready
    from vecsearch_gb300 import datasets as D
    x, q = _clustered(80_000, 200, 128, 64, True, 270)
    gpu = vsg.GpuBruteForceIndex(128, "cosine")
    gpu.add(x)
    mask = D.portable_mask(len(x), 0.2, seed=271)
    for m in ("bf16", "fp8"):
        gpu.set_tunable("shortlist_oversample", 8)
        bi, bd = gpu.search(q, 10, method=m, filter=mask)
        pi, pd = gpu.search(q, 10, method="skinny", filter=mask)
        assert mask[bi[bi >= 0]].all()
        same = (bi == pi).all(1)
        assert same.mean() >= 0.97, (m, same.mean())
        np.testing.assert_array_equal(bd[same].view(np.uint32), pd[same].view(np.uint32))


def test_auto_small_batches_on_large_index(gpu_ready):
    # 360,000 x 384 = 138 M elements >= 2^27: method auto sends even one query to the certified
    # path (reading the bf16 copy, half the bytes), with the scan kernel's answers bit for bit.
    vsg = gpu_ready
    x, q = _clustered(360_000, 32, 384, 256, True, 290)
    gpu = vsg.GpuBruteForceIndex(384, "cosine")
    gpu.add(x)
    assert gpu.get_tunable("tc_exact_min_elements") == 2 ** 27
    q0 = gpu.tc_exact_stats()[0]
    k0 = gpu.kernel_launches()
    for b in (1, 3, 17):
        _same(gpu.search(q[:b], 10), gpu.search(q[:b], 10, method="skinny"))
    assert gpu.tc_exact_stats()[0] - q0 == 21
    assert gpu.kernel_launches() > k0
    gpu.set_tunable("tc_exact_min_elements", 1e12)  # small batches back to the FP32 kernels
    gpu.search(q[:4], 10)
    assert gpu.tc_exact_stats()[0] - q0 == 21
    with pytest.raises(ValueError):
        gpu.set_tunable("tc_exact_min_elements", -1)


@pytest.mark.parametrize("metric,unit,d", [("cosine", True, 384), ("l2", False, 200), ("cosine", True, 1024)])
def test_fp32_sample_small_batches(gpu_ready, metric, unit, d):
    # Up to 4 queries on an index with many splits: the query preparation computes the 4K-row
    # sample in FP32 (no tensor-core sample pass). Every batch size 1-4, k = 10 and 100 (the k-th
    # sampled distance decides the start), padded dims 384, 200 and 1,024 (the largest it takes):
    # the scan kernel's results bit for bit.
    vsg = gpu_ready
    x, q = _clustered(150_001, 12, d, 64, unit, 300 + d)
    gpu = vsg.GpuBruteForceIndex(d, metric)
    gpu.add(x)
    for k in (10, 100):
        want = gpu.search(q, k, method="skinny")
        for b in (1, 2, 3, 4):
            for s in range(0, 12, b):
                got = gpu.search(q[s:s + b], k, method="tc_exact")
                _same(got, (want[0][s:s + b], want[1][s:s + b]))


@pytest.mark.parametrize("metric,unit", [("cosine", True), ("l2", False)])
def test_tc_exact_neighbours_in_few_splits(gpu_ready, metric, unit):
    # Rows ordered by cluster: a query's near rows sit in a few splits, so those splits' lists hold
    # many entries within the finish kernel's bound from the lists' heads (sorted lists are then
    # read in several runs) while most lists hold none. Batches 1-8 (sorted lists) and 20 (lists
    # with only their smallest entry first), k = 10, 100 and 128: the scan kernel's results bit
    # for bit.
    vsg = gpu_ready
    from vecsearch_gb300 import datasets as D
    x, labels = D.portable_clustered(200_000, 256, 32, 0.35, seed=310, centroid_seed=311, unit=unit)
    x = np.ascontiguousarray(x[np.argsort(labels, kind="stable")])
    q, _ = D.portable_clustered(20, 256, 32, 0.35, seed=312, centroid_seed=311, unit=unit)
    gpu = vsg.GpuBruteForceIndex(256, metric)
    gpu.add(x)
    for k in (10, 100, 128):
        want = gpu.search(q, k, method="skinny")
        for b in (1, 3, 8, 20):
            _same(gpu.search(q[:b], k, method="tc_exact"), (want[0][:b], want[1][:b]))


@pytest.mark.parametrize("metric,unit,d", [("cosine", True, 384), ("l2", False, 200)])
def test_tc_exact_over_e4m3_copy(gpu_ready, metric, unit, d):
    # "cert_fp8_max_batch": small batches of the certified path read the e4m3 copy (one scale per
    # row and per query) with a bound E that covers its roundings; a wider margin keeps more rows
    # (about a whole cluster of these ~290-row clusters; clusters larger than the finish kernel's
    # 2,048 reranked rows would leave the queries to the scan), and the results are still the scan
    # kernel's bit for bit. Batches 1-4 (FP32 sample) and 8 (tensor-core sample), k = 10 and 100.
    vsg = gpu_ready
    x, q = _clustered(150_000, 24, d, 512, unit, 330 + d)
    gpu = vsg.GpuBruteForceIndex(d, metric)
    gpu.add(x)
    gpu.set_tunable("cert_fp8_max_batch", 8)
    assert gpu.get_tunable("cert_prefetch_max_batch") == 16
    # the finish kernel's rerank on one CTA, or shared by 8 in a cluster; the kept rows prefetched
    # into L2 by the main pass ("cert_prefetch_max_batch") or by a one-CTA finish kernel
    for cluster, prefetch in ((1, 16), (8, 16), (16, 16), (1, 0)):
        gpu.set_tunable("finish_cluster", cluster)
        gpu.set_tunable("finish_cluster_one", cluster)
        gpu.set_tunable("cert_prefetch_max_batch", prefetch)
        for k in (10, 100):
            want = gpu.search(q, k, method="skinny")
            for b in (1, 3, 8):
                for s in range(0, 16, b):
                    _same(gpu.search(q[s:s + b], k, method="tc_exact"), (want[0][s:s + b], want[1][s:s + b]))
    q0, s0, f0 = gpu.tc_exact_stats()
    gpu.search(q[:8], 10, method="tc_exact")
    q1, s1, f1 = gpu.tc_exact_stats()
    assert q1 - q0 == 8 and s1 - s0 <= 2  # the certificate holds for nearly every query
    with pytest.raises(ValueError):
        gpu.set_tunable("cert_prefetch_max_batch", -1)


@pytest.mark.parametrize("cluster", [2, 8, 16])
def test_tc_exact_finish_cluster(gpu_ready, cluster):
    # "finish_cluster": the finish kernel of a small batch runs as a cluster of CTAs per query,
    # rank 0 staging and cutting, every rank reranking a share through distributed shared memory;
    # batches whose CTAs would exceed the SM count run with one CTA a query. Bit for bit the scan's.
    vsg = gpu_ready
    x, q = _clustered(200_000, 160, 256, 128, True, 360 + cluster)
    gpu = vsg.GpuBruteForceIndex(256, "cosine")
    gpu.add(x)
    gpu.set_tunable("finish_cluster", cluster)
    assert gpu.get_tunable("finish_cluster") == cluster
    for k in (10, 100):
        want = gpu.search(q, k, method="skinny")
        for b in (1, 5, 16, 40, 160):
            _same(gpu.search(q[:b], k, method="tc_exact"), (want[0][:b], want[1][:b]))
    gpu.set_tunable("finish_cluster_one", cluster)  # (batch 1 has its own, default 16)
    for b in (1, 3):
        _same(gpu.search(q[:b], 10, method="tc_exact"), (want[0][:b, :10], want[1][:b, :10]))
    with pytest.raises(ValueError):
        gpu.set_tunable("finish_cluster", 17)


def test_tc_exact_e4m3_wide_rows_use_bf16(gpu_ready):
    # Rows wider than the e4m3 query preparation takes (1,100 dims -> 1,104 > 1,024) stay on the
    # bf16 copy under cert_fp8_max_batch: still the scan kernel's results.
    vsg = gpu_ready
    x, q = _clustered(20_000, 6, 1100, 64, True, 390)
    gpu = vsg.GpuBruteForceIndex(1100, "cosine")
    gpu.add(x)
    gpu.set_tunable("cert_fp8_max_batch", 8)
    gpu.set_tunable("finish_cluster", 8)
    want = gpu.search(q, 10, method="skinny")
    for b in (1, 6):
        _same(gpu.search(q[:b], 10, method="tc_exact"), (want[0][:b], want[1][:b]))
