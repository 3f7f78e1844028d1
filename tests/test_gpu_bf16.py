"""GPU: the precision form (BF16 tcgen05 shortlist + exact FP32 rerank) against the plain path.

The rerank recomputes each shortlisted row with the streaming scan kernel's arithmetic, so for
every query whose shortlist holds the true top-k the result is bit-identical to method "skinny".
Recall@k is checked against the FP64 oracle.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _data(n, nq, d, clusters, unit, seed):
    from vecsearch_gb300 import datasets as D
    x, _ = D.portable_clustered(n, d, clusters, 0.35, seed=seed, centroid_seed=seed + 1, unit=unit)
    q, _ = D.portable_clustered(nq, d, clusters, 0.35, seed=seed + 2, centroid_seed=seed + 1, unit=unit)
    return x, q


@pytest.mark.parametrize("metric,unit", [("ip", True), ("l2", False)])
def test_bf16_shortlist_equals_plain(gpu_ready, metric, unit):
    vsg = gpu_ready
    x, q = _data(100_000, 300, 384, 256, unit, 40)
    gpu = vsg.GpuBruteForceIndex(384, metric)
    gpu.add(x)
    pi, pd = gpu.search(q, 10, method="skinny")
    bi, bd = gpu.search(q, 10, method="bf16")
    same = (bi == pi).all(1)
    assert same.mean() >= 0.99, same.mean()
    np.testing.assert_array_equal(bd[same].view(np.uint32), pd[same].view(np.uint32))
    gi, _ = O.fp64_topk(x, q, 10, metric)
    assert vsg.recall_at_k(bi, gi, 10) >= 0.999
    assert np.all(np.diff(bd, axis=1) >= 0)


def test_bf16_odd_shapes(gpu_ready):
    # dim not a multiple of 64, fewer rows than a tile, queries not a multiple of 128, k > rows
    vsg = gpu_ready
    from vecsearch_gb300 import datasets as D
    for n, d, nq, k in ((90, 37, 5, 10), (5000, 40, 131, 17), (300, 200, 1, 128)):
        x = D.portable(n, d, 50 + n, normalize=True)
        q = D.portable(nq, d, 60 + n, normalize=True)
        gpu = vsg.GpuBruteForceIndex(d, "cosine")
        gpu.add(x)
        pi, pd = gpu.search(q, k, method="skinny")
        bi, bd = gpu.search(q, k, method="bf16")
        np.testing.assert_array_equal(bi, pi)
        np.testing.assert_array_equal(bd, pd)


def test_bf16_copy_follows_adds(gpu_ready):
    vsg = gpu_ready
    x, q = _data(20_000, 40, 128, 64, True, 70)
    gpu = vsg.GpuBruteForceIndex(128, "cosine")
    gpu.add(x[:5000])
    gpu.search(q, 10, method="bf16")  # builds the bf16 copy of 5000 rows
    gpu.add(x[5000:])                 # the copy must follow (and survive the buffer growth)
    bi, bd = gpu.search(q, 10, method="bf16")
    pi, pd = gpu.search(q, 10, method="skinny")
    np.testing.assert_array_equal(bi, pi)
    np.testing.assert_array_equal(bd, pd)


def test_bf16_k100_recall(gpu_ready):
    vsg = gpu_ready
    x, q = _data(50_000, 64, 384, 128, True, 80)
    gpu = vsg.GpuBruteForceIndex(384, "cosine")
    gpu.add(x)
    bi, _ = gpu.search(q, 100, method="bf16")  # k' = 128
    gi, _ = O.fp64_topk(x, q, 100, "ip")
    assert vsg.recall_at_k(bi, gi, 100) >= 0.99
    gpu.set_tunable("shortlist_oversample", 1.0)
    assert gpu.get_tunable("shortlist_oversample") == 1.0


@pytest.mark.parametrize("metric,unit", [("ip", True), ("l2", False)])
def test_bf16_large_shortlist_many_items(gpu_ready, metric, unit):
    # k = 100 (k' = 120): candidate buffers of 256, several (query block, split) items per CTA and
    # thresholds shared across splits; ids must still match the plain path wherever the shortlist
    # holds the top k (recall 1.0 against FP64).
    vsg = gpu_ready
    x, q = _data(120_000, 300, 128, 128, unit, 80)
    q = np.concatenate([q, q[:212] + 0.001])  # 512 queries: 4 query blocks
    gpu = vsg.GpuBruteForceIndex(128, metric)
    gpu.add(x)
    pi, pd = gpu.search(q, 100, method="skinny")
    bi, bd = gpu.search(q, 100, method="bf16")
    same = (bi == pi).all(1)
    assert same.mean() >= 0.99, same.mean()
    np.testing.assert_array_equal(bd[same].view(np.uint32), pd[same].view(np.uint32))
    gi, _ = O.fp64_topk(x, q[:64], 100, metric)
    assert vsg.recall_at_k(bi[:64], gi, 100) >= 0.999


def test_bf16_wide_rows_stream_query_chunks(gpu_ready):
    # dim 700 (> 640): the query block does not stay resident; each ring slot carries its chunk.
    vsg = gpu_ready
    from vecsearch_gb300 import datasets as D
    x = D.portable(30_000, 700, 81, normalize=True)
    q = np.concatenate([x[:150] * 0.9 + D.portable(150, 700, 82, normalize=True) * 0.1])
    gpu = vsg.GpuBruteForceIndex(700, "cosine")
    gpu.add(x)
    pi, pd = gpu.search(q, 10, method="skinny")
    bi, bd = gpu.search(q, 10, method="bf16")
    same = (bi == pi).all(1)
    assert same.mean() >= 0.99, same.mean()
    np.testing.assert_array_equal(bd[same].view(np.uint32), pd[same].view(np.uint32))


@pytest.mark.parametrize("metric,unit", [("ip", True), ("l2", False)])
def test_bf16_sample_sizes_agree(gpu_ready, metric, unit, tmp_path):
    # 300 queries make 3 query blocks (the last one padded). With or without the sample pass the
    # shortlist holds the same top 10 here, so the reranked results are the same bits; a tuning
    # file of the older format (a third bf16 column) still loads.
    vsg = gpu_ready
    x, q = _data(150_000, 300, 256, 128, unit, 83)
    gpu = vsg.GpuBruteForceIndex(256, metric)
    gpu.add(x)
    base_i, base_d = None, None
    for version, sample in ((1, 0), (2, 0), (2, 4096), (2, 16384)):
        t = tmp_path / f"t{version}{sample}.txt"
        extra = " 4" if version == 1 else ""
        t.write_text(f"vsg-tuning {version} dim 256 rows 150000 metric 0 sms 0\nbf16 1 {sample}{extra}\n")
        gpu.load_tuning(t)
        assert gpu.tuning("bf16") == [{"batch": 1, "sample": sample}]
        bi, bd = gpu.search(q, 10, method="bf16")
        if base_i is None:
            base_i, base_d = bi, bd
            pi, pd = gpu.search(q, 10, method="skinny")
            same = (bi == pi).all(1)
            assert same.mean() >= 0.99, same.mean()
        else:
            np.testing.assert_array_equal(bi, base_i)
            np.testing.assert_array_equal(bd.view(np.uint32), base_d.view(np.uint32))


@pytest.mark.parametrize("metric,unit", [("ip", True), ("l2", False)])
def test_fp8_shortlist(gpu_ready, metric, unit):
    # FP8-e4m3 copy with per-row scales: a coarser shortlist (k' = 8k here), the same exact rerank.
    vsg = gpu_ready
    x, q = _data(100_000, 300, 384, 256, unit, 90)
    gpu = vsg.GpuBruteForceIndex(384, metric)
    gpu.add(x)
    gpu.set_tunable("shortlist_oversample", 8)
    pi, pd = gpu.search(q, 10, method="skinny")
    fi, fd = gpu.search(q, 10, method="fp8")
    same = (fi == pi).all(1)
    assert same.mean() >= 0.97, same.mean()
    np.testing.assert_array_equal(fd[same].view(np.uint32), pd[same].view(np.uint32))
    gi, _ = O.fp64_topk(x, q, 10, metric)
    assert vsg.recall_at_k(fi, gi, 10) >= 0.99
    assert np.all(np.diff(fd, axis=1) >= 0)


def test_fp8_odd_shapes(gpu_ready):
    # dim not a multiple of 16, fewer rows than a tile, k' >= rows (then the shortlist is exact)
    vsg = gpu_ready
    from vecsearch_gb300 import datasets as D
    for n, d, nq, k in ((90, 37, 5, 10), (300, 200, 1, 120), (5000, 40, 131, 17)):
        x = D.portable(n, d, 70 + n, normalize=True)
        q = D.portable(nq, d, 80 + n, normalize=True)
        gpu = vsg.GpuBruteForceIndex(d, "cosine")
        gpu.add(x)
        gpu.set_tunable("shortlist_oversample", 8)
        pi, pd = gpu.search(q, k, method="skinny")
        fi, fd = gpu.search(q, k, method="fp8")
        if min(120, 8 * k) >= n:
            np.testing.assert_array_equal(fi, pi)
            np.testing.assert_array_equal(fd, pd)
        else:
            assert vsg.recall_at_k(fi, pi, k) >= 0.95


@pytest.mark.parametrize("sample_rows", [0, 16384])
def test_merge_gather_and_overflow(gpu_ready, sample_rows):
    # k = 100 (k' = 120) over ~130 splits of 1,536 rows. Without a sample pass every split keeps
    # 120 rows, ~15,700 per query, more than the merge's gather staging (4,096): the list merge
    # runs. With the 16K-row sample, ~1,200 rows per query survive: the gather merge sorts ten
    # 128-entry chunks over eight warps. Both must give the same answers as the scan kernel.
    vsg = gpu_ready
    x, q = _data(200_000, 8, 64, 128, True, 85)
    gpu = vsg.GpuBruteForceIndex(64, "cosine")
    gpu.add(x)
    gpu.set_tunable("sample_rows", sample_rows)
    pi, pd = gpu.search(q, 100, method="skinny")
    ei, ed = gpu.search(q, 100, method="tc_exact")
    np.testing.assert_array_equal(ei, pi)
    np.testing.assert_array_equal(ed.view(np.uint32), pd.view(np.uint32))
    bi, bd = gpu.search(q, 100, method="bf16")
    same = (bi == pi).all(1)
    assert same.mean() >= 0.75, same.mean()
    np.testing.assert_array_equal(bd[same].view(np.uint32), pd[same].view(np.uint32))
    gi, _ = O.fp64_topk(x, q, 100, "ip")
    assert vsg.recall_at_k(bi, gi, 100) >= 0.99
