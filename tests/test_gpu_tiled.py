"""GPU: the tiled FP32 path (method "tiled") equals the streaming scan kernel bit for bit.

The tiled kernel sums each distance's products in one FMA chain, in another order than the scan
kernel, so near-ties may order differently. Its per-split lists hold a few more than k rows; the
finish kernel reranks the rows near each query's k-th best with the scan kernel's arithmetic and
proves from a bound on the difference of the two FP32 evaluations that no row left out can enter
the top k. Queries it cannot prove run in the scan kernel. Whatever the mix, the result must be
the scan kernel's (method "skinny"), ids and distance bits.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _same(a, b):
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1].view(np.uint32), b[1].view(np.uint32))


@pytest.mark.parametrize("metric,unit", [("ip", True), ("l2", False)])
@pytest.mark.parametrize("k", [1, 10, 32, 33, 100, 128])
def test_tiled_equals_scan(gpu_ready, metric, unit, k):
    vsg = gpu_ready
    from vecsearch_gb300 import datasets as D
    x, _ = D.portable_clustered(50_000, 384, 64, 0.35, seed=400, centroid_seed=401, unit=unit)
    q, _ = D.portable_clustered(200, 384, 64, 0.35, seed=402, centroid_seed=401, unit=unit)
    gpu = vsg.GpuBruteForceIndex(384, metric)
    gpu.add(x)
    t0, f0 = gpu.tiled_stats()
    _same(gpu.search(q, k, method="tiled"), gpu.search(q, k, method="skinny"))
    t1, f1 = gpu.tiled_stats()
    assert t1 - t0 == 200
    assert f1 - f0 < 20  # the certificate holds for most queries


@pytest.mark.parametrize("n,d,nq,k", [(90, 37, 5, 10), (5000, 40, 131, 17), (3000, 8, 70, 100), (300, 200, 1, 120),
                                      (40, 16, 9, 50)])
def test_tiled_shapes(gpu_ready, n, d, nq, k):
    # small and ragged shapes, k above the row count (padded with -1 / +inf)
    vsg = gpu_ready
    from vecsearch_gb300 import datasets as D
    for metric in ("ip", "l2"):
        x = D.portable(n, d, 420 + n, normalize=metric == "ip")
        q = D.portable(nq, d, 430 + n, normalize=metric == "ip")
        gpu = vsg.GpuBruteForceIndex(d, metric)
        gpu.add(x)
        _same(gpu.search(q, k, method="tiled"), gpu.search(q, k, method="skinny"))


def test_tiled_falls_back_when_it_cannot_prove(gpu_ready):
    # Each of the first 30 rows has 60 exact copies at higher ids, and the queries sit next to
    # them: a split's list fills with copies at one distance, so the certificate cannot separate
    # what it kept from what it left out and the scan kernel answers (ties to the lower id).
    vsg = gpu_ready
    from vecsearch_gb300 import datasets as D
    base = D.portable(20_000, 64, 440, normalize=True)
    x = np.concatenate([base] + [base[:30]] * 60)
    q = vsg.normalize(base[:30] + 1e-3 * D.portable(30, 64, 441))
    q = np.concatenate([q, D.portable(70, 64, 442, normalize=True)])
    gpu = vsg.GpuBruteForceIndex(64, "cosine")
    gpu.add(x)
    t0, f0 = gpu.tiled_stats()
    got = gpu.search(q, 10, method="tiled")
    _same(got, gpu.search(q, 10, method="skinny"))
    t1, f1 = gpu.tiled_stats()
    assert t1 - t0 == 100 and f1 - f0 > 0
    assert (got[0][:30, 0] == np.arange(30)).all()


def test_tiled_rows_added_later(gpu_ready):
    # The rows' norm bound follows every add: rows with a larger norm added after a first search.
    vsg = gpu_ready
    from vecsearch_gb300 import datasets as D
    x = D.portable(20_000, 128, 450)
    q = D.portable(150, 128, 451)
    gpu = vsg.GpuBruteForceIndex(128, "l2")
    gpu.add(x[:10_000])
    _same(gpu.search(q, 10, method="tiled"), gpu.search(q, 10, method="skinny"))
    gpu.add(x[10_000:] * 8.0)
    _same(gpu.search(q, 10, method="tiled"), gpu.search(q, 10, method="skinny"))
