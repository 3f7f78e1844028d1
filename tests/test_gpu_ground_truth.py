"""GPU: exact ground truth for ANN benchmarks (replaces bench/ground_truth.py's FAISS search)."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_ground_truth_matches_oracle_and_cli(gpu_ready, tmp_path):
    from vecsearch_gb300 import datasets as D
    from vecsearch_gb300 import ground_truth as G
    xb = D.portable(30_000, 64, 120, normalize=True)
    xq = D.portable(300, 64, 121, normalize=True)
    gt, gd = G.ground_truth(xb, xq, k=100, metric="ip", batch=128, return_distances=True)
    assert gt.dtype == np.int64 and gt.shape == (300, 100)
    wi, wd = O.search(xb, xq, 100, "ip")
    np.testing.assert_allclose(gd, wd, rtol=1e-5, atol=2e-6)
    O.check_ids(gt, O.ids_to_int64(wi), xb, xq, "ip", rel=1e-6)
    # batching does not change the answer
    np.testing.assert_array_equal(G.ground_truth(xb, xq, k=100, batch=300), gt)
    np.save(tmp_path / "base.npy", xb)
    np.save(tmp_path / "queries.npy", xq)
    assert G.main(["--data", str(tmp_path), "--k", "100", "--batch", "64"]) == 0
    np.testing.assert_array_equal(np.load(tmp_path / "gt.npy"), gt)


def test_ground_truth_small_base_pads(gpu_ready):
    from vecsearch_gb300 import datasets as D
    from vecsearch_gb300 import ground_truth as G
    xb = D.portable(50, 16, 122)
    xq = D.portable(3, 16, 123)
    gt = G.ground_truth(xb, xq, k=64, metric="l2")
    assert (gt[:, 50:] == -1).all() and (gt[:, :50] >= 0).all()
    with pytest.raises(ValueError):
        G.ground_truth(xb, xq[:, :8], k=5)
