"""GPU: the schedule autotuner (vsg_autotune) and its saved tables.

A tuned schedule changes only which kernel runs and how the rows are split, never the arithmetic
per row, so tuned method-"auto" results are bit-identical to the pinned kernel's results.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _index(vsg, n=60_000, d=96, metric="l2", seed=90):
    from vecsearch_gb300 import datasets as D
    x = D.portable(n, d, seed, normalize=(metric != "l2"))
    idx = vsg.GpuBruteForceIndex(d, metric)
    idx.add(x)
    return idx, x


def test_autotune_table_and_results(gpu_ready, tmp_path):
    vsg = gpu_ready
    from vecsearch_gb300 import datasets as D
    idx, x = _index(vsg)
    batches = (1, 16, 100, 300)
    table = idx.autotune(batches, k=10)
    assert [e["batch"] for e in table] == list(batches)
    assert all(e["kernel"] in ("skinny", "tiled", "tc_exact") and e["split"] in (1.0, 2.0) for e in table)
    for e in table:
        q = D.portable(e["batch"], 96, 1000 + e["batch"])
        ti, td = idx.search(q, 10)  # method auto consults the table
        pi, pd = idx.search(q, 10, method=e["kernel"])
        np.testing.assert_array_equal(ti, pi)
        np.testing.assert_array_equal(td.view(np.uint32), pd.view(np.uint32))
        wi, wd = O.search(x, q, 10, "l2")
        np.testing.assert_allclose(td, wd, rtol=1e-5, atol=2e-6)
        O.check_ids(ti, O.ids_to_int64(wi), x, q, "l2", rel=1e-6)

    path = tmp_path / "tuning.txt"
    idx.save_tuning(path)
    other, _ = _index(vsg, n=1000)
    assert other.tuning() == []
    other.load_tuning(path)
    assert other.tuning() == table
    assert path.read_text().startswith("vsg-tuning 2 dim 96")


def test_autotune_bf16(gpu_ready):
    vsg = gpu_ready
    from vecsearch_gb300 import datasets as D
    idx, x = _index(vsg, n=80_000, d=128, metric="cosine", seed=91)
    table = idx.autotune((8, 64, 256), k=10, method="bf16")
    assert [e["batch"] for e in table] == [8, 64, 256]
    assert all(set(e) == {"batch", "sample"} and e["sample"] in (0, 4096, 16384) for e in table)
    q = D.portable(256, 128, 92, normalize=True)
    bi, bd = idx.search(q, 10, method="bf16")
    gi, _ = O.fp64_topk(x, q, 10, "cosine")
    assert vsg.recall_at_k(bi, gi, 10) >= 0.999
    assert idx.tuning("auto") == []  # the FP32 table is separate


def test_autotune_rejects_bad_arguments(gpu_ready, tmp_path):
    vsg = gpu_ready
    idx, _ = _index(vsg, n=500)
    with pytest.raises(ValueError):
        idx.autotune((0,), k=10)
    with pytest.raises(ValueError):
        idx.autotune((8,), k=129)
    with pytest.raises(ValueError):
        idx.autotune((8,), k=10, method="tiled")
    bad = tmp_path / "bad.txt"
    bad.write_text("not a table\n")
    with pytest.raises(ValueError):
        idx.load_tuning(bad)
    with pytest.raises(ValueError):
        idx.load_tuning(tmp_path / "missing.txt")
    empty = vsg.GpuBruteForceIndex(16, "l2")
    with pytest.raises(ValueError):
        empty.autotune((8,), k=10)
    with pytest.raises(ValueError):
        idx.autotune((8,), k=10, queries=np.zeros((4, 7), np.float32))  # wrong dim


def test_autotune_with_query_sample(gpu_ready):
    vsg = gpu_ready
    from vecsearch_gb300 import datasets as D
    idx, x = _index(vsg, n=50_000, d=64, metric="l2", seed=95)
    sample = D.portable(37, 64, 96)  # fewer than the largest batch: repeated to fill it
    table = idx.autotune((8, 200), k=10, queries=sample)
    assert [e["batch"] for e in table] == [8, 200]
    q = D.portable(200, 64, 97)
    ti, td = idx.search(q, 10)
    pi, pd = idx.search(q, 10, method="skinny")
    O.check_ids(ti, pi, x, q, "l2", rel=1e-6)
    np.testing.assert_allclose(td, pd, rtol=1e-5, atol=2e-6)
