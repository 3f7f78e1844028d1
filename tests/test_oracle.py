"""CPU: the oracle against the reference's own outputs (golden fixtures) and its own tests."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from oracle.build_ref import reference_present
from tests.conftest import load_golden
from tests.golden.make_golden import CASES

BF_CASES = [c["name"] for c in CASES if not c["name"].startswith("filter")]
FILTER_CASES = [c["name"] for c in CASES if c["name"].startswith("filter")]


# The config-shape fixtures (100k x 384 rows) are checked on a prefix of their queries so that
# the CPU suite stays short: the reference answers each query on its own (batch == single,
# tests/cpp/test_brute_force.cpp:22-43), so a prefix of the queries has a prefix of the answers.
CONFIG_PREFIX = 48


@pytest.mark.parametrize("name", BF_CASES)
def test_oracle_matches_reference_bitwise(name):
    want_i, want_d, x, q, k, metric, _ = load_golden(name)
    big = x.shape[0] * x.shape[1] > 10_000_000
    if big:
        want_i, want_d, q = want_i[:CONFIG_PREFIX], want_d[:CONFIG_PREFIX], q[:CONFIG_PREFIX]
    for threads in ((4,) if big else (1, 3)):
        ids, dists = O.search(x, q, k, metric, num_threads=threads)
        np.testing.assert_array_equal(ids, want_i)
        np.testing.assert_array_equal(dists.view(np.uint32), want_d.view(np.uint32))


@pytest.mark.parametrize("name", FILTER_CASES)
def test_oracle_filtered_matches_reference_exact_path(name):
    # HNSW search with filter + exact_below -> search_exact (hnsw.cpp:325-328, :336-354)
    want_i, want_d, x, q, k, metric, extra = load_golden(name)
    ids, dists = O.search(x, q, k, metric, num_threads=2, allowed=extra["mask"])
    np.testing.assert_array_equal(ids, want_i)
    np.testing.assert_array_equal(dists, want_d)
    assert extra["mask"][want_i[want_i != O.NONE]].all()


def test_line_known_answer():
    # tests/cpp/test_brute_force.cpp:9-20
    want_i, _, x, q, k, _, _ = load_golden("line")
    assert want_i[0].tolist() == [3, 4, 2]
    assert O.search(x, q, 3, "l2")[0][0].tolist() == [3, 4, 2]


def test_padding_and_clamp():
    # tests/cpp/test_brute_force.cpp:45-65
    ids, d, *_ = load_golden("pad")
    assert ids[0, 0] == 0 and ids[0, 5] == O.NONE and np.isinf(d[0, 6])
    ids, d, *_ = load_golden("clamp")
    assert ids[0, 0] == 0 and (ids[0, 50:] == O.NONE).all() and (np.diff(d[0, :50]) >= 0).all()


def test_k_prefix_property():
    # top-k for k < 128 is the prefix of top-128 (tests/python/test_gpu.py:36-45 buckets)
    want_i, _, x, q, _, metric, _ = load_golden("kbuckets")
    for k in (1, 16, 17, 100):
        ids, _ = O.search(x, q, k, metric, num_threads=2)
        np.testing.assert_array_equal(ids, want_i[:, :k])


def test_fp64_parity_rule_on_reference_outputs():
    # The reference's FP32 ids agree with the FP64 oracle up to the near-tie rule.
    want_i, want_d, x, q, k, metric, _ = load_golden("c1")
    want_i, want_d, q = want_i[:200], want_d[:200], q[:200]
    gi, gd = O.fp64_topk(x, q, k, metric)
    O.check_ids(O.ids_to_int64(want_i), gi, x, q, metric)
    np.testing.assert_allclose(want_d, gd, rtol=0, atol=2e-6)


def test_check_ids_rejects_a_planted_mismatch():
    want_i, _, x, q, k, metric, _ = load_golden("gpu_cpu_d128_l2")
    bad = O.ids_to_int64(want_i).copy()
    bad[3, 2] = (bad[3, 2] + 1234) % x.shape[0]  # a far row planted in the oracle's output
    with pytest.raises(AssertionError):
        O.check_ids(bad, O.ids_to_int64(want_i), x, q, metric)


@pytest.mark.skipif(not reference_present(), reason="reference not built here")
def test_oracle_vs_live_reference_dims():
    # distance.h tails (tests/cpp/test_distance.cpp:24-25 dims) and single == batch
    from oracle.build_ref import build_reference
    if build_reference() is None:
        pytest.skip("reference sources absent")
    R = O.Reference()
    rng = np.random.default_rng(5)
    for d in (1, 3, 7, 8, 9, 15, 16, 17, 31, 128, 384, 385):
        for metric in ("l2", "ip"):
            x = rng.standard_normal((300, d), dtype=np.float32)
            q = rng.standard_normal((6, d), dtype=np.float32)
            ri, rd = R.bf_search(x, q, 10, metric, 2)
            oi, od = O.search(x, q, 10, metric, 2)
            np.testing.assert_array_equal(ri, oi)
            np.testing.assert_array_equal(rd.view(np.uint32), od.view(np.uint32))
            si, sd = R.bf_search_one(x, q, 10, metric)
            np.testing.assert_array_equal(si, oi)


def test_check_ids_rule():
    # Near-equal rows may swap places inside the list; clearly ordered rows may not; a different
    # row is allowed only at a k-th boundary near-tie.
    x = np.array([[1.0, 0.0], [2.0, 0.0], [2.0 + 1e-7, 0.0], [3.0, 0.0], [4.0, 0.0], [4.0 + 1e-7, 0.0]],
                 np.float32)
    q = np.zeros((1, 2), np.float32)
    want = np.array([[0, 1, 2, 3, 4]])
    assert O.check_ids(np.array([[0, 2, 1, 3, 4]]), want, x, q, "l2") == 2   # near-equal swap
    with pytest.raises(AssertionError):
        O.check_ids(np.array([[1, 0, 2, 3, 4]]), want, x, q, "l2")           # 1.0 vs 4.0
    assert O.check_ids(np.array([[0, 1, 2, 3, 5]]), want, x, q, "l2") == 1   # tie at the k-th place
    with pytest.raises(AssertionError):
        O.check_ids(np.array([[0, 1, 2, 4, 5]]), want, x, q, "l2")           # row 3 dropped
