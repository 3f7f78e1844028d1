"""GPU: blocking searches replayed from a CUDA graph (tunable "host_graph_max_batch").

A blocking unfiltered search of a small batch, repeated with the same shape, runs once call by
call, is captured on its second call and replays the captured chain (copies in and out included)
afterwards. Every replay must search the queries of its own call and return what the call-by-call
search returns, ids and distance bits; adding rows, setting a tunable or changing the shape must
drop the graph.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _same(a, b):
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1].view(np.uint32), b[1].view(np.uint32))


@pytest.mark.parametrize("method", ["tc_exact", "skinny", "auto", "bf16"])
def test_replays_equal_call_by_call(gpu_ready, method):
    vsg = gpu_ready
    from vecsearch_gb300 import datasets as D
    x, _ = D.portable_clustered(200_000, 256, 64, 0.35, seed=600, centroid_seed=601)
    q, _ = D.portable_clustered(64, 256, 64, 0.35, seed=602, centroid_seed=601)
    gpu = vsg.GpuBruteForceIndex(256, "cosine")
    gpu.add(x)
    ref = vsg.GpuBruteForceIndex(256, "cosine")
    ref.add(x)
    ref.set_tunable("host_graph_max_batch", 0)
    assert gpu.get_tunable("host_graph_max_batch") == 16
    gpu.set_tunable("host_graph_direct", 0)  # the copy into device memory (direct reads: below)
    for b, k in ((1, 10), (3, 100), (16, 10)):
        launches = []
        for rep in range(6):  # call by call, captured, then replays, each with other queries
            qq = q[(rep * b) % 48:(rep * b) % 48 + b]
            l0 = gpu.kernel_launches()
            _same(gpu.search(qq, k, method=method), ref.search(qq, k, method=method))
            launches.append(gpu.kernel_launches() - l0)
        # the capture and the replays count the graph's kernels (the first call may also build
        # the index's bf16 copy)
        assert min(launches) > 0 and len(set(launches[1:])) == 1 and launches[0] >= launches[1]


def test_direct_queries_equal_copied(gpu_ready):
    # host_graph_direct (the default): the certified path's kernels read the queries from the
    # pinned staging buffer themselves (no copy in); padded rows (dim 37 -> 40) included. The
    # copied form is checked by test_replays_equal_call_by_call with direct reads off.
    vsg = gpu_ready
    from vecsearch_gb300 import datasets as D
    for d in (200, 37):
        x, _ = D.portable_clustered(120_000, d, 64, 0.35, seed=620 + d, centroid_seed=621)
        q, _ = D.portable_clustered(24, d, 64, 0.35, seed=622 + d, centroid_seed=621)
        gpu = vsg.GpuBruteForceIndex(d, "cosine")
        gpu.add(x)
        assert gpu.get_tunable("host_graph_direct") == 1
        for b, k in ((1, 10), (4, 100)):
            want = gpu.search(q, k, method="skinny")
            for rep in range(5):
                s = (rep * b) % 20
                _same(gpu.search(q[s:s + b], k, method="tc_exact"), (want[0][s:s + b], want[1][s:s + b]))
    with pytest.raises(ValueError):
        gpu.set_tunable("host_graph_direct", 2)


def test_graph_dropped_on_changes(gpu_ready):
    vsg = gpu_ready
    from vecsearch_gb300 import datasets as D
    x, _ = D.portable_clustered(150_000, 128, 32, 0.35, seed=610, centroid_seed=611)
    q, _ = D.portable_clustered(8, 128, 32, 0.35, seed=612, centroid_seed=611)
    gpu = vsg.GpuBruteForceIndex(128, "l2")
    gpu.add(x)

    def check():
        want = gpu.search(q[:1], 10, method="skinny")
        for _ in range(3):
            _same(gpu.search(q[:1], 10, method="tc_exact"), want)

    check()
    # rows added after the capture: the next searches must see them (a copy of the nearest rows
    # with smaller ids is not possible, so add exact copies of the query: they become the top 1)
    gpu.add(np.repeat(q[:1], 2, axis=0))
    got = gpu.search(q[:1], 10, method="tc_exact")
    assert set(got[0][0, :2].tolist()) == {150_000, 150_001}
    check()
    gpu.set_tunable("cert_margin", 2.0)  # a tunable the graph captured by value
    check()
    gpu.set_tunable("cert_margin", 1.3)
    gpu.set_tunable("host_graph_max_batch", 0)
    check()
    gpu.set_tunable("host_graph_max_batch", 4)
    check()
    with pytest.raises(ValueError):
        gpu.set_tunable("host_graph_max_batch", -1)
