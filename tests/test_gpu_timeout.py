"""GPU: a bounded device wait that runs out ends the search with DeviceTimeoutError, and the index
stays usable.

Every wait of one kernel role on another (a copy landing, a ring slot or an accumulator freed) is
bounded by the tunable "wait_limit_s". The test hook "test_stall_wait" makes the next search's scan
or shortlist kernels first wait on a barrier that nothing completes, so that wait runs out; the
kernel then lets its own copies and MMAs finish, frees its tensor memory and returns, and the host
reads the status word. Nothing faults and nothing is left waiting: the next search, with the
default limit restored, must return the same results as before, bit for bit. The nearest
reference behaviour is its error surface: CUDA failures raise RuntimeError
(src/gpu_brute_force.cu:11-16); DeviceTimeoutError is a RuntimeError.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _same(a, b):
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1].view(np.uint32), b[1].view(np.uint32))


@pytest.mark.parametrize("method", ["skinny", "tc_exact", "bf16"])
def test_wait_runs_out_and_index_recovers(gpu_ready, method):
    vsg = gpu_ready
    from vecsearch_gb300 import datasets as D
    x, _ = D.portable_clustered(40_000, 128, 32, 0.35, seed=300, centroid_seed=301)
    q, _ = D.portable_clustered(64, 128, 32, 0.35, seed=302, centroid_seed=301)
    gpu = vsg.GpuBruteForceIndex(128, "cosine")
    gpu.add(x)
    want = gpu.search(q, 10, method=method)
    assert gpu.get_tunable("wait_limit_s") == pytest.approx(2.0)
    gpu.set_tunable("wait_limit_s", 0.002)
    gpu.set_tunable("test_stall_wait", 1)
    with pytest.raises(vsg.DeviceTimeoutError):
        gpu.search(q, 10, method=method)
    assert issubclass(vsg.DeviceTimeoutError, RuntimeError)
    assert gpu.get_tunable("test_stall_wait") == 0  # the hook covers one search
    gpu.set_tunable("wait_limit_s", 2.0)
    _same(gpu.search(q, 10, method=method), want)
    _same(gpu.search(q[:1], 10, method=method), (want[0][:1], want[1][:1]))


def test_wait_limit_range(gpu_ready):
    vsg = gpu_ready
    gpu = vsg.GpuBruteForceIndex(16)
    for bad in (0.0, -1.0, 61.0):
        with pytest.raises(ValueError):
            gpu.set_tunable("wait_limit_s", bad)
    with pytest.raises(ValueError):
        gpu.set_tunable("test_stall_wait", 2)
