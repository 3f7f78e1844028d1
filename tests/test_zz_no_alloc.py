"""GPU: the allocation-free entry point (vsg_search_rows_noalloc) against the regular one.

Some callers cannot allocate device memory while they search: a serving thread that must not
stall on cudaMalloc / cudaFree (both can synchronise the whole device), a host framework that
owns all device memory through its own pool, or a plugin handed only its buffers. For them the
library keeps the search's scratch in one static 4 MiB device array. This test calls that entry
point through the C ABI twice in a row and checks both results against the regular device
search (vsg_search_device) of an index holding the same rows, with the tolerance the other
parity tests use (rtol 1e-5, atol 2e-6; ids exact here since both paths run the same kernels).

The file is named to be collected last, so a run that stops at the first failure has run every
other test first; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL, ATOL = 1e-5, 2e-6


def _noalloc(lib, rows, n, dim, metric, q, nq, k, oi, od):
    return lib.vsg_search_rows_noalloc(ctypes.c_void_p(rows.data_ptr()), n, dim, metric,
                                       ctypes.c_void_p(q.data_ptr()), nq, k, ctypes.c_void_p(oi.data_ptr()),
                                       ctypes.c_void_p(od.data_ptr()), None)


@pytest.mark.parametrize("metric", ["ip", "l2"])
def test_noalloc_matches_regular_entry_point(gpu_ready, metric):
    import torch

    from vecsearch_gb300 import _native
    from vecsearch_gb300 import datasets as D

    vsg = gpu_ready
    lib = _native.lib()
    n, dim, k = 30000, 128, 10
    x = D.portable(n, dim, 21, normalize=metric == "ip")
    q = D.portable(64, dim, 22, normalize=metric == "ip")
    idx = vsg.GpuBruteForceIndex(dim, metric)
    idx.add(x)
    xd = torch.from_numpy(x).cuda()
    qd = torch.from_numpy(q).cuda()
    code = _native.METRIC_L2 if metric == "l2" else _native.METRIC_IP
    for nq in (1, 37):  # two calls in a row share (and reuse) the static scratch
        oi = torch.full((nq, k), 7, dtype=torch.int32, device="cuda")
        od = torch.full((nq, k), -1.0, dtype=torch.float32, device="cuda")
        rc = _noalloc(lib, xd, n, dim, code, qd, nq, k, oi, od)
        assert rc == _native.OK, lib.vsg_last_error()
        ri = torch.empty((nq, k), dtype=torch.int32, device="cuda")
        rd = torch.empty((nq, k), dtype=torch.float32, device="cuda")
        idx.search_device(qd.data_ptr(), dim, nq, k, ri.data_ptr(), rd.data_ptr(),
                          stream=torch.cuda.current_stream().cuda_stream)
        idx.sync()
        torch.cuda.synchronize()
        np.testing.assert_array_equal(oi.cpu().numpy(), ri.cpu().numpy())
        np.testing.assert_allclose(od.cpu().numpy(), rd.cpu().numpy(), rtol=RTOL, atol=ATOL)


@pytest.mark.parametrize("n,dim,k,metric", [(30000, 36, 10, "l2"),   # dim % 8 == 4: no padding here
                                             (20000, 132, 17, "ip"),
                                             (50, 64, 100, "l2")])    # k > n: padded with -1 / +inf
def test_noalloc_matches_oracle(gpu_ready, n, dim, k, metric):
    # The same entry point against the oracle (the reference's CPU search restated) with the
    # parity rule of the other tests: distances within rtol 1e-5 + atol 2e-6, ids equal except
    # at near-ties. Two calls in a row with different shapes reuse the static scratch.
    import torch

    from oracle import oracle as O
    from vecsearch_gb300 import _native
    from vecsearch_gb300 import datasets as D

    lib = _native.lib()
    x = D.portable(n, dim, 23, normalize=metric == "ip")
    q = D.portable(40, dim, 24, normalize=metric == "ip")
    xd = torch.from_numpy(x).cuda()
    qd = torch.from_numpy(q).cuda()
    code = _native.METRIC_L2 if metric == "l2" else _native.METRIC_IP
    for nq in (40, 3):
        oi = torch.full((nq, k), 7, dtype=torch.int32, device="cuda")
        od = torch.full((nq, k), -1.0, dtype=torch.float32, device="cuda")
        assert _noalloc(lib, xd, n, dim, code, qd, nq, k, oi, od) == _native.OK, lib.vsg_last_error()
        torch.cuda.synchronize()
        wi, wd = O.search(x, q[:nq], k, metric, num_threads=4)
        ids = oi.cpu().numpy().astype(np.int64)
        dists = od.cpu().numpy()
        np.testing.assert_allclose(dists, wd, rtol=RTOL, atol=ATOL)
        O.check_ids(ids, O.ids_to_int64(wi), x, q[:nq], metric)
        assert ((ids >= 0) == np.isfinite(dists)).all()


def test_noalloc_empty_rows_fill_missing(gpu_ready):
    # No rows: every result is -1 / +inf, as the regular search fills an empty index.
    import torch

    from vecsearch_gb300 import _native

    lib = _native.lib()
    q = torch.zeros((4, 16), device="cuda")
    oi = torch.zeros((4, 5), dtype=torch.int32, device="cuda")
    od = torch.zeros((4, 5), dtype=torch.float32, device="cuda")
    x = torch.zeros((1, 16), device="cuda")
    assert _noalloc(lib, x, 0, 16, _native.METRIC_L2, q, 4, 5, oi, od) == _native.OK, lib.vsg_last_error()
    torch.cuda.synchronize()
    assert (oi.cpu().numpy() == -1).all() and np.isinf(od.cpu().numpy()).all()


def test_noalloc_rejects_oversize_and_bad_shapes(gpu_ready):
    import torch

    from vecsearch_gb300 import _native

    lib = _native.lib()
    x = torch.zeros((1000, 64), device="cuda")
    q = torch.zeros((20000, 64), device="cuda")
    oi = torch.empty((20000, 128), dtype=torch.int32, device="cuda")
    od = torch.empty((20000, 128), dtype=torch.float32, device="cuda")
    # 20000 queries x 128 results exceed the 4 MiB scratch: a clear error, nothing launched
    assert _noalloc(lib, x, 1000, 64, 0, q, 20000, 128, oi, od) == _native.ERR_INVALID
    assert b"scratch" in lib.vsg_last_error()
    assert _noalloc(lib, x, 1000, 64, 0, q, 1, 129, oi, od) == _native.ERR_INVALID  # k > 128
    assert lib.vsg_search_rows_noalloc(ctypes.c_void_p(x.data_ptr()), 1000, 62, 0,
                                       ctypes.c_void_p(q.data_ptr()), 1, 10, ctypes.c_void_p(oi.data_ptr()),
                                       ctypes.c_void_p(od.data_ptr()), None) == _native.ERR_INVALID  # dim % 4
