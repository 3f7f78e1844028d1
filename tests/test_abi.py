"""CPU: the C-ABI library builds, loads, exports every declared symbol, and validates arguments."""
import ctypes
import os
import re

import numpy as np
import pytest

from tests.conftest import ROOT


def declared_symbols():
    names = []
    for f in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if f.endswith(".h"):
            text = open(os.path.join(ROOT, "include", f)).read()
            names += re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(vsg_\w+)\s*\(", text, re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from vecsearch_gb300 import build
    path = build.build()
    return ctypes.CDLL(path)


def test_exports_every_declared_symbol(lib):
    syms = declared_symbols()
    assert "vsg_search" in syms and "vsg_create" in syms and len(syms) >= 14
    for s in syms:
        assert hasattr(lib, s), s


def test_python_signatures_cover_header():
    from vecsearch_gb300 import _native
    assert set(declared_symbols()) <= set(_native.SIGNATURES), set(declared_symbols()) - set(_native.SIGNATURES)


def test_create_validates_before_touching_cuda():
    import vecsearch_gb300 as vsg
    with pytest.raises(ValueError):
        vsg.GpuBruteForceIndex(0)  # dim == 0 -> invalid_argument (gpu_brute_force.cu:387)
    with pytest.raises(ValueError):
        vsg.GpuBruteForceIndex(8, metric="hamming")  # parse_metric (bindings.cpp:38-42)


def test_cuda_available_is_false_without_gpu():
    import vecsearch_gb300 as vsg
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    assert vsg.cuda_available() is False


def test_null_index_is_rejected(lib):
    from vecsearch_gb300 import _native
    l = _native.lib()
    ids = np.zeros(4, np.uint32)
    assert l.vsg_search(None, None, 1, 1, ids.ctypes.data, ids.ctypes.data, 0) == _native.ERR_INVALID
    assert l.vsg_sync(None) == _native.ERR_INVALID
    assert b"NULL" in l.vsg_last_error()


def test_helpers():
    import vecsearch_gb300 as vsg
    x = np.array([[3.0, 4.0], [0.0, 0.0]], np.float32)
    n = vsg.normalize(x)
    assert np.allclose(n[0], [0.6, 0.8]) and np.all(np.isfinite(n))
    assert vsg.recall_at_k(np.array([[1, 2, 3]]), np.array([[3, 2, 9]]), 3) == pytest.approx(2 / 3)


def test_header_is_plain_c_and_links(lib, tmp_path):
    # What an FFI caller does: a C99 program includes the header, links the library and calls it.
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    from vecsearch_gb300 import build
    so = build.build()
    src = tmp_path / "caller.c"
    src.write_text(
        '#include "vsg.h"\n#include <stdio.h>\n'
        "int main(void) {\n"
        "  vsg_index* h = NULL;\n"
        "  int rc = vsg_create(0, VSG_METRIC_IP, 0, &h);  /* dim 0: rejected before any CUDA call */\n"
        '  printf("%d %d %d %s\\n", vsg_cuda_available(), rc == VSG_ERR_INVALID, h == NULL,\n'
        "         vsg_last_error()[0] ? \"msg\" : \"none\");\n"
        "  vsg_destroy(NULL);\n"
        "  return 0;\n}\n")
    exe = tmp_path / "caller"
    subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", os.path.join(ROOT, "include"),
                    str(src), so, "-Wl,-rpath," + os.path.dirname(so), "-o", str(exe)], check=True,
                   capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True, timeout=120).stdout.split()
    assert out[1:] == ["1", "1", "msg"]
    import torch
    if not torch.cuda.is_available():
        assert out[0] == "0"


def test_filter_masks_follow_as_mask():
    # python/bindings.cpp:18,28-36: None, or a 1-D array of len(index) entries cast to uint8
    # (forcecast: 0.5 -> 0, 256 -> 0), nonzero = allowed; here also one mask per query (nq x n).
    import vecsearch_gb300 as vsg

    class Rows:  # _mask_words needs only the index's length
        def __len__(self):
            return 70

    words = lambda f, nq=5: vsg.GpuBruteForceIndex._mask_words(Rows(), f, nq)
    m = np.zeros(70, bool)
    m[[0, 33, 69]] = True
    w, per_query, ld = words(m)
    assert (per_query, ld) == (0, 0) and w.tolist() == [1, 2, 32]
    for same in (m.astype(np.uint8), m.astype(np.int64) * 3, m.astype(np.float32)):
        assert words(same)[0].tolist() == [1, 2, 32]
    cast = m.astype(np.float64) * 0.5  # 0.5 casts to 0: nothing allowed
    cast[1] = 256.0  # wraps to 0 in the cast as well
    cast[2] = 1.5  # 1
    assert words(cast)[0].tolist() == [4, 0, 0]
    w, per_query, ld = words(np.stack([m, ~m, m, m, m]))
    assert (per_query, ld) == (1, 3) and w.shape == (5, 3) and w[1, 0] == (~1) & 0xFFFFFFFF
    for bad in (np.zeros(69, bool), np.zeros((4, 70), bool), np.zeros((5, 71), bool), np.zeros((1, 5, 70), bool)):
        with pytest.raises(ValueError):
            words(bad)


def test_k_converts_like_size_t():
    # bindings.cpp:167 and :79 take k as size_t: integers (and numpy integers) >= 0 only.
    import vecsearch_gb300 as vsg
    assert vsg._as_k(10) == 10 and vsg._as_k(np.int64(5)) == 5 and vsg._as_k(0) == 0
    for bad in (-1, 10.0, "10", None):
        with pytest.raises(TypeError):
            vsg._as_k(bad)


def test_exact_route_leaves_large_k_to_the_graph():
    # The GPU index answers k <= 128 (gpu_brute_force.h:27); HNSWIndex.search has no such limit,
    # so with a filter and k > 128 the route hands the call to the wrapped graph unchanged.
    import vecsearch_gb300 as vsg

    class Gpu:  # never reached for k > 128
        dim = 4
        _h = None

        def __len__(self):
            return 300

    class Graph:
        def search(self, queries, **kw):
            self.kw = kw
            return "graph"

    g = Graph()
    mask = np.ones(300, bool)
    q = np.zeros((2, 4), np.float32)
    assert vsg.HNSWExactRoute(Gpu(), graph=g).search(q, k=200, filter=mask, exact_below=300) == "graph"
    assert g.kw["k"] == 200 and g.kw["exact_below"] == 300 and g.kw["filter"] is mask
    with pytest.raises(ValueError):
        vsg.HNSWExactRoute(Gpu()).search(q, k=200, filter=mask, exact_below=300)


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    # No CPU fallback: without the built library every compute entry point raises.
    import vecsearch_gb300 as vsg
    from vecsearch_gb300 import _native
    monkeypatch.setattr(_native, "_lib", None)
    monkeypatch.setattr(_native, "LIB_PATH", str(tmp_path / "libvsg_gb300.so"))
    with pytest.raises(ImportError):
        _native.lib()
    with pytest.raises(ImportError):
        vsg.GpuBruteForceIndex(8)
    assert vsg.cuda_available() is False  # the probe answers as a build without CUDA does
