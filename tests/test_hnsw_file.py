"""The saved-HNSW-file reader (VSHNSW01, src/hnsw.cpp:368-420) against a file the reference wrote.

tests/golden/hnsw_small_l2.vshnsw is HNSWIndex::save's output for 150 x 13 portable rows
(tests/golden/make_golden.py). The CPU tests read its header through the C ABI; the GPU tests
load its vectors into a device index and search them.
"""
import numpy as np
import pytest

from tests.conftest import GOLDEN
from tests.golden.make_golden import HNSW_FILE, hnsw_file_rows

PATH = f"{GOLDEN}/{HNSW_FILE['name']}"


def test_fixture_layout():
    # the rows sit right after the 52-byte header, as hnsw.cpp:375-381 writes them
    raw = open(PATH, "rb").read()
    assert raw[:8] == b"VSHNSW01"
    hdr = np.frombuffer(raw[8:24], "<u8")
    assert hdr.tolist() == [13, 150]
    rows = np.frombuffer(raw[52:52 + 150 * 13 * 4], "<f4").reshape(150, 13)
    np.testing.assert_array_equal(rows, hnsw_file_rows())


def test_info():
    import vecsearch_gb300 as vsg
    assert vsg.hnsw_file_info(PATH) == (13, 150, "l2")


def test_info_errors(tmp_path):
    import vecsearch_gb300 as vsg
    with pytest.raises(RuntimeError, match="cannot open"):
        vsg.hnsw_file_info(tmp_path / "missing.bin")
    bad = tmp_path / "bad.bin"
    bad.write_bytes(b"NOTHNSW!" + bytes(44))
    with pytest.raises(RuntimeError, match="not a vecsearch HNSW file"):
        vsg.hnsw_file_info(bad)
    short = tmp_path / "short.bin"
    short.write_bytes(open(PATH, "rb").read()[:30])
    with pytest.raises(RuntimeError, match="truncated"):
        vsg.hnsw_file_info(short)


@pytest.mark.gpu
def test_load_and_search(gpu_ready, tmp_path):
    vsg = gpu_ready
    from vecsearch_gb300 import datasets as D
    x = hnsw_file_rows()
    q = D.portable(9, 13, 32)
    idx = vsg.GpuBruteForceIndex.from_hnsw_file(PATH)
    assert (idx.dim, len(idx), idx.metric) == (13, 150, "l2")
    ref = vsg.GpuBruteForceIndex(13, "l2")
    ref.add(x)
    for method in ("skinny", "tiled"):
        gi, gd = idx.search(q, 10, method=method)
        ri, rd = ref.search(q, 10, method=method)
        np.testing.assert_array_equal(gi, ri)
        np.testing.assert_array_equal(gd.view(np.uint32), rd.view(np.uint32))
    # appending the file again continues the ids
    assert idx.add_hnsw_file(PATH) == 150 and len(idx) == 300
    # a file cut inside its vectors leaves the index as it was
    cut = tmp_path / "cut.bin"
    cut.write_bytes(open(PATH, "rb").read()[:52 + 100 * 13 * 4])
    with pytest.raises(RuntimeError, match="truncated"):
        idx.add_hnsw_file(cut)
    assert len(idx) == 300
    other = vsg.GpuBruteForceIndex(16, "l2")
    with pytest.raises(ValueError):
        other.add_hnsw_file(PATH)
    ip = vsg.GpuBruteForceIndex(13, "ip")
    with pytest.raises(ValueError):
        ip.add_hnsw_file(PATH)
