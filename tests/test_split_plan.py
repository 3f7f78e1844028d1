"""CPU: the streaming scan's launch plan (vsg_index::plan in vecsearch_gb300/csrc/index_impl.cuh),
compiled from the library's own source into a host-only harness (tests/split_plan_main.cu, no
CUDA calls). The splits cover every row exactly once with 32-bit sizes up to 2^32 - 2 rows, and
the certified path's fallback scan splits as for at most 128 queries."""
import os
import subprocess

import pytest

from tests.conftest import ROOT

SMS = 152  # GB300


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    from vecsearch_gb300 import build
    nvcc = build.nvcc_path()
    if not os.path.exists(nvcc):
        pytest.skip("no nvcc")
    so = build.build()
    exe = str(tmp_path_factory.mktemp("plan") / "split_plan")
    lib_dir = os.path.dirname(so)
    subprocess.run([nvcc, *build.ARCH, "-std=c++17", "-O1", "--expt-relaxed-constexpr",
                    os.path.join(ROOT, "tests", "split_plan_main.cu"), "-o", exe, "-L", lib_dir, "-lvsg_gb300",
                    "-Xlinker", "-rpath=" + lib_dir], check=True, capture_output=True, timeout=600)

    def plan(cases):
        text = "".join(f"{n} {dp} {nq} {k} {s} {sms} {m}\n" for n, dp, nq, k, s, sms, m in cases)
        out = subprocess.run([exe], input=text, capture_output=True, text=True, check=True, timeout=120).stdout
        rows = []
        for line in out.splitlines():
            assert not line.startswith("error"), line
            qb, rw, stages, nqb, rps, nsplit = map(int, line.split())
            rows.append(dict(qb=qb, rw=rw, stages=stages, nqb=nqb, rps=rps, nsplit=nsplit))
        assert len(rows) == len(cases)
        return rows

    return plan


def test_splits_cover_every_row_once(harness):
    cases = [(n, dp, nq, 10, s, SMS, 1)
             for n in (1, 31, 32, 33, 1000, 20_000, 1_000_000, 2**31 + 5, 2**32 - 2)
             for dp in (8, 384)
             for nq in (1, 5, 8, 100, 128, 129, 300, 4096)
             for s in (0, 128)]
    for (n, dp, nq, _, _, _, _), p in zip(cases, harness(cases)):
        assert p["qb"] == min(8, 1 << (nq - 1).bit_length())
        assert p["nqb"] == -(-nq // p["qb"])
        rps, ns = p["rps"], p["nsplit"]
        assert rps % 32 == 0 and 0 < rps < 2**32
        assert ns == -(-n // rps) and (ns - 1) * rps < n <= ns * rps  # the last split holds rows
        assert p["stages"] >= 2


def test_fallback_splits_as_for_128_queries(harness):
    n = 1_000_000
    ref = harness([(n, 384, 128, 10, 0, SMS, 1)])[0]
    assert ref["nsplit"] == 9  # 152 SMs over 16 query blocks of 8
    for nq, whole_splits in ((129, 8), (512, 2), (4096, 1)):
        whole, capped = harness([(n, 384, nq, 10, 0, SMS, 1), (n, 384, nq, 10, 128, SMS, 1)])
        assert whole["nsplit"] == whole_splits  # at 4096: one split, one CTA over every row
        assert capped["nsplit"] == ref["nsplit"] and capped["rps"] == ref["rps"]
        assert capped["nqb"] == whole["nqb"] == -(-nq // 8)
    at, plain = harness([(n, 384, 100, 10, 128, SMS, 1), (n, 384, 100, 10, 0, SMS, 1)])
    assert at == plain  # batches of up to 128 queries keep their plan


def test_near_2_to_32_rows(harness):
    n = 2**32 - 2
    p = harness([(n, 8, 4096, 10, 0, SMS, 0)])[0]  # one split wanted: capped below 2^32
    assert p["rps"] == 2**32 - 32 and p["nsplit"] == 2
