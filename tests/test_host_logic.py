"""CPU: the index's planning logic (vecsearch_gb300/csrc/index_impl.cuh), compiled from the
library's own source into a host-only harness (tests/host_logic_main.cu, no CUDA calls).
- The streaming scan's launch plan: the splits cover every row exactly once with 32-bit sizes up to
  2^32 - 2 rows, and the certified path's fallback scan splits as for at most 128 queries.
- Method auto's routing between the certified path, the tiled and the scan kernel, at the
  boundaries include/vsg.h documents, and under a tuning table.
- The tuning file (vsg_autotune_save / _load through the C ABI): round trip, malformed lines
  skipped, files without the header rejected.
- Tunables' ranges (vsg_set_tunable / _get_tunable), the exact_below switch's branches that
  stay on the host (src/hnsw.cpp:325-328), and add / search argument rules and the empty index."""
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
    exe = str(tmp_path_factory.mktemp("plan") / "host_logic")
    lib_dir = os.path.dirname(so)
    subprocess.run([nvcc, *build.ARCH, "-std=c++17", "-O1", "--expt-relaxed-constexpr",
                    os.path.join(ROOT, "tests", "host_logic_main.cu"), "-o", exe, "-L", lib_dir, "-lvsg_gb300",
                    "-Xlinker", "-rpath=" + lib_dir], check=True, capture_output=True, timeout=600)

    def plan(cases):
        text = "".join(f"plan {n} {dp} {nq} {k} {s} {sms} {m}\n" for n, dp, nq, k, s, sms, m in cases)
        out = subprocess.run([exe], input=text, capture_output=True, text=True, check=True, timeout=120).stdout
        rows = []
        for line in out.splitlines():
            assert not line.startswith("error"), line
            qb, rw, stages, nqb, rps, nsplit = map(int, line.split())
            rows.append(dict(qb=qb, rw=rw, stages=stages, nqb=nqb, rps=rps, nsplit=nsplit))
        assert len(rows) == len(cases)
        return rows

    def route(cases):
        text = "".join("route %d %d %d %d %d %d %d %r\n" % c for c in cases)
        out = subprocess.run([exe], input=text, capture_output=True, text=True, check=True, timeout=120).stdout
        rows = [tuple(map(int, line.split())) for line in out.splitlines()]
        assert len(rows) == len(cases)
        return rows

    def raw(lines):
        out = subprocess.run([exe], input="".join(l + "\n" for l in lines), capture_output=True, text=True,
                             check=True, timeout=120).stdout
        return out.splitlines()

    plan.route = route
    plan.raw = raw
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


AUTO, SKINNY, TILED, BF16, TC_EXACT = 0, 2, 3, 4, 5


def test_auto_routing(harness):
    big, small = 1_000_000, 100_000  # rows at d = 384: above and below 2^27 elements
    edge = 2**27 // 384  # 349,525 rows: 2^27 - 128 elements; one more row reaches 2^27
    # (n, dp, nq, k, method, masked, gather, allowed) -> (certified path, tiled kernel)
    want = {
        (big, 384, 1, 10, AUTO, 0, 0, -1.0): (1, 0),       # a large index: every batch size
        (big, 384, 1, 32, AUTO, 0, 0, -1.0): (1, 0),
        (big, 384, 1, 33, AUTO, 0, 0, -1.0): (1, 0),       # every k <= 128
        (big, 384, 64, 100, AUTO, 0, 0, -1.0): (1, 1),
        (small, 384, 1, 10, AUTO, 0, 0, -1.0): (0, 0),
        (small, 384, 47, 10, AUTO, 0, 0, -1.0): (0, 0),
        (small, 384, 48, 10, AUTO, 0, 0, -1.0): (0, 1),    # tiled_min_batch
        (small, 384, 127, 10, AUTO, 0, 0, -1.0): (0, 1),
        (small, 384, 128, 10, AUTO, 0, 0, -1.0): (1, 1),   # tc_exact_min_batch (checked first)
        (edge, 384, 1, 10, AUTO, 0, 0, -1.0): (0, 0),
        (edge + 1, 384, 1, 10, AUTO, 0, 0, -1.0): (1, 0),  # tc_exact_min_elements
        (small, 384, 1, 120, TC_EXACT, 0, 0, -1.0): (1, 0),
        (small, 384, 1, 128, TC_EXACT, 0, 0, -1.0): (1, 0),  # k' up to 448 covers every k
        (big, 384, 500, 10, SKINNY, 0, 0, -1.0): (0, 0),
        (big, 384, 500, 10, TILED, 0, 0, -1.0): (0, 1),
        (big, 384, 500, 10, BF16, 0, 0, -1.0): (0, 0),
        # host masks, largest allowed fraction known
        (big, 384, 7, 10, AUTO, 1, 0, 0.5): (0, 0),        # fewer than 8 queries
        (big, 384, 8, 10, AUTO, 1, 1, 0.05): (1, 0),       # 8 x 0.05 >= 0.35
        (big, 384, 8, 10, AUTO, 1, 1, 0.04): (0, 0),       # 8 x 0.04 < 0.35, gather scan
        (big, 384, 8, 10, AUTO, 1, 0, 0.04): (1, 0),       # no gather: the masked full scan
        (big, 384, 63, 10, AUTO, 1, 1, 0.001): (0, 0),
        (big, 384, 64, 10, AUTO, 1, 1, 0.001): (1, 0),     # half of tc_exact_min_batch
        (big, 384, 64, 33, AUTO, 1, 0, 0.5): (0, 0),       # k > 32
        # device masks, fraction unknown
        (big, 384, 127, 10, AUTO, 1, 0, -1.0): (0, 0),
        (big, 384, 128, 10, AUTO, 1, 0, -1.0): (1, 0),
        (big, 384, 255, 10, AUTO, 1, 1, -1.0): (0, 0),
        (big, 384, 256, 10, AUTO, 1, 1, -1.0): (1, 0),     # twice the threshold with gather
    }
    got = harness.route(list(want))
    for case, g in zip(want, got):
        assert g == want[case], (case, g)


TUNING = """vsg-tuning 1 dim 384 rows 1000000 metric 1 sms 152
plain 1 2 1.000 120
plain 48 1 2.000 0
plain 128 2 1.000 200
plain 256 3 1.000 0
plain 512 1 0.000 0
plain 1024 0 1.500
bf16 8 16384 2
bf16 64 4096 3
bf16 128 0
bf16 256 2000000 1
junk line
"""
PLAIN_TABLE = [("1", "2", "1.000", "120"), ("48", "1", "2.000", "0"), ("128", "2", "1.000", "0"),
         ("1024", "0", "1.500", "0")]  # kernel 3, split 0 dropped; a first pass above 128 reads as none
# A third bf16 column (CTAs per cluster, version-1 files) is ignored; a sample above 2^20 is dropped.
BF16_TABLE = [("8", "16384", "1.000", "0"), ("64", "4096", "1.000", "0"), ("128", "0", "1.000", "0")]


def _tables(lines):
    out, i = [], 0
    while i < len(lines):
        n = int(lines[i])
        out.append([tuple(l.split()) for l in lines[i + 1:i + 1 + n]])
        i += 1 + n
    return out


def test_tuning_file_round_trip(harness, tmp_path):
    src, dst = tmp_path / "in.txt", tmp_path / "out.txt"
    src.write_text(TUNING)
    out = harness.raw([f"load {src}", "table 0", "table 4", f"save {dst}", "reset", "table 0",
                       f"load {dst}", "table 0", "table 4"])
    assert out[0] == "0"
    t = _tables(out[1:1 + 1 + len(PLAIN_TABLE) + 1 + len(BF16_TABLE)])
    assert t == [PLAIN_TABLE, BF16_TABLE]
    rest = out[1 + 1 + len(PLAIN_TABLE) + 1 + len(BF16_TABLE):]
    assert rest[0] == "0" and rest[1] == "0" and rest[2] == "0"  # saved; a fresh index is untuned; reloaded
    assert _tables(rest[3:]) == [PLAIN_TABLE, BF16_TABLE]
    assert dst.read_text().startswith("vsg-tuning 2 dim 0 rows 0 metric 0 sms 152")


def test_tuning_file_rejects(harness, tmp_path):
    bad = tmp_path / "bad.txt"
    bad.write_text("plain 1 2 1.000 120\n")  # no header
    out = harness.raw([f"load {bad}", f"load {tmp_path / 'missing.txt'}", "table 0"])
    assert out == ["1", "1", "0"]  # VSG_ERR_INVALID twice; the tables stay empty


def test_routing_follows_a_tuning_table(harness, tmp_path):
    src = tmp_path / "in.txt"
    src.write_text(TUNING)
    assert harness.raw([f"load {src}"]) == ["0"]
    small = 100_000  # below 2^27 elements: untuned, batch 1 would take the scan kernel
    cases = [(nq, want) for nq, want in ((1, "1 0"), (47, "1 0"), (48, "0 1"), (127, "0 1"), (128, "1 0"),
                                         (1023, "1 0"), (1024, "0 0"), (5000, "0 0"))]
    out = harness.raw([f"load {src}"] + [f"route {small} 384 {nq} 10 0 0 0 -1.0" for nq, _ in cases] +
                      [f"route {small} 384 200 10 0 1 0 0.5"])  # masks ignore the table
    assert out[0] == "0"
    assert out[1:-1] == [w for _, w in cases]
    assert out[-1] == "1 0"


def test_tunables_through_the_abi(harness):
    out = harness.raw(["get fallback_split_queries", "set fallback_split_queries 512", "get fallback_split_queries",
                       "set fallback_split_queries 0", "get fallback_split_queries",
                       "set fallback_split_queries -1", "set fallback_split_queries 2000000",
                       "get cert_margin", "set cert_margin 0.5", "set cert_margin 2", "get cert_margin",
                       "get tc_exact_min_elements", "set no_such_tunable 1", "get no_such_tunable"])
    assert out[0] == "0 128" and out[1] == "0" and out[2] == "0 512" and out[3] == "0" and out[4] == "0 0"
    assert out[5] == "1" and out[6] == "1"  # VSG_ERR_INVALID: out of range
    assert out[7] == "0 1.3" and out[8] == "1" and out[9] == "0" and out[10] == "0 2"
    assert out[11] == "0 134217728"
    assert out[12] == "1" and out[13].split()[0] == "1"


def test_certified_path_tunables(harness):
    # defaults and ranges of the certified path's tunables (include/vsg.h)
    names = {"finish_cluster": ("8", 16, 17), "finish_cluster_one": ("16", 1, 0),
             "cert_prefetch_max_batch": ("16", 0, -1), "cert_fp8_max_batch": ("16", 0, -1),
             "cert_fp8_sample_rows": ("32768", 65536, -1), "host_graph_max_batch": ("16", 0, 1025),
             "host_graph_direct": ("1", 0, 2)}
    for name, (default, ok, bad) in names.items():
        out = harness.raw([f"get {name}", f"set {name} {ok}", f"get {name}", f"set {name} {bad}", f"get {name}"])
        assert out[0] == f"0 {default}", (name, out)
        assert out[1] == "0" and out[2] == f"0 {ok}", (name, out)
        assert out[3] == "1" and out[4] == f"0 {ok}", (name, out)  # out of range: rejected, value kept


def test_exact_below_host_branches(harness):
    # src/hnsw.cpp:325-328: no allowed row -> empty results; more than exact_below -> the graph.
    out = harness.raw(["below 100 2 5 10 0",     # none allowed: handled, filled with none / +inf
                       "below 100 2 5 10 1",     # 100 allowed > 10: the graph path, nothing written
                       "below 100 2 5 0 3",      # exact_below 0, 34 allowed: the graph path
                       "below 100 2 5 10 -1",    # no mask: the graph path
                       "below 100 2 5 10 -2",    # a mask one row short: ValueError
                       "below 100 2 129 10 0",   # k > 128: ValueError
                       "below 100 0 5 10 0"])    # no queries: handled, nothing to write
    assert out[0] == "0 1 4294967295 inf"
    assert out[1] == "0 0 7 7" and out[2] == "0 0 7 7" and out[3] == "0 0 7 7"
    assert out[4].split()[0] == "1" and out[5].split()[0] == "1"
    assert out[6] == "0 1 7 7"


def test_add_and_search_argument_rules(harness):
    # src/gpu_brute_force.cu:408 (length_error past 2^32 - 2 rows), :294-298 (k > 128), :427-435
    # (empty index: none / +inf), bindings.cpp:165-186 (an unknown method is a ValueError).
    full = 2**32 - 2
    out = harness.raw([f"add {full} 1 0",         # 2^32 - 1 rows: VSG_ERR_LENGTH
                       f"add {full - 1} 2 0",
                       "add 10 0 1",              # m = 0: a no-op, even with NULL rows
                       "add 10 3 1",              # NULL rows: VSG_ERR_INVALID
                       "search 0 2 5 0 0 0",      # empty index: filled with none / +inf
                       "search 0 2 5 9 0 0",      # unknown method
                       "search 0 2 129 0 0 0",    # k > 128
                       "search 50 0 5 0 0 0",     # nq = 0: a no-op
                       "search 50 2 0 0 0 0",     # k = 0: a no-op
                       "search 100 2 5 0 1 3",    # per-query masks closer than ceil(100 / 32) words
                       "search 0 2 5 4 1 1"])     # empty index, any method and mask: filled
    assert out[0] == "2" and out[1] == "2"
    assert out[2] == "0" and out[3] == "1"
    assert out[4] == "0 4294967295 inf"
    assert out[5].split()[0] == "1" and out[6].split()[0] == "1"
    assert out[7] == "0 7 7" and out[8] == "0 7 7"
    assert out[9].split()[0] == "1"
    assert out[10] == "0 4294967295 inf"


def test_choose_splits_fills_whole_waves(harness):
    # The tiled and shortlist kernels' row splits: aligned to whole tiles, covering every row, and
    # never more than four times the wanted count (at least 1024 rows a split).
    cases = [(n, b, align, 1024, f, slots)
             for n in (5_000, 262_144, 1_000_000, 2**32 - 2)
             for b in (1, 3, 16, 32, 151, 400)
             for align in (128, 256)
             for f in (1.0, 2.0)
             for slots in (152, 304)]
    out = harness.raw(["splits %d %d %d %d %r %d" % c for c in cases])
    assert len(out) == len(cases)
    got = {}
    for (n, b, align, min_rows, f, slots), line in zip(cases, out):
        rps, ns = map(int, line.split())
        assert rps % align == 0 and 0 < rps < 2**32 and ns == -(-n // rps), (n, b, rps, ns)
        s0 = max(1, int(max(1, slots // b) * f))
        assert 1 <= ns <= max(1, min(-(-n // min_rows), 4 * s0))
        got[(n, b, align, f, slots)] = ns
    # One query block over 1M rows wants 152 splits; rounded to 256-row tiles they become 151
    # splits of 26 tiles (the ideal share is 25.7 tiles), so one of 152 SMs has no split.
    assert got[(1_000_000, 1, 256, 1.0, 152)] == 151
    assert got[(1_000_000, 16, 256, 1.0, 152)] * 16 % 152 == 0  # 16 blocks x 19 splits: 2 waves
