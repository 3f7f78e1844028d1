"""Regenerates tests/golden/*.npz from the reference's own CPU code.

Inputs come from vecsearch_gb300.datasets' portable generators (bit-identical on
every platform), so each fixture stores only its outputs plus the parameters
needed to regenerate the inputs. Outputs come from oracle/_ref/libvsref.so: the
reference's src/brute_force.cpp and src/hnsw.cpp compiled from its sources by
oracle/build_ref.py (x86, -O3 -march=native as the reference's CMake builds it).

The cases restate the reference's own tests:
  line          tests/cpp/test_brute_force.cpp:9-20   points (i, 0), query (3.2, 0), k = 3
  batch_single  tests/cpp/test_brute_force.cpp:22-43  500 x 37, 13 queries, both metrics
  pad           tests/cpp/test_brute_force.cpp:45-55  5 x 8, k = 7
  clamp         tests/cpp/test_brute_force.cpp:57-65  50 x 16, k = 100
  gpu_cpu_*     tests/python/test_gpu.py:17-33         3000 rows, d 37/128, 300 queries, both metrics
  kbuckets      tests/python/test_gpu.py:36-45         20000 x 64, 40 queries, k = 128 (prefixes: 1..128)
  chunks        tests/python/test_gpu.py:48-57         70000 x 16, 5000 queries, k = 10
  filter_exact  tests/cpp/test_filter.cpp:87-97        5000 x 32, 100 queries, ~1% mask, exact_below 1000
  filter_third  tests/python/test_bindings.py:76-91    3000 x 64, mask[::3], exact_below = n
  c1            config 1: 100k x 384 unit rows, 256-cluster mixture, IP, 1,000 queries, k = 10
  c1_k100       the same base, the first 256 of those queries, k = 100 (config 2's larger k)
  c2_l2_100k    config 2's L2 variant at 100k rows: unnormalised rows of the same mixture, 256
                queries, k = 10
  hnsw_small_l2.vshnsw   HNSWIndex::save (src/hnsw.cpp:375-389) of 150 x 13 rows, L2: the file
                the device index loads its vectors from (HNSW_FILE below regenerates the rows)

Run from the repository root: ``python tests/golden/make_golden.py``.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle.build_ref import build_reference  # noqa: E402
from oracle.oracle import Reference  # noqa: E402
from vecsearch_gb300 import datasets as D  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def inputs(case):
    """Regenerates the inputs of a case: (x, q, k, metric, extra)."""
    name = case["name"]
    if name == "line":
        x = np.array([[i, 0.0] for i in range(10)], np.float32)
        return x, np.array([[3.2, 0.0]], np.float32), 3, "l2", {}
    if name.startswith("batch_single"):
        m = case["metric"]
        return D.portable(500, 37, 3), D.portable(13, 37, 4), 10, m, {}
    if name == "pad":
        x = D.portable(5, 8, 9)
        return x, x[:1].copy(), 7, "l2", {}
    if name == "clamp":
        x = D.portable(50, 16, 7)
        return x, x[:1].copy(), 100, "l2", {}
    if name.startswith("gpu_cpu"):
        d, m = case["d"], case["metric"]
        unit = m == "ip"
        return D.portable(3000, d, 1, unit), D.portable(300, d, 2, unit), 10, m, {}
    if name == "kbuckets":
        return D.portable(20000, 64, 3), D.portable(40, 64, 4), 128, "l2", {}
    if name == "chunks":
        return D.portable(70000, 16, 5), D.portable(5000, 16, 6), 10, "l2", {}
    if name == "filter_exact":
        mask = D.portable_mask(5000, 0.01, 42)
        return D.portable(5000, 32, 30), D.portable(100, 32, 31), 10, "l2", {"mask": mask, "exact_below": 1000}
    if name == "filter_third":
        mask = np.zeros(3000, np.uint8)
        mask[::3] = 1
        return D.portable(3000, 64, 0), D.portable(100, 64, 11), 10, "l2", {"mask": mask, "exact_below": 3000}
    if name in ("c1", "c1_k100"):
        x, _ = D.portable_clustered(100_000, 384, 256, 0.35, seed=0, centroid_seed=2)
        nq = 1000 if name == "c1" else 256
        q, _ = D.portable_clustered(nq, 384, 256, 0.35, seed=1, centroid_seed=2)
        return x, q, 10 if name == "c1" else 100, "ip", {}
    if name == "c2_l2_100k":
        x, _ = D.portable_clustered(100_000, 384, 256, 0.35, seed=0, centroid_seed=2, unit=False)
        q, _ = D.portable_clustered(256, 384, 256, 0.35, seed=1, centroid_seed=2, unit=False)
        return x, q, 10, "l2", {}
    raise KeyError(name)


CASES = [
    {"name": "line"},
    {"name": "batch_single_l2", "metric": "l2"},
    {"name": "batch_single_ip", "metric": "ip"},
    {"name": "pad"},
    {"name": "clamp"},
    {"name": "gpu_cpu_d37_l2", "d": 37, "metric": "l2"},
    {"name": "gpu_cpu_d37_ip", "d": 37, "metric": "ip"},
    {"name": "gpu_cpu_d128_l2", "d": 128, "metric": "l2"},
    {"name": "gpu_cpu_d128_ip", "d": 128, "metric": "ip"},
    {"name": "kbuckets"},
    {"name": "chunks"},
    {"name": "filter_exact"},
    {"name": "filter_third"},
    {"name": "c1"},
    {"name": "c1_k100"},
    {"name": "c2_l2_100k"},
]


def case(name):
    for c in CASES:
        if c["name"] == name:
            return c
    raise KeyError(name)


def path(name):
    return os.path.join(OUT, name + ".npz")


HNSW_FILE = {"name": "hnsw_small_l2.vshnsw", "n": 150, "d": 13, "seed": 31, "metric": "l2"}


def hnsw_file_rows():
    return D.portable(HNSW_FILE["n"], HNSW_FILE["d"], HNSW_FILE["seed"])


def main(names=None):
    """Regenerates every fixture, or only the named cases."""
    if build_reference() is None:
        sys.exit("the reference sources are not present; fixtures can only be made where they are")
    ref = Reference()
    if not names:
        ref.hnsw_save(hnsw_file_rows(), os.path.join(OUT, HNSW_FILE["name"]), HNSW_FILE["metric"])
    for c in CASES:
        if names and c["name"] not in names:
            continue
        x, q, k, metric, extra = inputs(c)
        if "mask" in extra:
            ids, dists = ref.hnsw_exact(x, q, k, extra["mask"], extra["exact_below"], metric, num_threads=4)
        else:
            ids, dists = ref.bf_search(x, q, k, metric, num_threads=3)
        np.savez_compressed(path(c["name"]), ids=ids, dists=dists, metric=metric, k=k)
        print(c["name"], ids.shape)


if __name__ == "__main__":
    main(sys.argv[1:])
