#!/usr/bin/env python
"""Exact top-k QPS on one GB300: 1M x 384 unit rows (cosine), k = 10, by batch size.

Workload (the full-shape plain FP32 configuration): N = 1,000,000 base rows x d = 384
from a 1,024-cluster Gaussian mixture (centroids ~ N(0, 1), sigma = 0.35), each row
L2-normalised; 10,000 queries from the same mixture; inner product (cosine distance
1 - q.x); k = 10. Synthetic data stands in for the reference's tweet embeddings
(same 1M x 384 cosine shape).

A step is one exact search of one batch (default batch 1: the HBM-bound case). Method auto
runs it on the certified path on an index this large: a bf16 tensor-core pass over a bf16 copy
of the rows (half the FP32 bytes) keeps each query's candidates, an FP32 rerank computes their
exact distances with the scan kernel's arithmetic and proves that no other row can enter the
top k; unproven queries run in the FP32 scan kernel. Results equal the FP32 scan's bit for bit.
  value      queries/s with queries and results resident in HBM (device API), timed
             with CUDA events on the launching stream over exactly --steps steps.
  e2e        the same through the public host API (pinned host queries in, host
             results out, both copies inside the timed region).
  roofline   the dominant kernel of the timed steps (the bf16 shortlist pass, or the FP32 scan
             kernel): algorithmic bytes (the rows once, in the type it reads, plus queries) per
             launch / its CUDA-event time, against the measured HBM copy bandwidth.
  gpu_launches  this index's kernel launches in the timed steps (counted by the library).
  cpu_baseline  the reference's CPU algorithm (oracle port of brute_force.cpp
             search_batch) on this host's cores, on a bounded sample.
  autotune   the schedule tables vsg_autotune picked for the sweep's batch sizes (taken after
             the headline line; method auto in the sweep follows them).
  sweep      QPS for the batch sweep 1 .. 4096 (fewer steps each): method auto (tuned), the two
             FP32 kernels, the precision form (bf16) and the certified exact path (tc_exact, with
             the fraction of queries it left to the scan kernel).
The base (1.536 GB) is larger than L2 (129 MB), so no L2 flush is needed between steps.

--impl reference times the reference's CPU path (oracle port, all host threads) on the
same workload and prints the same JSON line with "impl": "reference".
--mode precision / serve / filtered run configs 4 / 5 / 3 on their own; --mode worker times the
GPU shard worker (one-query Search calls from concurrent clients).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# DRAM bytes per launch of the dominant kernel, measured by ncu (dram__bytes_read.sum +
# dram__bytes_write.sum) at batch 1, k = 10, cosine, 384 dims, on a case of the same kernel:
#   scan: the FP32 scan kernel, 262,144 rows: 402.69 MB read + 3.31 MB written
#   tc:   the certified path's bf16 shortlist main pass, 262,144 rows: 201.40 MB read + 3.15 MB
#         written
#   tc8:  the certified path's e4m3 shortlist main pass, 393,216 rows (the smallest base the
#         certified path takes at batch 1): 152.65 MB read + 0.10 MB written (mean of 4 launches)
# The rows dominate (reads equal the algorithmic bytes there), so a launch's traffic is taken as
# the measured bytes per row times the rows scanned, plus the configuration's own query, norm
# and list bytes: queries (dim x 4, bf16 copy dim x 2, e4m3 copy dim x 1) and, for L2, the rows'
# norms (4 a row).
MEASURED_TRAFFIC = {("scan", 384): (262_144, 406_000_000), ("tc", 384): (262_144, 204_550_000),
                    ("tc8", 384): (393_216, 152_748_800)}


def uses_e4m3(idx, batch, k, dim):
    """Whether a certified search of this shape reads the e4m3 copy (the library's rule)."""
    return batch <= idx.get_tunable("cert_fp8_max_batch") and k <= 16 and (dim + 15) // 16 * 16 <= 1024


def measured_traffic(kernel, n, dim, batch, k, metric):
    """(bytes per launch for n rows at this batch, k and metric, source) or (None, reason)."""
    m = MEASURED_TRAFFIC.get((kernel, dim))
    if m is None:
        return None, "no ncu capture of this kernel at this dim"
    rows, t = m
    qb = {"scan": 4, "tc": 2, "tc8": 1}[kernel]  # query bytes per dimension
    per_row = (t - dim * qb) / rows  # less the one query of the capture
    extra = batch * dim * qb + batch * k * 8 + (n * 4 if metric == "l2" and kernel != "scan" else 0)
    exact = batch == 1 and k == 10 and metric == "ip"
    src = (f"ncu capture at {rows:,} rows, scaled by rows" if exact else
           f"ncu capture at {rows:,} rows (batch 1, k 10, cosine): bytes per row scaled by rows, plus "
           "this configuration's query, list and norm bytes")
    return int(round(per_row * n + extra)), src


def parse():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--batch", type=int, default=1)
    ap.add_argument("--n", type=int, default=1_000_000)
    ap.add_argument("--dim", type=int, default=384)
    ap.add_argument("--k", type=int, default=10)
    ap.add_argument("--metric", default="ip", choices=["ip", "l2"])
    ap.add_argument("--clusters", type=int, default=1024)
    ap.add_argument("--queries", type=int, default=10_000)
    ap.add_argument("--sweep", default="1,8,16,32,48,64,96,128,256,512,1024,4096", help="comma list; empty to skip")
    ap.add_argument("--cpu-seconds", type=float, default=8.0, help="CPU-baseline sample budget")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-recall", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="sweep with the built-in schedule rules")
    ap.add_argument("--no-filtered", action="store_true", help="skip the filtered (config 3) sweep")
    ap.add_argument("--no-parity", action="store_true", help="skip the full-size parity checks")
    ap.add_argument("--no-serve", action="store_true", help="skip the short serving-latency check")
    ap.add_argument("--parity-queries", type=int, default=512, help="queries checked per cosine k=10 batch")
    ap.add_argument("--method", default="auto", choices=["auto", "skinny", "tiled", "bf16", "tc_exact"],
                    help="path of the main timed line (auto: the certified path on a large index, "
                         "else the FP32 kernels by batch size)")
    ap.add_argument("--rates", default="1000,5000,10000,20000,50000", help="serve mode: offered queries/s")
    ap.add_argument("--duration", type=float, default=2.0, help="serve mode: seconds of arrivals per rate")
    ap.add_argument("--plain-max-rate", type=int, default=10000, help="serve mode: highest rate for the plain path")
    ap.add_argument("--filter-targets", default="100,1000,10000,50000,100000,200000",
                    help="filtered mode: allowed-row counts to sweep")
    ap.add_argument("--filter-batch", type=int, default=16, help="filtered mode: queries per search")
    ap.add_argument("--mode", default="plain", choices=["plain", "precision", "serve", "filtered", "worker"],
                    help="precision: config 4 (BF16 shortlist + rerank) sweep instead of the default line")
    ap.add_argument("--big", action="store_true", help="precision mode: add the 4M x 384 base")
    return ap.parse_args()


def make_data(a):
    from vecsearch_gb300 import datasets as D
    unit = a.metric == "ip"
    x, _ = D.clustered(a.n, a.dim, a.clusters, 0.35, seed=0, centroid_seed=2, unit=unit)
    q, _ = D.clustered(a.queries, a.dim, a.clusters, 0.35, seed=1, centroid_seed=2, unit=unit)
    return x, q


def workload(a):
    return {
        "workload": f"exact top-{a.k} {'cosine' if a.metric == 'ip' else 'L2'}, {a.n:,} x {a.dim} fp32 rows "
                    f"({a.clusters}-cluster mixture, sigma 0.35{', unit rows' if a.metric == 'ip' else ''}), "
                    f"batch {a.batch}",
        "n": a.n, "dim": a.dim, "k": a.k, "batch": a.batch, "metric": a.metric, "global_batch": a.batch,
        "l2_flush": "none needed: base rows (%.3f GB) exceed the 129 MB L2" % (a.n * a.dim * 4 / 1e9),
    }


def peaks_bf16(key="bf16_tflops"):
    """Measured dense bf16 TFLOP/s from MEASURED_PEAKS.json (burst, or `key`), else the fallback
    (1,900 burst, 1,700 sustained)."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)[key])
    except (OSError, KeyError, ValueError):
        return 1700.0 if "sustained" in key else 1900.0


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)["hbm_gbs"], "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons while running."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.proc = None
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(gpu_index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.splitlines():
            f = [s.strip() for s in line.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for nm, v in zip(names, f[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(x, q, a, threads):
    """The reference's CPU search (oracle port) on a bounded sample: batches of a.batch queries."""
    from oracle import oracle as O
    O.search(x, q[:1], a.k, a.metric, num_threads=threads)  # warm-up
    t0 = time.perf_counter()
    calls = 0
    while True:
        s = (calls * a.batch) % (len(q) - a.batch + 1)
        O.search(x, q[s:s + a.batch], a.k, a.metric, num_threads=threads)
        calls += 1
        el = time.perf_counter() - t0
        if el >= a.cpu_seconds or calls >= 1000:
            break
    return {"value": round(calls * a.batch / el, 2), "unit": "queries/s", "cores": threads, "kind": "port",
            "sample": f"{calls} searches of batch {a.batch} over the full {a.n}x{a.dim} base, {el:.1f} s, "
                      f"{threads} threads (oracle/bf_oracle.c: brute_force.cpp search_batch restated)"}


def run_reference(a):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    x, q = make_data(a)
    from oracle import oracle as O
    O.search(x, q[:a.batch], a.k, a.metric, num_threads=threads)  # warm-up
    for _ in range(max(0, min(a.warmup, 2) - 1)):
        O.search(x, q[:a.batch], a.k, a.metric, num_threads=threads)
    t0 = time.perf_counter()
    steps = 0
    while steps < a.steps:
        s = (steps * a.batch) % (len(q) - a.batch + 1)
        O.search(x, q[s:s + a.batch], a.k, a.metric, num_threads=threads)
        steps += 1
        if time.perf_counter() - t0 > 120:  # bound the arm's run time
            break
    el = time.perf_counter() - t0
    v = steps * a.batch / el
    line = {
        "impl": "reference", "metric": f"exact top-{a.k} QPS at {a.n // 1000}Kx{a.dim}", "value": round(v, 2),
        "unit": "queries/s", "n_gpus": a.gpus, "steps": steps, "warmup": a.warmup,
        "ms_per_step": round(el * 1e3 / steps, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": dict(workload(a), parallelism=f"replicas{a.gpus}"),
        "cpu_baseline": {"value": round(v, 2), "unit": "queries/s", "cores": threads, "kind": "port",
                         "sample": f"{steps} searches of batch {a.batch} over the full base ({el:.1f} s)"},
        "e2e": {"value": round(v, 2), "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def time_device(idx, torch, qd, a, batch, steps, warmup, stream, dist=None, method="auto", out=None,
                profile_steps=None):
    """Device-resident search: (ms total over `steps`, scan ms total, merge ms total, searches
    profiled). The timed steps run without the library's kernel events (their launches chain as
    dependents); profile_steps more steps (default: as many) then record CUDA events around the
    dominant kernel and the one after it, each launched on its own. With `out` (a dict):
    out["kernels"] = this index's kernel launches in the timed steps, out["tc_exact"] = whether
    they ran the certified path."""
    k = a.k
    out_i = torch.empty((batch, k), dtype=torch.int32, device=qd.device)
    out_d = torch.empty((batch, k), dtype=torch.float32, device=qd.device)
    nq = qd.shape[0]
    sp = stream.cuda_stream

    def step(i):
        s = (i * batch) % (nq - batch + 1)
        idx.search_device(qd[s].data_ptr(), a.dim, batch, k, out_i.data_ptr(), out_d.data_ptr(), stream=sp,
                          method=method)

    for i in range(warmup):
        step(i)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    if out is not None:
        tq0 = idx.tc_exact_stats()[0]
        k0 = idx.kernel_launches()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for i in range(steps):
        step(warmup + i)
    e1.record(stream)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    ms = e0.elapsed_time(e1)
    if out is not None:
        out["kernels"] = idx.kernel_launches() - k0
        out["tc_exact"] = idx.tc_exact_stats()[0] > tq0
    idx.profile(True)
    for i in range(steps if profile_steps is None else profile_steps):
        step(warmup + steps + i)
    torch.cuda.synchronize()
    scan_ms, merge_ms, launches = idx.profile_read()
    idx.profile(False)
    idx.sync()
    return ms, scan_ms, merge_ms, launches


def filtered_sweep(idx, torch, x, q, a, stream, batch=16, targets=(100, 1000, 10000, 50000, 100000, 200000)):
    """Config 3: Zipf(1.1) group labels over 2,000 groups; each query filters to one group (per-query
    1M-bit masks on the device). For groups near each allowed count, device QPS of the gather scan
    (reads only allowed rows), the masked full scan (reads every tile holding an allowed row) and
    the certified tensor-core path with the masks (results equal the scans' bit for bit)."""
    from vecsearch_gb300 import datasets as D
    groups = D.zipf_groups(a.n, 2000, 1.1, seed=3)
    sizes = np.bincount(groups, minlength=2000)
    qd = torch.from_numpy(q[:batch]).to(x.device if hasattr(x, "device") else "cuda")
    out_i = torch.empty((batch, a.k), dtype=torch.int32, device=qd.device)
    out_d = torch.empty((batch, a.k), dtype=torch.float32, device=qd.device)
    res = []
    for t in targets:
        g = int(np.argmin(np.abs(sizes - t)))
        words = D.group_masks(groups, [g] * batch)
        wd = torch.from_numpy(words.view(np.int32)).to(qd.device)
        row = {"target": t, "allowed": int(sizes[g]), "batch": batch}
        for mode, frac, method in (("gather", 1.0, "skinny"), ("masked_full_scan", 0.0, "skinny"),
                                   ("tc_exact", 0.0, "tc_exact")):
            idx.set_tunable("gather_max_fraction", frac)
            steps = 20 if batch <= 64 else 5
            for i in range(steps + 3):
                if i == 3:
                    torch.cuda.synchronize()
                    e0 = torch.cuda.Event(enable_timing=True)
                    e1 = torch.cuda.Event(enable_timing=True)
                    e0.record(stream)
                idx.search_device(qd.data_ptr(), a.dim, batch, a.k, out_i.data_ptr(), out_d.data_ptr(),
                                  stream=stream.cuda_stream, mask_ptr=wd.data_ptr(), per_query=True,
                                  mask_ld=words.shape[1], method=method)
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / steps
            row[mode + "_qps"] = round(batch / (ms / 1e3), 1)
            row[mode + "_ms"] = round(ms, 4)
        res.append(row)
    idx.set_tunable("gather_max_fraction", 0.10)
    idx.sync()
    return res


def hbm_roofline(alg_bytes, kernel_ms, peak, peak_kind, traffic, traffic_source, kernel):
    achieved = alg_bytes / (kernel_ms / 1e3) / 1e9
    return {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "peak_source": peak_kind, "traffic": traffic,
            "traffic_source": traffic_source, "algorithmic_bytes_per_launch": alg_bytes, "kernel": kernel,
            "kernel_ms_avg": round(kernel_ms, 5)}


PARITY_RULE = ("distances within rtol 1e-5 + atol 2e-6 of the oracle port's; ids equal the oracle port's and the "
               "FP64 oracle's except at near-ties (a different row only at the k-th place within 1e-6 relative, "
               "rows of one list in another order within 1e-5 relative)")


def _parity_case(O, x, q, ids, dists, k, metric, cores, truth_i):
    """The parity rule for one set of results: against the oracle port (the reference's CPU
    algorithm restated, all host threads) and the FP64 oracle's ids."""
    wi, wd = O.search(x, q, k, metric, num_threads=cores)
    row = {"queries": int(len(q)), "vs_oracle": True, "vs_fp64": True, "near_ties_tolerated": 0}
    try:
        np.testing.assert_allclose(dists, wd, rtol=1e-5, atol=2e-6)
        row["near_ties_tolerated"] += O.check_ids(ids, O.ids_to_int64(wi), x, q, metric)
    except AssertionError as e:
        row["vs_oracle"] = False
        row["error"] = str(e)[:200]
    try:
        row["near_ties_tolerated"] += O.check_ids(ids, truth_i, x, q, metric)
    except AssertionError as e:
        row["vs_fp64"] = False
        row["error_fp64"] = str(e)[:200]
    return row


def parity_checks(vsg, idx, x, q, a):
    """Full-size parity of method auto (the drop-in's default) at 1M x 384: cosine k = 10 at
    batches 1, 128 and 4096 (the first --parity-queries queries of each), cosine k = 100 at batch
    128, and L2 k = 10 on unnormalised rows of the same mixture at batches 1 and 128. Each result
    set is checked against the oracle port of the reference's search_batch and the FP64 oracle.
    Returns (report, FP64 top-10 of the cosine queries, for reuse)."""
    from oracle import oracle as O
    from vecsearch_gb300 import datasets as D
    t0 = time.perf_counter()
    cores = os.cpu_count() or 1
    nchk = min(a.parity_queries, len(q))
    cases = []

    def run_case(index, xx, qq, k, metric, batch, truth_i):
        # every query of qq is searched in batches of `batch`; the first len(truth_i) are checked
        s0 = index.tc_exact_stats()
        parts = [index.search(qq[i:i + batch], k) for i in range(0, len(qq), batch)]
        ids = np.concatenate([p[0] for p in parts])[:len(truth_i)]
        dists = np.concatenate([p[1] for p in parts])[:len(truth_i)]
        s1 = index.tc_exact_stats()
        copy = "e4m3" if uses_e4m3(index, batch, k, xx.shape[1]) else "bf16"
        row = {"metric": metric, "k": k, "batch": batch, "method": "auto",
               "path": f"tc_exact ({copy} copy)" if s1[0] > s0[0] else "fp32 kernels",
               "uncertified_to_scan": int(s1[1] - s0[1])}
        row.update(_parity_case(O, xx, qq[:len(truth_i)], ids, dists, k, metric, cores, truth_i))
        cases.append(row)

    truth10 = O.fp64_topk(x, q[:nchk], 10, "ip")
    run_case(idx, x, q[:nchk], 10, "ip", 1, truth10[0])
    run_case(idx, x, q[:nchk], 10, "ip", 128, truth10[0])
    if len(q) >= 4096:
        run_case(idx, x, q[:4096], 10, "ip", 4096, truth10[0])
    n100 = min(128, len(q))
    run_case(idx, x, q[:n100], 100, "ip", 128, O.fp64_topk(x, q[:n100], 100, "ip")[0])
    # L2 on unnormalised rows of the same mixture (config 2's L2 variant)
    xl, _ = D.clustered(a.n, a.dim, a.clusters, 0.35, seed=0, centroid_seed=2, unit=False)
    ql, _ = D.clustered(128, a.dim, a.clusters, 0.35, seed=1, centroid_seed=2, unit=False)
    il = vsg.GpuBruteForceIndex(a.dim, "l2")
    il.add(xl)
    tl = O.fp64_topk(xl, ql, 10, "l2")[0]
    run_case(il, xl, ql[:32], 10, "l2", 1, tl[:32])
    run_case(il, xl, ql, 10, "l2", 128, tl)
    del il, xl
    return ({"rule": PARITY_RULE, "all_pass": all(c["vs_oracle"] and c["vs_fp64"] for c in cases), "cases": cases,
             "seconds": round(time.perf_counter() - t0, 1)}, truth10)


def precision_checks(vsg, idx, torch, qd, x, q, a, stream, truth):
    """Config 4 at batch 128 on the bench's base: the approximate precision forms (bf16 copy with
    k' = 40, e4m3 copy with k' = 80; exact FP32 rerank of the shortlist) - recall@10 and max
    |distance error| against the FP64 oracle on 128 queries, and device QPS."""
    from oracle import oracle as O
    nq = min(128, len(q))
    gi = truth[0][:nq] if truth is not None else O.fp64_topk(x, q[:nq], 10, "ip")[0]
    a2 = argparse.Namespace(**vars(a))
    a2.k = 10
    out = []
    for method, over in (("bf16", 4), ("fp8", 8)):
        idx.set_tunable("shortlist_oversample", over)
        ids, dists = idx.search(q[:nq], 10, method=method)
        err = 0.0
        for i in range(nq):
            ok = ids[i] >= 0
            d64 = O.fp64_distances(x, q[i:i + 1], "ip", ids[i][ok])[0]
            err = max(err, float(np.max(np.abs(dists[i][ok].astype(np.float64) - d64))))
        ms, _, _, _ = time_device(idx, torch, qd, a2, 128, 20, 3, stream, method=method, profile_steps=0)
        out.append({"copy": method, "k": 10, "k_prime": 10 * over, "batch": 128, "queries_checked": nq,
                    "recall_at_10_vs_fp64": vsg.recall_at_k(ids, gi, 10), "max_abs_dist_err_vs_fp64": err,
                    "qps": round(128 * 20 / (ms / 1e3), 1)})
    idx.set_tunable("shortlist_oversample", 4)
    return out


def serve_setup(a, idx, vsg):
    from vecsearch_gb300 import datasets as D
    groups = D.zipf_groups(a.n, 2000, 1.1, seed=3)
    sizes = np.bincount(groups, minlength=2000)
    cand = [g for g in range(2000) if sizes[g] >= 100][:64]
    words_by_group = {g: D.pack_bits(groups == g) for g in cand}
    return groups, words_by_group


def serve_check(vsg, idx, q, a, rates=(5000, 20000), duration=1.0):
    """Config 5's request mix through the continuous-batching server at two offered loads, one
    second each: achieved QPS and p50 / p99 latency (submit to completion)."""
    groups, words = serve_setup(a, idx, vsg)
    srv = vsg.Server(idx, max_batch=1024, max_k=100, slots=2)
    try:
        serve_load(idx, srv, None, q, groups, words, 2000, 0.3, 1)  # warm-up
        rows = [serve_load(idx, srv, None, q, groups, words, r, duration, 10 + i) for i, r in enumerate(rates)]
        st = srv.stats()
    finally:
        srv.close()
    return {"workload": "open-loop Poisson arrivals; requests of 1-64 queries (log-uniform), k 10 or 100, 30% "
                        "filtered to one Zipf(1.1) group of 2,000", "server": "2 slots x 1024 queries",
            "duration_s": duration, "loads": rows, "server_stats": st}


def run_ours(a):
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    import vecsearch_gb300 as vsg
    from vecsearch_gb300 import build as B
    B.build()

    x, q = make_data(a)
    idx = vsg.GpuBruteForceIndex(a.dim, "cosine" if a.metric == "ip" else "l2", device=local)
    idx.add(x)
    qd = torch.from_numpy(q).to(f"cuda:{local}")
    stream = torch.cuda.current_stream()

    sampler = ClockSampler(local)
    info = {}
    ms, scan_ms, merge_ms, launches = time_device(idx, torch, qd, a, a.batch, a.steps, a.warmup, stream, dist,
                                                  method=a.method, out=info, profile_steps=min(a.steps, 200))
    clocks = sampler.stop()
    if dist is not None:
        t = torch.tensor([ms], device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    qps = world * a.batch * a.steps / (ms / 1e3)

    # e2e: public host API with pinned buffers; copies inside the timed region.
    qh = torch.from_numpy(q).pin_memory()
    oi = torch.empty((a.batch, a.k), dtype=torch.int32).pin_memory()
    od = torch.empty((a.batch, a.k), dtype=torch.float32).pin_memory()
    nq = q.shape[0]
    e2e_steps = min(a.steps, max(20, int(2000 / a.batch)))
    for i in range(min(a.warmup, 5)):
        idx.search_host_ptr(qh[(i * a.batch) % (nq - a.batch + 1)].data_ptr(), a.batch, a.k, oi.data_ptr(),
                            od.data_ptr())
    if dist is not None:
        dist.barrier()
    t0 = time.perf_counter()
    for i in range(e2e_steps):
        s = (i * a.batch) % (nq - a.batch + 1)
        idx.search_host_ptr(qh[s].data_ptr(), a.batch, a.k, oi.data_ptr(), od.data_ptr())
    e2e_s = time.perf_counter() - t0
    if dist is not None:
        t = torch.tensor([e2e_s], device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_qps = world * a.batch * e2e_steps / e2e_s

    # roofline of the dominant kernel of the timed steps: the certified path's bf16 shortlist pass
    # (method auto on a large index), else the FP32 scan kernel
    scan_avg_ms = scan_ms / max(launches, 1)
    peak, peak_kind = peaks()
    if info.get("tc_exact") and uses_e4m3(idx, a.batch, a.k, a.dim):
        # the e4m3 rows once with their FP32 scales, the e4m3 queries (and, for L2, the row norms)
        d8 = (a.dim + 15) // 16 * 16
        alg_bytes = a.n * (d8 + 4) + a.batch * d8 + (a.n * 4 if a.metric == "l2" else 0)
        traffic, tsrc = measured_traffic("tc8", a.n, a.dim, a.batch, a.k, a.metric)
        kernel = "tc_shortlist_kernel (e4m3 tcgen05 pass over the rows; certified exact path)"
        dtype = "e4m3 products (FP32 scale per row and query), f32 accumulation and results"
    elif info.get("tc_exact"):
        alg_bytes = a.n * a.dim * 2 + a.batch * a.dim * 2  # the bf16 rows once, the bf16 queries
        traffic, tsrc = measured_traffic("tc", a.n, a.dim, a.batch, a.k, a.metric)
        kernel = "tc_shortlist_kernel (bf16 tcgen05 pass over the rows; certified exact path)"
        dtype = "bf16 products, f32 accumulation and results"
    else:
        alg_bytes = a.n * a.dim * 4 + a.batch * a.dim * 4 + a.batch * a.k * 8
        traffic, tsrc = measured_traffic("scan", a.n, a.dim, a.batch, a.k, a.metric)
        kernel = "scan_kernel (fused FP32 scan + top-k)"
        dtype = "f32"
    roofline = hbm_roofline(alg_bytes, scan_avg_ms, peak, peak_kind, traffic, tsrc, kernel)
    roofline["after_kernel_ms_avg"] = round(merge_ms / max(launches, 1), 5)

    extra = {}
    bf16_peak = peaks_bf16()
    bf16_sustained = peaks_bf16("bf16_tflops_sustained")
    if rank == 0 and a.sweep and world == 1:
        sweep = []
        tb = [int(s) for s in a.sweep.split(",") if s and int(s) <= q.shape[0]]
        if not a.no_autotune:  # method auto then follows the tuned table (after the headline line)
            t0 = time.perf_counter()
            # timed on a sample of the workload's own queries (the rest of the query set)
            tq = q[len(q) // 2:]
            extra["autotune"] = {"table": idx.autotune(tb, a.k, queries=tq),
                                 "bf16": idx.autotune(tb, a.k, method="bf16", queries=tq),
                                 "seconds": round(time.perf_counter() - t0, 2)}
        for b in [int(s) for s in a.sweep.split(",") if s]:
            if b > q.shape[0]:
                continue
            st = max(3, min(300, int(3e4 / b)))
            info_b = {}
            ms_b, scan_b, _, l_b = time_device(idx, torch, qd, a, b, st, 3, stream, out=info_b)
            flops = 2.0 * a.n * a.dim * b
            e8 = bool(info_b.get("tc_exact")) and uses_e4m3(idx, b, a.k, a.dim)
            # rows read by the auto path: e4m3 (+ its scales), bf16 or FP32
            row_bytes = a.n * ((a.dim + 15) // 16 * 16 + 4) if e8 else a.n * a.dim * (2 if info_b.get("tc_exact") else 4)
            row = {"batch": b, "qps": round(b * st / (ms_b / 1e3), 1), "ms_per_batch": round(ms_b / st, 4),
                   "auto_path": ("tc_exact_e4m3" if e8 else "tc_exact") if info_b.get("tc_exact") else "fp32",
                   "kernel_gbs": round(row_bytes / (scan_b / l_b / 1e3) / 1e9, 1),
                   "kernel_tflops": round(flops / (scan_b / l_b / 1e3) / 1e12, 2)}
            if b == 1:
                ms_m, _, _, _ = time_device(idx, torch, qd, a, b, max(3, st // 2), 3, stream, method="skinny",
                                            profile_steps=0)
                row["skinny_qps"] = round(b * max(3, st // 2) / (ms_m / 1e3), 1)
            if 8 <= b <= 256:  # both plain kernels near the auto crossover
                for m in ("skinny", "tiled"):
                    ms_m, _, _, _ = time_device(idx, torch, qd, a, b, max(3, st // 2), 3, stream, method=m,
                                                profile_steps=0)
                    row[m + "_qps"] = round(b * max(3, st // 2) / (ms_m / 1e3), 1)
            # precision form: BF16 tensor-core shortlist (k' = 4k) + exact FP32 rerank
            sb = max(3, min(200, int(2e5 / b)))
            ms_t, tc_t, rr_t, l_t = time_device(idx, torch, qd, a, b, sb, 3, stream, method="bf16")
            row["bf16_qps"] = round(b * sb / (ms_t / 1e3), 1)
            row["bf16_tc_tflops"] = round(flops / (tc_t / l_t / 1e3) / 1e12, 1)
            row["bf16_tc_gbs"] = round(a.n * a.dim * 2 / (tc_t / l_t / 1e3) / 1e9, 1)
            row["bf16_rerank_ms"] = round(rr_t / l_t, 4)
            # roofline fractions: HBM (measured copy) for the scan kernel at small batch, FP32 FMA
            # (nominal 80.5 TFLOP/s) for the FP32 kernels at large batch, bf16 tensor (measured)
            # for the shortlist kernel
            row["kernel_frac_hbm"] = round(row["kernel_gbs"] / peak, 4)
            if info_b.get("tc_exact"):  # the bf16 tensor-core pass, against the sustained bf16 peak
                row["kernel_frac_bf16_sustained"] = round(row["kernel_tflops"] / bf16_sustained, 4)
            else:
                row["kernel_frac_fp32"] = round(row["kernel_tflops"] / 80.5, 4)
            row["bf16_tc_frac"] = round(row["bf16_tc_tflops"] / bf16_peak, 4)
            if True:  # certified exact tensor-core path: the scan kernel's results, bit for bit
                q0, s0, f0 = idx.tc_exact_stats()
                ms_e, _, _, _ = time_device(idx, torch, qd, a, b, sb, 3, stream, method="tc_exact", profile_steps=0)
                q1, s1, f1 = idx.tc_exact_stats()
                row["tc_exact_qps"] = round(b * sb / (ms_e / 1e3), 1)
                row["tc_exact_uncertified"] = round((s1 - s0) / max(q1 - q0, 1), 4)
                row["tc_exact_scan_fallback"] = round((f1 - f0) / max(q1 - q0, 1), 4)
            sweep.append(row)
        extra["sweep"] = sweep

    if rank == 0 and world == 1 and a.metric == "ip" and not a.no_filtered:
        extra["filtered_sweep"] = filtered_sweep(idx, torch, qd, q, a, stream)
        extra["filtered_sweep_b256"] = filtered_sweep(idx, torch, qd, q, a, stream, batch=256)

    if rank == 0 and world == 1 and a.metric == "ip" and a.n >= 8 * a.dim:
        # the plain FP32 scan kernel at batch 1 (the drop-in's HBM-bound kernel)
        stp = max(20, min(a.steps, 300))
        _, sc_ms, _, sc_l = time_device(idx, torch, qd, a, 1, stp, 5, stream, method="skinny")
        t_plain, tsrc_plain = measured_traffic("scan", a.n, a.dim, 1, a.k, a.metric)
        extra["roofline_plain"] = hbm_roofline(a.n * a.dim * 4 + a.dim * 4 + a.k * 8, sc_ms / max(sc_l, 1), peak,
                                               peak_kind, t_plain, tsrc_plain,
                                               "scan_kernel (fused FP32 scan + top-k), batch 1, method skinny")

    truth = None
    if rank == 0 and world == 1 and not a.no_parity and a.metric == "ip":
        extra["parity"], truth = parity_checks(vsg, idx, x, q, a)
        extra["precision"] = precision_checks(vsg, idx, torch, qd, x, q, a, stream, truth)

    if rank == 0 and world == 1 and not a.no_serve and a.metric == "ip":
        extra["serve"] = serve_check(vsg, idx, q, a)

    if rank == 0 and not a.no_recall:
        from oracle import oracle as O
        nchk = min(a.batch, 16) if a.batch > 1 else 8
        ids, _ = idx.search(q[:nchk], a.k)
        gi = truth[0][:nchk] if truth is not None and truth[0].shape[1] == a.k else O.fp64_topk(x, q[:nchk], a.k,
                                                                                                 a.metric)[0]
        extra["recall_vs_fp64"] = vsg.recall_at_k(ids, gi, a.k)
        try:
            extra["near_ties_tolerated"] = O.check_ids(ids, gi, x, q[:nchk], a.metric)
            extra["ids_match_fp64_rule"] = True
        except AssertionError as e:
            extra["ids_match_fp64_rule"] = False
            extra["id_mismatch"] = str(e)[:200]

    cpu = None
    if rank == 0 and not a.no_cpu_baseline and world == 1:
        cpu = cpu_baseline(x, q, a, os.cpu_count() or 1)

    if rank == 0:
        line = {
            "metric": f"exact top-{a.k} QPS at {a.n // 1000}Kx{a.dim}", "value": round(qps, 2),
            "unit": "queries/s", "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": round(ms / a.steps, 5), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": dtype, "data": "synthetic",
            "config": dict(workload(a), parallelism=f"replicas{world}"),
            "roofline": roofline, "cpu_baseline": cpu,
            "e2e": {"value": round(e2e_qps, 2), "unit": "queries/s", "h2d_bytes_per_step": a.batch * a.dim * 4,
                    "d2h_bytes_per_step": a.batch * a.k * 8, "steps": e2e_steps},
            "gpu_launches": int(info.get("kernels", 0)), "clocks": clocks,
        }
        line.update(extra)
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def run_filtered(a):
    """Config 3 alone: per-query group masks over the base; gather scan, masked full scan and the
    certified path at --filter-batch queries for each allowed count in --filter-targets."""
    import torch
    import vecsearch_gb300 as vsg
    torch.cuda.set_device(0)
    x, q = make_data(a)
    idx = vsg.GpuBruteForceIndex(a.dim, "cosine" if a.metric == "ip" else "l2")
    idx.add(x)
    qd = torch.from_numpy(q).cuda()
    targets = tuple(int(t) for t in a.filter_targets.split(",") if t)
    rows = filtered_sweep(idx, torch, qd, q, a, torch.cuda.current_stream(), batch=a.filter_batch, targets=targets)
    print(json.dumps({"metric": "filtered exact top-k QPS by allowed rows", "unit": "queries/s", "data": "synthetic",
                      "config": dict(workload(a), batch=a.filter_batch), "results": rows}), flush=True)


def run_precision(a):
    """Config 4: BF16 and FP8-e4m3 shortlists (k' = 40 and 80 for k = 10, 120 for k = 100) + exact FP32 rerank vs the FP32
    path, on the 1M x 384 base (1,024 clusters) and, with --big, a 4M x 384 base (4,096 clusters):
    device QPS by batch, recall@k and max |distance error| against the FP64 oracle."""
    import torch
    import vecsearch_gb300 as vsg
    from oracle import oracle as O
    from vecsearch_gb300 import datasets as D
    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    bases = [(1_000_000, 1024)] + ([(4_000_000, 4096)] if a.big else [])
    batches = [int(b) for b in a.sweep.split(",") if b]
    out = []
    for n, clusters in bases:
        x, _ = D.clustered(n, a.dim, clusters, 0.35, seed=0, centroid_seed=2)
        q, _ = D.clustered(a.queries, a.dim, clusters, 0.35, seed=1, centroid_seed=2)
        idx = vsg.GpuBruteForceIndex(a.dim, "cosine")
        idx.add(x)
        qd = torch.from_numpy(q).cuda()
        nchk = 32
        truth = {k: O.fp64_topk(x, q[:nchk], k, "ip") for k in (10, 100)}
        for dtype in ("bf16", "fp8"):
            for k in (10, 100):
                for over in ((4, 8) if k == 10 else (1.2,)):  # k' = 40, 80 (k = 10) and 120 (k = 100)
                    idx.set_tunable("shortlist_oversample", over)
                    kp = min(448, int(np.ceil(over * k - 1e-9)))
                    tune = idx.autotune(batches, k, method="bf16", queries=q[len(q) // 2:])  # per batch, this k'
                    a2 = argparse.Namespace(**vars(a))
                    a2.k = k
                    row = {"n": n, "dtype": dtype, "k": k, "k_prime": kp, "qps": {}, "plain_qps": {},
                           "sample_rows": {e["batch"]: e["sample"] for e in tune}}
                    if dtype == "bf16" and over in (4, 1.2):
                        row["exact_tc_qps"] = {}  # the certified exact path, for comparison
                    for b in batches:
                        st = max(3, min(100, int(1e5 / b)))
                        ms, tc_ms, rr_ms, l = time_device(idx, torch, qd, a2, b, st, 3, stream, method=dtype)
                        row["qps"][b] = round(b * st / (ms / 1e3), 1)
                        if dtype == "bf16" and over in (4, 1.2) and b >= 8:
                            # plain: the faster FP32 kernel (scan or register-blocked tiled)
                            stp = max(3, min(50, int(2e4 / b)))
                            best = None
                            for m in (("skinny", "tiled") if b <= 512 else ("tiled",)):
                                msp, _, _, _ = time_device(idx, torch, qd, a2, b, stp, 2, stream, method=m,
                                                           profile_steps=0)
                                best = msp if best is None else min(best, msp)
                            row["plain_qps"][b] = round(b * stp / (best / 1e3), 1)
                            mse, _, _, _ = time_device(idx, torch, qd, a2, b, stp, 2, stream, method="tc_exact",
                                                       profile_steps=0)
                            row["exact_tc_qps"][b] = round(b * stp / (mse / 1e3), 1)
                    ids, dists = idx.search(q[:nchk], k, method=dtype)
                    gi, gd = truth[k]
                    row["recall_vs_fp64"] = vsg.recall_at_k(ids, gi, k)
                    errs = []
                    for i in range(nchk):
                        ok = ids[i] >= 0
                        d64 = O.fp64_distances(x, q[i:i + 1], "ip", ids[i][ok])[0]
                        errs.append(np.max(np.abs(dists[i][ok].astype(np.float64) - d64)))
                    row["max_abs_dist_err_vs_fp64"] = float(max(errs))
                    out.append(row)
                    print(json.dumps(row), flush=True)
        idx.set_tunable("shortlist_oversample", 4)
        del idx
    print(json.dumps({"metric": "precision form: BF16 / FP8 shortlist + FP32 rerank QPS by batch", "unit": "queries/s",
                      "data": "synthetic", "config": {"workload": "1M (and 4M) x 384 unit rows, cosine",
                                                        "batches": batches}, "results": out}), flush=True)


def serve_load(idx, srv, x, q, groups, words_by_group, rate, duration, seed, plain=False):
    """Open-loop Poisson arrivals at `rate` queries/s for `duration` s; each request 1-64 queries
    (log-uniform), k 10 or 100, 30% with one group's filter. Latency = completion - scheduled arrival."""
    import threading
    rng = np.random.default_rng(seed)
    mean_q = 63.0 / np.log(64.0)  # E[m] for m = floor(exp(U(0, ln 64))) is close to this
    req_rate = rate / mean_q
    t, reqs, pos = 0.0, [], 0
    while t < duration:
        t += rng.exponential(1.0 / req_rate)
        m = max(1, min(64, int(np.exp(rng.uniform(0, np.log(64))))))
        if pos + m > len(q):
            pos = 0
        k = int(rng.choice([10, 100]))
        g = int(rng.choice(list(words_by_group))) if rng.random() < 0.3 else None
        reqs.append((t, pos, m, k, g))
        pos += m
    lat = [0.0] * len(reqs)
    start = time.perf_counter() + 0.05
    if plain:
        for i, (ts, p0, m, k, g) in enumerate(reqs):
            now = time.perf_counter() - start
            if now < ts:
                time.sleep(ts - now)
            idx.search(q[p0:p0 + m], k, filter=None if g is None else (groups == g))
            lat[i] = (time.perf_counter() - start - ts) * 1e3
    else:
        tickets = [None] * len(reqs)
        done = threading.Event()

        def waiter():
            for i in range(len(reqs)):
                while tickets[i] is None:
                    time.sleep(20e-6)
                srv.wait(tickets[i], timeout=60)
                lat[i] = (time.perf_counter() - start - reqs[i][0]) * 1e3
            done.set()

        th = threading.Thread(target=waiter)
        th.start()
        for i, (ts, p0, m, k, g) in enumerate(reqs):
            now = time.perf_counter() - start
            if now < ts:
                time.sleep(ts - now)
            tickets[i] = srv.submit(q[p0:p0 + m], k, filter_words=None if g is None else words_by_group[g])
        th.join()
    end = time.perf_counter() - start
    nq = sum(r[2] for r in reqs)
    return {"offered_qps": rate, "requests": len(reqs), "queries": nq, "achieved_qps": round(nq / end, 1),
            "p50_ms": round(float(np.percentile(lat, 50)), 3), "p99_ms": round(float(np.percentile(lat, 99)), 3)}


def run_serve(a):
    """Config 5: the continuous-batching server vs the plain per-call FP32 path under open-loop load."""
    import torch
    import vecsearch_gb300 as vsg
    torch.cuda.set_device(0)
    x, q = make_data(a)
    idx = vsg.GpuBruteForceIndex(a.dim, "cosine")
    idx.add(x)
    groups, words_by_group = serve_setup(a, idx, vsg)
    srv = vsg.Server(idx, max_batch=1024, max_k=100, slots=2)
    rates = [int(r) for r in a.rates.split(",") if r]
    serve_load(idx, srv, x, q, groups, words_by_group, 2000, 0.3, 1)  # warm-up
    server_rows = [serve_load(idx, srv, x, q, groups, words_by_group, r, a.duration, 10 + i)
                   for i, r in enumerate(rates)]
    st = srv.stats()
    srv.close()
    plain_rows = [serve_load(idx, None, x, q, groups, words_by_group, r, min(a.duration, 1.0), 10 + i, plain=True)
                  for i, r in enumerate(rates) if r <= a.plain_max_rate]
    line = {"metric": "served p50/p99 latency and QPS (open-loop Poisson)", "unit": "ms",
            "data": "synthetic",
            "config": {"workload": f"{a.n:,} x {a.dim} unit rows, requests of 1-64 queries (log-uniform), k 10 or 100,"
                                   " 30% filtered to one Zipf(1.1) group of 2,000", "duration_s": a.duration,
                       "server": "2 slots x 1024 queries, certified path (BF16 shortlist, exact FP32 rerank, certificate, FP32 scan of unproven queries): results equal method skinny",
                       "plain": "one idx.search call per request (exact FP32 kernels), in arrival order"},
            "server": server_rows, "plain": plain_rows, "server_stats": st}
    print(json.dumps(line), flush=True)


def run_worker(a):
    """The GPU shard worker (vecsearch_gb300.shard_worker) behind its Searcher method bodies:
    `clients` threads each send one-query Search requests back to back (encoded as search.proto's
    SearchRequest, decoded replies), for --duration seconds per client count. The worker's batcher
    gathers concurrent calls into one exact device search. Reports calls/s, latency percentiles
    and the mean batch formed. gRPC transport is not included (the GPU image has no grpcio)."""
    import threading
    import torch
    import vecsearch_gb300 as vsg
    from vecsearch_gb300 import shard_worker as W
    torch.cuda.set_device(0)
    x, q = make_data(a)
    idx = vsg.GpuBruteForceIndex(a.dim, "cosine" if a.metric == "ip" else "l2")
    idx.add(x)
    reqs = [W.encode_search_request(q[i], a.k, 64) for i in range(len(q))]
    rows = []
    for clients in (1, 16, 64, 256):
        s = W.ShardSearcher(idx, offset=0, shard_id=0, max_batch=256, max_wait_ms=0.2)
        for i in range(8):  # warm-up
            s.search(reqs[i])
        lat = [[] for _ in range(clients)]
        stop = time.perf_counter() + a.duration
        b0, c0 = s.batches, s.calls

        def client(c):
            i = c
            while time.perf_counter() < stop:
                t = time.perf_counter()
                s.search(reqs[i % len(reqs)])
                lat[c].append(time.perf_counter() - t)
                i += clients

        t0 = time.perf_counter()
        ts = [threading.Thread(target=client, args=(c,)) for c in range(clients)]
        for t in ts:
            t.start()
        for t in ts:
            t.join()
        el = time.perf_counter() - t0
        calls, batches = s.calls - c0, s.batches - b0
        s.close()
        allv = np.sort(np.concatenate([np.asarray(v) for v in lat])) * 1e3
        rows.append({"clients": clients, "calls_per_s": round(calls / el, 1),
                     "p50_ms": round(float(np.percentile(allv, 50)), 3),
                     "p99_ms": round(float(np.percentile(allv, 99)), 3),
                     "mean_batch": round(calls / max(batches, 1), 1)})
        print(json.dumps(rows[-1]), file=sys.stderr, flush=True)
    print(json.dumps({"metric": "GPU shard worker: exact top-k Search calls/s and latency by concurrent clients",
                      "unit": "calls/s", "data": "synthetic",
                      "config": {"workload": f"one shard of {a.n:,} x {a.dim} rows, k = {a.k}, one query per call",
                                 "batcher": "up to 256 calls, 0.2 ms window, method auto"},
                      "results": rows}), flush=True)


def main():
    a = parse()
    if a.mode == "worker":
        run_worker(a)
        return
    if a.mode == "serve":
        run_serve(a)
        return
    if a.mode == "precision":
        run_precision(a)
        return
    if a.mode == "filtered":
        run_filtered(a)
        return
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
