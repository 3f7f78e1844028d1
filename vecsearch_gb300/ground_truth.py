"""Exact top-k ground truth for an ANN benchmark, computed on the GPU.

Replaces bench/ground_truth.py of vecsearch, which runs FAISS IndexFlatIP over every query
(:22-28) and saves the ids as int64 gt.npy (:29), then checks vecsearch's own BruteForceIndex
against it on a 200,000-row sample (:31-41). Here the exact FP32 GPU index does the search in
batches of queries resident in HBM; the result follows the reference's exact-search order
((dist, id), ties to the lower id).

    python -m vecsearch_gb300.ground_truth --data DIR --k 100 [--metric ip] [--batch 4096]

reads DIR/base.npy and DIR/queries.npy and writes DIR/gt.npy (int64, nq x k). When the
reference's ``vecsearch`` package is importable, the same agreement check as the reference's
script runs against its CPU BruteForceIndex on a sample.
"""
import argparse
import os
import time

import numpy as np

__all__ = ["ground_truth"]


def ground_truth(xb, xq, k=100, metric="ip", batch=4096, method="auto", device=0, return_distances=False):
    """Exact top-k ids (int64 [nq, k], -1 where the base has fewer than k rows) of every query.

    method "auto" by default: exact, through the FP32 kernels or (large indexes, k <= 32) the
    certified tensor-core path, whose results equal the FP32 scan's bit for bit; "tc_exact" forces
    the latter. "bf16" takes the tensor-core shortlist + FP32 rerank without the certificate
    (k <= 120): its ids equal the exact ones whenever each query's shortlist holds its top k.
    """
    from . import GpuBruteForceIndex
    xb = np.ascontiguousarray(xb, dtype=np.float32)
    xq = np.ascontiguousarray(xq, dtype=np.float32)
    if xb.ndim != 2 or xq.ndim != 2 or xb.shape[1] != xq.shape[1]:
        raise ValueError("xb and xq must be 2-D with the same number of columns")
    if batch < 1:
        raise ValueError("batch must be >= 1")
    idx = GpuBruteForceIndex(xb.shape[1], metric, device=device)
    idx.add(xb)
    ids = np.empty((len(xq), k), np.int64)
    dists = np.empty((len(xq), k), np.float32)
    for s in range(0, len(xq), batch):
        ids[s:s + batch], dists[s:s + batch] = idx.search(xq[s:s + batch], k, method=method)
    return (ids, dists) if return_distances else ids


def _agreement(xb, xq, metric, sample=200_000, nq=20, k=10):
    """The reference script's self-check, with the reference package when it is installed."""
    try:
        import vecsearch as vs
    except ImportError:
        return None
    n = min(len(xb), sample)
    bf = vs.BruteForceIndex(xb.shape[1], metric)
    bf.add(xb[:n])
    mine, _ = bf.search(xq[:nq], k)
    gpu = ground_truth(xb[:n], xq[:nq], k, metric)
    return vs.recall_at_k(mine, gpu, k)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--data", default="data/tweets")
    ap.add_argument("--k", type=int, default=100)
    ap.add_argument("--metric", default="ip", choices=["ip", "cosine", "l2"])
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--method", default="auto", choices=["auto", "tiled", "skinny", "tc_exact", "bf16"])
    ap.add_argument("--device", type=int, default=0)
    a = ap.parse_args(argv)
    xb = np.load(os.path.join(a.data, "base.npy"))
    xq = np.load(os.path.join(a.data, "queries.npy"))
    t = time.time()
    gt = ground_truth(xb, xq, a.k, a.metric, a.batch, a.method, a.device)
    print(f"exact search {len(xq):,} x {len(xb):,} in {time.time() - t:.1f}s")
    np.save(os.path.join(a.data, "gt.npy"), gt)
    agree = _agreement(xb, xq, "ip" if a.metric == "cosine" else a.metric)
    if agree is not None:
        print(f"vecsearch.BruteForce vs GPU exact agreement: {agree:.4f}")
        if agree <= 0.99:
            raise SystemExit("BruteForceIndex and the GPU index disagree")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
