// Launch interface of the exact-scan kernels (host side). Argument blocks are
// plain structs so they can be filled by the index code and by tests alike.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace vsg {

constexpr int kScanWarps = 8;                       // consumer warps per scan CTA
constexpr int kScanThreads = (kScanWarps + 1) * 32;  // + one producer warp
constexpr int kMaxStages = 8;

// One fused pass: distances of a block of QB queries against a row range, the
// filter applied per (query, row), and each warp's running top-k.
struct ScanArgs {
  const float* x;          // base rows, n x dp floats (dp: a multiple of 4; the index pads to 8)
  const float* q;          // queries, row stride ldq floats; rows >= nq are never read
  const uint32_t* mask;    // nullptr, or allow-bits: bit (r & 31) of word (r >> 5)
  uint64_t mask_ld;        // words between two queries' masks; 0 = one mask for all queries
  float* part_d;           // [nq][nsplit][k] per-split top-k, sorted by (dist, id)
  uint32_t* part_i;
  int* status;             // device status word (kDevOk / kDevTimeout)
  uint32_t n, dp, ldq, nq, k;
  uint32_t rows_per_split;  // multiple of 32
  uint32_t nsplit;
  uint32_t stages;          // ring depth (2..kMaxStages)
  uint32_t gather;          // with a mask: 1 = copy only allowed rows, 0 = masked full scan
  // Fused merge (optional): when `counters` is set, the last CTA of each query block to
  // finish merges all splits' lists and writes the final nq x k results to out_d / out_i.
  // counters: one zeroed uint32 per query block; the merging CTA resets its word to 0.
  uint32_t* counters;
  float* out_d;
  uint32_t* out_i;
  // Optional: the number of queries to search, read on the device (at most nq); the launch is
  // sized for nq and query blocks past the count return at once.
  const uint32_t* nq_dev;
  // Optional, instead of mask: one device pointer per query to its allow-bits, nullptr for a query
  // without a filter (a masked full scan: gather must be 0).
  const uint32_t* const* mask_ptrs;
  // Optional, with the fused merge: query j's final list goes to row out_map[j] of out_d / out_i
  // instead of row j (with nq_dev set, only queries j < *nq_dev are written).
  const uint32_t* out_map;
  // Limit of one wait on another role, in ns (0: 2 s). The waits that drain the CTA's own copies
  // before it exits always take 2 s.
  uint64_t wait_ns;
  // Test hook: 1 makes the consumer warps first wait on a barrier nothing completes, so that wait
  // runs out after wait_ns and the kernel winds down with kDevTimeout (needs stages < kMaxStages).
  uint32_t stall;
};

struct MergeArgs {
  const float* part_d;
  const uint32_t* part_i;
  float* out_d;            // [nq][k]
  uint32_t* out_i;
  uint32_t nq, nsplit, k;
  // Optional cut (the certified shortlist): with margin set, entries above (the kk-th best) +
  // margin[q], rounded up, are dropped (written as +inf / none) and lists that start above it are
  // not merged.
  const float* margin;
  uint32_t kk;
  // Optional: the number of queries to merge, read on the device (at most nq).
  const uint32_t* nq_dev;
};

// Rows per split as the kernels' 32-bit argument. Rounded up to `align`, a split can reach 2^32
// rows on an index of nearly 2^32 rows; it is capped at the largest multiple of `align` below
// 2^32, and callers derive the split count from the capped value.
inline uint32_t split_rows(size_t rows, size_t align) {
  const size_t cap = (size_t(0xFFFFFFFFu) / align) * align;
  return uint32_t(rows < cap ? rows : cap);
}

struct ScanShape {
  int qb;      // queries per CTA: 1, 2, 4 or 8
  int rw;      // rows per warp per tile: 1, 2 or 4 (tile = 8 * rw rows)
  bool l2;
};

// Shared-memory bytes the scan kernel needs for a shape, dim and k with `stages` ring slots.
size_t scan_smem_bytes(const ScanShape& s, uint32_t dp, uint32_t k, uint32_t stages);

// pdl: launched as a programmatic dependent of the previous kernel in the stream (the kernel
// waits for it before reading anything).
cudaError_t launch_scan(const ScanShape& s, const ScanArgs& a, dim3 grid, cudaStream_t stream, bool pdl = false);
// Sets the scan kernel's shared-memory limit for (shape, dp, k, stages) without launching, for a
// launch that is then captured into a CUDA graph.
cudaError_t scan_prepare(const ScanShape& s, uint32_t dp, uint32_t k, uint32_t stages);
cudaError_t launch_merge(const MergeArgs& m, cudaStream_t stream);
cudaError_t launch_fill_missing(float* out_d, uint32_t* out_i, size_t count, cudaStream_t stream);

}  // namespace vsg
