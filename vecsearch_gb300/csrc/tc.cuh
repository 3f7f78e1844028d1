// Launch interface of the tensor-core shortlist path (host side).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace vsg {

constexpr int kTcQueries = 128;  // queries per CTA (TMEM lanes, MMA M)
constexpr int kTcRows = 256;     // base rows per tile (MMA N; one accumulator of 256 TMEM columns)
constexpr int kTcKChunk = 64;    // bf16 dims per staged chunk (one 128-byte swizzle row)
// Largest per-query shortlist k' of one split's list: candidate buffers hold 64 (k' <= 16), 128
// (<= 48), 256 (<= 120) or 512 (<= 448) entries per query, so a list of k' always leaves room
// for 64 appends between compactions.
constexpr int kTcMaxShortlist = 448;
// Entries of the split lists the finish kernel stages in shared memory per query at most; beyond
// that its passes read the lists in global memory (176 KB of staging: with the query and the
// candidate arrays it fits the 227 KB of a CTA for every dim up to 4,096).
constexpr uint32_t kFinishStageMax = 22528;
// The shortlist kernel writes a query's final list of a split sorted by (dist, id) when the warp
// that holds the query has at most this many real queries (few queries: the sort lets the margin
// cut shorten the list), else unsorted with its smallest entry first. So a batch of at most this
// many queries has sorted lists only.
constexpr uint32_t kSortedListQueries = 8;

// Serving mode: one entry per query of a micro-batch (device memory).
struct ServeQuery {
  uint32_t k;              // results wanted
  uint32_t kp;             // shortlist entries (k <= kp <= TcArgs::kp)
  const uint32_t* mask;    // allow-bits of this query (device), or nullptr
  uint32_t out_off;        // first result slot of this query in the output block
  uint32_t pad;
};

// Serving mode: the micro-batch shape, written before each launch (device memory).
struct ServeHeader {
  uint32_t nq, nqb, nsplit, rows_per_split;
  uint32_t items;          // nqb * nsplit
  uint32_t next;           // work counter: CTAs claim items with atomicAdd (zeroed per launch)
  uint32_t sample_tiles;   // tiles per split scored by the sample pass
  uint32_t pad;
};

struct TcArgs {
  uint32_t n, dp, nq, kp;          // dp: padded elements per row of the operand copies; kp <= 448
  uint32_t rows_per_split, nsplit;  // rows_per_split: a multiple of kTcRows
  uint32_t stages;
  uint32_t resident;               // 1: the query block stays in shared memory for a whole item
  uint32_t l2;                     // 1: approximate L2 from norms, 0: 1 - q.x
  // 1: the operand copies are FP8 e4m3 with a scale per row (xscale) and per query (qscale), the
  // score being qscale * xscale * (q8 . x8); 0: bf16 copies without scales.
  uint32_t fp8;
  const float* xscale;
  const float* qscale;
  // Per-CTA candidate buffers in global memory: CTA c (linear index) owns entries
  // [c * 128 * cap, (c + 1) * 128 * cap), cap = tc_buffer_capacity(kp) per query slot.
  float* cbuf_d;
  uint32_t* cbuf_i;
  // Per-query shared thresholds (order keys of approximate distances, 0xFFFFFFFF = none),
  // or nullptr: a split whose list is full publishes its k'-th best with atomicMin and every
  // split of the query prunes against the smallest published value. Set to 0xFF bytes first.
  const float* xnorm;              // squared row norms (L2 only)
  const float* qnorm;              // squared query norms (L2 only)
  float* part_d;                   // [nq][nsplit][kp] approximate distances, sorted
  uint32_t* part_i;
  uint32_t* part_n;                // [nq][nsplit] real entries of each list, or nullptr
  int* status;
  uint32_t* gthr;
  // Serving mode (persistent): when hdr is set the grid has one CTA per SM, the batch shape
  // (nq, splits) comes from hdr, CTAs claim (query block, split) items from hdr->next, and each
  // query's shortlist size and filter come from sq. Otherwise CTA c takes items c, c + grid, ...
  // of the nqb * nsplit items (query block = item % nqb, split = item / nqb).
  ServeHeader* hdr;
  const ServeQuery* sq;
  // Sample pass: when dump is set, each CTA scores only the first sample_tiles tiles of its split
  // and writes the raw approximate distances (+inf where the filter or the range excludes a row)
  // to dump[q][split * sample_tiles * 128 + j]; no shortlist is kept.
  float* dump;
  uint32_t sample_tiles;
  // Sample pass with dump_min set: the smallest distance of each 32 rows only, to
  // dump[q][split * sample_tiles * 8 + j] (the k-th smallest of these minima still bounds the k-th
  // smallest sampled distance from above: k of the 32-row groups each hold a row at or below it).
  uint32_t dump_min;
  // Main pass: per-query starting threshold (the k'-th smallest sampled distance), or nullptr.
  const float* thr_init;
  // Certified path: per-query margin m, or nullptr. A compaction that holds at least kk entries
  // (serving mode: the query's k from sq) may then lower the threshold to (its kk-th best) + m, so
  // the list keeps the rows near the top kk instead of a fixed k'. Every threshold is published
  // to gthr, and the finish kernel's certificate takes the smallest, so any m keeps results exact.
  const float* margin;
  uint32_t kk;
  uint32_t nqb;  // query blocks (non-serving launches)
  // Non-serving launches: allow-bits (bit r & 31 of word r >> 5), one mask for every query
  // (mask_ld = 0) or one per query, mask_ld words apart; nullptr = no filter.
  const uint32_t* mask;
  uint32_t mask_ld;
  // Limit of one wait on another role, in ns (0: 2 s). The waits that drain the CTA's own copies
  // and MMAs before it exits always take 2 s.
  uint64_t wait_ns;
  // Test hook: 1 makes the epilogue warps first wait on a barrier nothing completes, so that wait
  // runs out after wait_ns and the kernel winds down with kDevTimeout.
  uint32_t stall;
  // Main pass of a small certified batch: the FP32 rows (xf_ld floats apart, xf_ld a multiple of
  // 4), or nullptr. Every row of a split's final list is prefetched into L2 (one bulk prefetch a
  // row) as the list is written, so the finish kernel's rerank of it reads L2 instead of DRAM.
  const float* xf;
  uint32_t xf_ld;
};

// Per-query k'-th smallest of `count` sampled distances (row q at in + q * count) -> thr[q]; plus
// margin[q] (rounded up) when margin != nullptr.
// pdl: launched as a programmatic dependent of the previous kernel in the stream (every launcher
// below with that flag; the kernels wait for their predecessors before touching their outputs).
cudaError_t launch_sample_select(const float* in, uint32_t count, uint32_t nq, const uint32_t* kp_per_query,
                                 uint32_t kp, float* thr, cudaStream_t stream, const float* margin = nullptr,
                                 bool pdl = false);
// Serving mode: the same with nq, count (nsplit * sample_tiles * 128) from hdr and each query's
// k' from sq (with margins: its k-th sampled distance plus margin[q]); CTAs past hdr->nq exit.
cudaError_t launch_serve_select(const ServeHeader* hdr, const ServeQuery* sq, const float* in, float* thr,
                                uint32_t max_queries, cudaStream_t stream, const float* margin = nullptr);

// Serving mode, the certified path's fallback after the scan (a launch sized for max_queries,
// reading the uncertified count on the device): the first sq.k of the scan's kmax results of slot
// j go to query fail_list[j]'s place in the output block, and the count is added to tally.
cudaError_t launch_serve_scatter(const uint32_t* count, const uint32_t* fail_list, const ServeQuery* sq,
                                 const float* src_d, const uint32_t* src_i, uint32_t kmax, float* out_d,
                                 uint32_t* out_i, unsigned long long* tally, uint32_t max_queries,
                                 cudaStream_t stream);

// count queries near rows of src (0.9 x_i + 0.1 x_j of its n rows, stride dp), for the autotuner.
cudaError_t launch_midpoint_rows(float* dst, const float* src, uint32_t dp, uint32_t n, uint32_t count,
                                 cudaStream_t stream);
// Epilogue groups of the shortlist kernel for a shortlist of kp: each writes its own list per
// (query, split), so a split has tc_groups(kp) lists (2 for kp <= 120, else 1); the candidate
// buffers hold tc_groups(kp) x 128 x tc_buffer_capacity(kp) entries per CTA.
uint32_t tc_groups(uint32_t kp);
// 128-byte chunks per row of an operand copy: dp bf16 (64 per chunk) or dp e4m3 (128 per chunk).
uint32_t tc_chunks(uint32_t dp, bool fp8);
// Shared memory of the shortlist kernel: ring depth, chunks per row, resident query block or not.
size_t tc_smem_bytes(uint32_t stages, uint32_t nkc, uint32_t resident);
// Ring depth for rows of nkc chunks that fits `budget` bytes (0 if none): the query block stays
// resident (*resident = 1) when that leaves at least 3 slots, else each slot carries a query chunk too.
uint32_t tc_pick_stages(uint32_t nkc, size_t budget, uint32_t* resident, bool l2, bool fp8);
// Candidate-buffer entries per query slot for a shortlist of kp (64, 128 or 256).
uint32_t tc_buffer_capacity(uint32_t kp);

// Encodes a 2-D tensor map over rows x dp elements (bf16: row stride dp * 2 bytes, 64 x box_rows
// box; fp8: dp bytes, 128 x box_rows box), 128-byte swizzle; box_rows <= 256 (128 for a query
// block). The driver's encoder is looked up through the runtime on first use.
cudaError_t tc_encode_map(CUtensorMap* map, const void* base, uint64_t rows, uint64_t dp, uint32_t box_rows,
                          bool fp8 = false);

// Operand copies of the rows are stored tile-major: for each tile of kTcRows rows, its 128-byte
// chunks one after another, each chunk holding that chunk of all kTcRows rows (chunk c of row r
// at byte ((r / kTcRows) * nkc + c) * kTcRows * 128 + (r % kTcRows) * 128). Every row-chunk box
// the shortlist kernel loads is then one contiguous 32 KB span. Bytes for `rows` rows:
size_t tc_tiled_bytes(size_t rows, uint32_t dp, bool fp8);
// Tensor map over such a copy of `rows` rows: a (64 bf16 | 128 e4m3) x (tiles * nkc * kTcRows)
// matrix of 128-byte chunk rows, box_rows per box (kTcRows), 128-byte swizzle.
cudaError_t tc_encode_tiled_map(CUtensorMap* map, const void* base, uint64_t rows, uint32_t dp, uint32_t box_rows,
                                bool fp8);

// Sets the shared-memory limit of the shortlist kernels of one variant (metric, operand type) for
// (stages, nkc, resident); launch_tc_shortlist does it too, but a launch being captured into a
// CUDA graph should find it done.
cudaError_t tc_prepare(uint32_t stages, uint32_t nkc, uint32_t resident, bool l2, bool fp8);
// grid: CTAs (x only); the candidate buffers must hold grid * tc_groups(kp) * 128 *
// tc_buffer_capacity(kp) entries, the lists nq * nsplit * tc_groups(kp) of kp (and their lengths).
cudaError_t launch_tc_shortlist(const CUtensorMap& qmap, const CUtensorMap& xmap, const TcArgs& a, unsigned grid,
                                cudaStream_t stream, bool pdl = false);
// FP32 -> bf16 rows (stride dp, padding copied as zeros) and, when norms != nullptr, squared norms.
// When bounds != nullptr, raises bounds[0..3) to the rows' max |x~ - x|, max |x| and max |x~|
// (x~ = the bf16 row; FP32 sums, not yet inflated for their rounding). With tile_row0 set, dst
// is a tile-major copy (tc_tiled_bytes) and the rows are its rows tile_row0, tile_row0 + 1, ...
constexpr size_t kRowMajor = ~size_t(0);
cudaError_t launch_to_bf16(const float* src, size_t ld_src, size_t rows, uint32_t dim, uint32_t dp, void* dst,
                           float* norms, cudaStream_t stream, float* bounds = nullptr, size_t tile_row0 = kRowMajor);
// The shortlist path's tail in one launch, one CTA per query: the real entries of the query's
// split lists (part_n of each, staged in shared memory when they fit in stage_cap), a cut at the
// target-th smallest approximate distance (k plus the query's margin on the certified path,
// else the shortlist size k'), the exact FP32 distances of every entry at or below the cut (at
// most 1,024) with the scan kernel's arithmetic, and the top k by (dist, id).
// Certification (exact results from the shortlist), when fail_count is set: every row outside the
// reranked set has an approximate distance >= L = min(sample threshold, the smallest shared
// threshold, the cut when it left entries out); the bound E on |approximate - FP32 distance|
// (from the bf16 rounding residuals of query and rows, Cauchy-Schwarz and accumulation terms; see
// launch_prepare_queries) then shows that none of them can enter the top k when L - E (rounded
// down) > the k-th FP32 distance found. Uncertified queries are counted (fail_count, atomic) and
// listed. Serving mode (hdr set): the batch shape comes from hdr, each query's k, k' and output
// offset from sq, and CTAs past hdr->nq exit. The kernel reads nothing when *status is set (a
// shortlist kernel gave up and its lists may be stale); row ids >= n are never dereferenced.
struct FinishArgs {
  const float* part_d;     // [nq][nsplit][kp] approximate distances (part_n of each list; its
                           // smallest by (order key, id) first, the rest in any order)
  const uint32_t* part_i;
  const uint32_t* part_n;  // [nq][nsplit x lists_per_split] real entries of each list
  uint32_t nq, nsplit, kp, k;  // kp: the lists' stride (<= kTcMaxShortlist) and, without margins, k'
  const float* margin;     // per-query margins (certified path), or nullptr
  const float* x;          // FP32 master rows, n x dp
  uint32_t n;
  const float* q;          // FP32 queries, row stride ldq
  uint32_t dp, ldq, l2;
  float* out_d;            // [nq][k], or at sq[q].out_off in serving mode
  uint32_t* out_i;
  const float* thr_init;   // per-query sample threshold, or nullptr (none)
  const uint32_t* gthr;    // the shortlist pass's shared thresholds (order keys), or nullptr
  const float* err;        // per-query E (launch_prepare_queries), needed when fail_count is set
  uint32_t* fail_count;    // number of uncertified queries, or nullptr: no certificate
  uint32_t* fail_list;     // their query indices
  const int* status;       // the shortlist kernels' status word, or nullptr
  const ServeHeader* hdr;  // serving mode, or nullptr
  const ServeQuery* sq;
  uint32_t stage_cap;      // list entries staged in shared memory at most (<= kFinishStageMax)
  uint32_t lists_per_split;  // lists of each split (the shortlist kernel's tc_groups(kp)); 0 = 1
  uint32_t sorted_lists;     // 1: every list is sorted by (dist, id) (kSortedListQueries)
  // CTAs per query (a thread-block cluster; at most 16, and nq x cluster at most the SM count,
  // else 1; 16 runs as 8 where such clusters do not fit): rank 0 does all but the rerank, which
  // the cluster shares. 0 or 1: one CTA.
  uint32_t cluster;
  // 1: the main pass prefetched the rows of its final lists into L2 (TcArgs::xf); otherwise a
  // one-CTA finish prefetches each staged row itself.
  uint32_t rows_in_l2;
  // The fallback's inputs, written for each uncertified query at its slot j in fail_list: its
  // FP32 row into fq row j (stride dp), its per-query mask (qmask row q, mask_ld words) into fmask
  // row j, or (serving) its filter pointer into fmask_ptrs[j]; tally counts them. Each optional.
  float* fq;
  const uint32_t* qmask;
  uint32_t* fmask;
  uint32_t mask_ld;
  const uint32_t** fmask_ptrs;
  unsigned long long* tally;
};
// Dynamic shared memory of the finish kernel, and its attribute set up to that size (done by
// launch_finish too; a launch captured into a CUDA graph should find it done). cluster16, when
// given, tells whether a cluster of 16 CTAs (a non-portable size: one GPC must hold them all) of
// the wide variant fits this device.
size_t finish_smem_bytes(uint32_t dp, uint32_t stage_cap);
cudaError_t finish_prepare(uint32_t dp, uint32_t stage_cap, bool* cluster16 = nullptr);
// grid: nq, or the largest batch in serving mode.
cudaError_t launch_finish(const FinishArgs& a, uint32_t grid, cudaStream_t stream, bool pdl = false);

// Small batches of the certified path: the sample is scored in FP32 by extra blocks of the query
// preparation, and its threshold selected there too, instead of a tensor-core sample pass and a
// select launch (two launches less before the main pass). The sample is the first 256 rows of
// each of `ranges` row ranges of rps rows (rows past n read +inf); each sample block writes, per
// query, the smallest distance of its rows to bmin[q * blocks + block]. The last block to finish
// (a ticket counter, zero between launches) sets thr[q] = the k-th smallest of the query's block
// minima plus the query's margin: k blocks each hold a row at or below it, so it bounds the k-th
// best FP32 sampled distance from above.
struct PrepSample {
  const float* x;   // FP32 rows, stride dp
  uint32_t n, rps, ranges;
  float* bmin;      // nq x sample blocks
  float* thr;       // nq thresholds out
  uint32_t k;
  uint32_t* ticket; // zero before the launch; the last block sets it back to zero
};
// The most queries and the largest padded dim the FP32 sample takes (its queries sit in shared
// memory: 8 x 1,024 floats).
constexpr uint32_t kPrepSampleQueries = 8, kPrepSampleDim = 1024;
// The most sampled rows it takes (ranges x 256): the last block selects from 512 block minima.
constexpr uint32_t kPrepSampleRows = 4096;

// The bf16 shortlist path's queries in one launch: bf16 copy qb (stride dp, padding zero) and
// squared norms qnorm (optional) of the FP32 queries (row stride ldq, dim columns read); gthr[q]
// reset to 0xFFFFFFFF (optional); with margin set (the certified path), err[q] = the certificate's
// bound E on |approximate - FP32 distance| over rows whose bf16 copies have the bounds xbound =
// [max |x~ - x|, max |x|, max |x~|] (x~ = bf16 row), and margin[q] = factor x E, both rounded up;
// and *fails = 0 when fails is set.
// qscale set: the certified path over the e4m3 copy; qb then receives e4m3 rows (stride dpo bytes,
// a multiple of 16, at most kPrepSampleDim) with qscale[q] = max |q| / 448, E covers the e4m3 roundings (xbound: the e4m3
// rows' bounds from launch_to_fp8), and the rest is as above.
cudaError_t launch_prepare_queries(const PrepSample* sample, const float* q, uint32_t ldq, uint32_t nq, uint32_t dim,
                                   uint32_t dp, void* qb,
                                   float* qnorm, uint32_t* gthr, const float* xbound, bool l2, float factor,
                                   float* margin, float* err, uint32_t* fails, cudaStream_t stream,
                                   float* qscale = nullptr, uint32_t dpo = 0);
// FP32 rows -> e4m3 rows (stride dp8 bytes, padding zero) with scale[r] = max |x_r| / 448 (1 for a
// zero row; saturating round to nearest of x / scale) and squared FP32 norms when norms != nullptr.
// With tile_row0 set, dst is a tile-major copy as in launch_to_bf16.
// bounds (optional): the rows' rounding bounds for the certificate, as launch_to_bf16 writes them.
cudaError_t launch_to_fp8(const float* src, size_t ld_src, size_t rows, uint32_t dim, uint32_t dp8, void* dst,
                          float* scale, float* norms, cudaStream_t stream, size_t tile_row0 = kRowMajor,
                          float* bounds = nullptr);

}  // namespace vsg
