/*
 * vsg.h - C ABI of the GB300 exact k-NN engine (libvsg_gb300.so).
 *
 * The drop-in boundary for vecsearch's exact-search path. Every entry point
 * below names the reference interface it replaces (paths relative to the
 * vecsearch project). Plain pointers and sizes only; no C++ or torch types.
 *
 * Conventions
 *   - Every function that can fail returns a status code (VSG_OK = 0) and
 *     leaves a message for the calling thread in vsg_last_error().
 *   - Results are nq x k, row-major, nearest first, ordered by (dist, id):
 *     equal distances go to the lower id. Missing results (k > rows, or fewer
 *     allowed rows than k) are id VSG_NONE with dist +inf.
 *   - Distances: VSG_METRIC_L2 = squared Euclidean (no sqrt);
 *     VSG_METRIC_IP = 1 - <q, x> (cosine distance on unit-norm rows).
 *   - One index serialises its own calls (a mutex, as the reference's
 *     GpuBruteForceIndex does); separate indexes may be used from separate
 *     threads.
 */
#ifndef VSG_H_
#define VSG_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. The reference throws instead (src/gpu_brute_force.cu:11-16,
 * :294-298, :387, :408); the C++ wrapper re-throws the same exception types. */
#define VSG_OK 0
#define VSG_ERR_INVALID 1        /* std::invalid_argument (Python: ValueError) */
#define VSG_ERR_LENGTH 2         /* std::length_error (Python: ValueError) */
#define VSG_ERR_CUDA 3           /* std::runtime_error from a CUDA call (Python: RuntimeError) */
#define VSG_ERR_DEVICE_TIMEOUT 4 /* a kernel's bounded wait ran out (Python: RuntimeError) */
#define VSG_ERR_NOMEM 5          /* device or pinned host allocation failed (Python: MemoryError) */
#define VSG_ERR_IO 6             /* a file could not be read (std::runtime_error; Python: RuntimeError) */

/* Same values as vecsearch::Metric (include/vecsearch/distance.h:15). */
#define VSG_METRIC_L2 0u
#define VSG_METRIC_IP 1u

/* Same values as vecsearch::GpuMethod (include/vecsearch/gpu_brute_force.h:16-21).
 * Methods 0-3 return the same exact top-k, bit for bit; the method only picks the kernel (naive
 * and skinny: the streaming scan kernel; tiled: the register-blocked kernel, whose per-split
 * lists of a few more than k rows are reranked with the scan kernel's arithmetic and certified,
 * its unproven queries answered by the scan kernel; auto: by batch size).
 * VSG_METHOD_BF16 (new) is the precision form: a BF16 tensor-core pass keeps a shortlist of
 * k' = min(448, max(k, oversample x k)) rows per query by approximate distance, then an exact
 * FP32 rerank of the shortlist returns the top-k with the streaming kernel's arithmetic. It is
 * exact whenever the shortlist holds the true top-k. Filters apply to the shortlist. */
#define VSG_METHOD_AUTO 0u
#define VSG_METHOD_NAIVE 1u
#define VSG_METHOD_SKINNY 2u
#define VSG_METHOD_TILED 3u
#define VSG_METHOD_BF16 4u
/* VSG_METHOD_TC_EXACT (new): the shortlist path with a certificate. The finish kernel (merge,
 * FP32 rerank, certificate) bounds the difference between each row's bf16 approximate distance
 * and its FP32 distance (from the bf16 rounding of the query and the rows), and proves that no
 * row outside the shortlist can enter the top k; the shortlist keeps each query's rows within
 * "cert_margin" x E of its k-th best (at most k' = 120 for k <= 16, 448 above). Queries it cannot
 * prove run in the streaming scan kernel, launched on the device's own count of them (nothing
 * waits on the host). Results equal VSG_METHOD_SKINNY bit for bit, with or without a filter, for
 * every k <= 128. Method AUTO uses it for unfiltered batches of at least "tc_exact_min_batch"
 * queries, or of any size on an index of at least "tc_exact_min_elements", or where the
 * autotuner picked it; for filtered batches (k <= 32) of 8+ queries whose size times the largest
 * allowed fraction of their host masks is at least 0.35, or with too many allowed rows for the
 * gather scan, and for every filtered batch of at least half "tc_exact_min_batch" (device-resident
 * masks: from "tc_exact_min_batch", or twice it when the gather scan applies). */
#define VSG_METHOD_TC_EXACT 5u
/* VSG_METHOD_FP8 (new): the precision form over an FP8-e4m3 copy of the rows with one FP32 scale
 * per row (and per query): half the bytes of the bf16 copy, a coarser score, the same exact FP32
 * rerank of a shortlist of k' = min(448, max(k, oversample x k)) rows. */
#define VSG_METHOD_FP8 6u

#define VSG_NONE 0xFFFFFFFFu /* GpuBruteForceIndex::kNone (gpu_brute_force.h:26) */
#define VSG_MAX_K 128u       /* GpuBruteForceIndex::kMaxK (gpu_brute_force.h:27) */

typedef struct vsg_index vsg_index;

/* cuda_available() (include/vecsearch/gpu_brute_force.h:24, src/gpu_brute_force.cu:334-341):
 * 1 if the CUDA runtime sees at least one device, else 0 (clears the sticky error). */
int vsg_cuda_available(void);

/* Message of the last failing call on this thread ("" if none). */
const char* vsg_last_error(void);

/* GpuBruteForceIndex(dim, metric, device) (gpu_brute_force.h:31, src/gpu_brute_force.cu:386-396).
 * dim == 0 or an unknown metric -> VSG_ERR_INVALID. */
int vsg_create(size_t dim, uint32_t metric, int device, vsg_index** out);

/* ~GpuBruteForceIndex(): frees every device and pinned buffer of the index. NULL is a no-op. */
void vsg_destroy(vsg_index* index);

/* GpuBruteForceIndex::add (gpu_brute_force.h:36, src/gpu_brute_force.cu:404-423).
 * n host rows, row-major with stride dim floats; ids continue from vsg_size().
 * More than 2^32 - 2 rows in total -> VSG_ERR_LENGTH. */
int vsg_add(vsg_index* index, const float* rows, size_t n);

/* GpuBruteForceIndex::search (gpu_brute_force.h:40-41, src/gpu_brute_force.cu:425-488).
 * nq host queries (stride dim) -> host out_ids / out_dists (nq x k). k > VSG_MAX_K or an
 * unknown method -> VSG_ERR_INVALID. nq == 0 or k == 0 is a no-op; an empty index fills
 * VSG_NONE / +inf. Blocks until the results are in the host arrays. */
int vsg_search(vsg_index* index, const float* queries, size_t nq, size_t k, uint32_t* out_ids,
               float* out_dists, uint32_t method);

/* search() with a filter (the spec extension of gpu_brute_force.h:40-41 with the semantics
 * of python/bindings.cpp:28-36 as_mask): a row may be returned only if its allow-bit is set.
 * mask_words: bit (r & 31) of word (r >> 5) is row r. per_query == 0: one mask of
 * ceil(size / 32) words for every query; per_query != 0: nq masks, mask_ld words apart
 * (mask_ld >= ceil(size / 32)). */
int vsg_search_filtered(vsg_index* index, const float* queries, size_t nq, size_t k,
                        const uint32_t* mask_words, int per_query, size_t mask_ld, uint32_t* out_ids,
                        float* out_dists, uint32_t method);

/* The HNSW index's exact_below switch (include/vecsearch/hnsw.h:29-33 SearchFilter,
 * src/hnsw.cpp:325-328). allowed: one byte per row (nonzero = allowed), allowed_len == size.
 * If the mask allows no row, fills VSG_NONE / +inf and sets *handled = 1 (hnsw.cpp:326).
 * If 0 < allowed rows <= exact_below, runs the exact filtered scan on the GPU (in place of
 * search_exact, hnsw.cpp:336-354) and sets *handled = 1. Otherwise sets *handled = 0 and
 * writes nothing: the caller runs its graph search (hnsw.cpp:329-333). k > VSG_MAX_K ->
 * VSG_ERR_INVALID: HNSWIndex has no such limit, so a caller keeps search_exact for larger k. */
int vsg_hnsw_exact_below(vsg_index* index, const float* queries, size_t nq, size_t k,
                         const uint8_t* allowed, size_t allowed_len, size_t exact_below,
                         uint32_t* out_ids, float* out_dists, int* handled);

/* Vectors of a saved HNSW index (the VSHNSW01 file of HNSWIndex::save, src/hnsw.cpp:368-389)
 * straight into a device index, so the exact_below route shares the HNSW file without a second
 * host copy of the base (HNSWIndex::load, hnsw.cpp:391-420, reads them into host memory).
 * vsg_hnsw_file_info reads the header (dim, rows, metric 0 = L2 / 1 = inner product) and needs no
 * GPU. vsg_add_hnsw_file appends the file's rows (ids continue from size) after checking that
 * its dim and metric equal the index's (else VSG_ERR_INVALID). Bad magic ("not a vecsearch HNSW
 * file"), an unreadable or truncated file -> VSG_ERR_IO, and the index is left unchanged. */
int vsg_hnsw_file_info(const char* path, size_t* dim, size_t* rows, uint32_t* metric);
int vsg_add_hnsw_file(vsg_index* index, const char* path, size_t* added);

/* Exact neighbour candidates for an HNSW build in insertion order (new). The reference's insert
 * (HNSWIndex::insert, src/hnsw.cpp:247-309, in id order from HNSWIndex::add) searches the graph of
 * the nodes before it for ef_construction candidates; here row i's list is the exact k nearest of
 * rows 0 .. i-1 by (dist, id), padded with VSG_NONE / +inf while i < k. rows: n x dim host floats
 * (stride dim); out_ids / out_dists: n x k host arrays. k <= VSG_MAX_K, else VSG_ERR_INVALID.
 * Rows go through the device in batches of `batch` (0: 1024): each batch is searched against the
 * rows before it (an index that grows with the build) and against its own earlier rows (one
 * prefix filter per query), and the two lists are merged by (dist, id). Distances are the scan
 * kernel's, so every list equals one exact search over rows 0 .. i-1. Blocks until done. */
int vsg_insert_candidates(const float* rows, size_t n, size_t dim, uint32_t metric, int device, size_t k,
                          size_t batch, uint32_t* out_ids, float* out_dists);

/* Device-resident search (new: the serving/throughput form of search()). Queries, mask and
 * outputs are device pointers; queries have row stride ldq floats (ldq >= dim). Work is queued
 * on `stream` (a cudaStream_t; NULL = legacy default stream) and the call returns without
 * waiting. Calls on one index are ordered on the device even across streams. Device-side
 * failures are reported by the next vsg_sync() or host-side search on the index. */
int vsg_search_device(vsg_index* index, const float* d_queries, size_t ldq, size_t nq, size_t k,
                      const uint32_t* d_mask_words, int per_query, size_t mask_ld, uint32_t* d_out_ids,
                      float* d_out_dists, uint32_t method, void* stream);

/* Waits for the index's queued device work; reports a device-side failure, if any. */
int vsg_sync(vsg_index* index);

/* size(), dim(), metric() (gpu_brute_force.h:44-46). */
size_t vsg_size(const vsg_index* index);
size_t vsg_dim(const vsg_index* index);
uint32_t vsg_metric(const vsg_index* index);

/* Device pointer to the resident rows (size x padded_dim floats, padding zero) and the padded
 * dim, for zero-copy consumers of the index (e.g. a ground-truth or rerank pass). */
const float* vsg_device_rows(const vsg_index* index, size_t* padded_dim);

/* Named tunables of an index (new; the reference fixes its tunables at compile time,
 * src/gpu_brute_force.cu:23-31). Unknown names or out-of-range values -> VSG_ERR_INVALID.
 *   "gather_max_fraction" (default 0.10): a filtered search reads only the allowed rows (gather
 *   mode) when the largest allowed fraction of its masks is at most this, else it scans every
 *   tile holding an allowed row (masked full scan). Device-resident masks are not counted:
 *   they use gather mode unless the value is 0.
 *   "tiled_min_batch" (default 48): method "auto" runs unfiltered batches of at least this many
 *   queries in the register-blocked tiled kernel, smaller ones in the streaming scan kernel.
 *   "shortlist_oversample" (default 4): shortlist size factor of VSG_METHOD_BF16.
 *   "tc_exact_min_batch" (default 128): method "auto" sends unfiltered batches of at least this
 *   many queries (k <= 32) to VSG_METHOD_TC_EXACT unless the autotuner decided otherwise.
 *   "sample_rows" (default 16384): rows the tensor-core paths score first, per query, for a
 *   starting threshold (batches of 8+ queries; at most 4096 for smaller batches, and for batches
 *   of up to 64 queries with k <= 16; unless tuned per batch size).
 *   "tc_exact_min_elements" (default 2^27): unfiltered batches below "tc_exact_min_batch" (k <=
 *   32), down to one query, take VSG_METHOD_TC_EXACT under method "auto" when the index holds at
 *   least this many elements (rows x padded dim): reading the bf16 copy (half the bytes) then
 *   saves more than the shortlist path's fixed costs.
 *   "cert_margin" (default 1.3, >= 1): VSG_METHOD_TC_EXACT keeps, per query, the rows within
 *   cert_margin x E of its k-th best approximate distance (E: the certificate's bound on
 *   |approximate - FP32 distance|). A smaller value keeps fewer rows; a query whose k-th FP32
 *   distance lies more than (cert_margin - 1) E above its k-th approximate one is then not
 *   certified and runs in the streaming scan kernel. Results are exact for every value.
 *   "fallback_split_queries" (default 128, 0 to 2^20): VSG_METHOD_TC_EXACT's scan of the
 *   queries it did not certify splits the rows as for at most this many queries, so that a few
 *   such queries in a large batch still spread over the SMs (0: split as for the whole batch).
 *   Results are the same for every value.
 *   "wait_limit_s" (default 2, 1e-6 to 60): how long one kernel wait on another part of the same
 *   kernel (a copy landing, a slot freed, an accumulator filled) may last before the kernel winds
 *   down and the search returns VSG_ERR_DEVICE_TIMEOUT; the index stays usable. A CTA always
 *   waits up to 2 s for its own copies and MMAs before it exits, whatever this value.
 *   "test_stall_wait" (0 or 1; for testing the failure path): 1 makes the next search's scan or
 *   shortlist kernels first wait on a barrier that nothing completes, so that wait runs out after
 *   "wait_limit_s" and the search returns VSG_ERR_DEVICE_TIMEOUT; it resets to 0 after that search.
 *   "host_graph_max_batch" (default 16, 0 to 1024): vsg_search (unfiltered) of at most this many
 *   queries, repeated with the same shape (queries, k, method), replays one CUDA graph of the
 *   whole search, copies included, instead of issuing it call by call; captured on the second
 *   search of a shape, dropped when rows are added, a tunable or tuning table is set or a buffer is
 *   reallocated. Results are the same for every value; 0 switches it off.
 *   "host_graph_direct" (default 1, 0 or 1): in those graphs the certified path's kernels read
 *   the queries from the pinned staging buffer themselves instead of a copy into device memory.
 *   "cert_fp8_max_batch" (default 16): VSG_METHOD_TC_EXACT batches of at most this many queries
 *   with k <= 16 read an e4m3 copy of the rows (one FP32 scale per row, built on first use; half
 *   the bf16 copy's bytes) with a bound E that covers its roundings; results stay bit-identical to
 *   VSG_METHOD_SKINNY. 0 keeps every batch on the bf16 copy.
 *   "cert_fp8_sample_rows" (default 32768): rows sampled for those searches' starting thresholds.
 *   "cert_prefetch_max_batch" (default 16): those searches of at most this many queries prefetch
 *   the rows of their shortlists into L2 as the pass over the rows writes them, for the exact
 *   rerank.
 *   "finish_cluster" (default 8, 1 to 16): CTAs per query sharing the certified path's FP32 rerank
 *   (a thread-block cluster) when the batch times this fits the SM count; else one CTA a query.
 *   "finish_cluster_one" (default 16, 1 to 16): the same for a search of one query. Sizes above 8
 *   run as 8 on a device where such a cluster does not fit. */
int vsg_set_tunable(vsg_index* index, const char* name, double value);
int vsg_get_tunable(vsg_index* index, const char* name, double* value);

/* Autotuner (new; the reference's tunables are compile-time constants, src/gpu_brute_force.cu:23-31).
 * vsg_autotune times candidate schedules for each batch size (queries 0.9 x_i + 0.1 x_j of rows;
 * CUDA events, the mean over 3 different batches after a warm-up) and keeps the fastest per batch size:
 *   method VSG_METHOD_AUTO: streaming scan, tiled kernel or certified shortlist (VSG_METHOD_TC_EXACT),
 *     with 1x or 2x the row splits for the FP32 kernels (the certified path runs with its default k';
 *     a table loaded from a file may name a narrower first pass), used by
 *     unfiltered method-auto searches of at least that many queries (largest tuned batch <= nq);
 *   method VSG_METHOD_BF16: how many rows the shortlist path samples for its starting thresholds
 *     (0, 4096 or 16384; 0 = no sample pass).
 * vsg_autotune_table copies a table out (count: capacity in, entries out; choice = kernel or
 * sampled rows; exact_kp: first-pass shortlist of certified entries, 0 for bf16 entries).
 * vsg_autotune_save / _load persist both tables as a small text file ("vsg-tuning 2"; files of
 * version 1 load too, their bf16 lines' third column ignored). */
int vsg_autotune(vsg_index* index, const size_t* batches, size_t count, size_t k, uint32_t method);
/* The same timed on a sample of the caller's queries (nq host rows, stride dim; repeated to fill
 * the largest batch): the certified path's choices depend on how queries sit among the rows. */
int vsg_autotune_with_queries(vsg_index* index, const float* queries, size_t nq, const size_t* batches,
                              size_t count, size_t k, uint32_t method);
int vsg_autotune_table(vsg_index* index, uint32_t method, size_t* count, uint32_t* batch, uint32_t* choice,
                       double* split, uint32_t* exact_kp);
int vsg_autotune_save(vsg_index* index, const char* path);
int vsg_autotune_load(vsg_index* index, const char* path);

/* Certified exact path counters since the index was created: queries searched, queries the
 * shortlist pass could not certify, and queries that ran in the scan kernel (the same queries:
 * there is one shortlist pass). The uncertified count is kept on the device, so
 * this call waits for the index's queued work. */
int vsg_tc_exact_stats(vsg_index* index, uint64_t* queries, uint64_t* second, uint64_t* fallbacks);

/* Tiled path counters since the index was created (new): queries searched by the tiled FP32
 * kernel, and those its certificate could not prove, which the scan kernel answered. Waits for
 * the index's queued work. */
int vsg_tiled_stats(vsg_index* index, uint64_t* queries, uint64_t* fallbacks);

/* Kernels this index has launched since it was created (searches, conversions; not the
 * serving loop's graphs), for benchmarks that report their launch count. */
int vsg_kernel_launches(vsg_index* index, uint64_t* launches);

/* Kernel timing (new; the reference has none). While enabled, every search records CUDA events
 * on its stream around the scan kernel and around the merge kernel. vsg_profile_read waits for
 * the recorded events, returns the summed milliseconds and the number of searches, and clears
 * them. Enabling or disabling also clears. */
int vsg_profile_enable(vsg_index* index, int enable);
int vsg_profile_read(vsg_index* index, double* scan_ms, double* merge_ms, size_t* searches);

/* Serving loop (new; the reference answers one call at a time, python/bindings.cpp:165-186, and its
 * shard worker calls the index per request, distributed/shard_worker.py:26-36). A worker thread
 * batches requests continuously onto the certified tensor-core path: requests that arrive while
 * others run join the next free slot; each slot replays one CUDA graph (query preparation with the
 * certificate's bounds, sample pass, persistent shortlist kernel, finish kernel with the
 * certificate, and the FP32 scan of the queries it could not prove, launched on the device's count
 * of them). Every result equals vsg_search with VSG_METHOD_SKINNY bit for bit and does not depend
 * on the other requests in a batch.
 *   vsg_server_create: max_batch queries per slot (a request may not exceed it), k <= max_k <= 128,
 *     up to `slots` slots, fewer if half of the free HBM cannot hold them (VSG_ERR_NOMEM if none
 *     fits). The index must not be added to while a server uses it.
 *   vsg_server_submit: host queries (nq x dim), optional host allow-bits (ceil(size / 32) words,
 *     shared by the request's queries; NULL = no filter) and host outputs (nq x k) that must stay
 *     valid until vsg_server_wait returns; returns a ticket.
 *   vsg_server_wait: blocks until the request is done (or timeout_s > 0 passes:
 *     VSG_ERR_DEVICE_TIMEOUT); latency_ms = submit to completion. A ticket is waited for once.
 *   vsg_server_stats: micro-batches launched, queries and requests submitted, slots.
 *   vsg_server_uncertified: queries of finished micro-batches that the certificate could not
 *     prove (answered by the FP32 scan in the same graph). */
typedef struct vsg_server vsg_server;
int vsg_server_create(vsg_index* index, size_t max_batch, size_t max_k, size_t slots, vsg_server** out);
int vsg_server_submit(vsg_server* server, const float* queries, size_t nq, size_t k, const uint32_t* mask_words,
                      uint32_t* out_ids, float* out_dists, uint64_t* ticket);
int vsg_server_wait(vsg_server* server, uint64_t ticket, double timeout_s, double* latency_ms);
int vsg_server_stats(vsg_server* server, uint64_t* batches, uint64_t* queries, uint64_t* requests,
                     uint64_t* slots);
int vsg_server_uncertified(vsg_server* server, uint64_t* queries);
void vsg_server_destroy(vsg_server* server);

/* Exact top-k over caller-owned device buffers, for callers that cannot allocate device memory
 * on their search path (a serving thread that must not stall on cudaMalloc / cudaFree, which can
 * synchronise the device; a host framework that owns all device memory through its own pool; a
 * plugin handed only its buffers). No counterpart in the reference: it has no allocation-free form.
 *
 * d_rows: n x dim device floats (row stride dim); d_queries: nq x dim device floats; dim a multiple
 * of 4, both pointers 16-byte aligned. Results go to d_out_ids / d_out_dists (nq x k, device), with
 * the same order and padding as vsg_search (n == 0 fills every result with VSG_NONE / +inf). Work
 * is queued on `stream` (a cudaStream_t, NULL = legacy default stream), and the call waits for it
 * so it can report a device-side failure.
 *
 * It allocates nothing: its scratch (the per-split top-k lists and a status word) is one static
 * 4 MiB device array in the library, which every GPU that loads the library holds until exit.
 * The first call on a device looks up that array's device address (set-up, once per device, with
 * the device current); make that first call before any stream capture. nq x splits x k top-k
 * entries beyond the array (at most 524,256; splits is up to one per SM for small batches) are
 * rejected with VSG_ERR_INVALID. Every call shares the array and it keeps the last call's contents;
 * calls whose device work overlaps (two streams, two threads) race on it and give wrong results. */
int vsg_search_rows_noalloc(const float* d_rows, size_t n, size_t dim, uint32_t metric, const float* d_queries,
                            size_t nq, size_t k, uint32_t* d_out_ids, float* d_out_dists, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* VSG_H_ */
