// Internal definition of the index (host side), shared by the C ABI (index.cu) and the
// serving loop (serve.cu). Not part of the public interface.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/vsg.h"
#include "scan.cuh"
#include "tc.cuh"
#include "tiled.cuh"

namespace vsg_detail {

extern thread_local std::string g_last_error;

struct DeviceTimeout : std::runtime_error {
  using std::runtime_error::runtime_error;
};

#define VSG_CUDA(expr)                                                                    \
  do {                                                                                    \
    cudaError_t err_ = (expr);                                                            \
    if (err_ != cudaSuccess) {                                                            \
      if (err_ == cudaErrorMemoryAllocation) {                                            \
        cudaGetLastError();                                                               \
        throw std::bad_alloc();                                                           \
      }                                                                                   \
      throw std::runtime_error(std::string(#expr) + ": " + cudaGetErrorString(err_));     \
    }                                                                                     \
  } while (0)

inline size_t ceil_div(size_t a, size_t b) { return (a + b - 1) / b; }

// Counts every (re)allocation of a DeviceBuffer or PinnedBuffer in the process: a CUDA graph
// captured at one value holds no pointer that has been freed since while the value is the same.
inline std::atomic<uint64_t> g_alloc_epoch{0};

// Grow-only device buffer, zero-filled when (re)allocated; `keep` bytes of the old
// contents are copied over (gpu_brute_force.cu:37-56).
class DeviceBuffer {
 public:
  DeviceBuffer() = default;
  DeviceBuffer(const DeviceBuffer&) = delete;
  DeviceBuffer& operator=(const DeviceBuffer&) = delete;
  ~DeviceBuffer() {
    if (p_) cudaFree(p_);
  }
  void* get() const { return p_; }
  size_t bytes() const { return n_; }
  void reserve(size_t bytes, size_t keep, cudaStream_t s) {
    if (bytes <= n_) return;
    keep = std::min(keep, n_);  // nothing to keep from a buffer not yet allocated
    void* raw = nullptr;
    VSG_CUDA(cudaMalloc(&raw, bytes));
    cudaError_t e = cudaMemsetAsync(raw, 0, bytes, s);
    if (e == cudaSuccess && keep) e = cudaMemcpyAsync(raw, p_, keep, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      cudaFree(raw);
      VSG_CUDA(e);
    }
    if (p_) cudaFree(p_);
    p_ = raw;
    n_ = bytes;
    g_alloc_epoch.fetch_add(1);
  }

 private:
  void* p_ = nullptr;
  size_t n_ = 0;
};

class PinnedBuffer {
 public:
  PinnedBuffer() = default;
  PinnedBuffer(const PinnedBuffer&) = delete;
  PinnedBuffer& operator=(const PinnedBuffer&) = delete;
  ~PinnedBuffer() {
    if (p_) cudaFreeHost(p_);
  }
  void* get() const { return p_; }
  void reserve(size_t bytes) {
    if (bytes <= n_) return;
    void* raw = nullptr;
    VSG_CUDA(cudaMallocHost(&raw, bytes));
    if (p_) cudaFreeHost(p_);
    p_ = raw;
    n_ = bytes;
    g_alloc_epoch.fetch_add(1);
  }

 private:
  void* p_ = nullptr;
  size_t n_ = 0;
};

inline bool host_is_pinned(const void* p) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeHost;
}

}  // namespace vsg_detail

using namespace vsg_detail;

struct vsg_index {
  size_t dim = 0, dp = 0;
  uint32_t metric = 0;
  int device = 0, sms = 1;
  size_t smem_optin = 0;
  size_t n = 0, cap = 0;
  DeviceBuffer x;       // cap x dp floats
  DeviceBuffer q;       // staged queries
  DeviceBuffer part;    // per-split top-k lists: dists then ids
  DeviceBuffer res;     // [status int | pad to 16][ids nq*k][dists nq*k]
  DeviceBuffer mask;    // staged filter words
  DeviceBuffer counters;  // per query block: CTAs done (the scan kernel's fused merge); kept zero
  // Precision form: BF16 copy of the rows (cap x dp) and FP32 squared norms, built on first use
  // and kept current by later adds; bf16 query staging; merged shortlist candidates.
  DeviceBuffer xb, xnorm, qb, qnorm, sample, thr;
  // method "fp8": e4m3 copy of the rows (cap x dp8 bytes, dp8 = dim rounded up to 16), one FP32
  // scale per row, FP32 squared norms; e4m3 query staging and query scales.
  DeviceBuffer x8, x8scale, x8norm, q8, q8scale;
  DeviceBuffer xbound8;  // the e4m3 rows' rounding bounds (certified path over the e4m3 copy)
  size_t fp8_rows = 0;
  CUtensorMap xmap8{};
  const void* xmap8_base = nullptr;
  size_t xmap8_rows = 0;
  DeviceBuffer cbuf;  // shortlist kernel: per-CTA candidate buffers (dists then ids)
  // Certified exact path (method tc_exact): rounding bounds of the bf16 rows, uncertified
  // queries ([count][ids]), their gathered queries and masks.
  DeviceBuffer xbound, fails, fq, fmask;
  double tc_exact_min_batch = 128;  // method auto, unfiltered: batches from this size
  uint64_t tc_exact_queries = 0;  // queries sent to the certified path
  DeviceBuffer tcstats;            // device tally of its uncertified queries (scan fallbacks)
  uint64_t kernel_launches = 0;    // this index's kernel launches (vsg_kernel_launches)
  DeviceBuffer gthr;  // shortlist kernel: per-query shared thresholds (order keys)
  DeviceBuffer qmargin;  // certified path: per-query margins, then error bounds (launch_prepare_queries)
  DeviceBuffer prep_ticket;  // the FP32 sample's block ticket (PrepSample), zero between launches
  size_t bf16_rows = 0;
  // Tiled path: an upper bound of the rows' norms (a float's bits) over the first xmax_rows rows,
  // the queries it searched and a device tally of those its certificate left to the scan kernel.
  DeviceBuffer xmax, tiledstats;
  size_t xmax_rows = 0;
  uint64_t tiled_queries = 0;
  CUtensorMap xmap{};
  const void* xmap_base = nullptr;
  size_t xmap_rows = 0;
  PinnedBuffer pin_in, pin_out;
  // Blocking host searches (search_host) of one repeated shape replay a CUDA graph of the whole
  // chain: the copy of the queries in (from pin_in), every kernel, the copy of the result block
  // out (to pin_out). One launch call queues everything, so the device never waits for the host
  // between kernels; issuing the chain call by call took ~20 us of host time at batch 1, longer
  // than the kernels before the main pass. The graph is captured on the second search of a shape
  // (the first allocates every buffer it needs) and dropped when what it captured may change:
  // another shape, rows added, a tunable or tuning table set (config_gen), any buffer reallocated
  // (g_alloc_epoch).
  struct HostGraph {
    cudaGraphExec_t exec = nullptr;
    size_t nq = 0, k = 0, n = 0;
    uint32_t method = 0;
    uint64_t gen = 0, epoch = 0;
    uint64_t launches = 0, tc_queries = 0, tiled_q = 0;  // counted per replay
    bool ran = false;     // the shape ran once without the graph
    bool failed = false;  // its capture failed: it runs without a graph
    bool direct = false;  // the kernels read the queries in pin_in (stride dp) themselves
  } hgraph;
  uint64_t config_gen = 0;
  double host_graph_max_batch = 16;  // blocking searches of at most this many queries; 0: none
  // Certified searches of at most this many queries, k <= 16, read the e4m3 copy of the rows
  // (0: none), starting from a sample of cert_fp8_sample_rows rows. Measured at 1M x 384, k = 10:
  // 1.14-1.24x the bf16 copy's QPS at batches 1-16, 0.89-0.93x at 32-64; k = 100 needs ~1,000
  // reranked rows a query and ran at 0.15-0.5x.
  double cert_fp8_max_batch = 16;
  double cert_fp8_sample_rows = 32768;
  // Certified searches over the e4m3 copy of at most this many queries prefetch the rows of their
  // final lists into L2 as the main pass writes them (one bulk prefetch a row), for the finish
  // kernel's rerank of ~1,000 rows a query; 0: none.
  double cert_prefetch_max_batch = 16;
  // Certified path: CTAs per query in the finish kernel when the batch times it fits the SMs
  // (1-16; k = 100 at batches 1-8 on the bf16 copy ran 9-10 % faster with 8 than with 1), and for
  // a search of one query (finish_cluster_one: 16 ran batch 1 at 1M x 384 2.7 % faster than 8,
  // while 16 at batch 8 ran 5 % slower than 8).
  double finish_cluster = 8;
  double finish_cluster_one = 16;
  // 1: on the certified path the graph's kernels read the queries straight from the pinned
  // staging buffer (no copy in; measured 1.5 us less a blocking search at batch 1)
  double host_graph_direct = 1;
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;  // last queued search on this index (any stream)
  std::mutex mu;
  // Filtered searches read only the allowed rows (gather mode) when the allowed fraction is
  // at most this; above it they scan every tile that holds an allowed row (masked full scan).
  // 0.10 from the filtered sweep on GB300 (1M x 384, batch 16): gather wins up to ~8 % allowed,
  // the masked full scan from ~17 %, where it shares each loaded tile among 8 queries.
  double gather_max_fraction = 0.10;
  // method "auto" uses the register-blocked tiled kernel from this batch size up.
  double tiled_min_batch = 48;
  // method "bf16": the tensor-core pass keeps k' = min(448, max(k, oversample x k)) per query.
  double shortlist_oversample = 4;
  // method "bf16": rows sampled for the starting thresholds (0: no sample pass) when nothing
  // else is tuned for the batch size; batches under 8 queries skip it.
  double sample_rows = 16384;
  // method "auto": unfiltered batches below tc_exact_min_batch take the certified path when the
  // index holds at least this many elements (rows x padded dim; 2^27 is ~350K rows at d = 384).
  double tc_exact_min_elements = 134217728.0;
  // method "tc_exact": rows within cert_margin x E of a query's k-th best are kept (E: the
  // certificate's error bound). Any value >= 1 gives exact results; it trades kept rows against
  // queries left uncertified.
  double cert_margin = 1.3;
  // method "tc_exact": the uncertified queries' scan splits the rows as for at most this many
  // queries (0: as for the whole batch).
  double fallback_split_queries = 128;
  // Limit of one kernel wait on another role (seconds); past it the kernel winds down and the
  // search reports VSG_ERR_DEVICE_TIMEOUT. The waits that drain a CTA's own copies keep 2 s.
  double wait_limit_s = 2.0;
  // Test hook ("test_stall_wait"): the next search's scan or shortlist kernels first wait on a
  // barrier that nothing completes, so that wait runs out after wait_limit_s.
  bool stall_next = false;
  uint64_t wait_ns() const { return uint64_t(wait_limit_s * 1e9); }

  // ---- autotuned schedules (vsg_autotune) ----
  // plain: for unfiltered method "auto" searches of at least `batch` queries (largest such entry),
  // which kernel (0 streaming scan, 1 tiled) and a factor on the number of row splits.
  // bf16: rows the sampled-threshold pass scores (0: none).
  struct TuneEntry {
    uint32_t batch = 0, kernel = 0, sample = 16384;
    uint32_t exact_kp = 0;  // exact methods, kernel 2: first-pass shortlist of the certified path (0: default)
    double split = 1.0;
  };
  std::vector<TuneEntry> tune_plain, tune_bf16;
  // Overrides used while the tuner times a candidate (-1 / 0 = not forced).
  int force_kernel = -1, force_sample = -1, force_exact_kp = -1;
  double force_split = 0.0;

  static const TuneEntry* lookup(const std::vector<TuneEntry>& t, size_t nq) {
    const TuneEntry* best = nullptr;
    for (const TuneEntry& e : t)
      if (e.batch <= nq && (!best || e.batch > best->batch)) best = &e;
    return best;
  }
  double split_factor(size_t nq, bool filtered) const {
    if (force_split > 0) return force_split;
    if (filtered) return 1.0;
    const TuneEntry* e = lookup(tune_plain, nq);
    return e ? e->split : 1.0;
  }

  ~vsg_index() {
    if (stream) {
      cudaSetDevice(device);
      cudaStreamSynchronize(stream);
    }
    destroy_timings();
    if (hgraph.exec) cudaGraphExecDestroy(hgraph.exec);
    if (done) cudaEventDestroy(done);
    if (stream) cudaStreamDestroy(stream);
  }

  int* status_word() const { return static_cast<int*>(res.get()); }

  // Allocates the result block (and status word) for nq x k results.
  void reserve_results(size_t nq, size_t k) {
    res.reserve(16 + nq * k * 8, 0, stream);
  }
  uint32_t* res_ids() const { return reinterpret_cast<uint32_t*>(static_cast<char*>(res.get()) + 16); }
  float* res_dists(size_t nq, size_t k) const {
    return reinterpret_cast<float*>(static_cast<char*>(res.get()) + 16 + nq * k * 4);
  }

  // Reads and clears the device status word (the result block must exist).
  void check_status_sync() {
    int st = 0;
    VSG_CUDA(cudaMemcpyAsync(&st, status_word(), sizeof(int), cudaMemcpyDeviceToHost, stream));
    VSG_CUDA(cudaStreamSynchronize(stream));
    if (st != 0) {
      reset_after_failure();
      throw DeviceTimeout("a search kernel's wait ran past its time limit");
    }
  }

  // After a kernel gave up on a wait: clear the status word and the merge counters.
  void reset_after_failure() {
    VSG_CUDA(cudaMemsetAsync(status_word(), 0, sizeof(int), stream));
    if (counters.get()) VSG_CUDA(cudaMemsetAsync(counters.get(), 0, counters.bytes(), stream));
    if (prep_ticket.get()) VSG_CUDA(cudaMemsetAsync(prep_ticket.get(), 0, prep_ticket.bytes(), stream));
    VSG_CUDA(cudaStreamSynchronize(stream));
  }

  struct Plan {
    vsg::ScanShape shape;
    uint32_t stages, nsplit, rows_per_split, nqb;
  };

  // filtered: the scan runs in gather mode; per_query: every query has its own mask.
  // split_nq (unfiltered only): when nonzero and below nq, the row range is split as for that
  // many queries, with factor 1, while the launch still covers all nq.
  Plan plan(size_t nq, size_t k, bool filtered = false, bool per_query = false, size_t split_nq = 0) const {
    Plan p{};
    p.shape.l2 = metric == VSG_METRIC_L2;
    p.shape.qb = 1;  // next power of two >= nq, at most 8; one query per CTA for per-query masks,
                     // so a CTA never loads rows only other queries may return
    while (!per_query && size_t(p.shape.qb) < nq && p.shape.qb < 8) p.shape.qb *= 2;
    const size_t budget = smem_optin - 1024;  // headroom for the kernel's static shared memory
    p.stages = 0;
    for (int rw : {4, 2, 1}) {
      p.shape.rw = rw;
      const size_t fixed = vsg::scan_smem_bytes(p.shape, uint32_t(dp), uint32_t(k), 0);
      const size_t tile = size_t(vsg::kScanWarps) * rw * dp * sizeof(float);
      if (fixed + 2 * tile > budget) continue;
      p.stages = uint32_t(std::min<size_t>(4, (budget - fixed) / tile));
      break;
    }
    if (p.stages < 2)
      throw std::invalid_argument("dim " + std::to_string(dim) + " with k " + std::to_string(k) +
                                  " does not fit the scan kernel's shared memory");
    p.nqb = uint32_t(ceil_div(nq, size_t(p.shape.qb)));
    size_t want;
    if (!filtered && split_nq && nq > split_nq) {
      const size_t blocks = ceil_div(split_nq, size_t(p.shape.qb));
      want = std::max<size_t>(1, size_t(sms) / blocks);
      want = std::min(want, std::max<size_t>(1, ceil_div(n, 256)));
    } else if (!filtered) {
      want = std::max<size_t>(1, size_t(double(std::max<size_t>(1, size_t(sms) / p.nqb)) * split_factor(nq, false)));
      want = std::min(want, std::max<size_t>(1, ceil_div(n, 256)));  // >= 256 rows per split
    } else {
      // Allowed rows are spread unevenly over queries and row ranges: cap a split at 32K rows
      // and aim for two CTAs per SM, with at least 1024 rows per split.
      want = std::max(ceil_div(n, 32768), ceil_div(2 * size_t(sms), p.nqb));
      want = std::max<size_t>(1, std::min(want, ceil_div(n, 1024)));
    }
    p.rows_per_split = vsg::split_rows(ceil_div(ceil_div(n, want), 32) * 32, 32);
    p.nsplit = uint32_t(ceil_div(n, p.rows_per_split));
    return p;
  }

  // Queues the scan + merge for device queries (stride ldq floats) on `s`. Results go to
  // out_ids / out_dists (device). Caller holds mu and has validated k, nq, n > 0.
  // Splits of a row range for `blocks` CTA columns: at least `min_splits`, rows per split a
  // multiple of `align`, and a total CTA count that fills whole waves of one CTA per SM.
  void choose_splits(size_t blocks, size_t align, size_t min_rows, uint32_t* rows_per_split, uint32_t* nsplit,
                     double factor = 1.0, size_t slots = 0) const {
    // slots: work items that run at once (one per SM unless given)
    if (slots == 0) slots = size_t(sms);
    const size_t s0 = std::max<size_t>(1, size_t(double(std::max<size_t>(1, slots / blocks)) * factor));
    const size_t smax = std::max<size_t>(1, std::min(ceil_div(n, min_rows), 4 * s0));
    size_t best = std::min(s0, smax);
    double best_eff = 0;
    for (size_t sp = std::min(s0, smax); sp <= smax; ++sp) {
      const size_t ctas = blocks * sp;
      const double eff = double(ctas) / double(ceil_div(ctas, slots) * slots);
      if (eff > best_eff + 1e-9) {
        best_eff = eff;
        best = sp;
      }
    }
    const size_t rps = vsg::split_rows(ceil_div(ceil_div(n, best), align) * align, align);
    *rows_per_split = uint32_t(rps);
    *nsplit = uint32_t(ceil_div(n, rps));
  }

  // Raises the rows' norm bound over rows added since the last call.
  void ensure_xmax() {
    if (xmax_rows == n && xmax.get()) return;
    xmax.reserve(16, 0, stream);
    VSG_CUDA(vsg::launch_row_norm_max(static_cast<const float*>(x.get()) + xmax_rows * dp, n - xmax_rows,
                                      uint32_t(dp), static_cast<uint32_t*>(xmax.get()), stream));
    ++kernel_launches;
    xmax_rows = n;
  }

  // The tiled FP32 kernel as a shortlist with a certificate, like the tensor-core path: the
  // kernel keeps each split's best kp = tiled_list_size(k) rows by its own FP32 arithmetic and
  // publishes every full list's last entry; the finish kernel reranks the rows within the margin
  // of each query's k-th best with the scan kernel's arithmetic and proves that no row left out
  // can enter the top k (E: launch_prepare_fp32_queries); unproven queries run in the scan kernel
  // (launched on the device's count of them, as in enqueue_tc_exact). Results equal method skinny
  // bit for bit.
  void enqueue_tiled(const float* dq, size_t ldq, size_t nq, size_t k, uint32_t* out_ids, float* out_dists,
                     cudaStream_t s) {
    const uint32_t kp = vsg::tiled_list_size(uint32_t(k));
    const size_t bm = size_t(vsg::tiled_block_queries(kp, uint32_t(nq)));
    const size_t nqb = ceil_div(nq, bm);
    vsg::TiledArgs a{};
    choose_splits(nqb, 128, 1024, &a.rows_per_split, &a.nsplit, split_factor(nq, false));
    const size_t parts = nq * a.nsplit * kp;
    part.reserve(parts * 8 + nq * a.nsplit * 4, 0, stream);  // lists, then their lengths
    ensure_xmax();
    fails.reserve((nq + 1) * sizeof(uint32_t), 0, stream);
    tiledstats.reserve(sizeof(unsigned long long), 0, stream);
    gthr.reserve(nq * sizeof(uint32_t), 0, stream);
    qmargin.reserve(2 * nq * sizeof(float), 0, stream);  // margins, then the bounds E
    fq.reserve(nq * dp * sizeof(float), 0, stream);
    float* mgn = static_cast<float*>(qmargin.get());
    uint32_t* d_fail = static_cast<uint32_t*>(fails.get());
    VSG_CUDA(vsg::launch_prepare_fp32_queries(dq, uint32_t(ldq), uint32_t(nq), uint32_t(dp), metric == VSG_METRIC_L2,
                                              static_cast<const uint32_t*>(xmax.get()), float(cert_margin),
                                              static_cast<uint32_t*>(gthr.get()), mgn, mgn + nq, d_fail, s));
    ++kernel_launches;
    a.x = static_cast<const float*>(x.get());
    a.q = dq;
    a.ldq = uint32_t(ldq);
    a.part_d = static_cast<float*>(part.get());
    a.part_i = reinterpret_cast<uint32_t*>(static_cast<char*>(part.get()) + parts * 4);
    a.part_n = reinterpret_cast<uint32_t*>(static_cast<char*>(part.get()) + parts * 8);
    a.gthr = static_cast<uint32_t*>(gthr.get());
    a.n = uint32_t(n);
    a.dp = uint32_t(dp);
    a.nq = uint32_t(nq);
    a.kp = kp;
    Timing* tm = profiling ? next_timing() : nullptr;
    if (tm) VSG_CUDA(cudaEventRecord(tm->ev[0], s));
    VSG_CUDA(vsg::launch_tiled(a, metric == VSG_METRIC_L2, dim3(unsigned(nqb), a.nsplit), s));
    ++kernel_launches;
    if (tm) VSG_CUDA(cudaEventRecord(tm->ev[1], s));
    vsg::FinishArgs fa{};
    fa.part_d = a.part_d;
    fa.part_i = a.part_i;
    fa.part_n = a.part_n;
    fa.nq = uint32_t(nq);
    fa.nsplit = a.nsplit;
    fa.kp = kp;
    fa.k = uint32_t(k);
    fa.margin = mgn;  // the cut keeps the rows within the margin of the k-th best
    fa.x = a.x;
    fa.n = uint32_t(n);
    fa.q = dq;
    fa.dp = uint32_t(dp);
    fa.ldq = uint32_t(ldq);
    fa.l2 = metric == VSG_METRIC_L2 ? 1u : 0u;
    fa.out_d = out_dists;
    fa.out_i = out_ids;
    fa.stage_cap = uint32_t(std::min<size_t>(vsg::kFinishStageMax, size_t(a.nsplit) * kp));
    fa.sorted_lists = 1;  // the tiled kernel keeps every list sorted
    fa.gthr = a.gthr;
    fa.err = mgn + nq;
    fa.fail_count = d_fail;
    fa.fail_list = d_fail + 1;
    fa.fq = static_cast<float*>(fq.get());
    fa.tally = static_cast<unsigned long long*>(tiledstats.get());
    const bool pdl = !profiling;
    VSG_CUDA(vsg::launch_finish(fa, uint32_t(nq), s, pdl));
    ++kernel_launches;
    if (tm) VSG_CUDA(cudaEventRecord(tm->ev[2], s));
    tiled_queries += nq;
    const bool prof = profiling;
    profiling = false;
    try {
      enqueue(static_cast<const float*>(fq.get()), dp, nq, k, nullptr, false, 0, false, out_ids, out_dists, s,
              VSG_METHOD_SKINNY, -1.0, d_fail, d_fail + 1, pdl);
    } catch (...) {
      profiling = prof;
      throw;
    }
    profiling = prof;
  }

  // Queries of the tiled path that the scan kernel answered (waits for the index's work).
  uint64_t tiled_stats_sync() {
    if (!tiledstats.get()) return 0;
    unsigned long long v = 0;
    VSG_CUDA(cudaStreamWaitEvent(stream, done, 0));
    VSG_CUDA(cudaMemcpyAsync(&v, tiledstats.get(), sizeof(v), cudaMemcpyDeviceToHost, stream));
    VSG_CUDA(cudaStreamSynchronize(stream));
    return uint64_t(v);
  }

  // Brings the BF16 copy (tile-major, see vsg::tc_tiled_bytes) and the norms up to the current
  // rows (after a grow they are rebuilt).
  void ensure_bf16() {
    const size_t need = vsg::tc_tiled_bytes(cap, uint32_t(dp), false);
    if (bf16_rows == n && xb.bytes() >= need) return;
    const size_t keep = xb.bytes() >= need ? bf16_rows : 0;
    xb.reserve(need, vsg::tc_tiled_bytes(keep, uint32_t(dp), false), stream);
    xnorm.reserve(cap * sizeof(float), keep * sizeof(float), stream);
    xbound.reserve(16, 0, stream);
    if (keep == 0) VSG_CUDA(cudaMemsetAsync(xbound.get(), 0, 16, stream));  // every row is converted again
    VSG_CUDA(vsg::launch_to_bf16(static_cast<const float*>(x.get()) + keep * dp, dp, n - keep, uint32_t(dp),
                                 uint32_t(dp), xb.get(), static_cast<float*>(xnorm.get()) + keep, stream,
                                 static_cast<float*>(xbound.get()), keep));
    ++kernel_launches;
    VSG_CUDA(cudaStreamSynchronize(stream));
    bf16_rows = n;
  }

  size_t dp8() const { return (dim + 15) / 16 * 16; }

  // The e4m3 copy (tile-major), its row scales and norms, and its tensor map.
  void ensure_fp8() {
    const uint32_t d8 = uint32_t(dp8());
    const size_t need = vsg::tc_tiled_bytes(cap, d8, true);
    if (fp8_rows == n && x8.bytes() >= need) return;
    const size_t keep = x8.bytes() >= need ? fp8_rows : 0;
    x8.reserve(need, vsg::tc_tiled_bytes(keep, d8, true), stream);
    x8scale.reserve(cap * sizeof(float), keep * sizeof(float), stream);
    x8norm.reserve(cap * sizeof(float), keep * sizeof(float), stream);
    xbound8.reserve(16, 0, stream);
    if (keep == 0) VSG_CUDA(cudaMemsetAsync(xbound8.get(), 0, 16, stream));  // every row is converted again
    VSG_CUDA(vsg::launch_to_fp8(static_cast<const float*>(x.get()) + keep * dp, dp, n - keep, uint32_t(dim), d8,
                                x8.get(), static_cast<float*>(x8scale.get()) + keep,
                                static_cast<float*>(x8norm.get()) + keep, stream, keep,
                                static_cast<float*>(xbound8.get())));
    ++kernel_launches;
    VSG_CUDA(cudaStreamSynchronize(stream));
    fp8_rows = n;
    if (xmap8_base != x8.get() || xmap8_rows != n) {
      VSG_CUDA(vsg::tc_encode_tiled_map(&xmap8, x8.get(), n, d8, uint32_t(vsg::kTcRows), true));
      xmap8_base = x8.get();
      xmap8_rows = n;
    }
  }

  // Tensor map of the bf16 rows (re-encoded after a grow or an add).
  void ensure_xmap() {
    if (xmap_base != xb.get() || xmap_rows != n) {
      VSG_CUDA(vsg::tc_encode_tiled_map(&xmap, xb.get(), n, uint32_t(dp), uint32_t(vsg::kTcRows), false));
      xmap_base = xb.get();
      xmap_rows = n;
    }
  }

  // Certified exact path: the list keeps the rows within each query's margin of its k-th best,
  // up to k' entries. For k <= 16, k' = 120: the rows within the margin (about 50-120 for
  // k = 10 on 1M clustered unit rows) fit, and the 256-entry candidate buffers sort fast; larger
  // k take the widest list (448; about 260-420 rows lie within the margin of the 100th-128th
  // best there). A table entry may still name another k'.
  static uint32_t exact_shortlist_size(size_t k) { return k <= 16 ? 120u : uint32_t(vsg::kTcMaxShortlist); }

  uint32_t shortlist_size(size_t k) const {
    const double want = std::max<double>(double(k), shortlist_oversample * double(k));
    return uint32_t(std::min<double>(double(vsg::kTcMaxShortlist), std::ceil(want)));
  }

  // The shortlist path over the bf16 copy (f8 = false) or the e4m3 copy with row scales (f8).
  void enqueue_bf16(const float* dq, size_t ldq, size_t nq, size_t k, uint32_t* out_ids, float* out_dists,
                    cudaStream_t s, bool certify = false, uint32_t kp_force = 0, bool f8 = false,
                    const uint32_t* dmask = nullptr, size_t mask_ld = 0) {
    const uint32_t kp = kp_force ? kp_force : certify ? exact_shortlist_size(k) : shortlist_size(k);
    // The operand copy, its norms (and rounding bounds or scales) cover every row before any
    // kernel reads them.
    if (f8) {
      ensure_fp8();
      if (!x8.get() || !x8scale.get() || !x8norm.get() || !xbound8.get() || fp8_rows != n)
        throw std::runtime_error("the e4m3 copy of the rows is missing");
    } else {
      ensure_bf16();
      if (!xb.get() || !xnorm.get() || !xbound.get() || bf16_rows != n)
        throw std::runtime_error("the bf16 copy of the rows is missing");
    }
    const size_t dpo = f8 ? dp8() : dp;  // padded elements per row of the operand copies
    const uint32_t nkc = vsg::tc_chunks(uint32_t(dpo), f8);
    uint32_t resident = 0;
    const uint32_t stages = vsg::tc_pick_stages(nkc, smem_optin - 1024, &resident, metric == VSG_METRIC_L2, f8);
    if (stages < 2) throw std::invalid_argument("rows do not fit the tensor-core kernel's shared memory");
    // Queries to bf16 / e4m3 (rows past nq are zero-filled by the copy engine) and their norms.
    qnorm.reserve(nq * sizeof(float), 0, stream);
    CUtensorMap qmap;
    // bf16 queries (and e4m3 queries on the certified path): one launch (the queries and their
    // norms, shared thresholds reset, and on the certified path the bounds E, the margins and the
    // zeroed uncertified count), made below once it is known whether it also computes the sample
    // (small batches).
    float* mgn = nullptr;
    auto launch_prep = [&](const vsg::PrepSample* smp) {
      VSG_CUDA(vsg::launch_prepare_queries(smp, dq, uint32_t(ldq), uint32_t(nq), uint32_t(dim), uint32_t(dp),
                                           f8 ? q8.get() : qb.get(), static_cast<float*>(qnorm.get()),
                                           static_cast<uint32_t*>(gthr.get()),
                                           static_cast<const float*>(f8 ? xbound8.get() : xbound.get()),
                                           metric == VSG_METRIC_L2, float(cert_margin), mgn, mgn ? mgn + nq : nullptr,
                                           certify ? static_cast<uint32_t*>(fails.get()) : nullptr, s,
                                           f8 ? static_cast<float*>(q8scale.get()) : nullptr, uint32_t(dpo)));
      ++kernel_launches;
    };
    bool prep_done = f8 && !certify;
    if (f8 && certify) {  // e4m3 queries, their bounds and margins in the query preparation
      q8.reserve(nq * dpo, 0, stream);
      q8scale.reserve(nq * sizeof(float), 0, stream);
      gthr.reserve(nq * sizeof(uint32_t), 0, stream);
      qmargin.reserve(2 * nq * sizeof(float), 0, stream);  // margins, then the bounds E
      mgn = static_cast<float*>(qmargin.get());
      VSG_CUDA(vsg::tc_encode_map(&qmap, q8.get(), nq, dpo, uint32_t(vsg::kTcQueries), true));
    } else if (f8) {
      q8.reserve(nq * dpo, 0, stream);
      q8scale.reserve(nq * sizeof(float), 0, stream);
      VSG_CUDA(vsg::launch_to_fp8(dq, ldq, nq, uint32_t(dim), uint32_t(dpo), q8.get(),
                                  static_cast<float*>(q8scale.get()), static_cast<float*>(qnorm.get()), s));
      ++kernel_launches;
      VSG_CUDA(vsg::tc_encode_map(&qmap, q8.get(), nq, dpo, uint32_t(vsg::kTcQueries), true));
    } else {
      qb.reserve(nq * dp * 2, 0, stream);
      gthr.reserve(nq * sizeof(uint32_t), 0, stream);
      if (certify) {
        qmargin.reserve(2 * nq * sizeof(float), 0, stream);  // margins, then the bounds E
        mgn = static_cast<float*>(qmargin.get());
      }
      VSG_CUDA(vsg::tc_encode_map(&qmap, qb.get(), nq, dp, uint32_t(vsg::kTcQueries)));
      ensure_xmap();
    }
    const size_t nqb = ceil_div(nq, size_t(vsg::kTcQueries));
    const TuneEntry* te = lookup(tune_bf16, nq);
    // Items are (query block, split), taken round-robin by one CTA per SM.
    const size_t slots = size_t(sms);
    vsg::TcArgs a{};
    choose_splits(nqb, vsg::kTcRows, 1024, &a.rows_per_split, &a.nsplit, 1.0, slots);
    const size_t groups = vsg::tc_groups(kp);  // lists per (query, split)
    const size_t parts = nq * a.nsplit * groups * kp;
    part.reserve(parts * 8 + nq * a.nsplit * groups * 4, 0, stream);  // lists, then their lengths
    // Candidate buffers: one set per epilogue group of each CTA.
    const unsigned grid = unsigned(std::min<size_t>(nqb * a.nsplit, slots));
    const CUtensorMap& rowmap = f8 ? xmap8 : xmap;
    const size_t cbuf_entries = size_t(grid) * groups * vsg::kTcQueries * vsg::tc_buffer_capacity(kp);
    cbuf.reserve(cbuf_entries * 8, 0, stream);
    if (f8 && !certify) {  // (the query preparation resets them)
      gthr.reserve(nq * sizeof(uint32_t), 0, stream);
      VSG_CUDA(cudaMemsetAsync(gthr.get(), 0xFF, nq * sizeof(uint32_t), s));
    }
    // Certified path: each query keeps only the rows within its margin of its k-th best (k' caps
    // the list), which is all the certificate needs.
    const bool margins = certify;
    if (margins) {
      a.margin = static_cast<const float*>(qmargin.get());
      a.kk = uint32_t(k);
    }
    a.n = uint32_t(n);
    a.dp = uint32_t(dpo);
    a.nq = uint32_t(nq);
    a.nqb = uint32_t(nqb);
    a.fp8 = f8 ? 1u : 0u;
    a.mask = dmask;  // mask_ld = 0: one mask for every query
    a.mask_ld = uint32_t(mask_ld);
    a.xscale = f8 ? static_cast<const float*>(x8scale.get()) : nullptr;
    a.qscale = f8 ? static_cast<const float*>(q8scale.get()) : nullptr;
    a.kp = kp;
    a.stages = stages;
    a.resident = resident;
    a.cbuf_d = static_cast<float*>(cbuf.get());
    a.cbuf_i = reinterpret_cast<uint32_t*>(static_cast<char*>(cbuf.get()) + cbuf_entries * 4);
    a.gthr = static_cast<uint32_t*>(gthr.get());
    a.l2 = metric == VSG_METRIC_L2 ? 1u : 0u;
    a.xnorm = static_cast<const float*>(f8 ? x8norm.get() : xnorm.get());
    a.qnorm = static_cast<const float*>(qnorm.get());
    a.part_d = static_cast<float*>(part.get());
    a.part_i = reinterpret_cast<uint32_t*>(static_cast<char*>(part.get()) + parts * 4);
    a.part_n = reinterpret_cast<uint32_t*>(static_cast<char*>(part.get()) + parts * 8);
    a.status = status_word();
    a.wait_ns = wait_ns();
    a.stall = stall_next ? 1u : 0u;
    if (certify && f8 && double(nq) <= cert_prefetch_max_batch) {
      a.xf = static_cast<const float*>(x.get());  // (dp: a multiple of 4)
      a.xf_ld = uint32_t(dp);
    }
    Timing* tm = profiling ? next_timing() : nullptr;
    // Batches first score a sample of rows (whole tiles at the head of every split; 16K rows for
    // 8+ queries, 4K below, unless tuned) and start each query at the k'-th best sampled distance, so the
    // main pass keeps only rows that can still make the shortlist.
    const uint32_t tiles_per_split = uint32_t(ceil_div(a.rows_per_split, size_t(vsg::kTcRows)));
    // (batches under 8 queries, and batches of up to 64 with k <= 16, sample at most 4K rows;
    // without a sample every row is a candidate until the first compactions, which made batch 1 at
    // 1M x 384 21 % slower. Measured at 1M x 384 on the certified path: k = 10 ran 2.6-4 % faster
    // with 4K than with 16K sampled rows at batches 8-64, but 6 % slower at 1024, where the
    // epilogue sets the pace and a looser start costs appends; k = 100 up to 1.9x slower with 4K)
    // The certified path over the e4m3 copy samples cert_fp8_sample_rows: its margin is ~16x the
    // bf16 copy's, and a start from 4K rows (about 4 rows of a query's 1,000-row cluster at
    // 1M x 384) kept every list full of rows far above the cluster for the whole pass.
    const bool small_sample = nq < 8 || (k <= 16 && nq <= 64);
    // (the tuning table's sample sizes are timed on the bf16 copy: not for the e4m3 copy, whose
    // margin needs the larger start; a 16K sample picked for batch 16 ran it 30 % slower)
    const size_t srows = force_sample >= 0 ? size_t(force_sample)
                         : f8 && certify ? size_t(cert_fp8_sample_rows)
                         : te ? size_t(te->sample)
                         : small_sample ? std::min<size_t>(size_t(sample_rows), 4096) : size_t(sample_rows);
    // After the query preparation the path's kernels run as a chain of programmatic dependent
    // launches (each may start while the one before it finishes); not while profiling, whose
    // events time the main pass on its own.
    const bool pdl = !(f8 && !certify) && !profiling;
    if (srows > 0 && tiles_per_split > 1) {
      vsg::TcArgs sa = a;
      uint32_t st = uint32_t(std::min<size_t>(tiles_per_split, ceil_div(srows, size_t(a.nsplit) * vsg::kTcRows)));
      unsigned sgrid = grid;
      if (size_t(a.nsplit) * vsg::kTcRows > srows) {
        // One tile per split would sample more rows than asked for (many splits, a small batch):
        // sample the first tile of each of ceil(srows / 256) ranges spread over the rows instead.
        const size_t tiles = ceil_div(size_t(n), size_t(vsg::kTcRows));
        const size_t rps =
            vsg::split_rows(ceil_div(tiles, ceil_div(srows, size_t(vsg::kTcRows))) * vsg::kTcRows, vsg::kTcRows);
        sa.rows_per_split = uint32_t(rps);
        sa.nsplit = uint32_t(ceil_div(size_t(n), rps));
        st = 1;
        sgrid = unsigned(std::min<size_t>(nqb * sa.nsplit, slots));
      }
      // (with margins and k <= 32, the sample pass writes each 32 rows' smallest distance only:
      // the select then reads 32x fewer values; its bound is the k-th smallest of those minima)
      sa.dump_min = margins && k <= 32 ? 1u : 0u;
      const size_t per_query = size_t(sa.nsplit) * st * (sa.dump_min ? vsg::kTcRows / 32 : vsg::kTcRows);
      sample.reserve(nq * size_t(sa.nsplit) * st * vsg::kTcRows * sizeof(float), 0, stream);
      thr.reserve(nq * sizeof(float), 0, stream);
      sa.dump = static_cast<float*>(sample.get());
      sa.sample_tiles = st;
      sa.gthr = nullptr;
      // Certified path, up to 4 queries with ranges sampled: the query preparation scores the
      // sample in FP32 and selects the thresholds itself (two launches less before the main pass).
      // A k-th distance in FP32 plus the margin m = f E (f > 1) still lets at least k sampled rows
      // through (each approximate distance lies within E of the FP32 one), and every bound the
      // certificate takes stays a bound.
      const bool fp32_sample = margins && !prep_done && st == 1 && nq <= 4 && nq <= vsg::kPrepSampleQueries &&
                               dp <= vsg::kPrepSampleDim && size_t(sa.nsplit) * vsg::kTcRows <= vsg::kPrepSampleRows;
      if (fp32_sample) {
        prep_ticket.reserve(sizeof(uint32_t), 0, stream);  // zero-filled; each launch leaves it zero
        vsg::PrepSample smp{static_cast<const float*>(x.get()), uint32_t(n), sa.rows_per_split, sa.nsplit,
                            sa.dump, static_cast<float*>(thr.get()), uint32_t(k),
                            static_cast<uint32_t*>(prep_ticket.get())};
        launch_prep(&smp);
        prep_done = true;
      } else {
        if (!prep_done) launch_prep(nullptr);
        prep_done = true;
        VSG_CUDA(vsg::launch_tc_shortlist(qmap, rowmap, sa, sgrid, s, pdl));
        ++kernel_launches;
        // (with margins: the k-th best sampled distance plus the margin)
        VSG_CUDA(vsg::launch_sample_select(sa.dump, uint32_t(per_query), uint32_t(nq), nullptr,
                                           margins ? uint32_t(k) : kp, static_cast<float*>(thr.get()), s,
                                           a.margin, pdl));
        ++kernel_launches;
      }
      a.thr_init = static_cast<const float*>(thr.get());
    }
    if (!prep_done) launch_prep(nullptr);
    if (tm) VSG_CUDA(cudaEventRecord(tm->ev[0], s));  // the profile times the main pass alone
    VSG_CUDA(vsg::launch_tc_shortlist(qmap, rowmap, a, grid, s, pdl));
    ++kernel_launches;
    if (tm) VSG_CUDA(cudaEventRecord(tm->ev[1], s));
    // Cut, rerank and (certified path) certificate in one launch.
    vsg::FinishArgs fa{};
    fa.part_d = a.part_d;
    fa.part_i = a.part_i;
    fa.part_n = a.part_n;
    fa.nq = uint32_t(nq);
    fa.nsplit = a.nsplit;
    fa.kp = kp;
    fa.k = uint32_t(k);
    fa.margin = margins ? a.margin : nullptr;  // the cut keeps the rows within the margin
    fa.x = static_cast<const float*>(x.get());
    fa.n = uint32_t(n);
    fa.q = dq;
    fa.dp = uint32_t(dp);
    fa.ldq = uint32_t(ldq);
    fa.l2 = a.l2;
    fa.out_d = out_dists;
    fa.out_i = out_ids;
    fa.status = status_word();
    fa.lists_per_split = uint32_t(groups);
    fa.sorted_lists = nq <= vsg::kSortedListQueries ? 1u : 0u;
    // Small batches rerank over a cluster of CTAs per query (the e4m3 copy's wider margin keeps
    // ~1,000 rows to rerank at 1M x 384, ~20 us on one SM).
    const size_t fc = size_t(nq == 1 ? finish_cluster_one : finish_cluster);
    fa.cluster = certify && double(nq * fc) <= double(sms) ? uint32_t(fc) : 1u;
    fa.rows_in_l2 = a.xf ? 1u : 0u;
    fa.stage_cap = uint32_t(std::min<size_t>(vsg::kFinishStageMax, size_t(a.nsplit) * groups * kp));
    if (certify) {
      fa.thr_init = a.thr_init;
      fa.gthr = a.gthr;
      fa.err = static_cast<const float*>(qmargin.get()) + nq;
      fa.fail_count = static_cast<uint32_t*>(fails.get());
      fa.fail_list = fa.fail_count + 1;
      // each uncertified query's FP32 row (and per-query mask) goes to its fallback slot
      fq.reserve(nq * dp * sizeof(float), 0, stream);
      fa.fq = static_cast<float*>(fq.get());
      if (dmask && mask_ld) {
        fmask.reserve(nq * mask_ld * sizeof(uint32_t), 0, stream);
        fa.qmask = dmask;
        fa.fmask = static_cast<uint32_t*>(fmask.get());
        fa.mask_ld = uint32_t(mask_ld);
      }
      tcstats.reserve(sizeof(unsigned long long), 0, stream);
      fa.tally = static_cast<unsigned long long*>(tcstats.get());
    }
    VSG_CUDA(vsg::launch_finish(fa, uint32_t(nq), s, pdl));
    ++kernel_launches;
    if (tm) VSG_CUDA(cudaEventRecord(tm->ev[2], s));
  }

  // Exact top-k through the shortlist. Queries whose result the finish kernel cannot certify (see
  // vsg::FinishArgs) run in the streaming scan kernel, so results equal method skinny bit for bit.
  // Nothing waits on the host: the finish kernel leaves the uncertified queries' count, indices,
  // FP32 rows (and per-query masks) on the device, and one scan launch sized for all nq queries,
  // its blocks past that count returning at once, writes their results over theirs (its fused
  // merge maps slot j to query fail_list[j]; row splits: plan()). A tally of uncertified queries
  // stays on the device (tc_stats_sync reads it).
  void enqueue_tc_exact(const float* dq, size_t ldq, size_t nq, size_t k, uint32_t* out_ids, float* out_dists,
                        cudaStream_t s, const uint32_t* dmask = nullptr, size_t mask_ld = 0) {
    fails.reserve((nq + 1) * sizeof(uint32_t), 0, stream);
    tcstats.reserve(sizeof(unsigned long long), 0, stream);
    // Shortlist cap: a tuned entry may name one; else exact_shortlist_size(k).
    const TuneEntry* te = dmask ? nullptr : lookup(tune_plain, nq);
    uint32_t kp1 = force_exact_kp > 0 ? uint32_t(force_exact_kp) : te && te->kernel == 2 ? te->exact_kp : 0u;
    kp1 = kp1 ? std::max<uint32_t>(std::min<uint32_t>(kp1, uint32_t(vsg::kTcMaxShortlist)), uint32_t(k))
              : exact_shortlist_size(k);
    // zeroes the count; the finish kernel fills the fallback's rows and masks. Batches of up to
    // cert_fp8_max_batch queries read the e4m3 copy (half the bytes; a wider margin).
    const bool f8 = double(nq) <= cert_fp8_max_batch && k <= 16 && dp8() <= vsg::kPrepSampleDim;  // (the query preparation's width)
    enqueue_bf16(dq, ldq, nq, k, out_ids, out_dists, s, true, kp1, f8, dmask, mask_ld);
    tc_exact_queries += nq;
    const uint32_t* d_count = static_cast<const uint32_t*>(fails.get());
    const uint32_t* d_list = d_count + 1;
    // Per-query masks follow their queries (a shared mask stays as it is).
    const uint32_t* m1 = dmask && mask_ld ? static_cast<const uint32_t*>(fmask.get()) : dmask;
    // The scan kernel's masked full scan (its gather mode gives the same results); not profiled.
    const bool prof = profiling;
    profiling = false;
    try {
      enqueue(static_cast<const float*>(fq.get()), dp, nq, k, m1, dmask && mask_ld, mask_ld, false, out_ids,
              out_dists, s, VSG_METHOD_SKINNY, -1.0, d_count, d_list, !prof);
    } catch (...) {
      profiling = prof;
      throw;
    }
    profiling = prof;
  }

  // Queries of the certified path that the scan kernel answered (waits for the index's work).
  uint64_t tc_stats_sync() {
    if (!tcstats.get()) return 0;
    unsigned long long v = 0;
    VSG_CUDA(cudaStreamWaitEvent(stream, done, 0));
    VSG_CUDA(cudaMemcpyAsync(&v, tcstats.get(), sizeof(v), cudaMemcpyDeviceToHost, stream));
    VSG_CUDA(cudaStreamSynchronize(stream));
    return uint64_t(v);
  }

  bool use_tc_exact(uint32_t method, size_t nq, size_t k, const uint32_t* dmask, bool gather,
                    double allowed = -1.0) const {
    if (k > size_t(vsg::kTcMaxShortlist) || k > VSG_MAX_K || n == 0) return false;
    if (method == VSG_METHOD_TC_EXACT) return true;
    if (method != VSG_METHOD_AUTO) return false;
    // Filtered: the gather scan reads only the allowed rows of each query, about 3.3 us per query
    // plus 0.375 ns per (query, allowed row) at d = 384, while the shortlist pass costs about the
    // same at any selectivity (0.2 ms at 16 queries over 1M rows). So with the largest allowed
    // fraction f known, the certified path takes batches of 8+ where nq f >= 0.35, and every
    // batch from half the threshold (measured at 1M x 384). Without f (device masks): from the
    // threshold when the scan would not gather, from twice it otherwise.
    if (dmask) {
      if (k > 32) return false;
      if (allowed >= 0.0)
        return nq >= 8 && (double(nq) >= 0.5 * tc_exact_min_batch || (!gather) || double(nq) * allowed >= 0.35);
      return (!gather || double(nq) >= 2 * tc_exact_min_batch) && double(nq) >= tc_exact_min_batch;
    }
    if (force_kernel >= 0) return force_kernel == 2;
    if (const TuneEntry* e = lookup(tune_plain, nq)) return e->kernel == 2;
    // Large batches amortise the shortlist path's fixed costs at any index size; smaller ones,
    // down to one query, when the index is large enough that reading half the bytes (the bf16
    // copy instead of the FP32 rows) saves more than those costs (about 30 us).
    return double(nq) >= tc_exact_min_batch || double(n) * double(dp) >= tc_exact_min_elements;
  }

  bool use_tiled(uint32_t method, size_t nq, const uint32_t* dmask) const {
    if (dmask) return false;  // filters run in the scan kernel
    if (method == VSG_METHOD_TILED) return true;
    if (method != VSG_METHOD_AUTO) return false;
    if (force_kernel >= 0) return force_kernel == 1;
    if (const TuneEntry* e = lookup(tune_plain, nq)) return e->kernel == 1;
    return double(nq) >= tiled_min_batch;
  }

  // Times each candidate schedule for every batch size and keeps the fastest (CUDA events, the
  // mean over 3 different batches after a warm-up). family: VSG_METHOD_AUTO for the
  // FP32 kernels, VSG_METHOD_BF16 for the shortlist path. Caller holds mu.
  // sample / nsample: host queries (stride dim) to time with, repeated to fill the largest batch;
  // nullptr: queries near the index's rows.
  void autotune(const size_t* batches, size_t count, size_t k, uint32_t family, const float* sample = nullptr,
                size_t nsample = 0) {
    if (n == 0) throw std::invalid_argument("the index is empty");
    if (k == 0 || k > VSG_MAX_K) throw std::invalid_argument("k must be in [1, 128]");
    if (family == VSG_METHOD_BF16) {
      if (k > size_t(vsg::kTcMaxShortlist)) throw std::invalid_argument("k is above the bf16 path's shortlist");
      ensure_bf16();
    }
    size_t bmax = 0;
    for (size_t i = 0; i < count; ++i) bmax = std::max(bmax, batches[i]);
    if (bmax == 0) throw std::invalid_argument("batch sizes must be > 0");
    // Each timed repetition takes another slice of the queries, so that costs that only some
    // batches pay (the certified path's scan of unproven queries) are averaged in.
    constexpr int kReps = 4;
    const size_t qrows = std::max(bmax, std::min<size_t>(sample && nsample ? nsample : bmax * kReps, bmax * kReps));
    DeviceBuffer qbuf, obuf;
    qbuf.reserve(qrows * dp * sizeof(float), 0, stream);
    obuf.reserve(bmax * k * 8, 0, stream);
    if (sample && nsample) {  // the caller's queries, repeated to fill qrows
      for (size_t r = 0; r < qrows; r += nsample)
        VSG_CUDA(cudaMemcpy2DAsync(static_cast<float*>(qbuf.get()) + r * dp, dp * sizeof(float), sample,
                                   dim * sizeof(float), dim * sizeof(float), std::min(nsample, qrows - r),
                                   cudaMemcpyHostToDevice, stream));
    } else {  // queries near the index's rows (0.9 x_i + 0.1 x_j; none coincides with a row)
      VSG_CUDA(vsg::launch_midpoint_rows(static_cast<float*>(qbuf.get()), static_cast<const float*>(x.get()),
                                         uint32_t(dp), uint32_t(n), uint32_t(qrows), stream));
      ++kernel_launches;
    }
    cudaEvent_t e0, e1;
    VSG_CUDA(cudaEventCreate(&e0));
    VSG_CUDA(cudaEventCreate(&e1));
    auto time_it = [&](size_t b, uint32_t method) {
      float sum = 0.f;
      for (int rep = 0; rep < kReps; ++rep) {
        const size_t first = (size_t(rep) * b) % (qrows - b + 1);
        VSG_CUDA(cudaEventRecord(e0, stream));
        enqueue(static_cast<const float*>(qbuf.get()) + first * dp, dp, b, k, nullptr, false, 0, false,
                static_cast<uint32_t*>(obuf.get()), reinterpret_cast<float*>(static_cast<char*>(obuf.get()) + b * k * 4),
                stream, method);
        VSG_CUDA(cudaEventRecord(e1, stream));
        VSG_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        VSG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (rep > 0) sum += ms;  // the first run warms up
      }
      return sum / float(kReps - 1);  // the mean over different batches
    };
    std::vector<TuneEntry> table;
    try {
      for (size_t i = 0; i < count; ++i) {
        const size_t b = batches[i];
        TuneEntry pick;
        pick.batch = uint32_t(b);
        float best = 1e30f;
        if (family == VSG_METHOD_BF16) {
          for (int smp : {0, 4096, 16384}) {
            force_sample = smp;
            const float t = time_it(b, VSG_METHOD_BF16);
            if (t < best) {
              best = t;
              pick.sample = uint32_t(smp);
            }
          }
        } else {
          for (int kern : {0, 1, 2}) {
            if (kern == 1 && b < 8) continue;  // the tiled kernel's tile is 64 queries at least
            if (kern == 2 && k > size_t(vsg::kTcMaxShortlist)) continue;
            // FP32 kernels: 1x or 2x the row splits; the certified path sizes its own splits
            for (int o = 0; o < 2; ++o) {
              const double f = kern == 2 ? 1.0 : (o == 0 ? 1.0 : 2.0);
              const int kp = kern == 2 ? int(exact_shortlist_size(k)) : -1;
              if (kern == 2 && o == 1) continue;
              force_kernel = kern;
              force_split = f;
              force_exact_kp = kp;
              const float t = time_it(b, VSG_METHOD_AUTO);
              if (t < best) {
                best = t;
                pick.kernel = uint32_t(kern);
                pick.split = f;
                pick.exact_kp = kern == 2 ? uint32_t(kp) : 0u;
              }
            }
          }
        }
        table.push_back(pick);
      }
    } catch (...) {
      force_kernel = -1;
      force_sample = -1;
      force_exact_kp = -1;
      force_split = 0;
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      throw;
    }
    force_kernel = -1;
    force_sample = -1;
    force_exact_kp = -1;
    force_split = 0;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    (family == VSG_METHOD_BF16 ? tune_bf16 : tune_plain) = table;
  }

  // allowed: the largest allowed fraction of the masks when known (host masks), else -1.
  // nq_dev: scan path only, a device count of the queries to search (at most nq).
  // out_map (with nq_dev): query j's results go to row out_map[j] of the outputs. pdl: the scan
  // is launched as a dependent of the kernel before it (the certified path's finish kernel).
  void enqueue(const float* dq, size_t ldq, size_t nq, size_t k, const uint32_t* dmask, bool per_query,
               size_t mask_ld, bool gather, uint32_t* out_ids, float* out_dists, cudaStream_t s,
               uint32_t method = VSG_METHOD_AUTO, double allowed = -1.0, const uint32_t* nq_dev = nullptr,
               const uint32_t* out_map = nullptr, bool pdl = false) {
    // (A shortlist holds at most kTcMaxShortlist rows per query, which every k <= 128 fits.)
    const size_t mld = dmask && per_query ? mask_ld : 0;  // 0: one mask for every query
    if ((method == VSG_METHOD_BF16 || method == VSG_METHOD_FP8) && k <= size_t(vsg::kTcMaxShortlist)) {
      enqueue_bf16(dq, ldq, nq, k, out_ids, out_dists, s, false, 0, method == VSG_METHOD_FP8, dmask, mld);
      return;
    }
    if (use_tc_exact(method, nq, k, dmask, gather, allowed)) {
      enqueue_tc_exact(dq, ldq, nq, k, out_ids, out_dists, s, dmask, mld);
      return;
    }
    if (use_tiled(method, nq, dmask)) {
      enqueue_tiled(dq, ldq, nq, k, out_ids, out_dists, s);
      return;
    }
    gather = gather && dmask != nullptr;
    // With a device count (the certified path's fallback) only the few queries at the front run:
    // split the rows as for at most fallback_split_queries so that one lone query block still
    // spans many SMs. Planned for all nq, a batch of 4096 would give that block one split, one
    // CTA over every row. The blocks past the count cost one launch and one load each.
    const Plan p = plan(nq, k, gather, gather && per_query, nq_dev && !gather ? size_t(fallback_split_queries) : 0);
    const size_t parts = nq * p.nsplit * k;
    part.reserve(parts * 8, 0, stream);
    vsg::ScanArgs a{};
    a.x = static_cast<const float*>(x.get());
    a.q = dq;
    a.ldq = uint32_t(ldq);
    a.mask = dmask;
    a.mask_ld = per_query ? mask_ld : 0;
    a.part_d = static_cast<float*>(part.get());
    a.part_i = reinterpret_cast<uint32_t*>(static_cast<char*>(part.get()) + parts * 4);
    a.status = status_word();
    a.n = uint32_t(n);
    a.dp = uint32_t(dp);
    a.nq = uint32_t(nq);
    a.k = uint32_t(k);
    a.rows_per_split = p.rows_per_split;
    a.nsplit = p.nsplit;
    a.stages = p.stages;
    a.gather = gather ? 1u : 0u;
    a.wait_ns = wait_ns();
    a.stall = stall_next ? 1u : 0u;
    Timing* tm = profiling ? next_timing() : nullptr;
    if (tm) VSG_CUDA(cudaEventRecord(tm->ev[0], s));
    // The last CTA of each query block merges the splits in the scan kernel itself.
    counters.reserve(size_t(p.nqb) * sizeof(uint32_t), 0, stream);
    a.counters = static_cast<uint32_t*>(counters.get());
    a.out_d = out_dists;
    a.out_i = out_ids;
    a.nq_dev = nq_dev;
    a.out_map = out_map;
    VSG_CUDA(vsg::launch_scan(p.shape, a, dim3(p.nqb, p.nsplit), s, pdl));
    ++kernel_launches;
    if (tm) VSG_CUDA(cudaEventRecord(tm->ev[1], s));
    if (tm) VSG_CUDA(cudaEventRecord(tm->ev[2], s));
  }

  // ---- kernel timing (vsg_profile_*) ----
  struct Timing {
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
  };
  bool profiling = false;
  std::vector<Timing> timings;  // event pool; the first `used` are recorded
  size_t used = 0;

  Timing* next_timing() {
    if (used == timings.size()) {
      Timing t;
      for (auto& e : t.ev) VSG_CUDA(cudaEventCreate(&e));
      timings.push_back(t);
    }
    return &timings[used++];
  }

  void read_timings(double* scan_ms, double* merge_ms, size_t* count) {
    double a = 0, b = 0;
    for (size_t i = 0; i < used; ++i) {
      VSG_CUDA(cudaEventSynchronize(timings[i].ev[2]));
      float x = 0, y = 0;
      VSG_CUDA(cudaEventElapsedTime(&x, timings[i].ev[0], timings[i].ev[1]));
      VSG_CUDA(cudaEventElapsedTime(&y, timings[i].ev[1], timings[i].ev[2]));
      a += x;
      b += y;
    }
    if (scan_ms) *scan_ms = a;
    if (merge_ms) *merge_ms = b;
    if (count) *count = used;
    used = 0;
  }

  void destroy_timings() {
    for (auto& t : timings)
      for (auto& e : t.ev)
        if (e) cudaEventDestroy(e);
    timings.clear();
    used = 0;
  }

  // Host queries -> device staging (dp stride). Pageable inputs go through pinned staging.
  const float* stage_queries(const float* host_q, size_t nq) {
    q.reserve(nq * dp * sizeof(float), 0, stream);
    float* dq = static_cast<float*>(q.get());
    if (host_is_pinned(host_q)) {
      VSG_CUDA(cudaMemcpy2DAsync(dq, dp * sizeof(float), host_q, dim * sizeof(float), dim * sizeof(float), nq,
                                 cudaMemcpyHostToDevice, stream));
    } else {
      pin_in.reserve(nq * dim * sizeof(float));
      std::memcpy(pin_in.get(), host_q, nq * dim * sizeof(float));
      VSG_CUDA(cudaMemcpy2DAsync(dq, dp * sizeof(float), pin_in.get(), dim * sizeof(float), dim * sizeof(float),
                                 nq, cudaMemcpyHostToDevice, stream));
    }
    return dq;
  }

  const uint32_t* stage_mask(const uint32_t* host_words, size_t words) {
    mask.reserve(words * 4, 0, stream);
    VSG_CUDA(cudaMemcpyAsync(mask.get(), host_words, words * 4, cudaMemcpyHostToDevice, stream));
    return static_cast<const uint32_t*>(mask.get());
  }

  // Largest fraction of rows any of `masks` masks (ld words apart) allows.
  double allowed_fraction(const uint32_t* words, size_t masks, size_t ld) const {
    const size_t nw = ceil_div(n, 32);
    size_t best = 0;
    for (size_t m = 0; m < masks; ++m) {
      const uint32_t* w = words + m * ld;
      size_t c = 0;
      for (size_t i = 0; i + 1 < nw; ++i) c += size_t(__builtin_popcount(w[i]));
      const uint32_t tail = (n % 32) ? (1u << (n % 32)) - 1u : 0xFFFFFFFFu;
      c += size_t(__builtin_popcount(w[nw - 1] & tail));
      best = std::max(best, c);
    }
    return n ? double(best) / double(n) : 0.0;
  }

  void drop_graph() {
    if (hgraph.exec) cudaGraphExecDestroy(hgraph.exec);
    hgraph.exec = nullptr;
  }

  // Captures the chain of an unfiltered blocking search of nq queries (host_graph_search); false
  // (nothing kept, no error left set) when the chain cannot be captured.
  bool capture_graph(size_t nq, size_t k, uint32_t method) {
    drop_graph();
    pin_in.reserve(nq * dp * sizeof(float));
    pin_out.reserve(16 + nq * k * 8);
    reserve_results(nq, k);
    q.reserve(nq * dp * sizeof(float), 0, stream);
    // Direct: the kernels read the pinned staging buffer through its device address (the
    // certified path only, whose kernels read the queries with plain loads).
    float* hq = nullptr;
    if (host_graph_direct > 0 && use_tc_exact(method, nq, k, nullptr, false, -1.0)) {
      cudaPointerAttributes at{};
      if (cudaPointerGetAttributes(&at, pin_in.get()) == cudaSuccess && at.devicePointer)
        hq = static_cast<float*>(at.devicePointer);
      cudaGetLastError();
    }
    hgraph.direct = hq != nullptr;
    const uint64_t l0 = kernel_launches, t0 = tc_exact_queries, i0 = tiled_queries;
    cudaGraph_t graph = nullptr;
    if (cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    bool ok = true;
    try {
      float* dq = hq ? hq : static_cast<float*>(q.get());
      if (!hq)
        VSG_CUDA(cudaMemcpy2DAsync(dq, dp * sizeof(float), pin_in.get(), dim * sizeof(float), dim * sizeof(float),
                                   nq, cudaMemcpyHostToDevice, stream));
      enqueue(dq, dp, nq, k, nullptr, false, 0, false, res_ids(), res_dists(nq, k), stream, method, -1.0);
      VSG_CUDA(cudaMemcpyAsync(pin_out.get(), res.get(), 16 + nq * k * 8, cudaMemcpyDeviceToHost, stream));
    } catch (...) {
      ok = false;  // (an allocation or a sync inside the chain: capture refuses both)
    }
    const cudaError_t e = cudaStreamEndCapture(stream, &graph);
    cudaGraphExec_t exec = nullptr;
    if (ok && e == cudaSuccess && graph && cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) exec = nullptr;
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    hgraph.launches = kernel_launches - l0;
    hgraph.tc_queries = tc_exact_queries - t0;
    hgraph.tiled_q = tiled_queries - i0;
    kernel_launches = l0;  // nothing ran: the replays count
    tc_exact_queries = t0;
    tiled_queries = i0;
    if (!exec) return false;
    hgraph.exec = exec;
    hgraph.epoch = g_alloc_epoch.load();
    return true;
  }

  // A blocking unfiltered search through the shape's graph; false when it does not apply (the
  // caller runs the search without it).
  bool host_graph_search(const float* host_q, size_t nq, size_t k, uint32_t method, uint32_t* out_ids,
                         float* out_dists) {
    HostGraph& g = hgraph;
    if (!(g.nq == nq && g.k == k && g.method == method && g.n == n && g.gen == config_gen)) {
      drop_graph();  // a new shape: it runs once without a graph, and is captured the next time
      g.nq = nq;
      g.k = k;
      g.method = method;
      g.n = n;
      g.gen = config_gen;
      g.ran = false;
      g.failed = false;
      return false;
    }
    if (!g.ran || g.failed) return false;
    VSG_CUDA(cudaSetDevice(device));
    VSG_CUDA(cudaStreamWaitEvent(stream, done, 0));
    if (!g.exec || g.epoch != g_alloc_epoch.load()) {
      if (!capture_graph(nq, k, method)) {
        g.failed = true;
        return false;
      }
    }
    if (g.direct) {  // rows dp apart, padding zero
      float* hq = static_cast<float*>(pin_in.get());
      for (size_t i = 0; i < nq; ++i) {
        std::memcpy(hq + i * dp, host_q + i * dim, dim * sizeof(float));
        std::fill(hq + i * dp + dim, hq + (i + 1) * dp, 0.f);
      }
    } else {
      std::memcpy(pin_in.get(), host_q, nq * dim * sizeof(float));
    }
    VSG_CUDA(cudaGraphLaunch(g.exec, stream));
    kernel_launches += g.launches;
    tc_exact_queries += g.tc_queries;
    tiled_queries += g.tiled_q;
    VSG_CUDA(cudaEventRecord(done, stream));
    VSG_CUDA(cudaStreamSynchronize(stream));
    const char* h = static_cast<const char*>(pin_out.get());
    int st = 0;
    std::memcpy(&st, h, sizeof(int));
    if (st != 0) {
      reset_after_failure();
      throw DeviceTimeout("a search kernel's wait ran past its time limit");
    }
    std::memcpy(out_ids, h + 16, nq * k * 4);
    std::memcpy(out_dists, h + 16 + nq * k * 4, nq * k * 4);
    return true;
  }

  // Full host-to-host search: stage, enqueue, copy the result block back, check status.
  void search_host(const float* host_q, size_t nq, size_t k, const uint32_t* host_mask, bool per_query,
                   size_t mask_ld, uint32_t* out_ids, float* out_dists, uint32_t method = VSG_METHOD_AUTO) {
    const bool graphable = !host_mask && !stall_next && !profiling && double(nq) <= host_graph_max_batch;
    if (graphable) {
      if (method == VSG_METHOD_BF16 && k <= size_t(vsg::kTcMaxShortlist)) ensure_bf16();
      if (host_graph_search(host_q, nq, k, method, out_ids, out_dists)) return;
    }
    VSG_CUDA(cudaSetDevice(device));
    VSG_CUDA(cudaStreamWaitEvent(stream, done, 0));
    reserve_results(nq, k);
    const float* dq = stage_queries(host_q, nq);
    const uint32_t* dm = nullptr;
    bool gather = false;
    double allowed = -1.0;
    if (host_mask) {
      const size_t words = per_query ? nq * mask_ld : ceil_div(n, 32);
      dm = stage_mask(host_mask, words);
      allowed = allowed_fraction(host_mask, per_query ? nq : 1, per_query ? mask_ld : ceil_div(n, 32));
      gather = allowed <= gather_max_fraction;
    }
    uint32_t* di = res_ids();
    float* dd = res_dists(nq, k);
    if (method == VSG_METHOD_BF16 && !dm && k <= size_t(vsg::kTcMaxShortlist)) ensure_bf16();
    try {
      enqueue(dq, dp, nq, k, dm, per_query, mask_ld, gather, di, dd, stream, method, allowed);
    } catch (...) {
      stall_next = false;
      throw;
    }
    stall_next = false;  // the test hook covers one search
    const size_t bytes = 16 + nq * k * 8;
    pin_out.reserve(bytes);
    VSG_CUDA(cudaMemcpyAsync(pin_out.get(), res.get(), bytes, cudaMemcpyDeviceToHost, stream));
    VSG_CUDA(cudaEventRecord(done, stream));
    VSG_CUDA(cudaStreamSynchronize(stream));
    const char* h = static_cast<const char*>(pin_out.get());
    int st = 0;
    std::memcpy(&st, h, sizeof(int));
    if (st != 0) {
      reset_after_failure();
      throw DeviceTimeout("a search kernel's wait ran past its time limit");
    }
    std::memcpy(out_ids, h + 16, nq * k * 4);
    std::memcpy(out_dists, h + 16 + nq * k * 4, nq * k * 4);
    if (graphable) hgraph.ran = true;  // its buffers exist: the next search of the shape is captured
  }
};
