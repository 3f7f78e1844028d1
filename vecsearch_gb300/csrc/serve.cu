// Serving loop: continuous batching over the certified tensor-core path (exact results).
//
// The reference serves queries one call at a time (python/bindings.cpp:165-186; its gRPC shard
// worker, distributed/shard_worker.py:26-36, calls the index per request). Here a worker thread
// keeps requests of any size, k and filter flowing onto the GPU:
//   * a request (host queries, k, optional allow-bits, host outputs) is queued by submit();
//   * each slot owns device and pinned buffers sized for `max_batch` queries and a CUDA graph
//     captured once: the query preparation (bf16 queries, norms, certificate bounds E and
//     margins), reset of the work counter, the sample pass and its select, the persistent
//     shortlist kernel (one CTA per SM claiming (query block, split) items; per-query k, k',
//     margin and filter), the finish kernel (cut, exact FP32 rerank, certificate; it hands each
//     query it could not certify, with its filter, to the fallback), the FP32 scan kernel
//     launched on the device's count of those queries, and their results scattered into place.
//     So every served result equals the FP32 scan's (method skinny) bit for bit;
//   * the worker admits queued requests into every free slot as soon as it frees (up to the
//     slot's query and filter capacity), copies the micro-batch in, launches the graph and the
//     copies out on the slot's stream, and completes requests when the slot's event fires. So
//     requests that arrive while others are on the GPU join the next free slot, and the slots'
//     copies and kernels overlap on the device;
//   * the number of slots is bounded by free HBM at creation (half of it at most).
// A request's result does not depend on the other requests in its micro-batch: every query's
// scores, shortlist, rerank, certificate and fallback scan are computed independently (bitwise).
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <thread>
#include <unordered_map>

#include "index_impl.cuh"

namespace vsg {
void set_last_error(const std::string& msg);
}

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  const float* q = nullptr;
  size_t nq = 0;
  uint32_t k = 0;
  const uint32_t* mask = nullptr;
  uint32_t* out_i = nullptr;
  float* out_d = nullptr;
  Clock::time_point t_submit, t_done;
  int status = -1;  // -1 pending, else a VSG_* code
  std::string error;
};

size_t align256(size_t v) { return (v + 255) & ~size_t(255); }

struct Slot {
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  DeviceBuffer d_in, d_qb, d_qn, d_part, d_out, d_sample, d_thr, d_cbuf, d_gthr;
  // certified path: margins then bounds E; [uncertified count | their indices]; the fallback
  // scan's queries, filter pointers, split lists, results and fused-merge counters
  DeviceBuffer d_margin, d_fails, d_fq, d_mptr, d_spart, d_fout, d_counters;
  PinnedBuffer h_in, h_out;
  CUtensorMap qmap{};
  std::vector<Request*> reqs;
  bool busy = false;
  uint32_t total_k = 0;
};

}  // namespace

constexpr size_t kSampleRows = 16384;

struct vsg_server {
  vsg_index* idx = nullptr;
  size_t sample_per_query = 0;  // capacity of a query's sampled distances
  size_t cap_q = 0, cap_masks = 0, max_k = 0, kp_max = 0, mwords = 0, stages = 0;
  uint32_t resident = 0;
  size_t off_sq = 0, off_q = 0, off_m = 0, in_bytes = 0, out_k = 0;
  std::vector<std::unique_ptr<Slot>> slots;
  std::deque<Request*> queue;
  std::unordered_map<uint64_t, std::unique_ptr<Request>> reqs;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::thread worker;
  bool stop = false;
  uint64_t next_ticket = 1;
  uint64_t n_batches = 0, n_queries = 0, n_requests = 0, n_uncertified = 0;
  vsg_index::Plan fb;  // the fallback scan's plan: cap_q queries, rows split as for a few

  uint32_t shortlist(uint32_t k) const { return vsg_index::exact_shortlist_size(k); }

  void build_slot(Slot& s) {
    VSG_CUDA(cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking));
    VSG_CUDA(cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming));
    s.d_in.reserve(in_bytes, 0, s.stream);
    s.h_in.reserve(in_bytes);
    std::memset(s.h_in.get(), 0, in_bytes);
    s.d_qb.reserve(cap_q * idx->dp * 2, 0, s.stream);
    s.d_qn.reserve(cap_q * sizeof(float), 0, s.stream);
    // split lists and their lengths: at most max(cap_q, 128 * SMs) (query, split) pairs, each with
    // tc_groups lists of kp_max
    const size_t groups = vsg::tc_groups(uint32_t(kp_max));
    const size_t pairs = std::max(cap_q, size_t(vsg::kTcQueries) * size_t(idx->sms)) * groups;
    s.d_part.reserve(pairs * kp_max * 8 + pairs * 4, 0, s.stream);
    s.d_out.reserve(out_k * 8 + 16, 0, s.stream);
    // sample pass: per query nsplit * sample_tiles * 128 <= max(kSample + one split's tiles, ...) distances
    s.d_sample.reserve(cap_q * sample_per_query * sizeof(float), 0, s.stream);
    s.d_thr.reserve(cap_q * sizeof(float), 0, s.stream);
    // one candidate buffer per CTA of the persistent kernel, one shared threshold per query
    const size_t cbuf_entries = size_t(idx->sms) * groups * vsg::kTcQueries * vsg::tc_buffer_capacity(uint32_t(kp_max));
    s.d_cbuf.reserve(cbuf_entries * 8, 0, s.stream);
    s.d_gthr.reserve(cap_q * sizeof(uint32_t), 0, s.stream);
    s.d_margin.reserve(2 * cap_q * sizeof(float), 0, s.stream);
    s.d_fails.reserve((1 + cap_q) * sizeof(uint32_t), 0, s.stream);
    s.d_fq.reserve(cap_q * idx->dp * sizeof(float), 0, s.stream);
    s.d_mptr.reserve(cap_q * sizeof(const uint32_t*), 0, s.stream);
    const size_t sparts = cap_q * size_t(fb.nsplit) * max_k;
    s.d_spart.reserve(sparts * 8, 0, s.stream);
    s.d_fout.reserve(cap_q * max_k * 8, 0, s.stream);
    s.d_counters.reserve(size_t(fb.nqb) * sizeof(uint32_t), 0, s.stream);  // zero: the scan keeps them so
    s.h_out.reserve(out_k * 8 + 16);
    char* din = static_cast<char*>(s.d_in.get());
    auto* hdr = reinterpret_cast<vsg::ServeHeader*>(din);
    auto* sq = reinterpret_cast<vsg::ServeQuery*>(din + off_sq);
    float* dq = reinterpret_cast<float*>(din + off_q);
    VSG_CUDA(vsg::tc_encode_map(&s.qmap, s.d_qb.get(), cap_q, idx->dp, uint32_t(vsg::kTcQueries)));
    float* out_d = static_cast<float*>(s.d_out.get());
    uint32_t* out_i = reinterpret_cast<uint32_t*>(out_d + out_k);
    int* status = reinterpret_cast<int*>(out_i + out_k);
    float* margin = static_cast<float*>(s.d_margin.get());
    uint32_t* fails = static_cast<uint32_t*>(s.d_fails.get());
    const bool l2 = idx->metric == VSG_METRIC_L2;
    vsg::TcArgs a{};
    a.n = uint32_t(idx->n);
    a.dp = uint32_t(idx->dp);
    a.kp = uint32_t(kp_max);
    a.stages = uint32_t(stages);
    a.resident = resident;
    a.l2 = l2 ? 1u : 0u;
    a.cbuf_d = static_cast<float*>(s.d_cbuf.get());
    a.cbuf_i = reinterpret_cast<uint32_t*>(static_cast<char*>(s.d_cbuf.get()) + cbuf_entries * 4);
    a.gthr = static_cast<uint32_t*>(s.d_gthr.get());
    a.xnorm = static_cast<const float*>(idx->xnorm.get());
    a.qnorm = static_cast<const float*>(s.d_qn.get());
    a.part_d = static_cast<float*>(s.d_part.get());
    a.part_i = reinterpret_cast<uint32_t*>(static_cast<char*>(s.d_part.get()) + pairs * kp_max * 4);
    a.part_n = reinterpret_cast<uint32_t*>(static_cast<char*>(s.d_part.get()) + pairs * kp_max * 8);
    a.status = status;
    a.hdr = hdr;
    a.sq = sq;
    a.margin = margin;  // each query keeps the rows within its margin of its k-th best
    vsg::FinishArgs f{};
    f.part_d = a.part_d;
    f.part_i = a.part_i;
    f.part_n = a.part_n;
    f.kp = uint32_t(kp_max);
    f.margin = margin;
    f.x = static_cast<const float*>(idx->x.get());
    f.n = uint32_t(idx->n);
    f.q = dq;
    f.dp = uint32_t(idx->dp);
    f.ldq = uint32_t(idx->dp);
    f.l2 = a.l2;
    f.out_d = out_d;
    f.out_i = out_i;
    f.thr_init = static_cast<const float*>(s.d_thr.get());
    f.gthr = a.gthr;
    f.err = margin + cap_q;
    f.fail_count = fails;
    f.fail_list = fails + 1;
    f.status = status;
    f.hdr = hdr;
    f.sq = sq;
    f.stage_cap = 4096;  // more entries: the finish kernel reads the lists in global memory
    f.lists_per_split = uint32_t(groups);
    f.fq = static_cast<float*>(s.d_fq.get());  // uncertified queries' rows and filters, for the scan
    f.fmask_ptrs = static_cast<const uint32_t**>(s.d_mptr.get());
    // The fallback scan: gathered queries, their filters by pointer, cap_q queries of which only
    // the device's uncertified count run; the fused merge writes max_k results per query.
    vsg::ScanArgs sc{};
    sc.x = static_cast<const float*>(idx->x.get());
    sc.q = static_cast<const float*>(s.d_fq.get());
    sc.ldq = uint32_t(idx->dp);
    sc.mask_ptrs = static_cast<const uint32_t* const*>(s.d_mptr.get());
    sc.part_d = static_cast<float*>(s.d_spart.get());
    sc.part_i = reinterpret_cast<uint32_t*>(static_cast<char*>(s.d_spart.get()) + sparts * 4);
    sc.status = status;
    sc.n = uint32_t(idx->n);
    sc.dp = uint32_t(idx->dp);
    sc.nq = uint32_t(cap_q);
    sc.k = uint32_t(max_k);
    sc.rows_per_split = fb.rows_per_split;
    sc.nsplit = fb.nsplit;
    sc.stages = fb.stages;
    sc.counters = static_cast<uint32_t*>(s.d_counters.get());
    float* fout_d = static_cast<float*>(s.d_fout.get());
    uint32_t* fout_i = reinterpret_cast<uint32_t*>(fout_d + cap_q * max_k);
    sc.out_d = fout_d;
    sc.out_i = fout_i;
    sc.nq_dev = fails;
    // kernel attributes before capture
    VSG_CUDA(vsg::tc_prepare(a.stages, vsg::tc_chunks(a.dp, false), a.resident, l2, false));
    VSG_CUDA(vsg::finish_prepare(f.dp, f.stage_cap));
    VSG_CUDA(vsg::scan_prepare(fb.shape, sc.dp, sc.k, sc.stages));
    VSG_CUDA(cudaStreamBeginCapture(s.stream, cudaStreamCaptureModeThreadLocal));
    VSG_CUDA(vsg::launch_prepare_queries(nullptr, dq, uint32_t(idx->dp), uint32_t(cap_q), uint32_t(idx->dp), uint32_t(idx->dp),
                                         s.d_qb.get(), static_cast<float*>(s.d_qn.get()), a.gthr,
                                         static_cast<const float*>(idx->xbound.get()), l2, float(idx->cert_margin),
                                         margin, margin + cap_q, fails, s.stream));
    // Sample pass: the head tiles of every split give each query a starting threshold (its k-th
    // best sampled distance plus its margin).
    vsg::TcArgs sa = a;
    sa.dump = static_cast<float*>(s.d_sample.get());
    sa.gthr = nullptr;
    VSG_CUDA(cudaMemsetAsync(&hdr->next, 0, sizeof(uint32_t), s.stream));
    VSG_CUDA(vsg::launch_tc_shortlist(s.qmap, idx->xmap, sa, unsigned(idx->sms), s.stream));
    VSG_CUDA(vsg::launch_serve_select(hdr, sq, sa.dump, static_cast<float*>(s.d_thr.get()), uint32_t(cap_q),
                                      s.stream, margin));
    a.thr_init = static_cast<const float*>(s.d_thr.get());
    VSG_CUDA(cudaMemsetAsync(&hdr->next, 0, sizeof(uint32_t), s.stream));
    VSG_CUDA(vsg::launch_tc_shortlist(s.qmap, idx->xmap, a, unsigned(idx->sms), s.stream));
    VSG_CUDA(vsg::launch_finish(f, uint32_t(cap_q), s.stream));
    VSG_CUDA(vsg::launch_scan(fb.shape, sc, dim3(fb.nqb, fb.nsplit), s.stream));
    VSG_CUDA(vsg::launch_serve_scatter(fails, fails + 1, sq, fout_d, fout_i, uint32_t(max_k), out_d, out_i, nullptr,
                                       uint32_t(cap_q), s.stream));
    VSG_CUDA(cudaStreamEndCapture(s.stream, &s.graph));
    VSG_CUDA(cudaGraphInstantiate(&s.exec, s.graph, 0));
  }

  ~vsg_server() {
    {
      std::lock_guard<std::mutex> g(mu);
      stop = true;
    }
    cv_work.notify_all();
    if (worker.joinable()) worker.join();
    for (auto& sp : slots) {
      Slot& s = *sp;
      if (s.stream) cudaStreamSynchronize(s.stream);
      if (s.exec) cudaGraphExecDestroy(s.exec);
      if (s.graph) cudaGraphDestroy(s.graph);
      if (s.done) cudaEventDestroy(s.done);
      if (s.stream) cudaStreamDestroy(s.stream);
    }
  }

  // Packs `batch` into slot s and queues copies in, the graph and copies out. Caller holds no lock.
  void launch(Slot& s, std::vector<Request*> batch) {
    char* hin = static_cast<char*>(s.h_in.get());
    auto* hdr = reinterpret_cast<vsg::ServeHeader*>(hin);
    auto* sq = reinterpret_cast<vsg::ServeQuery*>(hin + off_sq);
    float* hq = reinterpret_cast<float*>(hin + off_q);
    uint32_t* hm = reinterpret_cast<uint32_t*>(hin + off_m);
    const char* din = static_cast<const char*>(s.d_in.get());
    const uint32_t* dm = reinterpret_cast<const uint32_t*>(din + off_m);
    size_t nq = 0, nm = 0;
    uint32_t out = 0;
    for (Request* r : batch) {
      const uint32_t* mask_dev = nullptr;
      if (r->mask) {
        std::memcpy(hm + nm * mwords, r->mask, mwords * sizeof(uint32_t));
        mask_dev = dm + nm * mwords;
        ++nm;
      }
      const uint32_t kp = shortlist(r->k);
      for (size_t i = 0; i < r->nq; ++i, ++nq) {
        std::memcpy(hq + nq * idx->dp, r->q + i * idx->dim, idx->dim * sizeof(float));
        sq[nq] = vsg::ServeQuery{r->k, kp, mask_dev, out, 0};
        out += r->k;
      }
    }
    const size_t nqb = ceil_div(nq, size_t(vsg::kTcQueries));
    const size_t want = std::max<size_t>(1, size_t(idx->sms) / nqb);
    const size_t rps = vsg::split_rows(ceil_div(ceil_div(idx->n, want), size_t(vsg::kTcRows)) * vsg::kTcRows,
                                       vsg::kTcRows);
    hdr->nq = uint32_t(nq);
    hdr->nqb = uint32_t(nqb);
    hdr->rows_per_split = uint32_t(rps);
    hdr->nsplit = uint32_t(ceil_div(idx->n, rps));
    hdr->items = hdr->nqb * hdr->nsplit;
    hdr->next = 0;
    // Sample at least 16K rows per query (whole tiles at the head of each split).
    const size_t tiles_per_split = ceil_div(rps, size_t(vsg::kTcRows));
    hdr->sample_tiles = uint32_t(std::min(tiles_per_split, ceil_div(kSampleRows, size_t(hdr->nsplit) * vsg::kTcRows)));
    s.reqs = std::move(batch);
    s.total_k = out;
    char* dout = static_cast<char*>(s.d_out.get());
    char* hout = static_cast<char*>(s.h_out.get());
    cudaError_t e = cudaMemcpyAsync(s.d_in.get(), hin, off_q + nq * idx->dp * sizeof(float), cudaMemcpyHostToDevice,
                                    s.stream);
    if (e == cudaSuccess && nm)
      e = cudaMemcpyAsync(const_cast<uint32_t*>(dm), hm, nm * mwords * sizeof(uint32_t), cudaMemcpyHostToDevice,
                          s.stream);
    if (e == cudaSuccess) e = cudaGraphLaunch(s.exec, s.stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hout, dout, size_t(out) * 4, cudaMemcpyDeviceToHost, s.stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(hout + out_k * 4, dout + out_k * 4, size_t(out) * 4, cudaMemcpyDeviceToHost, s.stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(hout + out_k * 8, dout + out_k * 8, sizeof(int), cudaMemcpyDeviceToHost, s.stream);
    if (e == cudaSuccess)  // the certified path's uncertified count of this micro-batch
      e = cudaMemcpyAsync(hout + out_k * 8 + 4, s.d_fails.get(), sizeof(uint32_t), cudaMemcpyDeviceToHost, s.stream);
    if (e == cudaSuccess) e = cudaEventRecord(s.done, s.stream);
    if (e != cudaSuccess) {
      cudaGetLastError();
      fail_slot(s, std::string("serving launch: ") + cudaGetErrorString(e));
    }
  }

  void fail_slot(Slot& s, const std::string& msg) {
    std::lock_guard<std::mutex> g(mu);
    for (Request* r : s.reqs) {
      r->status = VSG_ERR_CUDA;
      r->error = msg;
      r->t_done = Clock::now();
    }
    s.reqs.clear();
    s.busy = false;
    cv_done.notify_all();
  }

  // Results of a finished slot into the requests' host arrays.
  void complete(Slot& s) {
    const char* hout = static_cast<const char*>(s.h_out.get());
    const float* od = reinterpret_cast<const float*>(hout);
    const uint32_t* oi = reinterpret_cast<const uint32_t*>(hout + out_k * 4);
    int st = 0;
    uint32_t unproven = 0;
    std::memcpy(&st, hout + out_k * 8, sizeof(int));
    std::memcpy(&unproven, hout + out_k * 8 + 4, sizeof(uint32_t));
    uint32_t off = 0;
    const auto now = Clock::now();
    for (Request* r : s.reqs) {
      const size_t cnt = r->nq * r->k;
      if (st == 0) {
        std::memcpy(r->out_d, od + off, cnt * sizeof(float));
        std::memcpy(r->out_i, oi + off, cnt * sizeof(uint32_t));
      }
      off += uint32_t(cnt);
    }
    if (st != 0) {  // a kernel gave up on a wait: clear the status word and the fallback scan's
                    // merge counters before the slot is reused
      char* dout = static_cast<char*>(s.d_out.get());
      cudaMemsetAsync(dout + out_k * 8, 0, sizeof(int), s.stream);
      cudaMemsetAsync(s.d_counters.get(), 0, s.d_counters.bytes(), s.stream);
      cudaStreamSynchronize(s.stream);
    }
    std::lock_guard<std::mutex> g(mu);
    for (Request* r : s.reqs) {
      r->status = st == 0 ? VSG_OK : VSG_ERR_DEVICE_TIMEOUT;
      if (st != 0) r->error = "a search kernel's wait ran past its time limit";
      r->t_done = now;
    }
    n_batches += 1;
    if (st == 0) n_uncertified += unproven;
    s.reqs.clear();
    s.busy = false;
    cv_done.notify_all();
  }

  void run() {
    cudaSetDevice(idx->device);
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
      bool progressed = false;
      for (auto& sp : slots) {
        Slot& s = *sp;
        if (!s.busy) continue;
        const cudaError_t e = cudaEventQuery(s.done);
        if (e == cudaErrorNotReady) continue;
        lk.unlock();
        if (e == cudaSuccess) {
          complete(s);
        } else {
          cudaGetLastError();
          fail_slot(s, std::string("serving slot: ") + cudaGetErrorString(e));
        }
        lk.lock();
        progressed = true;
      }
      for (auto& sp : slots) {
        Slot& s = *sp;
        if (s.busy || queue.empty()) continue;
        std::vector<Request*> batch;
        size_t nq = 0, nm = 0;
        while (!queue.empty()) {
          Request* r = queue.front();
          if (nq + r->nq > cap_q || nm + (r->mask ? 1 : 0) > cap_masks) break;
          nq += r->nq;
          nm += r->mask ? 1 : 0;
          batch.push_back(r);
          queue.pop_front();
        }
        if (batch.empty()) continue;
        s.busy = true;
        n_queries += nq;
        lk.unlock();
        launch(s, std::move(batch));
        lk.lock();
        progressed = true;
      }
      bool any_busy = false;
      for (auto& sp : slots) any_busy = any_busy || sp->busy;
      if (stop && queue.empty() && !any_busy) break;
      if (!progressed) {
        if (any_busy)
          cv_work.wait_for(lk, std::chrono::microseconds(20));
        else
          cv_work.wait(lk, [&] { return stop || !queue.empty(); });
      }
    }
  }
};

namespace {

int sfail(int code, const std::string& msg) {
  vsg::set_last_error(msg);
  return code;
}

}  // namespace

extern "C" {

int vsg_server_create(vsg_index* h, size_t max_batch, size_t max_k, size_t slots, vsg_server** out) {
  if (!h || !out) return sfail(VSG_ERR_INVALID, "index or out is NULL");
  *out = nullptr;
  vsg::set_last_error("");
  try {
    if (max_batch == 0 || slots == 0) throw std::invalid_argument("max_batch and slots must be > 0");
    if (max_k == 0 || max_k > size_t(VSG_MAX_K))
      throw std::invalid_argument("max_k must be in [1, " + std::to_string(VSG_MAX_K) + "]");
    std::unique_ptr<vsg_server> s(new vsg_server());
    s->idx = h;
    {
      std::lock_guard<std::mutex> g(h->mu);
      if (h->n == 0) throw std::invalid_argument("the index is empty");
      VSG_CUDA(cudaSetDevice(h->device));
      h->ensure_bf16();
      h->ensure_xmap();
      // the fallback scan of uncertified queries: rows split as for a few queries
      s->fb = h->plan(max_batch, max_k, false, false, std::max<size_t>(1, size_t(h->fallback_split_queries)));
    }
    s->cap_q = max_batch;
    s->cap_masks = std::min<size_t>(max_batch, 128);
    s->max_k = max_k;
    s->kp_max = vsg_index::exact_shortlist_size(max_k);
    s->stages = vsg::tc_pick_stages(vsg::tc_chunks(uint32_t(h->dp), false), h->smem_optin - 1024, &s->resident,
                                    h->metric == VSG_METRIC_L2, false);
    if (s->stages < 2) throw std::invalid_argument("shortlist does not fit the tensor-core kernel's shared memory");
    s->mwords = ceil_div(h->n, 32);
    s->off_sq = 256;
    s->off_q = align256(s->off_sq + max_batch * sizeof(vsg::ServeQuery));
    s->off_m = align256(s->off_q + max_batch * h->dp * sizeof(float));
    s->in_bytes = s->off_m + s->cap_masks * s->mwords * sizeof(uint32_t);
    s->out_k = max_batch * max_k;
    // nsplit * sample_tiles * 128 < kSampleRows + nsplit * 128 <= kSampleRows + 128 * SMs
    s->sample_per_query = kSampleRows + size_t(vsg::kTcRows) * size_t(h->sms);
    // Admission by free HBM: each slot's workspace is fixed; use at most half of what is free.
    const size_t groups = vsg::tc_groups(uint32_t(s->kp_max));
    const size_t pairs = std::max(max_batch, size_t(vsg::kTcQueries) * size_t(h->sms)) * groups;
    const size_t per_slot = s->in_bytes + max_batch * h->dp * 2 + max_batch * 4 + pairs * (s->kp_max * 8 + 4) +
                            s->out_k * 8 + 16 + max_batch * (s->sample_per_query + 2) * sizeof(float) +
                            size_t(h->sms) * groups * vsg::kTcQueries * vsg::tc_buffer_capacity(uint32_t(s->kp_max)) * 8 +
                            max_batch * (3 * sizeof(float) + sizeof(uint32_t) + sizeof(void*)) +  // margins, E, fails
                            max_batch * h->dp * sizeof(float) +                                    // fallback queries
                            max_batch * max_k * 8 * (size_t(s->fb.nsplit) + 1) + size_t(s->fb.nqb) * 4;
    size_t free_b = 0, total_b = 0;
    VSG_CUDA(cudaMemGetInfo(&free_b, &total_b));
    const size_t fit = (free_b / 2) / std::max<size_t>(per_slot, 1);
    if (fit == 0) throw std::bad_alloc();
    const size_t nslots = std::min(slots, fit);
    for (size_t i = 0; i < nslots; ++i) {
      s->slots.emplace_back(new Slot());
      s->build_slot(*s->slots.back());
    }
    vsg_server* raw = s.get();
    s->worker = std::thread([raw] { raw->run(); });
    *out = s.release();
    return VSG_OK;
  } catch (const std::invalid_argument& e) {
    return sfail(VSG_ERR_INVALID, e.what());
  } catch (const std::bad_alloc&) {
    return sfail(VSG_ERR_NOMEM, "not enough device or pinned host memory for one serving slot");
  } catch (const std::exception& e) {
    return sfail(VSG_ERR_CUDA, e.what());
  }
}

void vsg_server_destroy(vsg_server* s) { delete s; }

int vsg_server_submit(vsg_server* s, const float* queries, size_t nq, size_t k, const uint32_t* mask_words,
                      uint32_t* out_ids, float* out_dists, uint64_t* ticket) {
  if (!s || !queries || !out_ids || !out_dists || !ticket) return sfail(VSG_ERR_INVALID, "NULL argument");
  if (nq == 0 || nq > s->cap_q)
    return sfail(VSG_ERR_INVALID, "a request must hold 1.." + std::to_string(s->cap_q) + " queries");
  if (k == 0 || k > s->max_k) return sfail(VSG_ERR_INVALID, "k must be in [1, " + std::to_string(s->max_k) + "]");
  std::unique_ptr<Request> r(new Request());
  r->q = queries;
  r->nq = nq;
  r->k = uint32_t(k);
  r->mask = mask_words;
  r->out_i = out_ids;
  r->out_d = out_dists;
  r->t_submit = Clock::now();
  {
    std::lock_guard<std::mutex> g(s->mu);
    *ticket = s->next_ticket++;
    s->queue.push_back(r.get());
    s->reqs.emplace(*ticket, std::move(r));
    s->n_requests += 1;
  }
  s->cv_work.notify_one();
  return VSG_OK;
}

int vsg_server_wait(vsg_server* s, uint64_t ticket, double timeout_s, double* latency_ms) {
  if (!s) return sfail(VSG_ERR_INVALID, "server is NULL");
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return sfail(VSG_ERR_INVALID, "unknown ticket");
  Request* r = it->second.get();
  const auto deadline = Clock::now() + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(
                                           timeout_s > 0 ? timeout_s : 1e9));
  if (!s->cv_done.wait_until(lk, deadline, [&] { return r->status != -1; }))
    return sfail(VSG_ERR_DEVICE_TIMEOUT, "request not finished before the timeout");
  const int st = r->status;
  const std::string err = r->error;
  if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
  s->reqs.erase(it);
  if (st != VSG_OK) return sfail(st, err);
  return VSG_OK;
}

int vsg_server_stats(vsg_server* s, uint64_t* batches, uint64_t* queries, uint64_t* requests, uint64_t* slots) {
  if (!s) return sfail(VSG_ERR_INVALID, "server is NULL");
  std::lock_guard<std::mutex> g(s->mu);
  if (batches) *batches = s->n_batches;
  if (queries) *queries = s->n_queries;
  if (requests) *requests = s->n_requests;
  if (slots) *slots = s->slots.size();
  return VSG_OK;
}

int vsg_server_uncertified(vsg_server* s, uint64_t* queries) {
  if (!s || !queries) return sfail(VSG_ERR_INVALID, "server or output is NULL");
  std::lock_guard<std::mutex> g(s->mu);
  *queries = s->n_uncertified;
  return VSG_OK;
}

}  // extern "C"
