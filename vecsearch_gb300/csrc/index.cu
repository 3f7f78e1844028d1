// Host side of the GB300 exact index: device-resident rows, search planning,
// kernel launches and the C ABI of include/vsg.h.
//
// Mirrors the reference's GpuBruteForceIndex (src/gpu_brute_force.cu:343-488):
// grow-only device storage with zero-padded rows, one mutex per index, CUDA
// errors surfaced as runtime errors with the failing expression. Unlike the
// reference, the search never materialises a query x row distance block: one
// fused scan kernel per search plus one merge kernel, on the index's own
// stream, with queries in and results out through pinned staging buffers.
#include "index_impl.cuh"

#include <cstdio>

namespace vsg_detail {
thread_local std::string g_last_error;
}  // namespace vsg_detail

namespace vsg {
// The calling thread's vsg_last_error() text, for entry points defined in other files.
void set_last_error(const std::string& msg) { vsg_detail::g_last_error = msg; }
}  // namespace vsg


namespace {

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

template <class F>
int guarded(F&& f) {
  try {
    g_last_error.clear();
    f();
    return VSG_OK;
  } catch (const std::invalid_argument& e) {
    return fail(VSG_ERR_INVALID, e.what());
  } catch (const std::length_error& e) {
    return fail(VSG_ERR_LENGTH, e.what());
  } catch (const DeviceTimeout& e) {
    return fail(VSG_ERR_DEVICE_TIMEOUT, e.what());
  } catch (const std::bad_alloc&) {
    return fail(VSG_ERR_NOMEM, "out of device or pinned host memory");
  } catch (const std::exception& e) {
    return fail(VSG_ERR_CUDA, e.what());
  } catch (...) {
    return fail(VSG_ERR_CUDA, "unknown error");
  }
}

void check_method(uint32_t method) {
  if (method > VSG_METHOD_FP8)
    throw std::invalid_argument("method must be 'auto', 'naive', 'skinny', 'tiled', 'bf16', 'tc_exact' or 'fp8'");
}

void check_k(size_t k) {
  if (k > VSG_MAX_K) throw std::invalid_argument("k must be <= " + std::to_string(VSG_MAX_K));
}

void fill_missing_host(uint32_t* ids, float* dists, size_t count) {
  std::fill(ids, ids + count, VSG_NONE);
  std::fill(dists, dists + count, __builtin_inff());
}

}  // namespace

extern "C" {

int vsg_cuda_available(void) {
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return count > 0 ? 1 : 0;
}

const char* vsg_last_error(void) { return g_last_error.c_str(); }

int vsg_create(size_t dim, uint32_t metric, int device, vsg_index** out) {
  if (!out) return fail(VSG_ERR_INVALID, "out is NULL");
  *out = nullptr;
  return guarded([&] {
    if (dim == 0) throw std::invalid_argument("dim must be > 0");
    if (metric != VSG_METRIC_L2 && metric != VSG_METRIC_IP)
      throw std::invalid_argument("metric must be 'l2', 'ip' or 'cosine' (cosine expects normalized vectors)");
    auto* h = new vsg_index();
    try {
      h->dim = dim;
      h->dp = (dim + 7) / 8 * 8;
      h->metric = metric;
      h->device = device;
      VSG_CUDA(cudaSetDevice(device));
      cudaDeviceProp prop;
      VSG_CUDA(cudaGetDeviceProperties(&prop, device));
      h->sms = prop.multiProcessorCount;
      h->smem_optin = prop.sharedMemPerBlockOptin;
      VSG_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
      VSG_CUDA(cudaEventCreateWithFlags(&h->done, cudaEventDisableTiming));
      VSG_CUDA(cudaEventRecord(h->done, h->stream));
      h->reserve_results(1, 1);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}

void vsg_destroy(vsg_index* h) { delete h; }

int vsg_add(vsg_index* h, const float* rows, size_t m) {
  if (!h) return fail(VSG_ERR_INVALID, "index is NULL");
  return guarded([&] {
    std::lock_guard<std::mutex> g(h->mu);
    if (m == 0) return;
    if (!rows) throw std::invalid_argument("rows is NULL");
    if (h->n + m >= VSG_NONE) throw std::length_error("GpuBruteForceIndex holds at most 2^32 - 2 vectors");
    VSG_CUDA(cudaSetDevice(h->device));
    VSG_CUDA(cudaStreamWaitEvent(h->stream, h->done, 0));
    if (h->n + m > h->cap) {
      const size_t cap = std::max({h->n + m, h->cap * 2, size_t(1024)});
      h->x.reserve(cap * h->dp * sizeof(float), h->n * h->dp * sizeof(float), h->stream);
      h->cap = cap;
    }
    float* dst = static_cast<float*>(h->x.get()) + h->n * h->dp;
    VSG_CUDA(cudaMemcpy2DAsync(dst, h->dp * sizeof(float), rows, h->dim * sizeof(float), h->dim * sizeof(float), m,
                               cudaMemcpyHostToDevice, h->stream));
    VSG_CUDA(cudaEventRecord(h->done, h->stream));
    VSG_CUDA(cudaStreamSynchronize(h->stream));
    h->n += m;
    ++h->config_gen;
  });
}

int vsg_search(vsg_index* h, const float* queries, size_t nq, size_t k, uint32_t* out_ids, float* out_dists,
               uint32_t method) {
  return vsg_search_filtered(h, queries, nq, k, nullptr, 0, 0, out_ids, out_dists, method);
}

int vsg_search_filtered(vsg_index* h, const float* queries, size_t nq, size_t k, const uint32_t* mask_words,
                        int per_query, size_t mask_ld, uint32_t* out_ids, float* out_dists, uint32_t method) {
  if (!h) return fail(VSG_ERR_INVALID, "index is NULL");
  return guarded([&] {
    check_method(method);
    check_k(k);
    if (nq == 0 || k == 0) return;
    if (!queries || !out_ids || !out_dists) throw std::invalid_argument("NULL query or output pointer");
    std::lock_guard<std::mutex> g(h->mu);
    if (mask_words && per_query && mask_ld < ceil_div(h->n, 32))
      throw std::invalid_argument("mask_ld must be >= ceil(size / 32)");
    if (h->n == 0) {
      fill_missing_host(out_ids, out_dists, nq * k);
      return;
    }
    h->search_host(queries, nq, k, mask_words, mask_words && per_query, mask_ld, out_ids, out_dists, method);
  });
}

int vsg_hnsw_exact_below(vsg_index* h, const float* queries, size_t nq, size_t k, const uint8_t* allowed,
                         size_t allowed_len, size_t exact_below, uint32_t* out_ids, float* out_dists,
                         int* handled) {
  if (!h || !handled) return fail(VSG_ERR_INVALID, "index or handled is NULL");
  *handled = 0;
  return guarded([&] {
    check_k(k);
    if (!allowed) return;  // no filter: the graph path (hnsw.cpp:329-333)
    std::lock_guard<std::mutex> g(h->mu);
    if (allowed_len != h->n) throw std::invalid_argument("filter must be a 1-D bool array of length " +
                                                         std::to_string(h->n));
    size_t n_allowed = 0;
    for (size_t i = 0; i < allowed_len; ++i) n_allowed += allowed[i] != 0;
    if (n_allowed != 0 && n_allowed > exact_below) return;  // graph path
    *handled = 1;
    if (nq == 0 || k == 0) return;
    if (!queries || !out_ids || !out_dists) throw std::invalid_argument("NULL query or output pointer");
    if (n_allowed == 0) {
      fill_missing_host(out_ids, out_dists, nq * k);
      return;
    }
    std::vector<uint32_t> words(ceil_div(h->n, 32), 0u);
    for (size_t i = 0; i < allowed_len; ++i)
      if (allowed[i]) words[i >> 5] |= 1u << (i & 31);
    h->search_host(queries, nq, k, words.data(), false, 0, out_ids, out_dists);
  });
}

int vsg_search_device(vsg_index* h, const float* d_queries, size_t ldq, size_t nq, size_t k,
                      const uint32_t* d_mask_words, int per_query, size_t mask_ld, uint32_t* d_out_ids,
                      float* d_out_dists, uint32_t method, void* stream) {
  if (!h) return fail(VSG_ERR_INVALID, "index is NULL");
  return guarded([&] {
    check_method(method);
    check_k(k);
    if (nq == 0 || k == 0) return;
    if (!d_queries || !d_out_ids || !d_out_dists) throw std::invalid_argument("NULL query or output pointer");
    if (ldq < h->dim) throw std::invalid_argument("ldq must be >= dim");
    std::lock_guard<std::mutex> g(h->mu);
    if (d_mask_words && per_query && mask_ld < ceil_div(h->n, 32))
      throw std::invalid_argument("mask_ld must be >= ceil(size / 32)");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    VSG_CUDA(cudaSetDevice(h->device));
    VSG_CUDA(cudaStreamWaitEvent(s, h->done, 0));
    if (h->n == 0) {
      VSG_CUDA(vsg::launch_fill_missing(d_out_dists, d_out_ids, nq * k, s));
    } else {
      const float* dq = d_queries;
      size_t ld = ldq;
      // The kernel reads dp floats per query row and 16-byte chunks: use the caller's rows in
      // place only when they need no zero padding and are aligned; else repack (pads stay zero).
      const bool direct = h->dim == h->dp && ldq % 4 == 0 && reinterpret_cast<uintptr_t>(d_queries) % 16 == 0;
      if (!direct) {
        h->q.reserve(nq * h->dp * sizeof(float), 0, h->stream);
        VSG_CUDA(cudaMemcpy2DAsync(h->q.get(), h->dp * sizeof(float), d_queries, ldq * sizeof(float),
                                   h->dim * sizeof(float), nq, cudaMemcpyDeviceToDevice, s));
        dq = static_cast<const float*>(h->q.get());
        ld = h->dp;
      }
      // Device masks cannot be counted here without a sync: gather unless it is switched off.
      if (method == VSG_METHOD_BF16 && !d_mask_words && k <= size_t(vsg::kTcMaxShortlist)) h->ensure_bf16();
      h->enqueue(dq, ld, nq, k, d_mask_words, d_mask_words && per_query, mask_ld, h->gather_max_fraction > 0.0,
                 d_out_ids, d_out_dists, s, method);
    }
    VSG_CUDA(cudaEventRecord(h->done, s));
  });
}

int vsg_sync(vsg_index* h) {
  if (!h) return fail(VSG_ERR_INVALID, "index is NULL");
  return guarded([&] {
    std::lock_guard<std::mutex> g(h->mu);
    VSG_CUDA(cudaSetDevice(h->device));
    VSG_CUDA(cudaStreamWaitEvent(h->stream, h->done, 0));
    h->check_status_sync();
  });
}

size_t vsg_size(const vsg_index* h) { return h ? h->n : 0; }
size_t vsg_dim(const vsg_index* h) { return h ? h->dim : 0; }
uint32_t vsg_metric(const vsg_index* h) { return h ? h->metric : 0; }

const float* vsg_device_rows(const vsg_index* h, size_t* padded_dim) {
  if (!h) return nullptr;
  if (padded_dim) *padded_dim = h->dp;
  return static_cast<const float*>(h->x.get());
}

int vsg_set_tunable(vsg_index* h, const char* name, double value) {
  if (!h || !name) return fail(VSG_ERR_INVALID, "index or name is NULL");
  return guarded([&] {
    std::lock_guard<std::mutex> g(h->mu);
    const std::string nm(name);
    if (nm == "gather_max_fraction") {
      if (!(value >= 0.0 && value <= 1.0)) throw std::invalid_argument("gather_max_fraction must be in [0, 1]");
      h->gather_max_fraction = value;
    } else if (nm == "tiled_min_batch") {
      if (!(value >= 1.0)) throw std::invalid_argument("tiled_min_batch must be >= 1");
      h->tiled_min_batch = value;
    } else if (nm == "shortlist_oversample") {
      if (!(value >= 1.0)) throw std::invalid_argument("shortlist_oversample must be >= 1");
      h->shortlist_oversample = value;
    } else if (nm == "tc_exact_min_batch") {
      if (!(value >= 1.0)) throw std::invalid_argument("tc_exact_min_batch must be >= 1");
      h->tc_exact_min_batch = value;
    } else if (nm == "sample_rows") {
      if (!(value >= 0.0 && value <= 1048576.0)) throw std::invalid_argument("sample_rows must be in [0, 2^20]");
      h->sample_rows = value;
    } else if (nm == "tc_exact_min_elements") {
      if (!(value >= 0.0)) throw std::invalid_argument("tc_exact_min_elements must be >= 0");
      h->tc_exact_min_elements = value;
    } else if (nm == "cert_margin") {
      if (!(value >= 1.0 && value <= 100.0)) throw std::invalid_argument("cert_margin must be in [1, 100]");
      h->cert_margin = value;
    } else if (nm == "fallback_split_queries") {
      if (!(value >= 0.0 && value <= 1048576.0))
        throw std::invalid_argument("fallback_split_queries must be in [0, 2^20]");
      h->fallback_split_queries = std::floor(value);
    } else if (nm == "wait_limit_s") {
      if (!(value >= 1e-6 && value <= 60.0)) throw std::invalid_argument("wait_limit_s must be in [1e-6, 60]");
      h->wait_limit_s = value;
    } else if (nm == "test_stall_wait") {
      if (value != 0.0 && value != 1.0) throw std::invalid_argument("test_stall_wait must be 0 or 1");
      h->stall_next = value != 0.0;
    } else if (nm == "host_graph_max_batch") {
      if (!(value >= 0.0 && value <= 1024.0)) throw std::invalid_argument("host_graph_max_batch must be in [0, 1024]");
      h->host_graph_max_batch = std::floor(value);
    } else if (nm == "cert_fp8_max_batch") {
      if (!(value >= 0.0 && value <= 1048576.0)) throw std::invalid_argument("cert_fp8_max_batch must be in [0, 2^20]");
      h->cert_fp8_max_batch = std::floor(value);
    } else if (nm == "cert_fp8_sample_rows") {
      if (!(value >= 0.0 && value <= 1048576.0)) throw std::invalid_argument("cert_fp8_sample_rows must be in [0, 2^20]");
      h->cert_fp8_sample_rows = std::floor(value);
    } else if (nm == "cert_prefetch_max_batch") {
      if (!(value >= 0.0 && value <= 1048576.0)) throw std::invalid_argument("cert_prefetch_max_batch must be in [0, 2^20]");
      h->cert_prefetch_max_batch = std::floor(value);
    } else if (nm == "finish_cluster" || nm == "finish_cluster_one") {
      if (!(value >= 1.0 && value <= 16.0)) throw std::invalid_argument(nm + " must be in [1, 16]");
      (nm == "finish_cluster" ? h->finish_cluster : h->finish_cluster_one) = std::floor(value);
    } else if (nm == "host_graph_direct") {
      if (value != 0.0 && value != 1.0) throw std::invalid_argument("host_graph_direct must be 0 or 1");
      h->host_graph_direct = value;
    } else {
      throw std::invalid_argument("unknown tunable '" + nm + "'");
    }
    ++h->config_gen;  // a captured search graph may hold the old value
  });
}

int vsg_get_tunable(vsg_index* h, const char* name, double* value) {
  if (!h || !name || !value) return fail(VSG_ERR_INVALID, "index, name or value is NULL");
  return guarded([&] {
    std::lock_guard<std::mutex> g(h->mu);
    const std::string nm(name);
    if (nm == "gather_max_fraction") *value = h->gather_max_fraction;
    else if (nm == "tiled_min_batch") *value = h->tiled_min_batch;
    else if (nm == "shortlist_oversample") *value = h->shortlist_oversample;
    else if (nm == "sample_rows") *value = h->sample_rows;
    else if (nm == "tc_exact_min_batch") *value = h->tc_exact_min_batch;
    else if (nm == "cert_margin") *value = h->cert_margin;
    else if (nm == "tc_exact_min_elements") *value = h->tc_exact_min_elements;
    else if (nm == "fallback_split_queries") *value = h->fallback_split_queries;
    else if (nm == "wait_limit_s") *value = h->wait_limit_s;
    else if (nm == "test_stall_wait") *value = h->stall_next ? 1.0 : 0.0;
    else if (nm == "host_graph_max_batch") *value = h->host_graph_max_batch;
    else if (nm == "host_graph_direct") *value = h->host_graph_direct;
    else if (nm == "cert_fp8_max_batch") *value = h->cert_fp8_max_batch;
    else if (nm == "cert_fp8_sample_rows") *value = h->cert_fp8_sample_rows;
    else if (nm == "cert_prefetch_max_batch") *value = h->cert_prefetch_max_batch;
    else if (nm == "finish_cluster") *value = h->finish_cluster;
    else if (nm == "finish_cluster_one") *value = h->finish_cluster_one;
    else throw std::invalid_argument("unknown tunable '" + nm + "'");
  });
}

int vsg_autotune_with_queries(vsg_index* h, const float* queries, size_t nq, const size_t* batches, size_t count,
                              size_t k, uint32_t method) {
  if (!h || (!batches && count)) return fail(VSG_ERR_INVALID, "index or batches is NULL");
  return guarded([&] {
    if (method != VSG_METHOD_AUTO && method != VSG_METHOD_BF16)
      throw std::invalid_argument("the tuner covers method auto (exact methods) and bf16");
    if (nq && !queries) throw std::invalid_argument("queries is NULL");
    std::lock_guard<std::mutex> g(h->mu);
    VSG_CUDA(cudaSetDevice(h->device));
    VSG_CUDA(cudaStreamWaitEvent(h->stream, h->done, 0));
    h->autotune(batches, count, k, method, queries, nq);
    ++h->config_gen;
    VSG_CUDA(cudaEventRecord(h->done, h->stream));
  });
}

int vsg_autotune(vsg_index* h, const size_t* batches, size_t count, size_t k, uint32_t method) {
  return vsg_autotune_with_queries(h, nullptr, 0, batches, count, k, method);
}

int vsg_autotune_table(vsg_index* h, uint32_t method, size_t* count, uint32_t* batch, uint32_t* choice,
                       double* split, uint32_t* exact_kp) {
  if (!h || !count) return fail(VSG_ERR_INVALID, "index or count is NULL");
  return guarded([&] {
    std::lock_guard<std::mutex> g(h->mu);
    const auto& t = method == VSG_METHOD_BF16 ? h->tune_bf16 : h->tune_plain;
    const size_t cap = *count;
    *count = t.size();
    for (size_t i = 0; i < t.size() && i < cap; ++i) {
      if (batch) batch[i] = t[i].batch;
      if (choice) choice[i] = method == VSG_METHOD_BF16 ? t[i].sample : t[i].kernel;
      if (split) split[i] = t[i].split;
      if (exact_kp) exact_kp[i] = method == VSG_METHOD_BF16 ? 0u : t[i].exact_kp;
    }
  });
}

int vsg_autotune_save(vsg_index* h, const char* path) {
  if (!h || !path) return fail(VSG_ERR_INVALID, "index or path is NULL");
  return guarded([&] {
    std::lock_guard<std::mutex> g(h->mu);
    FILE* f = std::fopen(path, "w");
    if (!f) throw std::runtime_error(std::string("cannot open ") + path);
    std::fprintf(f, "vsg-tuning 2 dim %zu rows %zu metric %u sms %d\n", h->dim, h->n, h->metric, h->sms);
    for (const auto& e : h->tune_plain)
      std::fprintf(f, "plain %u %u %.3f %u\n", e.batch, e.kernel, e.split, e.exact_kp);
    for (const auto& e : h->tune_bf16) std::fprintf(f, "bf16 %u %u\n", e.batch, e.sample);
    const bool ok = std::fclose(f) == 0;
    if (!ok) throw std::runtime_error(std::string("write failed: ") + path);
  });
}

int vsg_autotune_load(vsg_index* h, const char* path) {
  if (!h || !path) return fail(VSG_ERR_INVALID, "index or path is NULL");
  return guarded([&] {
    FILE* f = std::fopen(path, "r");
    if (!f) throw std::invalid_argument(std::string("cannot open ") + path);
    std::vector<vsg_index::TuneEntry> plain, bf16;
    char line[256];
    bool header = false;
    while (std::fgets(line, sizeof line, f)) {
      vsg_index::TuneEntry e;
      unsigned b = 0, c = 0;
      double sp = 1.0;
      // Version 1 files carried a third bf16 column (CTAs per cluster); it is read and ignored.
      if (std::strncmp(line, "vsg-tuning 1", 12) == 0 || std::strncmp(line, "vsg-tuning 2", 12) == 0) {
        header = true;
      } else if (std::sscanf(line, "plain %u %u %lf", &b, &c, &sp) == 3 && c <= 2 && sp > 0) {
        unsigned kp = 0;
        std::sscanf(line, "plain %*u %*u %*f %u", &kp);  // first-pass shortlist of kernel 2 (optional)
        e.batch = b;
        e.kernel = c;
        e.split = sp;
        e.exact_kp = kp <= 128 ? kp : 0;
        plain.push_back(e);
      } else if (std::strncmp(line, "bf16 ", 5) == 0) {
        if (std::sscanf(line, "bf16 %u %u", &b, &c) == 2 && c <= (1u << 20)) {
          e.batch = b;
          e.sample = c;
          bf16.push_back(e);
        }
      }
    }
    std::fclose(f);
    if (!header) throw std::invalid_argument(std::string(path) + " is not a vsg tuning file");
    std::lock_guard<std::mutex> g(h->mu);
    h->tune_plain = plain;
    h->tune_bf16 = bf16;
    ++h->config_gen;
  });
}

int vsg_tc_exact_stats(vsg_index* h, uint64_t* queries, uint64_t* second, uint64_t* fallbacks) {
  if (!h || !queries || !second || !fallbacks) return fail(VSG_ERR_INVALID, "index or output is NULL");
  return guarded([&] {
    std::lock_guard<std::mutex> g(h->mu);
    VSG_CUDA(cudaSetDevice(h->device));
    const uint64_t scanned = h->tc_stats_sync();
    *queries = h->tc_exact_queries;
    *second = scanned;  // uncertified after the one shortlist pass (k' = 120 is the first pass)
    *fallbacks = scanned;
  });
}

int vsg_tiled_stats(vsg_index* h, uint64_t* queries, uint64_t* fallbacks) {
  if (!h || !queries || !fallbacks) return fail(VSG_ERR_INVALID, "index or output is NULL");
  return guarded([&] {
    std::lock_guard<std::mutex> g(h->mu);
    VSG_CUDA(cudaSetDevice(h->device));
    *fallbacks = h->tiled_stats_sync();
    *queries = h->tiled_queries;
  });
}

int vsg_kernel_launches(vsg_index* h, uint64_t* launches) {
  if (!h || !launches) return fail(VSG_ERR_INVALID, "index or output is NULL");
  return guarded([&] {
    std::lock_guard<std::mutex> g(h->mu);
    *launches = h->kernel_launches;
  });
}

int vsg_profile_enable(vsg_index* h, int enable) {
  if (!h) return fail(VSG_ERR_INVALID, "index is NULL");
  return guarded([&] {
    std::lock_guard<std::mutex> g(h->mu);
    VSG_CUDA(cudaSetDevice(h->device));
    h->read_timings(nullptr, nullptr, nullptr);
    h->profiling = enable != 0;
  });
}

int vsg_profile_read(vsg_index* h, double* scan_ms, double* merge_ms, size_t* searches) {
  if (!h) return fail(VSG_ERR_INVALID, "index is NULL");
  return guarded([&] {
    std::lock_guard<std::mutex> g(h->mu);
    VSG_CUDA(cudaSetDevice(h->device));
    h->read_timings(scan_ms, merge_ms, searches);
  });
}

}  // extern "C"
