// TEST INFRASTRUCTURE ONLY: a C entry layer over the reference's own CPU
// classes, so that tests and fixture scripts can run the unmodified reference
// (BruteForceIndex, HNSWIndex) through ctypes. oracle/build_ref.py compiles
// this file together with the reference's sources into oracle/_ref/; nothing
// in the product links it.
//
// Reference interfaces used: include/vecsearch/brute_force.h:10-25
// (BruteForceIndex ctor/add/search/search_batch), include/vecsearch/hnsw.h:29-62
// (SearchFilter, HNSWIndex ctor/add/search_batch/save).
#include <cstddef>
#include <cstdint>
#include <exception>

#include "vecsearch/brute_force.h"
#include "vecsearch/hnsw.h"

using vecsearch::BruteForceIndex;
using vecsearch::HNSWIndex;
using vecsearch::Metric;

extern "C" {

void* vsref_bf_create(size_t dim, int metric) {
  try {
    return new BruteForceIndex(dim, metric == 0 ? Metric::L2 : Metric::InnerProduct);
  } catch (const std::exception&) {
    return nullptr;
  }
}

void vsref_bf_destroy(void* h) { delete static_cast<BruteForceIndex*>(h); }

void vsref_bf_add(void* h, const float* x, size_t n) { static_cast<BruteForceIndex*>(h)->add(x, n); }

void vsref_bf_search_batch(void* h, const float* q, size_t nq, size_t k, uint32_t* ids, float* dists,
                           int threads) {
  static_cast<BruteForceIndex*>(h)->search_batch(q, nq, k, ids, dists, threads);
}

// Single-query search(): returns the number of results written (<= k).
size_t vsref_bf_search_one(void* h, const float* q, size_t k, uint32_t* ids, float* dists) {
  auto r = static_cast<BruteForceIndex*>(h)->search(q, k);
  for (size_t j = 0; j < r.size(); ++j) {
    ids[j] = r[j].id;
    dists[j] = r[j].dist;
  }
  return r.size();
}

void* vsref_hnsw_create(size_t dim, size_t max_elements, int metric) {
  try {
    return new HNSWIndex(dim, max_elements, metric == 0 ? Metric::L2 : Metric::InnerProduct);
  } catch (const std::exception&) {
    return nullptr;
  }
}

void vsref_hnsw_destroy(void* h) { delete static_cast<HNSWIndex*>(h); }

int vsref_hnsw_add(void* h, const float* x, size_t n, int threads) {
  try {
    static_cast<HNSWIndex*>(h)->add(x, n, threads);
    return 0;
  } catch (const std::exception&) {
    return -1;
  }
}

int vsref_hnsw_save(void* h, const char* path) {
  try {
    static_cast<HNSWIndex*>(h)->save(path);
    return 0;
  } catch (const std::exception&) {
    return -1;
  }
}

// HNSWIndex::search_batch with a byte mask; n_allowed is counted here the way
// python/bindings.cpp:86-91 counts it.
void vsref_hnsw_search(void* h, const float* q, size_t nq, size_t k, size_t ef, const uint8_t* allowed,
                       size_t exact_below, uint32_t* ids, float* dists, int threads) {
  auto* idx = static_cast<HNSWIndex*>(h);
  vecsearch::SearchFilter f;
  if (allowed) {
    f.allowed = allowed;
    size_t cnt = 0;
    for (size_t i = 0; i < idx->size(); ++i) cnt += allowed[i] != 0;
    f.n_allowed = cnt;
    f.exact_below = exact_below;
  }
  idx->search_batch(q, nq, k, ef, ids, dists, threads, f);
}

}  // extern "C"
