// vsg_insert_candidates: exact neighbour candidates for an HNSW build, in insertion order.
//
// The reference builds its graph one node at a time (HNSWIndex::insert, src/hnsw.cpp:247-309,
// called in id order by HNSWIndex::add, :311-): node i searches the graph of nodes 0 .. i-1 for
// ef_construction candidates (search_layer) and keeps M of them (select_neighbors). Here the
// candidate step is exact and batched on the GPU: row i's list is the k nearest of rows
// 0 .. i-1 by (dist, id). Rows go through in batches [i0, i1):
//   * against rows 0 .. i0-1: one index that grows with the build (every row of it comes before
//     the batch), one unfiltered search of the whole batch;
//   * against the batch's own earlier rows: a second index holding the batch, searched with one
//     prefix filter per query (query j allows local rows < j);
//   * the two sorted lists merge on the host by (dist, id), then the batch is added.
// Every exact method returns the scan kernel's distances bit for bit, and a (query, row) distance
// depends only on the two rows (not on the index or batch), so the merged list equals one exact
// search over rows 0 .. i-1. Host code only: it drives the library through its own C ABI.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/vsg.h"

namespace vsg {
void set_last_error(const std::string& msg);  // index.cu: the thread's vsg_last_error() text
}

namespace {

struct Owned {
  vsg_index* h = nullptr;
  ~Owned() { vsg_destroy(h); }
};

// Merges two lists sorted by (dist, id) (missing entries VSG_NONE / +inf last) into out (k).
void merge_lists(const uint32_t* ai, const float* ad, const uint32_t* bi, const float* bd, size_t k,
                 uint32_t* oi, float* od) {
  size_t a = 0, b = 0;
  for (size_t j = 0; j < k; ++j) {
    const bool a_ok = a < k && ai[a] != VSG_NONE;
    const bool b_ok = b < k && bi[b] != VSG_NONE;
    bool take_a;
    if (a_ok && b_ok)
      take_a = ad[a] < bd[b] || (ad[a] == bd[b] && ai[a] < bi[b]);
    else
      take_a = a_ok;
    if (a_ok || b_ok) {
      oi[j] = take_a ? ai[a] : bi[b];
      od[j] = take_a ? ad[a] : bd[b];
      (take_a ? a : b) += 1;
    } else {
      oi[j] = VSG_NONE;
      od[j] = __builtin_inff();
    }
  }
}

}  // namespace

extern "C" int vsg_insert_candidates(const float* rows, size_t n, size_t dim, uint32_t metric, int device, size_t k,
                                     size_t batch, uint32_t* out_ids, float* out_dists) {
  if (n == 0 || k == 0) return VSG_OK;
  if (!rows || !out_ids || !out_dists) {
    vsg::set_last_error("NULL rows or output pointer");
    return VSG_ERR_INVALID;
  }
  if (k > VSG_MAX_K) {
    vsg::set_last_error("k must be <= " + std::to_string(VSG_MAX_K));
    return VSG_ERR_INVALID;
  }
  if (batch == 0) batch = 1024;
  Owned built, local;
  int rc = vsg_create(dim, metric, device, &built.h);
  if (rc != VSG_OK) return rc;
  std::vector<uint32_t> pi, li, mask;
  std::vector<float> pd, ld;
  for (size_t i0 = 0; i0 < n; i0 += batch) {
    const size_t m = std::min(batch, n - i0);
    const float* q = rows + i0 * dim;
    pi.assign(m * k, VSG_NONE);
    pd.assign(m * k, __builtin_inff());
    if (i0 > 0) {  // every row of the grown index comes before this batch
      rc = vsg_search(built.h, q, m, k, pi.data(), pd.data(), VSG_METHOD_AUTO);
      if (rc != VSG_OK) return rc;
    }
    // The batch's own earlier rows: query j allows local rows 0 .. j-1.
    const size_t words = (m + 31) / 32;
    mask.assign(m * words, 0u);
    for (size_t j = 0; j < m; ++j) {
      uint32_t* w = mask.data() + j * words;
      for (size_t r = 0; r < j; r += 32) w[r / 32] = j - r >= 32 ? 0xFFFFFFFFu : (1u << (j - r)) - 1u;
    }
    vsg_destroy(local.h);
    local.h = nullptr;
    rc = vsg_create(dim, metric, device, &local.h);
    if (rc == VSG_OK) rc = vsg_add(local.h, q, m);
    li.assign(m * k, VSG_NONE);
    ld.assign(m * k, __builtin_inff());
    if (rc == VSG_OK && m > 1)
      rc = vsg_search_filtered(local.h, q, m, k, mask.data(), 1, words, li.data(), ld.data(), VSG_METHOD_AUTO);
    if (rc != VSG_OK) return rc;
    for (size_t j = 0; j < m * k; ++j)
      if (li[j] != VSG_NONE) li[j] += uint32_t(i0);
    for (size_t j = 0; j < m; ++j)
      merge_lists(pi.data() + j * k, pd.data() + j * k, li.data() + j * k, ld.data() + j * k, k,
                  out_ids + (i0 + j) * k, out_dists + (i0 + j) * k);
    rc = vsg_add(built.h, q, m);
    if (rc != VSG_OK) return rc;
  }
  return VSG_OK;
}
