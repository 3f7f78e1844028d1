// Test harness (host only, no CUDA calls) for the index's host logic in
// vecsearch_gb300/csrc/index_impl.cuh and index.cu. One index lives across the commands read
// from stdin, one per line:
//   plan  n dp nq k split_nq sms metric          -> "qb rw stages nqb rows_per_split nsplit"
//   route n dp nq k method masked gather allowed -> "tc_exact tiled" (1 / 0 each)
//   load PATH | save PATH                        -> the status of vsg_autotune_load / _save
//   table method                                 -> "count" then "batch choice split extra" lines
//   splits n blocks align min_rows factor slots  -> "rows_per_split nsplit" of choose_splits
//   reset                                        -> a fresh index (empty tuning tables)
//   set NAME value | get NAME                    -> vsg_set_tunable's status | "status value"
//   below n nq k exact_below pattern             -> "status handled id dist" after
//       vsg_hnsw_exact_below on a byte mask of n rows (pattern 0: none allowed, 1: all, m > 1:
//       every m-th row; -1: no mask; -2: a mask one row short), outputs preset to 7 / 7.0.
//       Only cases that stay on the host: no mask, too many allowed rows, or none allowed.
//   add held m null                              -> vsg_add's status on an index holding `held` rows
//       (only cases that fail or return before a copy: m = 0, NULL rows, too many rows)
//   search n nq k method per_query mask_ld       -> "status id dist" of vsg_search_filtered with a
//       mask when mask_ld > 0 (only cases that stay on the host: bad arguments, nq or k = 0, n = 0)
// (metric 0 = L2, 1 = IP; method as VSG_METHOD_*; allowed < 0 = unknown). The load, save, table,
// set, get, below, add and search commands go through the library's C ABI with this host-built
// index. Built and run by tests/test_host_logic.py.
#include <cstdio>
#include <cstring>
#include <memory>
#include <vector>

#include "../vecsearch_gb300/csrc/index_impl.cuh"

static std::unique_ptr<vsg_index> fresh() {
  std::unique_ptr<vsg_index> h(new vsg_index);  // no stream, events or buffers: nothing here touches the device
  h->sms = 152;
  h->smem_optin = 232448;  // 227 KB, the opt-in shared memory of a GB300 CTA
  return h;
}

int main() {
  std::unique_ptr<vsg_index> idx = fresh();
  char cmd[16];
  while (std::scanf("%15s", cmd) == 1) {
    unsigned long long n, dp, nq, k;
    if (std::strcmp(cmd, "plan") == 0) {
      unsigned long long split_nq, sms, metric;
      if (std::scanf("%llu %llu %llu %llu %llu %llu %llu", &n, &dp, &nq, &k, &split_nq, &sms, &metric) != 7) return 1;
      idx->dim = idx->dp = dp;
      idx->n = n;
      idx->sms = int(sms);
      idx->metric = uint32_t(metric);
      try {
        const auto p = idx->plan(nq, k, false, false, split_nq);
        std::printf("%d %d %u %u %u %u\n", p.shape.qb, p.shape.rw, p.stages, p.nqb, p.rows_per_split, p.nsplit);
      } catch (const std::exception& e) {
        std::printf("error %s\n", e.what());
      }
    } else if (std::strcmp(cmd, "route") == 0) {
      unsigned long long method, masked, gather;
      double allowed;
      if (std::scanf("%llu %llu %llu %llu %llu %llu %llu %lf", &n, &dp, &nq, &k, &method, &masked, &gather,
                     &allowed) != 8)
        return 1;
      idx->dim = idx->dp = dp;
      idx->n = n;
      static const uint32_t word = ~0u;  // stands for a mask; never read
      const uint32_t* m = masked ? &word : nullptr;
      std::printf("%d %d\n", idx->use_tc_exact(uint32_t(method), nq, k, m, gather != 0, allowed) ? 1 : 0,
                  idx->use_tiled(uint32_t(method), nq, m) ? 1 : 0);
    } else if (std::strcmp(cmd, "load") == 0 || std::strcmp(cmd, "save") == 0) {
      char path[4096];
      if (std::scanf("%4095s", path) != 1) return 1;
      const int rc = cmd[0] == 'l' ? vsg_autotune_load(idx.get(), path) : vsg_autotune_save(idx.get(), path);
      std::printf("%d\n", rc);
    } else if (std::strcmp(cmd, "table") == 0) {
      unsigned method;
      if (std::scanf("%u", &method) != 1) return 1;
      size_t count = 64;
      uint32_t batch[64], choice[64], extra[64];
      double split[64];
      if (vsg_autotune_table(idx.get(), method, &count, batch, choice, split, extra) != VSG_OK) return 1;
      std::printf("%zu\n", count);
      for (size_t i = 0; i < count && i < 64; ++i)
        std::printf("%u %u %.3f %u\n", batch[i], choice[i], split[i], extra[i]);
    } else if (std::strcmp(cmd, "set") == 0 || std::strcmp(cmd, "get") == 0) {
      char name[64];
      double v = 0;
      if (std::scanf("%63s", name) != 1) return 1;
      if (cmd[0] == 's') {
        if (std::scanf("%lf", &v) != 1) return 1;
        std::printf("%d\n", vsg_set_tunable(idx.get(), name, v));
      } else {
        const int rc = vsg_get_tunable(idx.get(), name, &v);
        std::printf("%d %.17g\n", rc, v);
      }
    } else if (std::strcmp(cmd, "below") == 0) {
      unsigned long long eb;
      long long pattern;
      if (std::scanf("%llu %llu %llu %llu %lld", &n, &nq, &k, &eb, &pattern) != 5) return 1;
      idx->n = n;
      idx->dim = idx->dp = 8;
      std::vector<uint8_t> mask(n + 1, 0);
      for (size_t i = 0; i < n; ++i) mask[i] = pattern == 1 || (pattern > 1 && i % size_t(pattern) == 0);
      std::vector<float> q(nq * 8 + 8, 0.f);
      std::vector<uint32_t> ids(nq * k + 1, 7u);
      std::vector<float> d(nq * k + 1, 7.f);
      int handled = -1;
      const int rc = vsg_hnsw_exact_below(idx.get(), q.data(), nq, k, pattern == -1 ? nullptr : mask.data(),
                                          pattern == -2 ? n - 1 : n, eb, ids.data(), d.data(), &handled);
      std::printf("%d %d %u %g\n", rc, handled, ids[0], double(d[0]));
    } else if (std::strcmp(cmd, "add") == 0) {
      unsigned long long held, m, null_rows;
      if (std::scanf("%llu %llu %llu", &held, &m, &null_rows) != 3) return 1;
      idx->n = held;
      idx->dim = idx->dp = 8;
      float row[8] = {0};
      std::printf("%d\n", vsg_add(idx.get(), null_rows ? nullptr : row, m));
    } else if (std::strcmp(cmd, "search") == 0) {
      unsigned long long method, per_query, mask_ld;
      if (std::scanf("%llu %llu %llu %llu %llu %llu", &n, &nq, &k, &method, &per_query, &mask_ld) != 6) return 1;
      idx->n = n;
      idx->dim = idx->dp = 8;
      std::vector<float> q(nq * 8 + 8, 0.f);
      std::vector<uint32_t> words(nq * (mask_ld + 1) + 1, ~0u);
      std::vector<uint32_t> ids(nq * k + 1, 7u);
      std::vector<float> d(nq * k + 1, 7.f);
      const int rc = vsg_search_filtered(idx.get(), q.data(), nq, k, mask_ld ? words.data() : nullptr, int(per_query),
                                         mask_ld, ids.data(), d.data(), uint32_t(method));
      std::printf("%d %u %g\n", rc, ids[0], double(d[0]));
    } else if (std::strcmp(cmd, "splits") == 0) {
      unsigned long long blocks, align, min_rows, slots;
      double factor;
      if (std::scanf("%llu %llu %llu %llu %lf %llu", &n, &blocks, &align, &min_rows, &factor, &slots) != 6) return 1;
      idx->n = n;
      uint32_t rps = 0, nsplit = 0;
      idx->choose_splits(blocks, align, min_rows, &rps, &nsplit, factor, slots);
      std::printf("%u %u\n", rps, nsplit);
    } else if (std::strcmp(cmd, "reset") == 0) {
      idx = fresh();
    } else {
      return 1;
    }
    std::fflush(stdout);
  }
  return 0;
}
