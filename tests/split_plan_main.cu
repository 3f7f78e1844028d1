// Test harness (host only, no CUDA calls) for the index's planning logic in
// vecsearch_gb300/csrc/index_impl.cuh. Reads cases from stdin, one per line:
//   plan  n dp nq k split_nq sms metric         -> "qb rw stages nqb rows_per_split nsplit"
//   route n dp nq k method masked gather allowed -> "tc_exact tiled" (1 / 0 each)
// (metric 0 = L2, 1 = IP; method as VSG_METHOD_*; allowed < 0 = unknown). Built and run by
// tests/test_split_plan.py.
#include <cstdio>
#include <cstring>

#include "../vecsearch_gb300/csrc/index_impl.cuh"

int main() {
  char cmd[16];
  while (std::scanf("%15s", cmd) == 1) {
    vsg_index idx;  // no stream, events or buffers: nothing here touches the device
    idx.sms = 152;
    idx.smem_optin = 232448;  // 227 KB, the opt-in shared memory of a GB300 CTA
    unsigned long long n, dp, nq, k;
    if (std::strcmp(cmd, "plan") == 0) {
      unsigned long long split_nq, sms, metric;
      if (std::scanf("%llu %llu %llu %llu %llu %llu %llu", &n, &dp, &nq, &k, &split_nq, &sms, &metric) != 7) return 1;
      idx.dim = idx.dp = dp;
      idx.n = n;
      idx.sms = int(sms);
      idx.metric = uint32_t(metric);
      try {
        const auto p = idx.plan(nq, k, false, false, split_nq);
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
      idx.dim = idx.dp = dp;
      idx.n = n;
      static const uint32_t word = ~0u;  // stands for a mask; never read
      const uint32_t* m = masked ? &word : nullptr;
      std::printf("%d %d\n", idx.use_tc_exact(uint32_t(method), nq, k, m, gather != 0, allowed) ? 1 : 0,
                  idx.use_tiled(uint32_t(method), nq, m) ? 1 : 0);
    } else {
      return 1;
    }
  }
  return 0;
}
