// Test harness (host only, no CUDA calls): prints the streaming scan's launch plan for the
// cases read from stdin, one per line: "n dp nq k split_nq sms metric" (metric 0 = L2, 1 = IP).
// Output per case: "qb rw stages nqb rows_per_split nsplit". Built and run by
// tests/test_split_plan.py against the library's own plan() (vecsearch_gb300/csrc/index_impl.cuh).
#include <cstdio>

#include "../vecsearch_gb300/csrc/index_impl.cuh"

int main() {
  unsigned long long n, dp, nq, k, split_nq, sms, metric;
  while (std::scanf("%llu %llu %llu %llu %llu %llu %llu", &n, &dp, &nq, &k, &split_nq, &sms, &metric) == 7) {
    vsg_index idx;  // no stream, events or buffers: nothing here touches the device
    idx.dim = dp;
    idx.dp = dp;
    idx.n = n;
    idx.sms = int(sms);
    idx.metric = uint32_t(metric);
    idx.smem_optin = 232448;  // 227 KB, the opt-in shared memory of a GB300 CTA
    try {
      const auto p = idx.plan(nq, k, false, false, split_nq);
      std::printf("%d %d %u %u %u %u\n", p.shape.qb, p.shape.rw, p.stages, p.nqb, p.rows_per_split, p.nsplit);
    } catch (const std::exception& e) {
      std::printf("error %s\n", e.what());
    }
  }
  return 0;
}
