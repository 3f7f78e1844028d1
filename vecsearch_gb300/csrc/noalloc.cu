// vsg_search_rows_noalloc: the exact scan + merge for callers that must not allocate.
//
// Some callers cannot call cudaMalloc or cudaFree on their search path: a serving thread
// that must not stall (cudaMalloc and cudaFree can synchronise the whole device and take
// milliseconds), a host framework that owns every byte of device memory through its own
// pool and forbids allocations outside it, or a plugin that is handed only the buffers it
// works on. This entry point takes every input and output from the caller and keeps its
// scratch (the per-split top-k lists and the status word) in one fixed array of device
// memory defined in this file.
//
// The array is kNoAllocScratchBytes (4 MiB). Every GPU that loads the library holds it
// until the process exits. All calls share it and it keeps the last call's contents: the
// status word is cleared on each call; the lists are fully rewritten before they are read.
// Calls whose device work overlaps (for example on two streams at once, or from two host
// threads) race on the array and give wrong results.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <string>

#include "../../include/vsg.h"
#include "scan.cuh"

namespace vsg {
void set_last_error(const std::string& msg);  // index.cu: the thread's vsg_last_error() text
}

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(4) << 20;
constexpr size_t kStatusBytes = 256;  // status word, padded to keep the lists 256-byte aligned
constexpr int kMaxDevices = 64;

__device__ __align__(256) static unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_setup_mu;
void* g_scratch_addr[kMaxDevices] = {};  // device address of g_noalloc_scratch, per device
int g_sms[kMaxDevices] = {};
size_t g_smem_optin[kMaxDevices] = {};

size_t ceil_div(size_t a, size_t b) { return (a + b - 1) / b; }

int fail(int code, const std::string& msg) {
  vsg::set_last_error(msg);  // reported by vsg_last_error(), like every other entry point
  return code;
}

// Once per device, with that device current: the array's device address and the limits
// the plan needs. The host-side symbol is only a stand-in and is never passed to a kernel.
int setup_device(int dev) {
  std::lock_guard<std::mutex> g(g_setup_mu);
  if (g_scratch_addr[dev]) return VSG_OK;
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p)
    return fail(VSG_ERR_CUDA, std::string("cudaGetSymbolAddress(g_noalloc_scratch): ") + cudaGetErrorString(e));
  cudaDeviceProp prop;
  e = cudaGetDeviceProperties(&prop, dev);
  if (e != cudaSuccess) return fail(VSG_ERR_CUDA, std::string("cudaGetDeviceProperties: ") + cudaGetErrorString(e));
  g_sms[dev] = prop.multiProcessorCount;
  g_smem_optin[dev] = prop.sharedMemPerBlockOptin;
  g_scratch_addr[dev] = p;
  return VSG_OK;
}

}  // namespace

extern "C" int vsg_search_rows_noalloc(const float* d_rows, size_t n, size_t dim, uint32_t metric,
                                       const float* d_queries, size_t nq, size_t k, uint32_t* d_out_ids,
                                       float* d_out_dists, void* stream) {
  vsg::set_last_error("");
  if (metric != VSG_METRIC_L2 && metric != VSG_METRIC_IP) return fail(VSG_ERR_INVALID, "unknown metric");
  if (k > VSG_MAX_K) return fail(VSG_ERR_INVALID, "k must be <= " + std::to_string(VSG_MAX_K));
  if (nq == 0 || k == 0) return VSG_OK;
  if (n >= VSG_NONE) return fail(VSG_ERR_LENGTH, "at most 2^32 - 2 rows");
  if (dim == 0 || dim % 4 != 0) return fail(VSG_ERR_INVALID, "dim must be a positive multiple of 4");
  if (!d_queries || !d_out_ids || !d_out_dists || (n && !d_rows)) return fail(VSG_ERR_INVALID, "NULL pointer");
  if (reinterpret_cast<uintptr_t>(d_rows) % 16 || reinterpret_cast<uintptr_t>(d_queries) % 16)
    return fail(VSG_ERR_INVALID, "rows and queries must be 16-byte aligned");
  if (n == 0) {  // no rows: every result is missing (VSG_NONE / +inf), as vsg_search fills it
    cudaStream_t s0 = static_cast<cudaStream_t>(stream);
    cudaError_t e0 = vsg::launch_fill_missing(d_out_dists, d_out_ids, nq * k, s0);
    if (e0 == cudaSuccess) e0 = cudaStreamSynchronize(s0);
    if (e0 != cudaSuccess) return fail(VSG_ERR_CUDA, std::string("fill: ") + cudaGetErrorString(e0));
    return VSG_OK;
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(VSG_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return fail(VSG_ERR_INVALID, "device ordinal too large");
  int rc = setup_device(dev);
  if (rc != VSG_OK) return rc;

  // Same plan as the index's search: queries per CTA, rows per tile, ring depth, splits.
  vsg::ScanShape shape{1, 4, metric == VSG_METRIC_L2};
  while (size_t(shape.qb) < nq && shape.qb < 8) shape.qb *= 2;
  uint32_t stages = 0;
  for (int rw : {4, 2, 1}) {
    shape.rw = rw;
    const size_t fixed = vsg::scan_smem_bytes(shape, uint32_t(dim), uint32_t(k), 0);
    const size_t tile = size_t(vsg::kScanWarps) * rw * dim * sizeof(float);
    if (fixed + 2 * tile > g_smem_optin[dev]) continue;
    stages = uint32_t(std::min<size_t>(4, (g_smem_optin[dev] - fixed) / tile));
    break;
  }
  if (stages < 2) return fail(VSG_ERR_INVALID, "dim too large for the scan kernel's shared memory");
  const size_t nqb = ceil_div(nq, size_t(shape.qb));
  size_t want = std::max<size_t>(1, size_t(g_sms[dev]) / nqb);
  want = std::min(want, std::max<size_t>(1, ceil_div(n, 256)));
  const size_t rows_per_split = vsg::split_rows(ceil_div(ceil_div(n, want), 32) * 32, 32);
  const size_t nsplit = ceil_div(n, rows_per_split);
  const size_t parts = nq * nsplit * k;
  if (kStatusBytes + parts * 8 > kNoAllocScratchBytes)
    return fail(VSG_ERR_INVALID, "nq x splits x k = " + std::to_string(parts) +
                                     " top-k entries exceed the 4 MiB scratch (at most " +
                                     std::to_string((kNoAllocScratchBytes - kStatusBytes) / 8) +
                                     "); split the batch");

  unsigned char* base = static_cast<unsigned char*>(g_scratch_addr[dev]);
  int* status = reinterpret_cast<int*>(base);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  e = cudaMemsetAsync(status, 0, sizeof(int), s);
  if (e != cudaSuccess) return fail(VSG_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));

  vsg::ScanArgs a{};
  a.x = d_rows;
  a.q = d_queries;
  a.ldq = uint32_t(dim);
  a.mask = nullptr;
  a.mask_ld = 0;
  a.part_d = reinterpret_cast<float*>(base + kStatusBytes);
  a.part_i = reinterpret_cast<uint32_t*>(base + kStatusBytes + parts * 4);
  a.status = status;
  a.n = uint32_t(n);
  a.dp = uint32_t(dim);
  a.nq = uint32_t(nq);
  a.k = uint32_t(k);
  a.rows_per_split = uint32_t(rows_per_split);
  a.nsplit = uint32_t(nsplit);
  a.stages = stages;
  e = vsg::launch_scan(shape, a, dim3(unsigned(nqb), unsigned(nsplit)), s);
  if (e != cudaSuccess) return fail(VSG_ERR_CUDA, std::string("scan launch: ") + cudaGetErrorString(e));
  vsg::MergeArgs m{a.part_d, a.part_i, d_out_dists, d_out_ids, uint32_t(nq), uint32_t(nsplit), uint32_t(k)};
  e = vsg::launch_merge(m, s);
  if (e != cudaSuccess) return fail(VSG_ERR_CUDA, std::string("merge launch: ") + cudaGetErrorString(e));

  int st = 0;  // read back on the caller's stream into host stack memory: no allocation
  e = cudaMemcpyAsync(&st, status, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail(VSG_ERR_CUDA, std::string("status read: ") + cudaGetErrorString(e));
  if (st != 0) return fail(VSG_ERR_DEVICE_TIMEOUT, "a search kernel's wait ran past its time limit");
  return VSG_OK;
}
