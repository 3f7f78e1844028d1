// _vecsearch_gb300: a pybind11 module with the reference's GPU class surface over the C ABI.
//
// The reference exposes GpuBruteForceIndex and cuda_available() from its pybind11 module
// (python/bindings.cpp:151-197, :199-205). This module has the same class, constructor,
// methods, argument names, defaults, coercions and exceptions, backed by libvsg_gb300.so
// through include/vsg.h, so the reference's Python package can import it in place of its own
// class (`GpuBruteForceIndex = _vecsearch_gb300.GpuBruteForceIndex`). Additions, all optional:
// search's `filter` (None, a 1-D bool/uint8 array over the rows, or a 2-D one with one row per
// query), the methods "bf16", "tc_exact" and "fp8", and the `metric` property.
//
// Inputs are coerced to contiguous float32 / uint8 (forcecast) as the reference's are; the GIL
// is released around add and search (bindings.cpp:161, :180). Status codes become the
// reference's exception types: VSG_ERR_INVALID / VSG_ERR_LENGTH -> ValueError, VSG_ERR_NOMEM ->
// MemoryError, anything else -> RuntimeError (a kernel's wait that ran out is reported with
// its message, as vecsearch_gb300.DeviceTimeoutError is in the ctypes front end).
#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>

#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/vsg.h"

namespace py = pybind11;

namespace {

using FloatArray = py::array_t<float, py::array::c_style | py::array::forcecast>;
using MaskArray = py::array_t<uint8_t, py::array::c_style | py::array::forcecast>;

void check(int rc) {
  if (rc == VSG_OK) return;
  const std::string msg = vsg_last_error();
  if (rc == VSG_ERR_INVALID || rc == VSG_ERR_LENGTH) throw py::value_error(msg);
  if (rc == VSG_ERR_NOMEM) throw std::bad_alloc();  // pybind11 raises MemoryError
  throw std::runtime_error(msg);
}

uint32_t parse_metric(const std::string& s) {
  if (s == "l2") return VSG_METRIC_L2;
  if (s == "ip" || s == "cosine") return VSG_METRIC_IP;
  throw py::value_error("metric must be 'l2', 'ip' or 'cosine' (cosine expects normalized vectors)");
}

uint32_t parse_method(const std::string& m) {
  if (m == "auto") return VSG_METHOD_AUTO;
  if (m == "naive") return VSG_METHOD_NAIVE;
  if (m == "skinny") return VSG_METHOD_SKINNY;
  if (m == "tiled") return VSG_METHOD_TILED;
  if (m == "bf16") return VSG_METHOD_BF16;
  if (m == "tc_exact") return VSG_METHOD_TC_EXACT;
  if (m == "fp8") return VSG_METHOD_FP8;
  throw py::value_error("method must be 'auto', 'naive', 'skinny', 'tiled', 'bf16', 'tc_exact' or 'fp8'");
}

void check_2d(const FloatArray& a, size_t dim) {
  if (a.ndim() != 2 || size_t(a.shape(1)) != dim)
    throw py::value_error("expected array of shape (n, " + std::to_string(dim) + ")");
}

// uint32 ids with VSG_NONE for a missing result -> int64 with -1 (bindings.cpp:50-56).
py::array_t<int64_t> ids_to_int64(const std::vector<uint32_t>& ids, size_t nq, size_t k) {
  py::array_t<int64_t> out({py::ssize_t(nq), py::ssize_t(k)});
  int64_t* dst = out.mutable_data();
  for (size_t i = 0; i < ids.size(); ++i) dst[i] = ids[i] == VSG_NONE ? -1 : int64_t(ids[i]);
  return out;
}

// Allow-bits (bit r & 31 of word r >> 5) from a byte mask, nonzero = allowed (as_mask,
// bindings.cpp:28-36: the array is cast to uint8 first, so 0.5 disallows a row).
void pack_bits(const uint8_t* m, size_t n, uint32_t* words) {
  const size_t nw = (n + 31) / 32;
  std::memset(words, 0, nw * sizeof(uint32_t));
  for (size_t r = 0; r < n; ++r)
    if (m[r]) words[r >> 5] |= 1u << (r & 31);
}

class GpuIndex {
 public:
  GpuIndex(size_t dim, const std::string& metric, int device) {
    if (dim == 0) throw py::value_error("dim must be > 0");
    const uint32_t mt = parse_metric(metric);
    check(vsg_create(dim, mt, device, &h_));
  }
  ~GpuIndex() { vsg_destroy(h_); }
  GpuIndex(const GpuIndex&) = delete;
  GpuIndex& operator=(const GpuIndex&) = delete;

  void add(FloatArray x) {
    check_2d(x, dim());
    const float* p = x.data();
    const size_t n = size_t(x.shape(0));
    int rc;
    {
      py::gil_scoped_release nogil;
      rc = vsg_add(h_, p, n);
    }
    check(rc);
  }

  py::tuple search(FloatArray q, size_t k, const std::string& method, const py::object& filter) {
    const uint32_t gm = parse_method(method);
    if (q.ndim() == 1) q = q.reshape({py::ssize_t(1), q.shape(0)});
    check_2d(q, dim());
    if (k > VSG_MAX_K) throw py::value_error("k must be <= " + std::to_string(VSG_MAX_K));
    const size_t nq = size_t(q.shape(0)), n = size();
    std::vector<uint32_t> ids(nq * k);
    py::array_t<float> dists({py::ssize_t(nq), py::ssize_t(k)});
    float* dd = dists.mutable_data();
    const float* qp = q.data();
    std::vector<uint32_t> words;
    int per_query = 0;
    size_t mask_ld = 0;
    if (!filter.is_none()) {
      MaskArray m = MaskArray::ensure(filter);
      const bool one = m && m.ndim() == 1 && size_t(m.shape(0)) == n;
      const bool each = m && m.ndim() == 2 && size_t(m.shape(0)) == nq && size_t(m.shape(1)) == n;
      if (!one && !each)
        throw py::value_error("filter must be a 1-D bool array of length " + std::to_string(n) +
                              " (or one such row per query)");
      mask_ld = (n + 31) / 32;
      per_query = each ? 1 : 0;
      words.resize(std::max<size_t>(1, (each ? nq : 1) * mask_ld));
      for (size_t i = 0; i < (each ? nq : 1); ++i) pack_bits(m.data() + i * n, n, words.data() + i * mask_ld);
    }
    int rc;
    {
      py::gil_scoped_release nogil;
      rc = filter.is_none() ? vsg_search(h_, qp, nq, k, ids.data(), dd, gm)
                            : vsg_search_filtered(h_, qp, nq, k, words.data(), per_query, mask_ld, ids.data(), dd,
                                                  gm);
    }
    check(rc);
    return py::make_tuple(ids_to_int64(ids, nq, k), dists);
  }

  size_t dim() const { return vsg_dim(h_); }
  size_t size() const { return vsg_size(h_); }
  std::string metric() const { return vsg_metric(h_) == VSG_METRIC_L2 ? "l2" : "ip"; }

 private:
  vsg_index* h_ = nullptr;
};

}  // namespace

PYBIND11_MODULE(_vecsearch_gb300, m) {
  m.doc() = "GB300 exact k-NN: the reference's GpuBruteForceIndex surface over libvsg_gb300.so";
  py::class_<GpuIndex>(m, "GpuBruteForceIndex")
      .def(py::init<size_t, const std::string&, int>(), py::arg("dim"), py::arg("metric") = "l2",
           py::arg("device") = 0)
      .def("add", &GpuIndex::add, py::arg("x"))
      .def("search", &GpuIndex::search, py::arg("queries"), py::arg("k") = 10, py::arg("method") = "auto",
           py::arg("filter") = py::none(),
           "Exact top-k on the GPU, k <= 128. Returns (ids[int64, nq x k], distances[float32, nq x k]).")
      .def_property_readonly("dim", &GpuIndex::dim)
      .def_property_readonly("metric", &GpuIndex::metric)
      .def("__len__", &GpuIndex::size);
  m.def("cuda_available", [] { return vsg_cuda_available() != 0; }, "True if a GPU is visible.");
}
