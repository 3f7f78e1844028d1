// Loading the vectors of a saved HNSW index (the VSHNSW01 file) straight into a device index.
//
// File layout (src/hnsw.cpp:368-389, HNSWIndex::save): the 8-byte magic "VSHNSW01", then
// dim u64, n u64, metric u32, M u64, ef_construction u64, max_level i32, entry_point u32
// (each written on its own, no padding: 52 bytes in all), then n x dim f32 vectors, then the
// levels and links. Only the header and the vectors are read here. The vectors stream from the
// file through two pinned chunks into the padded device rows, so no host copy of the whole base
// is made (the reference's load reads them into HNSWIndex::data_, hnsw.cpp:404).
#include <cstdio>
#include <cstring>

#include "index_impl.cuh"

using namespace vsg_detail;

namespace {

constexpr char kMagic[8] = {'V', 'S', 'H', 'N', 'S', 'W', '0', '1'};
constexpr size_t kHeaderBytes = 52;
constexpr size_t kChunkBytes = size_t(32) << 20;

struct IoError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

struct File {
  FILE* f = nullptr;
  explicit File(const char* path) : f(std::fopen(path, "rb")) {
    if (!f) throw IoError(std::string("cannot open ") + path);
  }
  ~File() {
    if (f) std::fclose(f);
  }
  void read(void* dst, size_t bytes, const char* path) {
    if (bytes && std::fread(dst, 1, bytes, f) != bytes) throw IoError(std::string("truncated index file: ") + path);
  }
};

template <class T>
T take(const unsigned char* p) {
  T v;
  std::memcpy(&v, p, sizeof(T));  // the file is little-endian, as are x86-64 and aarch64
  return v;
}

struct Header {
  uint64_t dim, n;
  uint32_t metric;
};

Header read_header(File& f, const char* path) {
  unsigned char h[kHeaderBytes];
  f.read(h, kHeaderBytes, path);
  if (std::memcmp(h, kMagic, 8) != 0) throw IoError("not a vecsearch HNSW file");
  Header r;
  r.dim = take<uint64_t>(h + 8);
  r.n = take<uint64_t>(h + 16);
  r.metric = take<uint32_t>(h + 24);
  if (r.dim == 0 || r.metric > 1) throw IoError(std::string("bad header in ") + path);
  return r;
}

template <class F>
int guarded_io(F&& f) {
  try {
    g_last_error.clear();
    f();
    return VSG_OK;
  } catch (const IoError& e) {
    g_last_error = e.what();
    return VSG_ERR_IO;
  } catch (const std::invalid_argument& e) {
    g_last_error = e.what();
    return VSG_ERR_INVALID;
  } catch (const std::length_error& e) {
    g_last_error = e.what();
    return VSG_ERR_LENGTH;
  } catch (const std::bad_alloc&) {
    g_last_error = "out of device or pinned host memory";
    return VSG_ERR_NOMEM;
  } catch (const std::exception& e) {
    g_last_error = e.what();
    return VSG_ERR_CUDA;
  }
}

}  // namespace

extern "C" {

int vsg_hnsw_file_info(const char* path, size_t* dim, size_t* n, uint32_t* metric) {
  return guarded_io([&] {
    if (!path) throw std::invalid_argument("path is NULL");
    File f(path);
    const Header h = read_header(f, path);
    if (dim) *dim = size_t(h.dim);
    if (n) *n = size_t(h.n);
    if (metric) *metric = h.metric;
  });
}

int vsg_add_hnsw_file(vsg_index* h, const char* path, size_t* added) {
  return guarded_io([&] {
    if (!h || !path) throw std::invalid_argument("index or path is NULL");
    File f(path);
    const Header hd = read_header(f, path);
    if (hd.dim != h->dim) throw std::invalid_argument("the file's dim differs from the index's");
    if (hd.metric != h->metric) throw std::invalid_argument("the file's metric differs from the index's");
    std::lock_guard<std::mutex> g(h->mu);
    const size_t m = size_t(hd.n);
    if (h->n + m >= VSG_NONE) throw std::length_error("GpuBruteForceIndex holds at most 2^32 - 2 vectors");
    VSG_CUDA(cudaSetDevice(h->device));
    VSG_CUDA(cudaStreamWaitEvent(h->stream, h->done, 0));
    if (h->n + m > h->cap) {
      const size_t cap = std::max({h->n + m, h->cap * 2, size_t(1024)});
      h->x.reserve(cap * h->dp * sizeof(float), h->n * h->dp * sizeof(float), h->stream);
      h->cap = cap;
    }
    const size_t row_bytes = h->dim * sizeof(float);
    const size_t chunk_rows = std::max<size_t>(1, kChunkBytes / row_bytes);
    PinnedBuffer buf[2];
    cudaEvent_t ev[2] = {nullptr, nullptr};
    auto cleanup = [&] {
      for (cudaEvent_t e : ev)
        if (e) {
          cudaEventSynchronize(e);
          cudaEventDestroy(e);
        }
    };
    try {
      for (int i = 0; i < 2; ++i) {
        buf[i].reserve(std::min(m, chunk_rows) * row_bytes + 1);
        VSG_CUDA(cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming));
      }
      float* dst = static_cast<float*>(h->x.get()) + h->n * h->dp;
      size_t done = 0;
      for (int slot = 0; done < m; slot ^= 1) {
        const size_t rows = std::min(chunk_rows, m - done);
        VSG_CUDA(cudaEventSynchronize(ev[slot]));  // the copy that last used this chunk has finished
        f.read(buf[slot].get(), rows * row_bytes, path);
        VSG_CUDA(cudaMemcpy2DAsync(dst + done * h->dp, h->dp * sizeof(float), buf[slot].get(), row_bytes, row_bytes,
                                   rows, cudaMemcpyHostToDevice, h->stream));
        VSG_CUDA(cudaEventRecord(ev[slot], h->stream));
        done += rows;
      }
      VSG_CUDA(cudaEventRecord(h->done, h->stream));
      VSG_CUDA(cudaStreamSynchronize(h->stream));
    } catch (...) {
      cleanup();
      throw;  // rows past h->n may hold part of the file; h->n is unchanged, so they are not searched
    }
    cleanup();
    h->n += m;
    if (added) *added = m;
  });
}

}  // extern "C"
