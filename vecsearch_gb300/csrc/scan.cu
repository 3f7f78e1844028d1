// Fused exact scan + top-k for FP32 rows resident in HBM (sm_103a).
//
// Replaces the reference's distance-block + select round trip
// (src/gpu_brute_force.cu:97-140 skinny_kernel, :220-292 select_kernel, :475-482
// merge loop): no query x row score block is ever written to memory.
//
// Grid (query blocks, row splits). Each CTA owns QB queries and one contiguous
// row range of the base:
//   * a producer warp streams tiles of R = 8*RW consecutive rows into a ring of
//     shared-memory slots with bulk (TMA) copies, one mbarrier pair per slot;
//   * 8 consumer warps each take RW rows of a tile. Lanes split the dims in
//     16-byte chunks (lane l reads chunks l, l+32, ...: conflict-free), every
//     lane accumulates RW x QB partial dot products (or squared differences),
//     and a warp reduce-scatter leaves one finished distance per lane;
//   * a distance enters the warp's sorted top-k list of its query when it beats
//     the list's last entry in (dist, id) order and the row passes the filter.
// With a filter, the producer warp instead reads the filter bits of 1024 rows per
// step, compacts the allowed rows (warp prefix sum of popcounts) and copies only
// those, R per slot: one copy for a run of consecutive rows, else one per row.
// The filtered scan therefore reads only allowed rows from HBM (the allowed-id
// gather scan), whether the mask is shared or per query, on the host or device.
// At the end the 8 warp lists of each query are merged and written as the
// split's top-k; merge_kernel then merges the splits.
#include <mutex>

#include "device_common.cuh"
#include "launch.cuh"
#include "scan.cuh"

namespace vsg {

namespace {

__host__ __device__ constexpr size_t align128(size_t v) { return (v + 127) & ~size_t(127); }

constexpr uint32_t kEndOfRows = 0xFFFFFFFFu;  // slot_rows value that ends a filtered scan
constexpr int kChunkRows = 1024;               // rows whose filter bits the producer warp reads per step

struct SmemLayout {
  size_t rows_off, q_off, ids_off, chunk_off, ring_off, ld_off, li_off, total;
};

// [full/empty mbarriers | rows per slot | queries | row ids per slot | compaction buffer |
//  ring of row tiles | per-warp top-k dists | per-warp top-k ids]
__host__ __device__ inline SmemLayout scan_layout(int qb, int rw, uint32_t dp, uint32_t k, uint32_t stages) {
  SmemLayout L;
  L.rows_off = 2 * kMaxStages * sizeof(uint64_t);
  L.q_off = align128(L.rows_off + kMaxStages * sizeof(uint32_t));
  L.ids_off = L.q_off + align128(size_t(qb) * dp * sizeof(float));
  L.chunk_off = L.ids_off + align128(size_t(kMaxStages) * 32 * sizeof(uint32_t));
  L.ring_off = L.chunk_off + align128(size_t(kChunkRows) * sizeof(uint32_t));
  const size_t tile = size_t(kScanWarps) * rw * dp * sizeof(float);
  L.ld_off = L.ring_off + align128(size_t(stages) * tile);
  const size_t lists = size_t(kScanWarps) * qb * k * sizeof(float);
  L.li_off = L.ld_off + align128(lists);
  L.total = L.li_off + align128(lists);
  return L;
}

template <bool L2>
__device__ __forceinline__ float acc4(const float4 q, const float4 x, float a) {
  if constexpr (L2) {
    float e = q.x - x.x;
    a = fmaf(e, e, a);
    e = q.y - x.y;
    a = fmaf(e, e, a);
    e = q.z - x.z;
    a = fmaf(e, e, a);
    e = q.w - x.w;
    return fmaf(e, e, a);
  } else {
    a = fmaf(q.x, x.x, a);
    a = fmaf(q.y, x.y, a);
    a = fmaf(q.z, x.z, a);
    return fmaf(q.w, x.w, a);
  }
}

// Filter bits of mask word w for the block's queries (their union), clipped to rows < row_end.
template <int QB>
__device__ __forceinline__ uint32_t block_bits(const ScanArgs& a, uint32_t qbase, uint32_t w, uint32_t row_end) {
  uint32_t bits = 0;
  if (a.mask_ptrs) {  // per-query pointers; no filter (nullptr) allows every row
#pragma unroll
    for (int b = 0; b < QB; ++b)
      if (qbase + b < a.nq) {
        const uint32_t* p = a.mask_ptrs[qbase + b];
        bits |= p ? __ldg(p + w) : 0xFFFFFFFFu;
      }
  } else if (a.mask_ld == 0) {
    bits = __ldg(a.mask + w);
  } else {
#pragma unroll
    for (int b = 0; b < QB; ++b)
      if (qbase + b < a.nq) bits |= __ldg(a.mask + size_t(qbase + b) * a.mask_ld + w);
  }
  const uint32_t lo = w * 32;
  if (row_end - lo < 32) bits &= (1u << (row_end - lo)) - 1u;  // lo < row_end (no wrap near 2^32)
  return bits;
}

// Masked full scan: true when no query of the block may return any row of the tile
// [r0, r0 + R). R divides 32 and tiles start at multiples of R, so one word covers a tile.
template <int QB, int R>
__device__ __forceinline__ bool tile_filtered_out(const ScanArgs& a, uint32_t qbase, uint32_t r0,
                                                  uint32_t row_end) {
  const uint32_t span = R >= 32 ? 0xFFFFFFFFu : (((1u << R) - 1u) << (r0 & 31));
  return (block_bits<QB>(a, qbase, r0 >> 5, row_end) & span) == 0;
}

// The scan kernel's tail. (1) Warp b merges the 8 warp lists of query b (registers, bitonic)
// and writes the split's top-k. (2) With a.counters set, the last CTA of the query block to
// finish stages every split's list of each query in the (now free) ring, the 8 consumer warps
// merge a share each, warp b merges the 8 results and writes the final top-k, and the
// block's counter is reset for the next launch.
template <int E, int QB>
__device__ __forceinline__ void scan_epilogue(const ScanArgs& a, const SmemLayout& L, float* ring, float* lst_d,
                                              uint32_t* lst_i, uint32_t qbase, uint32_t split, int tid, int warp,
                                              int lane) {
  const uint32_t k = a.k;
  if (warp < QB) {
    const int b = warp;
    WarpTopK<E> acc;
    acc.load(lst_d + size_t(b) * k, lst_i + size_t(b) * k, int(k), lane);
    warp_merge_lists<E>(acc, lst_d + size_t(QB + b) * k, lst_i + size_t(QB + b) * k, kScanWarps - 1,
                        size_t(QB) * k, int(k), lane);
    const uint32_t qg = qbase + b;
    if (qg < a.nq) {
      const size_t o = (size_t(qg) * a.nsplit + split) * k;
      acc.store(a.part_d + o, a.part_i + o, int(k), lane);
    }
  }
  if (a.counters == nullptr) return;

  __shared__ int last_cta;
  __threadfence();  // this CTA's lists are visible device-wide before it is counted
  __syncthreads();
  if (tid == 0) last_cta = atomicAdd(a.counters + blockIdx.x, 1u) == gridDim.y - 1;
  __syncthreads();
  if (!last_cta) return;
  __threadfence();
  const uint32_t nlive = a.nq_dev ? min(a.nq, *a.nq_dev) : a.nq;  // qbase < nlive (checked at the start)
  const uint32_t nvalid = min(uint32_t(QB), nlive - qbase);
  // Stage split lists in the ring, one query at a time, in rounds that fit (the ring holds at
  // least 512 entries; k <= 128).
  const size_t ring_entries = (L.ld_off - L.ring_off) / (2 * sizeof(float));
  float* st_d = ring;
  uint32_t* st_i = reinterpret_cast<uint32_t*>(ring + ring_entries);
  const size_t per_query = size_t(a.nsplit) * k;
  const uint32_t lists_per_round = uint32_t(ring_entries / k > 1 ? ring_entries / k : 1);
  for (uint32_t b = 0; b < nvalid; ++b) {
    WarpTopK<E> acc;
    acc.clear();
    for (uint32_t s0 = 0; s0 < a.nsplit; s0 += lists_per_round) {
      const uint32_t ns = min(lists_per_round, a.nsplit - s0);
      __syncthreads();  // the previous round's staged lists are merged
      stage_lists_cg(st_d, st_i, a.part_d + size_t(qbase + b) * per_query + size_t(s0) * k,
                     a.part_i + size_t(qbase + b) * per_query + size_t(s0) * k, size_t(ns) * k, tid, kScanThreads);
      __syncthreads();
      if (warp < kScanWarps && uint32_t(warp) < ns)
        warp_merge_lists<E>(acc, st_d + size_t(warp) * k, st_i + size_t(warp) * k,
                            int((ns - warp + kScanWarps - 1) / kScanWarps), size_t(kScanWarps) * k, int(k), lane);
    }
    if (warp < kScanWarps) acc.store(lst_d + (size_t(warp) * QB + b) * k, lst_i + (size_t(warp) * QB + b) * k,
                                     int(k), lane);
  }
  __syncthreads();
  if (warp < int(nvalid)) {
    const int b = warp;
    WarpTopK<E> acc;
    acc.load(lst_d + size_t(b) * k, lst_i + size_t(b) * k, int(k), lane);
    warp_merge_lists<E>(acc, lst_d + size_t(QB + b) * k, lst_i + size_t(QB + b) * k, kScanWarps - 1,
                        size_t(QB) * k, int(k), lane);
    const size_t row = a.out_map ? size_t(a.out_map[qbase + b]) : size_t(qbase + b);
    acc.store(a.out_d + row * k, a.out_i + row * k, int(k), lane);
  }
  if (tid == 0) a.counters[blockIdx.x] = 0;  // ready for the next launch
}

template <int QB, int RW, bool L2>
__global__ void __launch_bounds__(kScanThreads, 1) scan_kernel(const ScanArgs a) {
  constexpr int R = kScanWarps * RW;  // rows per tile
  constexpr int V = RW * QB;          // partial sums per lane
  constexpr int G = 32 / V;           // lanes sharing one finished distance
  static_assert(V <= 32 && (V & (V - 1)) == 0, "RW * QB must be a power of two <= 32");
  static_assert(R <= 32, "a tile's row ids fit one warp");

  extern __shared__ __align__(128) unsigned char smem[];
  const uint32_t dp = a.dp, nc = dp / 4, k = a.k;
  const SmemLayout L = scan_layout(QB, RW, dp, k, a.stages);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem);
  uint64_t* empty = full + kMaxStages;
  uint32_t* slot_rows = reinterpret_cast<uint32_t*>(smem + L.rows_off);
  float* qs = reinterpret_cast<float*>(smem + L.q_off);
  uint32_t* slot_ids = reinterpret_cast<uint32_t*>(smem + L.ids_off);
  uint32_t* chunk = reinterpret_cast<uint32_t*>(smem + L.chunk_off);
  float* ring = reinterpret_cast<float*>(smem + L.ring_off);
  float* lst_d = reinterpret_cast<float*>(smem + L.ld_off);
  uint32_t* lst_i = reinterpret_cast<uint32_t*>(smem + L.li_off);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t qbase = blockIdx.x * QB;
  pdl_trigger();
  pdl_wait();
  // A count read on the device: whole query blocks past it leave before touching anything (the
  // fused merge's counter of such a block is never used).
  if (a.nq_dev && qbase >= *a.nq_dev) return;
  const uint32_t split = blockIdx.y;
  const uint32_t row_begin = split * a.rows_per_split;  // a multiple of 32
  const uint64_t end64 = uint64_t(row_begin) + a.rows_per_split;  // can pass 2^32 near 2^32 rows
  const uint32_t row_end = end64 < a.n ? uint32_t(end64) : a.n;
  const uint32_t ntiles = row_end > row_begin ? (row_end - row_begin + R - 1) / R : 0;
  const uint32_t stages = a.stages;
  // Without a filter, or for a masked full scan, the producer copies whole tiles of
  // consecutive rows (skipping tiles with no allowed row). In gather mode it compacts the
  // allowed rows from the filter bits and copies only those.
  const bool gather = a.mask != nullptr && a.gather != 0;

  const unsigned long long wl = a.wait_ns ? a.wait_ns : kWaitLimitNs;
  const bool stall = a.stall != 0 && stages < uint32_t(kMaxStages);
  if (tid == 0) {
    for (uint32_t s = 0; s < stages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], kScanWarps);
    }
    if (stall) mbar_init(&full[kMaxStages - 1], 1);  // nothing ever arrives on it
    mbar_fence_init();
  }
  {  // queries of the block (rows >= nq become zeros), and empty lists
    float4* qs4 = reinterpret_cast<float4*>(qs);
    for (uint32_t i = tid; i < QB * nc; i += kScanThreads) {
      const uint32_t b = i / nc, c = i % nc;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (qbase + b < a.nq) v = *reinterpret_cast<const float4*>(a.q + size_t(qbase + b) * a.ldq + c * 4);
      qs4[i] = v;
    }
    for (uint32_t i = tid; i < kScanWarps * QB * k; i += kScanThreads) {
      lst_d[i] = __int_as_float(0x7f800000);
      lst_i[i] = kNone;
    }
  }
  __syncthreads();

  if (warp == kScanWarps) {
    // ---------------- producer warp ----------------
    const uint64_t policy = policy_evict_first();
    uint32_t s = 0, ph = 0;
    uint32_t pending = 0, last_ph = 0;  // lane 0: per-slot bit "a copy was issued", and its parity
    bool ok = true;
    auto note_issue = [&](uint32_t slot) {
      pending |= 1u << slot;
      last_ph = (last_ph & ~(1u << slot)) | (ph << slot);
    };
    auto advance = [&]() {
      if (++s == stages) {
        s = 0;
        ph ^= 1;
      }
    };
    if (!gather) {
      if (lane == 0) {
        for (uint32_t t = 0; t < ntiles; ++t) {
          const uint32_t r0 = row_begin + t * R;
          if ((a.mask || a.mask_ptrs) && tile_filtered_out<QB, R>(a, qbase, r0, row_end)) continue;
          if (!mbar_wait(&empty[s], ph ^ 1, wl)) {
            ok = false;
            break;
          }
          const uint32_t rows = min(uint32_t(R), row_end - r0);
          const uint32_t bytes = rows * dp * uint32_t(sizeof(float));
          mbar_arrive_expect_tx(&full[s], bytes);
          bulk_load_stream(ring + size_t(s) * R * dp, a.x + size_t(r0) * dp, bytes, &full[s], policy);
          note_issue(s);
          advance();
        }
      }
    } else {
      // Rows whose filter bit is set, in increasing order, R per slot; the slot's row ids go
      // to slot_ids. Consecutive rows are fetched with one copy, others one copy per row.
      uint32_t cnt = 0;  // rows placed in the open slot (warp-uniform)
      auto commit = [&]() {
        __syncwarp();
        const uint32_t first = slot_ids[s * 32], last = slot_ids[s * 32 + cnt - 1];
        const bool dense = last - first == cnt - 1;
        if (lane == 0) {
          slot_rows[s] = cnt;
          mbar_arrive_expect_tx(&full[s], cnt * dp * uint32_t(sizeof(float)));
          note_issue(s);
        }
        __syncwarp();
        float* dst = ring + size_t(s) * R * dp;
        if (dense) {
          if (lane == 0)
            bulk_load_stream(dst, a.x + size_t(first) * dp, cnt * dp * uint32_t(sizeof(float)), &full[s], policy);
        } else if (uint32_t(lane) < cnt) {
          bulk_load_stream(dst + size_t(lane) * dp, a.x + size_t(slot_ids[s * 32 + lane]) * dp,
                           dp * uint32_t(sizeof(float)), &full[s], policy);
        }
        advance();
        cnt = 0;
      };
      auto open_slot = [&]() -> bool {
        bool got = true;
        if (lane == 0) got = mbar_wait(&empty[s], ph ^ 1, wl);
        return __shfl_sync(kFull, got ? 1 : 0, 0) != 0;
      };
      const uint32_t wend = (row_end >> 5) + ((row_end & 31u) != 0u);
      // The next step's filter words are loaded before this step is processed, so the
      // global-load latency overlaps the compaction and the slot filling.
      uint32_t next = (row_begin >> 5) + lane < wend ? block_bits<QB>(a, qbase, (row_begin >> 5) + lane, row_end) : 0u;
      for (uint32_t w0 = row_begin >> 5; w0 < wend && ok; w0 += kChunkRows / 32) {
        const uint32_t w = w0 + lane;
        uint32_t bits = next;
        const uint32_t wn = w + kChunkRows / 32;
        next = wn < wend ? block_bits<QB>(a, qbase, wn, row_end) : 0u;
        const uint32_t pc = __popc(bits);
        uint32_t incl = pc;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const uint32_t t = __shfl_up_sync(kFull, incl, o);
          if (lane >= o) incl += t;
        }
        const uint32_t total = __shfl_sync(kFull, incl, 31);
        uint32_t e = incl - pc;
        while (bits) {
          const int i = __ffs(bits) - 1;
          bits &= bits - 1;
          chunk[e++] = w * 32 + uint32_t(i);
        }
        __syncwarp();
        for (uint32_t pos = 0; pos < total;) {
          if (cnt == 0 && !open_slot()) {
            ok = false;
            break;
          }
          const uint32_t take = min(uint32_t(R) - cnt, total - pos);
          if (uint32_t(lane) < take) slot_ids[s * 32 + cnt + lane] = chunk[pos + lane];
          cnt += take;
          pos += take;
          if (cnt == uint32_t(R)) commit();
        }
        __syncwarp();  // the compaction buffer is rewritten by the next step
      }
      if (ok && cnt > 0) commit();
      if (ok) {  // end marker: a slot with no rows
        if (!open_slot()) {
          ok = false;
        } else if (lane == 0) {
          // The slot was empty: its previous copy landed and was consumed. The marker moves
          // this barrier one more phase, so the drain below must not wait on that copy.
          pending &= ~(1u << s);
          slot_rows[s] = kEndOfRows;
          mbar_arrive(&full[s]);
        }
      }
    }
    if (lane == 0) {
      // Wait (bounded) until every issued copy has landed before the CTA may exit.
      for (uint32_t i = 0; i < stages; ++i)
        if ((pending >> i) & 1u)
          if (!mbar_wait(&full[i], (last_ph >> i) & 1u)) ok = false;
      if (!ok) atomicExch(a.status, kDevTimeout);
    }
  } else {
    // ---------------- consumer warps ----------------
    float* my_d = lst_d + size_t(warp) * QB * k;
    uint32_t* my_i = lst_i + size_t(warp) * QB * k;
    const float4* qs4 = reinterpret_cast<const float4*>(qs);
    const int vi = lane / G;  // value this lane finishes
    const int vr = vi / QB, vb = vi % QB;
    const bool owner = (lane % G) == 0;
    const uint32_t lrow = uint32_t(warp * RW + vr);  // the finished value's row within a tile
    // A masked full scan checks every pair; gather slots hold only allowed rows, but for
    // per-query masks with QB > 1 they hold the block's union.
    const bool check_bits = (a.mask != nullptr && (!gather || (a.mask_ld != 0 && QB > 1))) || a.mask_ptrs != nullptr;
    uint32_t s = 0, ph = 0;
    bool live = true;
    if (stall && !__all_sync(kFull, mbar_wait(&full[kMaxStages - 1], 0, wl))) {  // the test hook's wait
      if (lane == 0) atomicExch(a.status, kDevTimeout);
      live = false;
    }
    for (uint32_t t = 0; live && (gather || t < ntiles); ++t) {
      if (!gather && (a.mask || a.mask_ptrs) && tile_filtered_out<QB, R>(a, qbase, row_begin + t * R, row_end))
        continue;
      // warp-uniform decision, so no lane leaves while the others shuffle
      if (!__all_sync(kFull, mbar_wait(&full[s], ph, wl))) {
        if (lane == 0) atomicExch(a.status, kDevTimeout);
        break;
      }
      uint32_t rows, row;
      if (gather) {
        rows = slot_rows[s];
        if (rows == kEndOfRows) break;
        row = lrow < rows ? slot_ids[s * 32 + lrow] : kNone;  // read before the slot is released
      } else {
        const uint32_t r0 = row_begin + t * R;
        rows = min(uint32_t(R), row_end - r0);
        row = r0 + lrow;
      }
      const float4* xs4 = reinterpret_cast<const float4*>(ring + size_t(s) * R * dp) + size_t(warp) * RW * nc;
      float acc[V];
#pragma unroll
      for (int i = 0; i < V; ++i) acc[i] = 0.f;
#pragma unroll 2
      for (uint32_t c = lane; c < nc; c += 32) {
        float4 xv[RW];
#pragma unroll
        for (int r = 0; r < RW; ++r) xv[r] = xs4[r * nc + c];
#pragma unroll
        for (int b = 0; b < QB; ++b) {
          const float4 qv = qs4[b * nc + c];
#pragma unroll
          for (int r = 0; r < RW; ++r) acc[r * QB + b] = acc4<L2>(qv, xv[r], acc[r * QB + b]);
        }
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[s]);
      if (++s == stages) {
        s = 0;
        ph ^= 1;
      }

      ReduceScatter<V, 16>::run(acc, lane);
      const float dist = L2 ? acc[0] : 1.0f - acc[0];
      bool pass = owner && lrow < rows && qbase + vb < a.nq;  // padded query slots never compete
      if (pass && check_bits) {
        const uint32_t* p = a.mask_ptrs ? a.mask_ptrs[qbase + vb] : a.mask + size_t(qbase + vb) * a.mask_ld;
        pass = p == nullptr || ((__ldg(p + (row >> 5)) >> (row & 31)) & 1u);
      }
      if (pass) pass = nb_less(dist, row, my_d[vb * k + k - 1], my_i[vb * k + k - 1]);
      unsigned bal = __ballot_sync(kFull, pass);
      while (bal) {
        const int src = __ffs(bal) - 1;
        bal &= bal - 1;
        const float cd = __shfl_sync(kFull, dist, src);
        const uint32_t ci = __shfl_sync(kFull, row, src);
        const int cb = (src / G) % QB;
        float* ld = my_d + cb * k;
        uint32_t* li = my_i + cb * k;
        if (nb_less(cd, ci, ld[k - 1], li[k - 1])) list_insert(ld, li, int(k), cd, ci, lane);
      }
    }
  }
  __syncthreads();

  if (k <= 32) {
    scan_epilogue<1, QB>(a, L, ring, lst_d, lst_i, qbase, split, tid, warp, lane);
  } else if (k <= 64) {
    scan_epilogue<2, QB>(a, L, ring, lst_d, lst_i, qbase, split, tid, warp, lane);
  } else {
    scan_epilogue<4, QB>(a, L, ring, lst_d, lst_i, qbase, split, tid, warp, lane);
  }
}

// Warp w merges split lists w, w + 8, ... of query q into acc, in registers, and leaves its
// first k entries in sd[w] / si[w].
template <int E>
__device__ __forceinline__ void merge_split_lists(WarpTopK<E>& acc, const MergeArgs& m, uint32_t q, float (*sd)[kMaxK],
                                                  uint32_t (*si)[kMaxK], int warp, int lane, int kk, float mg) {
  const uint32_t k = m.k;
  const size_t base = size_t(q) * m.nsplit * k;
  if (uint32_t(warp) < m.nsplit)
    warp_merge_lists<E>(acc, m.part_d + base + size_t(warp) * k, m.part_i + base + size_t(warp) * k,
                        int((m.nsplit - warp + 7) / 8), size_t(8) * k, int(k), lane, kk, mg);
  acc.store(sd[warp], si[warp], int(k), lane);
}

// Warp 0, after every warp's list is in sd / si: merges lists 1..7 into its own (acc), applies
// the margin cut, and writes the query's k entries.
template <int E>
__device__ __forceinline__ void merge_finish(WarpTopK<E>& acc, const MergeArgs& m, uint32_t q, float (*sd)[kMaxK],
                                             uint32_t (*si)[kMaxK], int lane, int kk, float mg) {
  const uint32_t k = m.k;
  warp_merge_lists<E>(acc, sd[1], si[1], 7, kMaxK, int(k), lane, kk, mg);
  if (mg >= 0.f) {  // the cut: entries above the kk-th + mg (the list stays sorted)
    float td;
    uint32_t ti;
    acc.entry(kk - 1, td, ti);
    const float cut = __fadd_ru(td, mg);
#pragma unroll
    for (int e = 0; e < E; ++e)
      if (!nb_less(acc.d[e], acc.i[e], cut, kNone)) {
        acc.d[e] = __int_as_float(0x7f800000);
        acc.i[e] = kNone;
      }
  }
  acc.store(m.out_d + size_t(q) * k, m.out_i + size_t(q) * k, int(k), lane);
}

// One CTA per query: warp w merges split lists w, w + 8, ... in registers, then warp 0
// merges the 8 warp results.
template <int E>
__global__ void __launch_bounds__(256) merge_kernel(const MergeArgs m) {
  __shared__ float sd[8][kMaxK];
  __shared__ uint32_t si[8][kMaxK];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t q = blockIdx.x;
  if (m.nq_dev && q >= *m.nq_dev) return;
  const float mg = m.margin ? m.margin[q] : -1.f;
  const int kk = int(m.kk);
  WarpTopK<E> acc;
  acc.clear();
  merge_split_lists<E>(acc, m, q, sd, si, warp, lane, kk, mg);
  __syncthreads();
  if (warp == 0) merge_finish<E>(acc, m, q, sd, si, lane, kk, mg);
}

__global__ void fill_missing_kernel(float* d, uint32_t* i, size_t count) {
  for (size_t j = blockIdx.x * size_t(blockDim.x) + threadIdx.x; j < count; j += size_t(gridDim.x) * blockDim.x) {
    d[j] = __int_as_float(0x7f800000);
    i[j] = kNone;
  }
}

template <int QB, int RW, bool L2>
cudaError_t launch_one(const ScanArgs& a, dim3 grid, cudaStream_t stream, bool launch = true, bool pdl = false) {
  const size_t smem = scan_layout(QB, RW, a.dp, a.k, a.stages).total;
  // Largest dynamic shared-memory size already allowed for this instantiation, per device.
  static std::mutex mu;
  static size_t configured[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  {
    std::lock_guard<std::mutex> g(mu);
    if (dev >= 64 || smem > configured[dev]) {
      e = cudaFuncSetAttribute(scan_kernel<QB, RW, L2>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
      if (e != cudaSuccess) return e;
      if (dev < 64) configured[dev] = smem;
    }
  }
  if (!launch) return cudaSuccess;
  return launch_kernel(scan_kernel<QB, RW, L2>, grid, dim3(kScanThreads), smem, stream, pdl, a);
}

template <int QB, int RW>
cudaError_t launch_metric(const ScanShape& s, const ScanArgs& a, dim3 grid, cudaStream_t st, bool launch, bool pdl) {
  return s.l2 ? launch_one<QB, RW, true>(a, grid, st, launch, pdl) : launch_one<QB, RW, false>(a, grid, st, launch, pdl);
}

template <int QB>
cudaError_t launch_rw(const ScanShape& s, const ScanArgs& a, dim3 grid, cudaStream_t st, bool launch = true,
                      bool pdl = false) {
  switch (s.rw) {
    case 1: return launch_metric<QB, 1>(s, a, grid, st, launch, pdl);
    case 2: return launch_metric<QB, 2>(s, a, grid, st, launch, pdl);
    default: return launch_metric<QB, 4>(s, a, grid, st, launch, pdl);
  }
}

}  // namespace

size_t scan_smem_bytes(const ScanShape& s, uint32_t dp, uint32_t k, uint32_t stages) {
  return scan_layout(s.qb, s.rw, dp, k, stages).total;
}

cudaError_t launch_scan(const ScanShape& s, const ScanArgs& a, dim3 grid, cudaStream_t stream, bool pdl) {
  switch (s.qb) {
    case 1: return launch_rw<1>(s, a, grid, stream, true, pdl);
    case 2: return launch_rw<2>(s, a, grid, stream, true, pdl);
    case 4: return launch_rw<4>(s, a, grid, stream, true, pdl);
    default: return launch_rw<8>(s, a, grid, stream, true, pdl);
  }
}

cudaError_t scan_prepare(const ScanShape& s, uint32_t dp, uint32_t k, uint32_t stages) {
  ScanArgs a{};
  a.dp = dp;
  a.k = k;
  a.stages = stages;
  switch (s.qb) {
    case 1: return launch_rw<1>(s, a, dim3(1), nullptr, false);
    case 2: return launch_rw<2>(s, a, dim3(1), nullptr, false);
    case 4: return launch_rw<4>(s, a, dim3(1), nullptr, false);
    default: return launch_rw<8>(s, a, dim3(1), nullptr, false);
  }
}

cudaError_t launch_merge(const MergeArgs& m, cudaStream_t stream) {
  if (m.margin && (m.kk == 0 || m.kk > m.k)) return cudaErrorInvalidValue;
  if (m.nq == 0) return cudaSuccess;
  if (m.k <= 32) {
    merge_kernel<1><<<m.nq, 256, 0, stream>>>(m);
  } else if (m.k <= 64) {
    merge_kernel<2><<<m.nq, 256, 0, stream>>>(m);
  } else {
    merge_kernel<4><<<m.nq, 256, 0, stream>>>(m);
  }
  return cudaGetLastError();
}

cudaError_t launch_fill_missing(float* out_d, uint32_t* out_i, size_t count, cudaStream_t stream) {
  if (count == 0) return cudaSuccess;
  const unsigned blocks = unsigned(count / 256 + 1 < 1024 ? count / 256 + 1 : 1024);
  fill_missing_kernel<<<blocks, 256, 0, stream>>>(out_d, out_i, count);
  return cudaGetLastError();
}

}  // namespace vsg
