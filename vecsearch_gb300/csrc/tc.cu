// Tensor-core paths: BF16 (or FP8-e4m3) shortlist (tcgen05 + TMEM + TMA) and exact FP32 rerank,
// with an optional certificate that makes the result exact.
//
// The reference has no tensor-core path; its large-batch kernel is a CUDA-core SGEMM
// (src/gpu_brute_force.cu:142-218). Here the base keeps an FP32 master copy and a tile-major
// BF16 (or e4m3) copy.
//
// prepare_queries_kernel: bf16 queries and norms, shared thresholds reset, certificate bounds E
//   and margins (certified path).
// tc_shortlist_kernel: CTA = 128 queries x a range of rows, one CTA per SM; 6 warps.
//   warp 0   TMA producer: the query block stays resident in shared memory; each 256-row tile of
//            the row copy arrives as 128-byte chunks (32 KB, one contiguous span of the
//            tile-major copy) into a ring of `stages` slots.
//   warp 1   allocates all 512 TMEM columns (two 128 x 256 FP32 accumulators); one lane issues
//            tcgen05.mma (M = 128 queries, N = 256 rows, K = 16 bf16 or 32 e4m3) over each chunk
//            and commits the slot back to the producer and the finished tile to the epilogue.
//   warps 2-5 epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31, one query per thread; per
//            tile it tests all 256 scores against its threshold with bit masks and one vote per
//            half, appends the few candidates to its query's global buffer, and compacts a
//            buffer that may overflow (a warp bitonic sort keeping the best k', or with margins
//            only the rows within the margin of the k-th best); thresholds are shared across
//            a query's splits. At the end each thread writes its split's sorted list and length.
//   A dump mode (the sample pass) writes raw approximate distances instead.
// sample_select_kernel: per query, an upper bound of the k'-th (or k-th + margin) best sampled
//   distance: the starting threshold.
// finish_kernel: per query, the split lists merged, the exact FP32 distances of the merged rows
//   with the streaming scan kernel's arithmetic (so a shortlist that holds the true top k yields
//   the scan kernel's results bit for bit), the top k by (dist, id), and the certificate.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp8.h>

#include <algorithm>
#include <mutex>

#include "device_common.cuh"
#include "launch.cuh"
#include "tc.cuh"

namespace vsg {

namespace {

// Epilogue groups: with candidate buffers of up to 256 entries (k' <= 120) two groups of four
// epilogue warps share every accumulator tile, group g taking its columns 128 g .. 128 g + 127,
// so two warps share each SM sub-partition and a tile's epilogue takes half as long (with one
// warp per sub-partition the MMAs of the next tile but one waited on it about a fifth of the time
// at large batches: two accumulators leave the epilogue one tile's MMAs). Each group keeps its
// own candidate buffers and writes its own list per (query, split). Larger buffers keep one
// group: the warp sort of 512 entries needs more registers than two groups leave a thread.
// With two groups the CTA has ten warps: the TMA producer, the MMA issuer and the epilogue
// warps 2-9 (group 0: warps 2-5, group 1: warps 6-9; warp w reads TMEM lanes 32 (w % 4) ..).
// Two sub-partitions then hold three warps, so a thread has at most 168 registers.
__host__ __device__ constexpr int tc_groups_cap(uint32_t cap) { return cap <= 256u ? 2 : 1; }
__host__ __device__ constexpr int tc_threads_cap(uint32_t cap) { return 64 + 128 * tc_groups_cap(cap); }
// A row of either operand copy is cut into chunks of 128 bytes (64 bf16 or 128 e4m3 elements).
constexpr uint32_t kChunkBytes = kTcQueries * 128;    // 16 KB: a chunk of the 128-query block (A)
constexpr uint32_t kRowChunkBytes = kTcRows * 128;    // 32 KB: a chunk of a 256-row tile (B)
constexpr uint32_t kL2Ahead = 8;  // row chunks a CTA prefetches into L2 past its ring before its first wait
constexpr uint32_t kTmemCols = 2 * kTcRows;           // two accumulators: all 512 columns
constexpr int kMaxTcStages = 8;

// Instruction descriptor, kind::f16: D FP32 (bits 4-5 = 1), A BF16 (bits 7-9 = 1), B BF16
// (bits 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at 24-28.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(kTcRows >> 3) << 17) |
                            (uint32_t(kTcQueries >> 4) << 24);

// Shared memory: [resident query block: nkc chunks][ring of `stages` slots][barriers]. A slot
// holds a 32 KB chunk of a row tile, plus the matching query chunk when the block is not resident.
struct TcLayout {
  size_t a, ring, slot, bars, total;  // offsets from the 1024-aligned base; slot = bytes per slot
};

__host__ __device__ inline TcLayout tc_layout(uint32_t stages, uint32_t nkc, bool resident) {
  TcLayout L;
  L.a = 0;
  L.slot = resident ? kRowChunkBytes : kRowChunkBytes + kChunkBytes;
  L.ring = resident ? size_t(nkc) * kChunkBytes : 0;
  L.bars = L.ring + size_t(stages) * L.slot;
  L.total = L.bars + 256;
  return L;
}

// Candidate-buffer capacity per query: the kp kept entries plus room for many appends between
// compactions (one is due when the next 32 scores might not fit). The warp sort holds 32 E = cap.
__host__ __device__ inline uint32_t tc_capacity(uint32_t kp) {
  return kp <= 16 ? 64 : kp <= 48 ? 128 : kp <= 120 ? 256 : 512;
}

// Element offset of (row, column c) in a tile-major operand copy with nkc chunks of ce elements
// (64 bf16 or 128 e4m3) per row.
__host__ __device__ inline size_t tile_major_offset(size_t row, uint32_t c, uint32_t nkc, uint32_t ce) {
  return ((row / kTcRows) * nkc + c / ce) * size_t(kTcRows) * ce + (row % kTcRows) * ce + c % ce;
}

// Approximate L2 distance from squared norms and the bf16 score: |q|^2 + |x|^2 - 2 s, rounded
// the same way wherever it is computed (the prefilter, the append and the sample pass agree).
__device__ __forceinline__ float l2_approx(float qn, float xn, float sc) { return __fmaf_rn(-2.f, sc, __fadd_rn(qn, xn)); }

__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Sorts the first `cnt` buffered entries of one query (entry j at bd[j] / bi[j], global memory)
// and keeps the best min(cnt, kp): back into the buffer, or, when out_d is set, into out_d /
// out_i as a sorted list (its length is returned; nothing is written past it). thr becomes entry kp - 1 when
// cnt >= kp, else (+inf, none). With a margin (mg >= 0) and at least kk entries, thr drops to
// (entry kk - 1) + mg, rounded up, when that is lower, and only the entries at or below it are
// kept. Returns the kept count.
template <int E>
__device__ __forceinline__ uint32_t compact_query(float* bd, uint32_t* bi, uint32_t cnt, uint32_t kp, uint32_t kk,
                                                  float mg, int lane, float& thr_d, uint32_t& thr_i, float* out_d,
                                                  uint32_t* out_i) {
  __syncwarp();  // the lanes' appends are visible to the whole warp
  WarpTopK<E> w;
#pragma unroll
  for (int e = 0; e < E; ++e) {
    const uint32_t j = uint32_t(e * 32 + lane);
    w.d[e] = j < cnt ? bd[j] : __int_as_float(0x7f800000);
    w.i[e] = j < cnt ? bi[j] : kNone;
  }
  w.sort(lane);
  uint32_t keep = cnt < kp ? cnt : kp;
  thr_d = __int_as_float(0x7f800000);
  thr_i = kNone;
  if (keep == kp) w.entry(int(kp) - 1, thr_d, thr_i);
  if (mg >= 0.f && kk > 0 && cnt >= kk) {  // warp-uniform: cnt, kk and mg are one lane's
    float dk;
    uint32_t ik;
    w.entry(int(kk) - 1, dk, ik);
    const float tm = __fadd_ru(dk, mg);
    if (nb_less(tm, kNone, thr_d, thr_i)) {
      thr_d = tm;
      thr_i = kNone;
      uint32_t c = 0;  // the list is sorted: the entries at or below tm come first
#pragma unroll
      for (int e = 0; e < E; ++e) c += __popc(__ballot_sync(kFull, nb_less(w.d[e], w.i[e], tm, kNone)));
      keep = c < keep ? c : keep;
    }
  }
  if (out_d) {
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const uint32_t j = uint32_t(e * 32 + lane);
      if (j < keep) {
        out_d[j] = w.d[e];
        out_i[j] = w.i[e];
      }
    }
  } else {
    __syncwarp();  // every lane has read its entries before any is overwritten
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const uint32_t j = uint32_t(e * 32 + lane);
      if (j < keep) {
        bd[j] = w.d[e];
        bi[j] = w.i[e];
      }
    }
    __syncwarp();
  }
  return keep;
}

struct CompactResult {
  uint32_t keep;  // entries kept (this lane's query, if it was compacted)
  float td;       // its new threshold (compact_query's thr), or (+inf, none)
  uint32_t ti;
};

// Compacts the buffers (cap = 32 E entries apart from wd / wi) of the lanes in `lanes`
// (warp-uniform) one after another; each lane passes its own count, kp and, for the final lists,
// its output list (else nullptr). Kept out of line: it is large and rarely runs, and the loop
// that calls it must stay small enough for the instruction cache.
template <int E>
__device__ __noinline__ CompactResult compact_warp(float* wd, uint32_t* wi, unsigned lanes, uint32_t cnt,
                                                   uint32_t kp, uint32_t kk, float mg, float* out_d, uint32_t* out_i,
                                                   int lane, float thr_d, uint32_t thr_i) {
  CompactResult r{cnt, __int_as_float(0x7f800000), kNone};
  // Final lists of many queries at once (large batches) are copied without a sort; a few (small
  // batches, where the finish kernel's cost follows the lists' lengths) are sorted so that the
  // margin cut at their own k-th entry shortens them.
  const bool copy_final =
      __any_sync(kFull, out_d != nullptr) && __popc(lanes) > int(kSortedListQueries);  // warp-uniform
  while (lanes) {
    const int src = __ffs(lanes) - 1;
    lanes &= lanes - 1;
    float* od = reinterpret_cast<float*>(__shfl_sync(kFull, reinterpret_cast<unsigned long long>(out_d), src));
    uint32_t* oi = reinterpret_cast<uint32_t*>(__shfl_sync(kFull, reinterpret_cast<unsigned long long>(out_i), src));
    float td;
    uint32_t ti;
    const uint32_t n = __shfl_sync(kFull, cnt, src), k = __shfl_sync(kFull, kp, src);
    const uint32_t k1 = __shfl_sync(kFull, kk, src);
    const float m1 = __shfl_sync(kFull, mg, src);
    float* bd = wd + size_t(src) * (32 * E);
    uint32_t* bi = wi + size_t(src) * (32 * E);
    uint32_t keep;
    if (copy_final && n <= k) {
      // A final list that fits needs no sort: the warp copies the entries at or below the query's
      // threshold, 32 at a time, and then swaps the smallest (by order key, then id) to the front,
      // since the finish kernel bounds the k-th best from the lists' first entries.
      const float t_d = __shfl_sync(kFull, thr_d, src);
      const uint32_t t_i = __shfl_sync(kFull, thr_i, src);
      __syncwarp();  // the lanes' appends are visible to the whole warp
      keep = 0;
      unsigned long long best = ~0ull;
      uint32_t best_at = 0;
      for (uint32_t j0 = 0; j0 < n; j0 += 32) {
        const uint32_t j = j0 + uint32_t(lane);
        const float dv = j < n ? bd[j] : 0.f;
        const uint32_t iv = j < n ? bi[j] : kNone;
        const bool take = j < n && (nb_less(dv, iv, t_d, t_i) || (dv == t_d && iv == t_i));
        const unsigned bal = __ballot_sync(kFull, take);
        if (take) {
          const uint32_t at = keep + __popc(bal & ((1u << lane) - 1u));
          od[at] = dv;
          oi[at] = iv;
          const unsigned long long key = (static_cast<unsigned long long>(order_key(dv)) << 32) | iv;
          if (key < best) {
            best = key;
            best_at = at;
          }
        }
        keep += __popc(bal);
      }
      unsigned long long least = best;
#pragma unroll
      for (int o = 16; o >= 1; o >>= 1) {
        const unsigned long long other = __shfl_xor_sync(kFull, least, o);
        least = other < least ? other : least;
      }
      const unsigned holder = __ballot_sync(kFull, best == least && least != ~0ull);
      __syncwarp();  // every lane's copies are visible before the swap reads slot 0
      if (holder && lane == __ffs(holder) - 1 && best_at != 0) {
        const float d0 = od[0];
        const uint32_t i0 = oi[0];
        od[best_at] = d0;
        oi[best_at] = i0;
        od[0] = key_float(uint32_t(best >> 32));
        oi[0] = uint32_t(best);
      }
      td = __int_as_float(0x7f800000);
      ti = kNone;
    } else if (E > 1 && n <= 32)  // else the smallest sort that holds the buffered entries
      keep = compact_query<1>(bd, bi, n, k, k1, m1, lane, td, ti, od, oi);
    else if (E > 2 && n <= 64)
      keep = compact_query<(E > 2 ? 2 : E)>(bd, bi, n, k, k1, m1, lane, td, ti, od, oi);
    else if (E > 4 && n <= 128)
      keep = compact_query<(E > 4 ? 4 : E)>(bd, bi, n, k, k1, m1, lane, td, ti, od, oi);
    else if (E > 8 && n <= 256)
      keep = compact_query<(E > 8 ? 8 : E)>(bd, bi, n, k, k1, m1, lane, td, ti, od, oi);
    else
      keep = compact_query<E>(bd, bi, n, k, k1, m1, lane, td, ti, od, oi);
    if (lane == src) {
      r.keep = keep;
      r.td = td;
      r.ti = ti;
    }
  }
  return r;
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, rows 128 bytes apart, 8-row
// groups 1024 bytes apart (the layout a 64 x R box TMA copy with 128-byte swizzle writes).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = uint64_t((saddr & 0x3FFFFu) >> 4);  // start address
  d |= uint64_t(1) << 16;                          // leading byte offset (unused with this swizzle)
  d |= uint64_t(1024 >> 4) << 32;                  // stride byte offset: 8 rows x 128 bytes
  d |= uint64_t(1) << 46;                          // descriptor version
  d |= uint64_t(2) << 61;                          // 128-byte swizzle
  return d;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar,
                                            uint64_t policy) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint"
      " [%0], [%1, {%2, %3}], [%4], %5;" ::"r"(smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_addr(bar)), "l"(policy)
      : "memory");
}

// Brings the box at (x, y) of a tensor map into L2 (no shared memory, no barrier).
__device__ __forceinline__ void tma_prefetch_l2(const CUtensorMap* map, int x, int y) {
  asm volatile("cp.async.bulk.prefetch.tensor.2d.L2.global.tile [%0, {%1, %2}];" ::"l"(reinterpret_cast<uint64_t>(map)),
               "r"(x), "r"(y)
               : "memory");
}

__device__ __forceinline__ uint64_t policy_evict_last() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate)
      : "memory");
}

// Instruction descriptor, kind::f8f6f4: D FP32 (bits 4-5 = 1), A and B E4M3 (type 0 at bits 7-9
// and 10-12), both K-major, N >> 3 at bits 17-22, M >> 4 at 24-28. K = 32 per instruction.
constexpr uint32_t kIdescF8 = (1u << 4) | (uint32_t(kTcRows >> 3) << 17) | (uint32_t(kTcQueries >> 4) << 24);

__device__ __forceinline__ void tc_mma_f8(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(kIdescF8), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
               : "memory");
}

// tcgen05.ld and tcgen05.wait::ld are .sync.aligned: every lane of the warp must execute them
// together, so the warp is reconverged first (the score filter before them branches per lane).
// The load is asynchronous: its registers are valid only after tmem_wait32, which names them as
// read-write operands so that no use can be scheduled before it.
__device__ __forceinline__ void tmem_issue32(uint32_t taddr, uint32_t (&v)[32]) {
  __syncwarp();
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
        "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
        "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
        "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
      : "r"(taddr));
}

__device__ __forceinline__ void tmem_wait32(uint32_t (&v)[32]) {
  __syncwarp();
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(v[0]), "+r"(v[1]), "+r"(v[2]), "+r"(v[3]), "+r"(v[4]), "+r"(v[5]), "+r"(v[6]), "+r"(v[7]),
                 "+r"(v[8]), "+r"(v[9]), "+r"(v[10]), "+r"(v[11]), "+r"(v[12]), "+r"(v[13]), "+r"(v[14]),
                 "+r"(v[15]), "+r"(v[16]), "+r"(v[17]), "+r"(v[18]), "+r"(v[19]), "+r"(v[20]), "+r"(v[21]),
                 "+r"(v[22]), "+r"(v[23]), "+r"(v[24]), "+r"(v[25]), "+r"(v[26]), "+r"(v[27]), "+r"(v[28]),
                 "+r"(v[29]), "+r"(v[30]), "+r"(v[31])
               :
               : "memory");
}


// v[j] for a run-time j in [0, 32): a tree of selects over compile-time indices, so the array
// stays in registers (an indexed read would move it to local memory).
__device__ __forceinline__ uint32_t pick32(const uint32_t (&v)[32], uint32_t j) {
  uint32_t t16[16], t8[8], t4[4], t2[2];
#pragma unroll
  for (int i = 0; i < 16; ++i) t16[i] = (j & 16u) ? v[16 + i] : v[i];
#pragma unroll
  for (int i = 0; i < 8; ++i) t8[i] = (j & 8u) ? t16[8 + i] : t16[i];
#pragma unroll
  for (int i = 0; i < 4; ++i) t4[i] = (j & 4u) ? t8[4 + i] : t8[i];
#pragma unroll
  for (int i = 0; i < 2; ++i) t2[i] = (j & 2u) ? t4[2 + i] : t4[i];
  return (j & 1u) ? t2[1] : t2[0];
}

template <int E, bool L2, bool F8>
__global__ void __launch_bounds__(tc_threads_cap(32u * E), 1)
    tc_shortlist_kernel(const __grid_constant__ CUtensorMap qmap, const __grid_constant__ CUtensorMap xmap,
                        const TcArgs a) {
  extern __shared__ unsigned char smem_raw[];
  // 128-byte swizzled tiles need 1024-byte aligned addresses.
  const uint32_t raw = smem_addr(smem_raw);
  unsigned char* smem = smem_raw + ((1024u - (raw & 1023u)) & 1023u);
  const uint32_t stages = a.stages;
  const bool resident = a.resident != 0;
  // A 128-byte chunk of a row holds 64 bf16 or 128 e4m3 elements.
  constexpr uint32_t kChunkElems = F8 ? 128u : uint32_t(kTcKChunk);
  const uint32_t nkc = (a.dp + kChunkElems - 1) / kChunkElems;
  const TcLayout L = tc_layout(stages, nkc, resident);
  unsigned char* qres = smem + L.a;    // resident query block: chunk kc at kc * kChunkBytes
  unsigned char* ring = smem + L.ring;
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + L.bars);
  uint64_t* empty = full + kMaxTcStages;
  uint64_t* tfull = empty + kMaxTcStages;  // [2]
  uint64_t* tempty = tfull + 2;            // [2]
  uint64_t* afull = tempty + 2;            // resident query block landed
  uint64_t* aempty = afull + 1;            // ... and no MMA reads it any more
  uint64_t* done = aempty + 1;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
  uint64_t* stall_bar = done + 2;  // after the TMEM slot word; within the 256 bytes of barriers

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  constexpr uint32_t G = uint32_t(tc_groups_cap(32u * E));  // epilogue groups, lists per (query, split)
  constexpr int kEpi0 = 2;                                    // the first epilogue warp
  const bool persistent = a.hdr != nullptr;
  const uint32_t nq = persistent ? a.hdr->nq : a.nq;
  const uint32_t nqb = persistent ? a.hdr->nqb : a.nqb;
  const uint32_t nsplit = persistent ? a.hdr->nsplit : a.nsplit;
  const uint32_t rows_per_split = persistent ? a.hdr->rows_per_split : a.rows_per_split;
  const uint32_t nitems = persistent ? a.hdr->items : nqb * nsplit;
  constexpr uint32_t cap = 32u * E;
  __shared__ uint32_t item_slot;
  // Epilogue warps' row norms (L2) and row scales (e4m3 copies) of their group's columns of a
  // tile, two tiles' worth (the next tile's are copied in while this one's are used).
  constexpr uint32_t kGroupRows = kTcRows / G;
  __shared__ __align__(16) float xs_buf[4 * G][2][L2 ? kGroupRows : 4];
  __shared__ __align__(16) float xsc_buf[4 * G][2][F8 ? kGroupRows : 4];

  if (tid == 0) {
    for (uint32_t s = 0; s < stages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);  // the MMAs that read the slot have completed
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], 4 * G);  // one arrival per epilogue warp
    }
    mbar_init(afull, 1);
    mbar_init(aempty, 1);
    mbar_init(done, 1);
    if (a.stall) mbar_init(stall_bar, 1);  // nothing ever arrives on it
    mbar_fence_init();
  }
  if (warp == 1) {
    __syncwarp();  // .sync.aligned: the whole warp, converged
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmem_slot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;
  const unsigned long long wl = a.wait_ns ? a.wait_ns : kWaitLimitNs;
  pdl_trigger();
  // Launched as a dependent of the previous kernel: the producer of a non-serving launch with a
  // resident query block first fills the ring with row chunks (the operand copy of the rows was
  // written long before), then waits; every other thread waits before the first item.
  const bool prefetch_rows = !persistent && resident && warp == 0 && lane == 0;
  bool waited = false;
  if (!prefetch_rows) {
    pdl_wait();
    waited = true;
  }

  // Ring, accumulator and query-block positions carry over from one item to the next; every
  // role walks the same items and tiles in the same order, so they stay in step.
  uint32_t s = 0, ph = 0;      // smem ring (producer and MMA issuer)
  uint32_t tglob = 0;          // tiles so far (MMA issuer and epilogue): TMEM buffer tglob & 1
  uint32_t aitem = 0;          // items that loaded a resident query block (its barrier phases)
  uint32_t pending = 0, last_ph = 0;
  bool a_pending = false;
  uint32_t a_last = 0;
  bool ok = true;
  const uint64_t stream_policy = policy_evict_first();
  const uint64_t keep_policy = policy_evict_last();

  for (uint32_t iter = 0;; ++iter) {
    if (tid == 0) item_slot = persistent ? atomicAdd(&a.hdr->next, 1u) : blockIdx.x + iter * gridDim.x;
    __syncthreads();
    const uint32_t item = item_slot;
    __syncthreads();  // everyone has read the slot before thread 0 may overwrite it
    if (item >= nitems) break;
    const uint32_t qb = item % nqb, split = item / nqb;
    const uint32_t qbase = qb * kTcQueries;
    const uint32_t row_begin = split * rows_per_split;
    // No 32-bit wrap: with its FP32 rows and a bf16 or e4m3 copy (160+ bytes a row) an index
    // holds under 2^31 rows in HBM, so row_begin + rows_per_split < 2^32.
    uint32_t row_end = min(a.n, row_begin + rows_per_split);
    const uint32_t sample_tiles = persistent ? a.hdr->sample_tiles : a.sample_tiles;
    if (a.dump) row_end = min(row_end, row_begin + sample_tiles * kTcRows);  // sample pass
    const uint32_t ntiles = row_end > row_begin ? (row_end - row_begin + kTcRows - 1) / kTcRows : 0;
    const bool load_a = resident && ntiles > 0;
    const uint32_t aph = aitem & 1u;

    if (warp == 0) {
      // ---------------- TMA producer ----------------
      if (lane == 0) {
        // Row chunk c of this item: chunk c % nkc of tile c / nkc (tile-major copy: kTcRows chunk
        // rows starting at y).
        const uint32_t nch = ntiles * nkc;
        auto issue_rows = [&](uint32_t c) {
          const uint32_t tile = row_begin / kTcRows + c / nkc, kc = c % nkc;
          const int y = int((tile * nkc + kc) * kTcRows);
          if (!mbar_wait(&empty[s], ph ^ 1, wl)) {
            ok = false;
            return;
          }
          unsigned char* st = ring + size_t(s) * L.slot;
          unsigned char* sb = resident ? st : st + kChunkBytes;
          mbar_arrive_expect_tx(&full[s], resident ? kRowChunkBytes : kRowChunkBytes + kChunkBytes);
          if (!resident) tma_load_2d(st, &qmap, int(kc * kChunkElems), int(qbase), &full[s], keep_policy);
          tma_load_2d(sb, &xmap, 0, y, &full[s], stream_policy);
          pending |= 1u << s;
          last_ph = (last_ph & ~(1u << s)) | (ph << s);
          if (++s == stages) {
            s = 0;
            ph ^= 1;
          }
        };
        uint32_t c0 = 0;
        if (!waited) {  // first item: rows before the wait, the query block after it
          for (const uint32_t pre = min(nch, stages); c0 < pre && ok; ++c0) issue_rows(c0);
          // The next kL2Ahead chunks into L2 as well: at small batches HBM idles while the query
          // preparation runs, and these are the first bytes the ring asks for after the wait.
          for (uint32_t c = c0; c < min(nch, c0 + kL2Ahead); ++c) {
            const uint32_t tile = row_begin / kTcRows + c / nkc, kc = c % nkc;
            tma_prefetch_l2(&xmap, 0, int((tile * nkc + kc) * kTcRows));
          }
          pdl_wait();
          waited = true;
        }
        if (load_a) {
          // The previous block's MMAs have finished before its chunks are overwritten.
          if (!mbar_wait(aempty, aph ^ 1u, wl)) {
            ok = false;
          } else {
            mbar_arrive_expect_tx(afull, nkc * kChunkBytes);
            for (uint32_t kc = 0; kc < nkc; ++kc)
              tma_load_2d(qres + size_t(kc) * kChunkBytes, &qmap, int(kc * kChunkElems), int(qbase), afull,
                          keep_policy);
            a_pending = true;
            a_last = aph;
          }
        }
        for (uint32_t c = c0; c < nch && ok; ++c) issue_rows(c);
      }
    } else if (warp == 1) {
      // ---------------- MMA issuer ----------------
      if (lane == 0) {
        if (load_a) {
          if (!mbar_wait(afull, aph, wl)) ok = false;
          tc_fence_after();
        }
        for (uint32_t t = 0; t < ntiles && ok; ++t, ++tglob) {
          const uint32_t b = tglob & 1, use = tglob >> 1;
          if (!mbar_wait(&tempty[b], (use & 1) ^ 1, wl)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t d = tmem_base + b * kTcRows;
          for (uint32_t kc = 0; kc < nkc; ++kc) {
            if (!mbar_wait(&full[s], ph, wl)) {
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t slot = smem_addr(ring + size_t(s) * L.slot);
            const uint32_t sa = resident ? smem_addr(qres + size_t(kc) * kChunkBytes) : slot;
            const uint32_t sb = resident ? slot : slot + kChunkBytes;
#pragma unroll
            for (uint32_t kk = 0; kk < 4; ++kk) {  // 32 bytes of K per instruction
              if constexpr (F8)
                tc_mma_f8(d, sw128_desc(sa + kk * 32), sw128_desc(sb + kk * 32), (kc | kk) != 0 ? 1u : 0u);
              else
                tc_mma(d, sw128_desc(sa + kk * 32), sw128_desc(sb + kk * 32), (kc | kk) != 0 ? 1u : 0u);
            }
            tc_commit(&empty[s]);  // the slot is free once these MMAs have read it
            if (++s == stages) {
              s = 0;
              ph ^= 1;
            }
          }
          if (ok) tc_commit(&tfull[b]);  // the accumulator is complete once all MMAs so far are
        }
        if (load_a && ok) tc_commit(aempty);  // the block may be replaced once these MMAs are done
      }
    } else if (warp >= kEpi0) {
      // ---------------- epilogue: one query per thread ----------------
      // Each thread appends scores that beat its query's threshold to the query's buffer (global
      // memory, rarely touched once the threshold is tight); when a buffer may overflow in the
      // next 32 scores, the warp sorts it together and keeps the best kp (the new threshold).
      const uint32_t quarter = uint32_t(warp & 3);  // TMEM lanes 32 quarter .. + 31
      const uint32_t ew = uint32_t(warp - kEpi0);     // epilogue warp 0 .. 4 G - 1
      const uint32_t group = ew / 4;                  // takes columns [group, group + 1) x 256 / G
      const int m = int(quarter) * 32 + lane;
      const uint32_t qg = qbase + uint32_t(m);
      const bool qvalid = qg < nq;
      const uint32_t kp = (persistent && qvalid) ? a.sq[qg].kp : a.kp;
      const uint32_t kk = (persistent && qvalid) ? a.sq[qg].k : a.kk;  // the margin's rank (k)
      const uint32_t* qmask = !qvalid ? nullptr
                              : persistent ? a.sq[qg].mask
                              : a.mask ? a.mask + size_t(qg) * a.mask_ld : nullptr;
      const float qn = (L2 && qvalid) ? a.qnorm[qg] : 0.f;
      const float qsc = (F8 && qvalid) ? a.qscale[qg] : 1.f;  // e4m3 copies: the query's scale
      // Certified path: the margin above the kk-th best beyond which no row is needed (-1: none).
      const float mg = (a.margin && qvalid) ? a.margin[qg] : -1.f;
      // this warp's 32 buffers
      float* wd = a.cbuf_d + ((size_t(blockIdx.x) * G + group) * kTcQueries + quarter * 32) * cap;
      uint32_t* wi = a.cbuf_i + ((size_t(blockIdx.x) * G + group) * kTcQueries + quarter * 32) * cap;
      uint32_t* gq = (a.gthr && qvalid && !a.dump) ? a.gthr + qg : nullptr;
      // A sampled threshold bounds the k'-th best from above: rows at or below it are kept.
      float thr_d = (a.thr_init && qvalid) ? a.thr_init[qg] : __int_as_float(0x7f800000);
      uint32_t thr_i = kNone;
      uint32_t cnt = 0;
      // Inner product: a cheap prefilter on the raw score. 1 - s <= thr needs s >= 1 - thr up to
      // rounding; the bound is lowered by 8 ulps of max(1, |thr|) so no candidate is lost.
      auto score_bound = [](float td) { return (1.f - td) - 8.f * 1.1920929e-7f * fmaxf(1.f, fabsf(td)); };
      float s_lo = score_bound(thr_d);
      // Another split's k'-th best also bounds this query's k'-th best (ties kept).
      auto tighten = [&](uint32_t key) {
        if (key != kKeyNone) {
          const float g = key_float(key);
          if (g < thr_d) {
            thr_d = g;
            thr_i = kNone;
            s_lo = score_bound(g);
          }
        }
      };
      const uint32_t dump_per_tile = a.dump_min ? uint32_t(kTcRows / 32) : uint32_t(kTcRows);
      float* dump_row = (a.dump && qvalid) ? a.dump + (size_t(qg) * nsplit + split) * sample_tiles * dump_per_tile
                                           : nullptr;
      auto compact_lanes = [&](unsigned lanes, bool final_list) {
        if (!lanes) return;
        const bool mine = (lanes >> lane) & 1u;
        float* od = nullptr;
        uint32_t* oi = nullptr;
        if (final_list && mine) {  // this group's shortlist of the split (lists are a.kp apart)
          const size_t o = (size_t(qg) * nsplit * G + size_t(split) * G + group) * a.kp;
          od = a.part_d + o;
          oi = a.part_i + o;
        }
        const CompactResult r = compact_warp<E>(wd, wi, lanes, cnt, kp, kk, mg, od, oi, lane, thr_d, thr_i);
        if (mine) {
          cnt = r.keep;
          if (final_list && a.part_n) a.part_n[size_t(qg) * nsplit * G + size_t(split) * G + group] = r.keep;
          if (r.ti != kNone || r.td != __int_as_float(0x7f800000)) {  // a threshold was set
            if (nb_less(r.td, r.ti, thr_d, thr_i)) {
              thr_d = r.td;
              thr_i = r.ti;
              s_lo = score_bound(r.td);
            }
            if (gq) atomicMin(gq, order_key(r.td));
          }
        }
      };
      uint32_t gkey = kKeyNone;  // other splits' published k'-th best, loaded one tile ahead
      if (a.stall && !__all_sync(kFull, mbar_wait(stall_bar, 0, wl))) {  // the test hook's wait
        if (lane == 0) atomicExch(a.status, kDevTimeout);
        ok = false;
      }
      // The norms and scales of this group's columns of tile tt into buffer sb, copied without
      // registers (16 bytes a lane) one tile ahead of their use: loaded after the accumulator's
      // wait they put a DRAM round trip into every tile. Rows at or past n read row n - 1 (their
      // columns are never allowed). One commit group per call, also when there is nothing to copy.
      // A warp whose 32 query slots are all padding (small batches) only keeps the tile handshake.
      const bool live = __any_sync(kFull, qvalid);
      auto stage_rows = [&](uint32_t tt, uint32_t sb) {
        if constexpr (L2 || F8) {
          if (live && tt < ntiles) {
            const uint32_t rb = row_begin + tt * kTcRows + group * kGroupRows;
            for (uint32_t p = uint32_t(lane) * 4u; p < kGroupRows; p += 128u) {
              const uint32_t row = rb + p;
              if (row + 4u <= a.n) {  // (row is a multiple of 4: 16-byte aligned)
                if constexpr (L2) cp_async16(&xs_buf[ew][sb][p], a.xnorm + row, true);
                if constexpr (F8) cp_async16(&xsc_buf[ew][sb][p], a.xscale + row, true);
              } else {
#pragma unroll
                for (uint32_t i = 0; i < 4; ++i) {
                  const uint32_t r = min(row + i, a.n - 1);
                  if constexpr (L2) xs_buf[ew][sb][p + i] = __ldg(a.xnorm + r);
                  if constexpr (F8) xsc_buf[ew][sb][p + i] = __ldg(a.xscale + r);
                }
              }
            }
          }
          cp_async_commit();
        }
      };
      stage_rows(0, tglob & 1);
      for (uint32_t t = 0; t < ntiles && ok; ++t, ++tglob) {
        const uint32_t b = tglob & 1, use = tglob >> 1;
        tighten(gkey);
        gkey = gq ? ld_relaxed(gq) : kKeyNone;
        stage_rows(t + 1, b ^ 1u);  // (buffer b ^ 1 held the previous tile's, done with)
        if (!__all_sync(kFull, mbar_wait(&tfull[b], use & 1, wl))) {
          if (lane == 0) atomicExch(a.status, kDevTimeout);
          ok = false;
          break;
        }
        tc_fence_after();
        if constexpr (L2 || F8) {  // this tile's copies (the next tile's may still be in flight)
          cp_async_wait<1>();
          __syncwarp();
        }
        const float* xs = xs_buf[ew][b];    // column j of chunk cg at (cg - cg0) x 32 + j
        const float* xsc = xsc_buf[ew][b];
        const int cg0 = int(group) * (kTcRows / 32 / G);
        const uint32_t r0 = row_begin + t * kTcRows;
        const uint32_t tbase = tmem_base + ((quarter * 32) << 16) + b * kTcRows;
        // Allowed rows of chunk c (32 rows from c0): inside the split, real query, filter bit.
        auto allowed = [&](uint32_t c0) {
          uint32_t al = c0 < row_end ? (row_end - c0 >= 32 ? ~0u : (1u << (row_end - c0)) - 1u) : 0u;
          if (qmask && al) al &= __ldg(qmask + (c0 >> 5));
          return qvalid ? al : 0u;
        };
        if (!live) {
        } else if (a.dump) {  // sample pass: raw distances out, nothing kept. The branch is warp-
                              // uniform (a.dump): lanes of padded query slots take it too and store nothing.
#pragma unroll 1
          for (uint32_t c = group * (kTcRows / 32 / G); c < (group + 1) * (kTcRows / 32 / G); ++c) {
            uint32_t v[32];
            tmem_issue32(tbase + c * 32, v);
            tmem_wait32(v);
            const uint32_t c0 = r0 + c * 32;
            const uint32_t allow = allowed(c0);
            if (dump_row) {
              float o[32];
              const int at = (int(c) - cg0) * 32;
#pragma unroll
              for (int j = 0; j < 32; ++j) {
                const float sc = F8 ? __uint_as_float(v[j]) * (qsc * xsc[at + j]) : __uint_as_float(v[j]);
                const float dist = L2 ? l2_approx(qn, xs[at + j], sc) : 1.f - sc;
                o[j] = ((allow >> j) & 1u) ? dist : __int_as_float(0x7f800000);
              }
              if (a.dump_min) {  // the 32 rows' smallest distance only
                float m = o[0];
#pragma unroll
                for (int j = 1; j < 32; ++j) m = fminf(m, o[j]);
                dump_row[t * (kTcRows / 32) + c] = m;
              } else {
                // 16-byte stores (the row's 32 values are contiguous and 128-byte aligned).
                float4* d4 = reinterpret_cast<float4*>(dump_row + t * kTcRows + c * 32);
#pragma unroll
                for (int j = 0; j < 8; ++j) d4[j] = make_float4(o[4 * j], o[4 * j + 1], o[4 * j + 2], o[4 * j + 3]);
              }
            }
          }
        } else {
          // The tile's scores arrive in loads of 64 columns. One reduction per 32 columns
          // (the largest score, or the smallest distance with the same expression as the
          // append) and one vote per half; the per-score path runs only when some lane may have
          // a candidate.
          // (the rows' scales are shared by the warp; each lane applies its query's)
#pragma unroll 1
          for (int cg = cg0; cg < cg0 + kTcRows / 32 / G; ++cg) {
            const int at = (cg - cg0) * 32;
            // Room for this chunk's appends, made before its scores are loaded (the out-of-line
            // sort then runs with few live registers).
            compact_lanes(__ballot_sync(kFull, cnt + 32 > cap), false);
            uint32_t v[32];
            tmem_issue32(tbase + uint32_t(cg) * 32, v);
            tmem_wait32(v);
            // The chunk's entries that may beat the threshold (the prefilter's test) as a bit
            // mask; one vote per 32 columns, and only the columns some lane needs go further.
            uint32_t bits;
            {
              uint32_t m[4] = {0u, 0u, 0u, 0u};  // four interleaved chains
#pragma unroll
              for (int j = 0; j < 32; ++j) {
                const float sc = F8 ? __uint_as_float(v[j]) * (qsc * xsc[at + j]) : __uint_as_float(v[j]);
                const bool p = L2 ? l2_approx(qn, xs[at + j], sc) <= thr_d : sc >= s_lo;
                m[j & 3] |= p ? (1u << j) : 0u;
              }
              bits = (m[0] | m[1] | m[2] | m[3]) & allowed(r0 + uint32_t(cg) * 32);
            }
            if (__any_sync(kFull, bits != 0u)) {  // rare once the threshold is tight
              const uint32_t c0 = r0 + uint32_t(cg) * 32;
              // Each lane walks its own candidate columns; the scores are still in v, picked
              // by a select tree. The loop runs as often as the busiest lane needs.
              uint32_t mine = bits;
              while (__any_sync(kFull, mine != 0u)) {
                const bool has = mine != 0u;
                const uint32_t j = has ? uint32_t(__ffs(mine) - 1) : 0u;
                mine &= mine - 1u;
                const float raw = __uint_as_float(pick32(v, j));
                if (has) {
                  const float sc = F8 ? raw * (qsc * xsc[at + j]) : raw;
                  const float dist = L2 ? l2_approx(qn, xs[at + j], sc) : 1.f - sc;
                  if (nb_less(dist, c0 + j, thr_d, thr_i)) {
                    wd[size_t(lane) * cap + cnt] = dist;
                    wi[size_t(lane) * cap + cnt] = c0 + j;
                    ++cnt;
                  }
                }
              }
            }
          }
        }
        if (L2 || F8) __syncwarp();  // every lane is done with buffer b before it is copied into again
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&tempty[b]);
      }
      if constexpr (L2 || F8) cp_async_wait<0>();  // (an early exit may leave copies in flight)
      if (a.dump) {  // sample pass: tiles past the split's end read as +inf
        if (dump_row && group == 0)
          for (uint32_t j = ntiles * dump_per_tile; j < sample_tiles * dump_per_tile; ++j)
            dump_row[j] = __int_as_float(0x7f800000);
      } else {
        // Sort every buffer, keep the best kp and write the split's shortlist.
        compact_lanes(ok ? __ballot_sync(kFull, qvalid) : 0u, true);
        if (a.xf) {  // its rows into L2 for the finish kernel's rerank (which starts a few us
          __syncwarp();  // after the pass, once every split is done; the warp wrote the lists)
          if (ok && qvalid) {
            const uint32_t* li = a.part_i + (size_t(qg) * nsplit * G + size_t(split) * G + group) * a.kp;
            for (uint32_t e = 0; e < cnt; ++e) bulk_prefetch_l2(a.xf + size_t(li[e]) * a.xf_ld, a.xf_ld * 4u);
          }
        }
      }
    }
    if (load_a) ++aitem;
    if (!__syncthreads_and(ok)) break;  // a role gave up: no further items
  }

  if (!waited) pdl_wait();  // a CTA without items still waits before it exits
  if (warp == 0 && lane == 0) {
    // Wait (bounded) until every issued copy has landed before the CTA may exit.
    for (uint32_t i = 0; i < stages; ++i)
      if ((pending >> i) & 1u)
        if (!mbar_wait(&full[i], (last_ph >> i) & 1u)) ok = false;
    if (a_pending && !mbar_wait(afull, a_last)) ok = false;
    if (!ok) atomicExch(a.status, kDevTimeout);
  }
  if (warp == 1 && lane == 0) {
    // Every MMA has finished before TMEM may be released.
    tc_commit(done);
    if (!mbar_wait(done, 0)) ok = false;
    if (!ok) atomicExch(a.status, kDevTimeout);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    __syncwarp();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(kTmemCols)
                 : "memory");
  }
}

// FP32 rows -> bf16 rows of stride dp (columns >= dim are zero); optional squared norms (FP32)
// and, for certification, the rows' largest rounding residual and norms.
__global__ void to_bf16_kernel(const float* __restrict__ src, size_t ld_src, size_t rows, uint32_t dim,
                               uint32_t dp, __nv_bfloat16* __restrict__ dst, float* __restrict__ norms,
                               float* __restrict__ bounds, size_t tile_row0) {
  const size_t row = (size_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32;
  const int lane = threadIdx.x & 31;
  if (row >= rows) return;
  const float* s = src + row * ld_src;
  const bool tiled = tile_row0 != kRowMajor;
  const uint32_t nkc = (dp + kTcKChunk - 1) / kTcKChunk;
  const uint32_t width = tiled ? nkc * uint32_t(kTcKChunk) : dp;  // tile-major chunks are whole
  float acc = 0.f, res = 0.f, accb = 0.f;
  for (uint32_t c = lane; c < width; c += 32) {
    const float v = c < dim ? s[c] : 0.f;
    const __nv_bfloat16 b = __float2bfloat16_rn(v);
    acc = fmaf(v, v, acc);
    const float vb = __bfloat162float(b);
    const float e = vb - v;  // exact: v and its rounding are within a factor of 2
    res = fmaf(e, e, res);
    accb = fmaf(vb, vb, accb);
    dst[tiled ? tile_major_offset(tile_row0 + row, c, nkc, kTcKChunk) : row * dp + c] = b;
  }
  for (int o = 16; o > 0; o >>= 1) {
    acc += __shfl_xor_sync(kFull, acc, o);
    res += __shfl_xor_sync(kFull, res, o);
    accb += __shfl_xor_sync(kFull, accb, o);
  }
  if (lane == 0) {
    if (norms) norms[row] = acc;
    if (bounds) {  // non-negative floats order like their bit patterns
      atomicMax(reinterpret_cast<unsigned*>(bounds) + 0, __float_as_uint(sqrtf(res)));
      atomicMax(reinterpret_cast<unsigned*>(bounds) + 1, __float_as_uint(sqrtf(acc)));
      atomicMax(reinterpret_cast<unsigned*>(bounds) + 2, __float_as_uint(sqrtf(accb)));
    }
  }
}

// e4m3 byte -> its value (exact in FP32).
__device__ __forceinline__ float e4m3_value(uint8_t b) {
  return __half2float(__half(__nv_cvt_fp8_to_halfraw(__nv_fp8_storage_t(b), __NV_E4M3)));
}

// FP32 rows -> e4m3 rows of stride dp8 bytes (columns >= dim are zero), one FP32 scale per row
// (max |x| / 448, the largest finite e4m3; 1 for a zero row) and optional squared FP32 norms.
// With bounds set, the rows' rounding bounds as for the bf16 copy (max |x~ - x|, max |x|,
// max |x~|, raised with atomicMax), where x~ = e4m3 value x scale: the differences and the
// copy's norms are summed in FP64 from exact products (4 + 24 significant bits), and rounded up.
__global__ void to_fp8_kernel(const float* __restrict__ src, size_t ld_src, size_t rows, uint32_t dim, uint32_t dp8,
                              uint8_t* __restrict__ dst, float* __restrict__ scale, float* __restrict__ norms,
                              float* __restrict__ bounds, size_t tile_row0) {
  const size_t row = (size_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32;
  const int lane = threadIdx.x & 31;
  if (row >= rows) return;
  const float* s = src + row * ld_src;
  float mx = 0.f, acc = 0.f;
  for (uint32_t c = lane; c < dim; c += 32) {
    const float v = s[c];
    mx = fmaxf(mx, fabsf(v));
    acc = fmaf(v, v, acc);
  }
  for (int o = 16; o > 0; o >>= 1) {
    mx = fmaxf(mx, __shfl_xor_sync(kFull, mx, o));
    acc += __shfl_xor_sync(kFull, acc, o);
  }
  const float sc = mx > 0.f ? mx / 448.f : 1.f;
  const float inv = 1.f / sc;
  const bool tiled = tile_row0 != kRowMajor;
  const uint32_t nkc = (dp8 + 127) / 128;
  const uint32_t width = tiled ? nkc * 128u : dp8;  // tile-major chunks are whole
  double res = 0.0, accb = 0.0;
  for (uint32_t c = lane; c < width; c += 32) {
    const float v = c < dim ? s[c] : 0.f;
    const uint8_t b = c < dim ? uint8_t(__nv_cvt_float_to_fp8(v * inv, __NV_SATFINITE, __NV_E4M3)) : uint8_t(0);
    dst[tiled ? tile_major_offset(tile_row0 + row, c, nkc, 128) : row * dp8 + c] = b;
    if (bounds && c < dim) {
      const double xt = double(e4m3_value(b)) * double(sc);  // exact
      const double e = xt - double(v);
      res = fma(e, e, res);
      accb = fma(xt, xt, accb);
    }
  }
  if (bounds)
    for (int o = 16; o > 0; o >>= 1) {
      res += __shfl_xor_sync(kFull, res, o);
      accb += __shfl_xor_sync(kFull, accb, o);
    }
  if (lane == 0) {
    scale[row] = sc;
    if (norms) norms[row] = acc;
    if (bounds) {  // non-negative floats order like their bit patterns
      atomicMax(reinterpret_cast<unsigned*>(bounds) + 0, __float_as_uint(__double2float_ru(sqrt(res))));
      atomicMax(reinterpret_cast<unsigned*>(bounds) + 1, __float_as_uint(sqrtf(acc)));
      atomicMax(reinterpret_cast<unsigned*>(bounds) + 2, __float_as_uint(__double2float_ru(sqrt(accb))));
    }
  }
}

// Tuning queries: row r is 0.9 x_i + 0.1 x_j for two rows picked by a hash of r: near a row of
// the index, as a real query near its neighbours is, without coinciding with it.
__global__ void midpoint_rows_kernel(float* dst, const float* src, uint32_t dp, uint32_t n, uint32_t count) {
  const uint32_t r = blockIdx.x;
  if (r >= count) return;
  uint64_t h = 0x9E3779B97F4A7C15ull * (uint64_t(r) + 1);
  h ^= h >> 31;
  const uint32_t i = uint32_t(h % n), j = uint32_t((h >> 32) % n);
  for (uint32_t c = threadIdx.x; c < dp; c += blockDim.x)
    dst[size_t(r) * dp + c] = 0.9f * src[size_t(i) * dp + c] + 0.1f * src[size_t(j) * dp + c];
}

// Serving fallback, after the scan: the first k of slot j's kmax results go to query
// fail_list[j]'s place in the output block; the count is added to the tally.
__global__ void serve_scatter_kernel(const uint32_t* count, const uint32_t* fail_list, const ServeQuery* sq,
                                     const float* src_d, const uint32_t* src_i, uint32_t kmax, float* out_d,
                                     uint32_t* out_i, unsigned long long* tally) {
  const uint32_t j = blockIdx.x, cnt = *count;
  if (tally && j == 0 && threadIdx.x == 0) atomicAdd(tally, (unsigned long long)cnt);
  if (j >= cnt) return;
  const ServeQuery s = sq[fail_list[j]];
  for (uint32_t c = threadIdx.x; c < s.k; c += blockDim.x) {
    out_d[s.out_off + c] = src_d[size_t(j) * kmax + c];
    out_i[s.out_off + c] = src_i[size_t(j) * kmax + c];
  }
}

template <bool L2>
__device__ __forceinline__ float exact_distance(const float4* q4, const float4* x4, uint32_t nc, int lane) {
  float acc = 0.f;
  for (uint32_t c = lane; c < nc; c += 32) {
    const float4 qv = q4[c], xv = __ldg(x4 + c);
    if constexpr (L2) {
      float e = qv.x - xv.x;
      acc = fmaf(e, e, acc);
      e = qv.y - xv.y;
      acc = fmaf(e, e, acc);
      e = qv.z - xv.z;
      acc = fmaf(e, e, acc);
      e = qv.w - xv.w;
      acc = fmaf(e, e, acc);
    } else {
      acc = fmaf(qv.x, xv.x, acc);
      acc = fmaf(qv.y, xv.y, acc);
      acc = fmaf(qv.z, xv.z, acc);
      acc = fmaf(qv.w, xv.w, acc);
    }
  }
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) acc += __shfl_xor_sync(kFull, acc, o);
  return L2 ? acc : 1.0f - acc;
}

// exact_distance for G rows at once (row g at x4[g], nullptr: skipped): the same arithmetic per
// row, so the same bits, with the rows' loads in flight together.
template <bool L2, int G, int kAhead>
__device__ __forceinline__ void exact_distances(const float4* q4, const float4* const (&x4)[G], uint32_t nc, int lane,
                                                float (&out)[G]) {
  // The loads of kAhead chunk steps (kAhead x 16 bytes a row per lane) are issued before any is
  // used; the sums still take the chunks in increasing order.
  float acc[G];
#pragma unroll
  for (int g = 0; g < G; ++g) acc[g] = 0.f;
  for (uint32_t c0 = lane; c0 < nc; c0 += 32u * kAhead) {
    float4 xv[kAhead][G];
#pragma unroll
    for (int u = 0; u < kAhead; ++u) {
      const uint32_t c = c0 + 32u * u;
#pragma unroll
      for (int g = 0; g < G; ++g) xv[u][g] = (c < nc && x4[g]) ? __ldg(x4[g] + c) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int u = 0; u < kAhead; ++u) {
      const uint32_t c = c0 + 32u * u;
      if (c >= nc) break;
      const float4 qv = q4[c];
#pragma unroll
      for (int g = 0; g < G; ++g) {
        if constexpr (L2) {
          float e = qv.x - xv[u][g].x;
          acc[g] = fmaf(e, e, acc[g]);
          e = qv.y - xv[u][g].y;
          acc[g] = fmaf(e, e, acc[g]);
          e = qv.z - xv[u][g].z;
          acc[g] = fmaf(e, e, acc[g]);
          e = qv.w - xv[u][g].w;
          acc[g] = fmaf(e, e, acc[g]);
        } else {
          acc[g] = fmaf(qv.x, xv[u][g].x, acc[g]);
          acc[g] = fmaf(qv.y, xv[u][g].y, acc[g]);
          acc[g] = fmaf(qv.z, xv[u][g].z, acc[g]);
          acc[g] = fmaf(qv.w, xv[u][g].w, acc[g]);
        }
      }
    }
  }
#pragma unroll
  for (int g = 0; g < G; ++g) {
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) acc[g] += __shfl_xor_sync(kFull, acc[g], o);
    out[g] = L2 ? acc[g] : 1.0f - acc[g];
  }
}

// The certificate's bound E on |approximate - FP32 distance| for one query, from its sums
// |q|^2, |q~|^2 and |q~ - q|^2 (FP32, d terms each; q~ = the bf16 query) and the rows' bounds
// xbound = [max |x~ - x|, max |x|, max |x~|]. In FP32 with every operation rounded up: all terms
// are non-negative and every operation is monotone, so the result is at least the formula's
// exact value (FP64 would be as safe but is slow on GB300). F8: q~ and x~ are the e4m3 copies
// times their scales, and the score the kernel uses is (sum of e4m3 products) x (query scale x row
// scale), two more FP32 roundings: at most 2 u (1 + u) |q~||x~|, taken as 4 u |q~||x~|.
template <bool L2, bool F8 = false>
__device__ float cert_error(float sq2, float sqb2, float sr2, uint32_t dp, const float* xbound) {
  auto mul = [](float a, float b) { return __fmul_ru(a, b); };
  auto add = [](float a, float b) { return __fadd_ru(a, b); };
  const float u = 5.9604644775390625e-08f, dd = float(dp);  // 2^-24; dp is exact in FP32
  const float du = mul(dd, u);
  // FP32 sums of d non-negative terms: inflate by (1 + 2 d u) before use.
  const float infl = add(1.f, mul(2.f, du));
  const float qn = __fsqrt_ru(mul(sq2, infl)), qbn = __fsqrt_ru(mul(sqb2, infl)), rq = __fsqrt_ru(mul(sr2, infl));
  const float R = mul(xbound[0], infl), N = mul(xbound[1], infl), Nb = mul(xbound[2], infl);
  // |bf16 score - q.x| <= |q~||x~ - x| + |q~ - q||x| + accumulation (8 d u |q~||x~|);
  // |FP32 q.x - q.x| <= 2 d u |q||x|.
  float e_dot = add(add(mul(qbn, R), mul(rq, N)), add(mul(mul(8.f, du), mul(qbn, Nb)), mul(mul(2.f, du), mul(qn, N))));
  if (F8) e_dot = add(e_dot, mul(mul(4.f, u), mul(qbn, Nb)));
  float e;
  if (L2) {  // norms (d u each), two roundings of |q|^2 + |x|^2 - 2 s, FP32 squared differences
    const float q2n2 = add(mul(qn, qn), mul(N, N));
    const float qpn = add(qn, N);
    e = add(add(mul(2.f, e_dot), mul(du, q2n2)),
            add(mul(mul(4.f, u), add(q2n2, mul(2.f, mul(qbn, Nb)))), mul(mul(add(dd, 2.f), u), mul(qpn, qpn))));
  } else {  // the two roundings of 1 - s
    e = add(e_dot, mul(mul(4.f, u), add(1.f, mul(qn, N))));
  }
  return mul(e, 1.1f);  // margin over the (already worst-case) terms; 1.1f is above 1.1
}

// Thread-block cluster helpers (sm_90+): the CTA's rank and the cluster's size along x, a barrier
// over every thread of the cluster (release / acquire: shared-memory writes before it are seen
// after it), and 4-byte loads and stores in rank r's shared memory at the address a variable has
// in this CTA's.
__device__ __forceinline__ uint32_t cluster_nctarank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t cluster_ctarank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ uint32_t cluster_addr(const void* local, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(smem_addr(local)), "r"(rank));
  return r;
}
__device__ __forceinline__ uint32_t ld_cluster_u32(uint32_t addr) {
  uint32_t v;
  asm volatile("ld.shared::cluster.u32 %0, [%1];" : "=r"(v) : "r"(addr) : "memory");
  return v;
}
__device__ __forceinline__ void st_cluster_f32(uint32_t addr, float v) {
  asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(addr), "f"(v) : "memory");
}

// The shortlist path's tail (FinishArgs), one CTA of kFinishThreads per query.
//   1. Stage: the split lists' real entries (part_n of each) are copied into shared memory when
//      they fit (stage_cap entries), else the passes below read the lists in global memory. With
//      up to 1,024 lists the copy is flat: the lengths are scanned into offsets and every thread
//      copies independent entries (one thread per list left a few threads walking long lists
//      with dependent loads). With margins, each list's first entry is its smallest (every
//      producer writes them so), and these heads come in with the lengths: the k-th smallest head
//      h bounds the k-th best a_k from above (k lists hold an entry at or below it), so no entry
//      above c = h + margin can be reranked, and only the lists whose head is at or below c are
//      read, their entries above c dropped. (At batch 1 over the bf16 copy the lists held ~2,800
//      entries for ~70 reranked rows: no split sees enough of the query's near rows for its own
//      k-th best to be tight.) With margins and no more entries in all than the rerank takes in
//      one pass (two with a cluster), every entry is staged and reranked without a bound.
//   2. Cut: the `target`-th smallest approximate distance (k with margins, else the shortlist
//      size k') by exact radix selection on order keys (a min / max pass, then 8-bit rounds below
//      the highest bit where the keys differ); the cut is that value, plus the margin (rounded
//      up) on the certified path. Every entry at or below the cut is reranked, at most
//      kRerankMax: beyond that the cut drops to the entries strictly below the kRerankMax-th.
//   3. Rerank: the exact FP32 distance of every kept row with the scan kernel's arithmetic (lane
//      l sums 16-byte chunks l, l + 32, ... in order, then a butterfly over lanes 16 .. 1), so a
//      candidate set that holds the true top k yields the scan kernel's results bit for bit.
//   4. The top k by (FP32 dist, id): each candidate's rank among the (order key, id) pairs,
//      counted in shared memory (beyond 256 candidates, among those at or below a bound of the
//      k-th key only); the k-th FP32 distance D_k.
//   5. Certificate (fail_count set): every row left out has approximate distance >= L = min(sample
//      threshold, final shared threshold, the cut when it left entries out); if L - E > D_k
//      (rounded down) no such row can enter the top k, else the query is listed for the scan.
// Nothing is read when the status word says a shortlist kernel gave up (its lists may be stale),
// and row ids at or beyond n are never dereferenced.
constexpr int kFinishThreads = 512;
constexpr uint32_t kRerankMax = 2048;  // (the e4m3 copy's wider margin keeps ~1,000 rows at 1M x 384)
constexpr uint32_t kKeyAll = 0xFFFFFFFFu;  // cut key that keeps every entry
constexpr uint32_t kStageSplits = 1024;    // lists the flat staging copy handles at most
constexpr uint32_t kSmallSelect = 256;     // staged entries up to which the cut ranks them in one pass

struct FinishSmem {
  size_t qs, cd, ci, cx, sd, si, total;  // byte offsets: query, candidates (approx, id, exact), staging
};
__host__ __device__ inline FinishSmem finish_smem(uint32_t dp, uint32_t stage_cap) {
  FinishSmem L;
  const size_t qbytes = dp <= 4096 ? (size_t(dp) * 4 + 15) / 16 * 16 : 0;
  L.qs = 0;
  L.cd = qbytes;
  L.ci = L.cd + kRerankMax * 4;
  L.cx = L.ci + kRerankMax * 4;
  // (at least kRerankMax entries: the top-k sort reuses the staging area as 8-byte keys)
  const size_t stage = stage_cap > kRerankMax ? stage_cap : kRerankMax;
  L.sd = L.cx + kRerankMax * 4;
  L.si = L.sd + stage * 4;
  L.total = L.si + stage * 4;
  return L;
}

// kWide (a batch no larger than the SM count: one CTA per SM, registers to spare): the rerank
// loads three chunk steps of each row before using them, so a 384-dim row arrives in one round
// trip; otherwise one step at a time, with fewer registers, so two CTAs share an SM.
template <bool L2, bool kWide>
__global__ void __launch_bounds__(kFinishThreads) finish_kernel(const FinishArgs a) {
  extern __shared__ __align__(16) unsigned char fsm[];
  __shared__ uint32_t hist[256];
  __shared__ uint32_t s_total, s_cnt, s_kmin, s_kmax, s_prefix, s_rank, s_all, s_heads, s_staged;
  __shared__ uint32_t s_off[kStageSplits + 1];  // list offsets of the flat staging copy
  __shared__ float s_dk;
  pdl_trigger();
  pdl_wait();
  // A query may have a cluster of CTAs (launched so for small batches, wide variant): rank 0 does
  // everything but share the rerank, which every CTA of the cluster does (below).
  const uint32_t csize = kWide ? cluster_nctarank() : 1u, crank = csize > 1 ? cluster_ctarank() : 0u;
  const uint32_t q = blockIdx.x / csize;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  constexpr int nwarps = kFinishThreads / 32;
  const bool serving = a.hdr != nullptr;
  if (serving && q >= a.hdr->nq) return;
  // A shortlist kernel that gave up may have left stale lists: nothing is used then (the status is
  // read here and tested once the first loads, harmless either way, are issued; CTA-uniform, and
  // the same for every CTA of a cluster, before any cluster barrier).
  const bool stale = a.status && *reinterpret_cast<const volatile int*>(a.status) != 0;
  const uint32_t nsplit = (serving ? a.hdr->nsplit : a.nsplit) * max(1u, a.lists_per_split);  // lists
  uint32_t k, sel;
  size_t out_off;
  if (serving) {
    const ServeQuery s = a.sq[q];
    k = s.k;
    sel = s.kp;
    out_off = s.out_off;
  } else {
    k = a.k;
    sel = a.kp;
    out_off = size_t(q) * a.k;
  }
  const float mg = a.margin ? a.margin[q] : -1.f;
  const uint32_t target = mg >= 0.f ? k : sel;
  const FinishSmem L = finish_smem(a.dp, a.stage_cap);
  float* qs = reinterpret_cast<float*>(fsm + L.qs);
  float* cand_d = reinterpret_cast<float*>(fsm + L.cd);
  uint32_t* cand_i = reinterpret_cast<uint32_t*>(fsm + L.ci);
  float* cand_x = reinterpret_cast<float*>(fsm + L.cx);
  float* stg_d = reinterpret_cast<float*>(fsm + L.sd);
  uint32_t* stg_i = reinterpret_cast<uint32_t*>(fsm + L.si);
  const size_t base = size_t(q) * nsplit * a.kp;
  const uint32_t* lens = a.part_n + size_t(q) * nsplit;
  if (tid == 0) {
    s_total = 0;
    s_cnt = 0;
    s_kmin = 0xFFFFFFFFu;
    s_kmax = 0u;
    s_all = 0;
    s_heads = 0;
    s_staged = 0;
    s_dk = __int_as_float(0x7f800000);
  }
  const float* qrow = a.q + size_t(q) * a.ldq;
  constexpr int G = kWide ? 6 : 4;  // rows per warp in flight in the rerank (96 a pass of a CTA when wide)
  // The rerank's share of cluster rank crank: warps crank x nwarps + warp of all csize x nwarps,
  // G rows each in flight; rank 0's candidate ids in, FP32 distances out (its shared memory).
  auto rerank_share = [&](uint32_t nc) {
    const float4* q4 = reinterpret_cast<const float4*>(L.cd > 0 ? qs : qrow);
    const uint32_t nch = a.dp / 4, wall = csize * uint32_t(nwarps);
    for (uint32_t j0 = crank * uint32_t(nwarps) + uint32_t(warp); j0 < nc; j0 += G * wall) {
      const float4* x4[G];
#pragma unroll
      for (int g = 0; g < G; ++g) {
        const uint32_t j = j0 + uint32_t(g) * wall;
        uint32_t id = kNone;
        if (j < nc) id = csize > 1 ? ld_cluster_u32(cluster_addr(cand_i + j, 0)) : cand_i[j];
        x4[g] = id < a.n ? reinterpret_cast<const float4*>(a.x + size_t(id) * a.dp) : nullptr;
      }
      float d[G];
      exact_distances<L2, G, kWide ? 3 : 1>(q4, x4, nch, lane, d);
      if (lane == 0) {
#pragma unroll
        for (int g = 0; g < G; ++g) {
          const uint32_t j = j0 + uint32_t(g) * wall;
          if (j >= nc) continue;
          const float v = x4[g] ? d[g] : __int_as_float(0x7f800000);
          if (csize > 1) st_cluster_f32(cluster_addr(cand_x + j, 0), v);
          else cand_x[j] = v;
        }
      }
    }
  };
  if (crank != 0) {  // (CTA-uniform) a cluster member: the query, rank 0's candidates, a share
    if (stale) return;
    if (L.cd > 0)
      for (uint32_t c = tid; c < a.dp; c += kFinishThreads) qs[c] = qrow[c];
    __syncthreads();
    cluster_sync_all();  // rank 0 has collected its candidates
    rerank_share(ld_cluster_u32(cluster_addr(&s_cnt, 0)));
    cluster_sync_all();  // every share is in rank 0's shared memory
    return;
  }
  // The query and (for the flat copy below) the lists' lengths and heads load in the same round
  // trip; the heads' order keys sit in cand_x until the rerank needs it (kKeyAll: empty list).
  const bool flat = nsplit <= kStageSplits;
  const bool by_heads = flat && mg >= 0.f;
  uint32_t* hkey = reinterpret_cast<uint32_t*>(cand_x);
  if (L.cd > 0)
    for (uint32_t c = tid; c < a.dp; c += kFinishThreads) qs[c] = qrow[c];
  if (flat) {
    uint32_t sum = 0, nonempty = 0;
    for (uint32_t sp = tid; sp < nsplit; sp += kFinishThreads) {
      const uint32_t len = min(lens[sp], a.kp);
      // (read whatever the length: slot 0 of every list exists, and an empty list's is ignored)
      const float head = by_heads ? a.part_d[base + size_t(sp) * a.kp] : 0.f;
      s_off[sp + 1] = len;
      sum += len;
      nonempty += len ? 1u : 0u;
      if (by_heads) hkey[sp] = len ? order_key(head) : kKeyAll;
    }
    sum = __reduce_add_sync(kFull, sum);
    nonempty = __reduce_add_sync(kFull, nonempty);
    if (lane == 0 && sum) {
      atomicAdd(&s_all, sum);
      atomicAdd(&s_heads, nonempty);
    }
    if (tid == 0) s_off[0] = 0;
  }
  if (stale) return;
  __syncthreads();
  // ---- 2. the cut (selection; used on the heads first) ----
  // The rank-th smallest key of `each_key`'s keys (1 <= rank <= their count): exact after enough
  // 8-bit rounds, or after `rounds` rounds the largest key of the bucket holding it (an upper
  // bound). CTA-uniform result. each_key calls f(key, valid) for every key.
  auto radix_select = [&](auto&& each_key, uint32_t rank, int rounds) -> uint32_t {
    uint32_t lo = 0xFFFFFFFFu, hi = 0u;
    each_key([&](uint32_t key, bool ok) {
      if (ok) {
        lo = min(lo, key);
        hi = max(hi, key);
      }
    });
    lo = __reduce_min_sync(kFull, lo);
    hi = __reduce_max_sync(kFull, hi);
    if (lane == 0) {
      atomicMin(&s_kmin, lo);
      atomicMax(&s_kmax, hi);
    }
    __syncthreads();
    const uint32_t kmin = s_kmin, kmax = s_kmax;
    __syncthreads();
    if (tid == 0) {
      s_kmin = 0xFFFFFFFFu;  // ready for the next selection
      s_kmax = 0u;
    }
    __syncthreads();
    const uint32_t diff = kmin ^ kmax;
    if (!diff) return kmin;
    int lo_bit = 32 - __clz(diff);  // bits [0, lo_bit) remain to resolve; above them all keys agree
    uint32_t mask = lo_bit == 32 ? 0u : (0xFFFFFFFFu << lo_bit);
    uint32_t prefix = kmin & mask;
    uint32_t remaining = rank;
    for (int round = 0; lo_bit > 0 && round < rounds; ++round) {
      const int nb = min(8, lo_bit);
      const int shift = lo_bit - nb;
      const uint32_t bmask = (1u << nb) - 1u;
      for (int b = tid; b < 256; b += kFinishThreads) hist[b] = 0;
      __syncthreads();
      each_key([&](uint32_t key, bool ok) {
        if (ok && (key & mask) == prefix) atomicAdd(&hist[(key >> shift) & bmask], 1u);
      });
      __syncthreads();
      if (warp == 0) {  // the first bucket whose running count reaches `remaining`
        uint32_t c[8], sum = 0;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          c[i] = hist[lane * 8 + i];
          sum += c[i];
        }
        uint32_t incl = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const uint32_t t = __shfl_up_sync(kFull, incl, o);
          if (lane >= o) incl += t;
        }
        const unsigned reach = __ballot_sync(kFull, incl >= remaining);
        const int src = reach ? __ffs(reach) - 1 : 31;
        if (lane == src) {
          uint32_t rr = remaining - (incl - sum), bi = 7;
          bool found = false;
#pragma unroll
          for (int i = 0; i < 8; ++i)
            if (!found) {
              if (c[i] >= rr || i == 7) {
                bi = uint32_t(i);
                found = true;
              } else {
                rr -= c[i];
              }
            }
          s_prefix = prefix | ((uint32_t(lane) * 8u + bi) << shift);
          s_rank = rr;
        }
      }
      __syncthreads();
      prefix = s_prefix;
      remaining = s_rank;
      mask |= bmask << shift;
      lo_bit = shift;
      __syncthreads();
    }
    return prefix | ~mask;  // every unresolved bit set: the bucket's largest key (exact when none)
  };
  // The heads' bound c (order key): the k-th smallest head, to 16 bits below the heads' highest
  // differing bit (rounded up to its bucket's end), plus the margin, rounded up. Fewer than k
  // non-empty lists: every list is read.
  // Certified path with few entries in all (at most one rerank pass, two with a cluster): every
  // entry is staged and reranked, and no bound is needed (at batch 1 over the e4m3 copy every list
  // entry was under it, and its select took ~1.8 us).
  const uint32_t whole_cap = uint32_t(G * nwarps) * (csize > 1 ? 2u * csize : 1u);
  const bool few = by_heads && s_all <= whole_cap && s_all <= a.stage_cap;  // CTA-uniform
  uint32_t c_key = kKeyAll;
  bool direct = false;  // sorted lists under the heads' bound: read in runs (below)
  if (by_heads && !few && k > 0 && s_heads >= k) {  // CTA-uniform
    const uint32_t h = radix_select(
        [&](auto&& f) {
          for (uint32_t s0 = 0; s0 < nsplit; s0 += kFinishThreads) {
            const uint32_t sp = s0 + uint32_t(tid);
            const uint32_t key = sp < nsplit ? hkey[sp] : kKeyAll;
            f(key, key != kKeyAll);
          }
        },
        k, 2);
    c_key = order_key(__fadd_ru(key_float(h), mg));
    if (key_float(c_key) != key_float(c_key)) c_key = kKeyAll;  // NaN: no bound
    // (wide variant only: the shortlist's sorted lists come with at most kSortedListQueries
    // queries, and the run reader would push the narrow variant past its registers). Only lists
    // holding more entries than one load of every thread (four) covers: the flat copy below reads
    // those in one round trip, the runs take one a run.
    direct = kWide && a.sorted_lists != 0 && c_key != kKeyAll && s_all > 4u * kFinishThreads;
    if (!direct) {  // only the lists whose head is at or below c are read
      for (uint32_t sp = tid; sp < nsplit; sp += kFinishThreads)
        if (hkey[sp] > c_key) s_off[sp + 1] = 0;
      __syncthreads();
    }
  }
  // Appends (d, id) to the staging area when `keep` (warp-uniform call; any order); past
  // stage_cap nothing is written and the count alone grows (the passes then read the lists).
  // The row of a kept entry is also prefetched into L2 for the rerank (most kept entries are
  // reranked; the rows are scattered over HBM, so the rerank's loads otherwise wait on DRAM): not
  // when the main pass did so already, nor when a cluster shares the rerank (its CTAs load their
  // own rows; one SM issuing ~12,000 line prefetches for ~1,000 rows took 15 us).
  auto append = [&](bool keep, float d, uint32_t id) {
    const unsigned bal = __ballot_sync(kFull, keep);
    uint32_t at = 0;
    if (lane == 0 && bal) at = atomicAdd(&s_staged, uint32_t(__popc(bal)));
    at = __shfl_sync(kFull, at, 0) + __popc(bal & ((1u << lane) - 1u));
    if (keep && at < a.stage_cap) {
      stg_d[at] = d;
      stg_i[at] = id;
    }
    for (unsigned m = csize > 1 || a.rows_in_l2 ? 0u : bal; m; m &= m - 1) {  // a row's lines, one a lane
      const uint32_t rid = __shfl_sync(kFull, id, __ffs(m) - 1);
      if (rid < a.n) {
        const char* row = reinterpret_cast<const char*>(a.x + size_t(rid) * a.dp);
        for (uint32_t b = uint32_t(lane) * 128u; b < a.dp * 4u; b += 32u * 128u)
          asm volatile("prefetch.global.L2 [%0];" ::"l"(row + b));
      }
    }
  };
  // ---- 1. stage ----
  // Sorted lists under the heads' bound: the entries at or below c are a prefix of each list
  // whose head is at or below c, so the lists are read in runs of kDirectRun entries from the
  // head, every run of every such list at once (no offsets to scan, one round trip a run); a
  // list whose run ended at or below c with entries left goes on to the next run.
  // Otherwise, up to kStageSplits lists: their lengths are scanned into offsets, then every thread
  // copies entries of any list (found by binary search over the offsets), four at a time, so the
  // copy runs with many independent loads in flight (with the heads' bound, only the entries at
  // or below c). More lists: one list per thread.
  if (direct) {
    constexpr uint32_t kDirectRun = 8;
    uint32_t* cur = reinterpret_cast<uint32_t*>(cand_d);  // this run's lists (cand_d / cand_i
    uint32_t* nxt = cand_i;                               // are free until the collection)
    for (uint32_t w0 = uint32_t(tid) & ~31u; w0 < nsplit; w0 += kFinishThreads) {
      const uint32_t sp = w0 + uint32_t(lane);
      const bool take = sp < nsplit && hkey[sp] <= c_key;  // (an empty list's key is above c)
      const unsigned bal = __ballot_sync(kFull, take);
      uint32_t at = 0;
      if (lane == 0 && bal) at = atomicAdd(&s_total, uint32_t(__popc(bal)));
      at = __shfl_sync(kFull, at, 0) + __popc(bal & ((1u << lane) - 1u));
      if (take) cur[at] = sp;
    }
    __syncthreads();
    uint32_t nl = s_total;
    for (uint32_t j0 = 0; nl > 0; j0 += kDirectRun) {  // CTA-uniform
      if (tid == 0) s_rank = 0;  // the next run's list count
      __syncthreads();
      const uint32_t tot = nl * kDirectRun;
      // kDirectAhead entries a thread, all loaded before any is appended (one round trip)
      constexpr int kDirectAhead = 4;
      for (uint32_t w0 = uint32_t(tid) & ~31u; w0 < tot; w0 += kDirectAhead * kFinishThreads) {
        uint32_t sp[kDirectAhead], j[kDirectAhead], len[kDirectAhead], iv[kDirectAhead];
        float dv[kDirectAhead];
#pragma unroll
        for (int p = 0; p < kDirectAhead; ++p) {
          const uint32_t e = w0 + uint32_t(lane) + uint32_t(p) * kFinishThreads;
          sp[p] = 0;
          j[p] = 0;
          len[p] = 0;
          iv[p] = 0;
          dv[p] = 0.f;
          if (e < tot) {
            sp[p] = cur[e / kDirectRun];
            j[p] = j0 + e % kDirectRun;
            len[p] = s_off[sp[p] + 1];
            if (j[p] < len[p]) {
              const size_t at = base + size_t(sp[p]) * a.kp + j[p];
              dv[p] = a.part_d[at];
              iv[p] = a.part_i[at];
            }
          }
        }
#pragma unroll
        for (int p = 0; p < kDirectAhead; ++p) {
          const uint32_t e = w0 + uint32_t(lane) + uint32_t(p) * kFinishThreads;
          const bool keep = j[p] < len[p] && order_key(dv[p]) <= c_key;
          append(keep, dv[p], iv[p]);
          const bool more = keep && e % kDirectRun == kDirectRun - 1 && j[p] + 1 < len[p];
          const unsigned bal = __ballot_sync(kFull, more);
          uint32_t at = 0;
          if (lane == 0 && bal) at = atomicAdd(&s_rank, uint32_t(__popc(bal)));
          at = __shfl_sync(kFull, at, 0) + __popc(bal & ((1u << lane) - 1u));
          if (more) nxt[at] = sp[p];
        }
      }
      __syncthreads();
      nl = s_rank;
      uint32_t* t = cur;
      cur = nxt;
      nxt = t;
    }
  } else if (flat) {
    if (warp == 0) {  // inclusive scan of s_off[1 .. nsplit]: lane l sums a run of consecutive lists
      const uint32_t per = (nsplit + 31) / 32;
      const uint32_t b0 = min(nsplit, uint32_t(lane) * per), b1 = min(nsplit, b0 + per);
      uint32_t sum = 0;
      for (uint32_t i = b0; i < b1; ++i) sum += s_off[i + 1];
      uint32_t incl = sum;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += t;
      }
      uint32_t run = incl - sum;
      for (uint32_t i = b0; i < b1; ++i) {
        run += s_off[i + 1];
        s_off[i + 1] = run;
      }
      if (lane == 31) s_total = incl;
    }
    __syncthreads();
    const uint32_t tot = s_total;
    if (tot <= a.stage_cap) {
      // (warp-uniform loop: the heads' filter appends with one ballot per step)
      for (uint32_t w0 = uint32_t(tid) & ~31u; w0 < tot; w0 += 4 * kFinishThreads) {
        float dv[4];
        uint32_t iv[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          const uint32_t e = w0 + uint32_t(lane) + uint32_t(t) * kFinishThreads;
          dv[t] = 0.f;
          iv[t] = 0u;
          if (e < tot) {  // the list holding entry e: the largest sp with s_off[sp] <= e
            uint32_t lo = 0, hi = nsplit;
            while (hi - lo > 1) {
              const uint32_t mid = (lo + hi) >> 1;
              if (s_off[mid] <= e) lo = mid;
              else hi = mid;
            }
            const size_t at = base + size_t(lo) * a.kp + (e - s_off[lo]);
            dv[t] = a.part_d[at];
            iv[t] = a.part_i[at];
          }
        }
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          const uint32_t e = w0 + uint32_t(lane) + uint32_t(t) * kFinishThreads;
          if (c_key != kKeyAll) {  // CTA-uniform
            append(e < tot && order_key(dv[t]) <= c_key, dv[t], iv[t]);
          } else if (e < tot) {
            stg_d[e] = dv[t];
            stg_i[e] = iv[t];
          }
        }
      }
    }
  } else {
    for (uint32_t sp = tid; sp < nsplit; sp += kFinishThreads) {
      const uint32_t len = min(lens[sp], a.kp);
      if (!len) continue;
      const uint32_t pos = atomicAdd(&s_total, len);
      if (pos + len > a.stage_cap) continue;  // too many to stage: the passes read the lists
      const float* ld = a.part_d + base + size_t(sp) * a.kp;
      const uint32_t* li = a.part_i + base + size_t(sp) * a.kp;
      for (uint32_t j = 0; j < len; j += 8) {
        float dv[8];
        uint32_t iv[8];
#pragma unroll
        for (int t = 0; t < 8; ++t) {
          dv[t] = j + t < len ? ld[j + t] : 0.f;
          iv[t] = j + t < len ? li[j + t] : 0u;
        }
#pragma unroll
        for (int t = 0; t < 8; ++t)
          if (j + t < len) {
            stg_d[pos + j + t] = dv[t];
            stg_i[pos + j + t] = iv[t];
          }
      }
    }
  }
  __syncthreads();
  // all: every list entry; total: the entries the passes below take (the staged ones, or every
  // list entry when the lists to read did not fit). CTA-uniform.
  const uint32_t all = flat ? s_all : s_total;
  const bool staged = direct ? s_staged <= a.stage_cap : s_total <= a.stage_cap;
  const uint32_t total = !staged ? all : c_key != kKeyAll ? s_staged : s_total;
  // Every entry once, as (order key, approximate distance, id).
  auto each = [&](auto&& f) {
    if (staged) {
      for (uint32_t e = tid; e < total; e += kFinishThreads) f(order_key(stg_d[e]), stg_d[e], stg_i[e]);
    } else {
      for (uint32_t sp = warp; sp < nsplit; sp += nwarps) {
        const uint32_t len = min(lens[sp], a.kp);
        const float* ld = a.part_d + base + size_t(sp) * a.kp;
        const uint32_t* li = a.part_i + base + size_t(sp) * a.kp;
        for (uint32_t j = lane; j < len; j += 32) {
          const float d = ld[j];
          f(order_key(d), d, li[j]);
        }
      }
    }
  };
  // ---- 2. the cut ----
  // Exact rank-th smallest key (1 <= rank <= total): CTA-uniform result.
  auto select_key = [&](uint32_t rank) -> uint32_t {
    if (staged && total <= kSmallSelect) {
      // Few entries: each thread ranks its own entry against all of them in one pass (shared
      // reads every thread makes at once), ties by position, so the ranks are a permutation.
      if (uint32_t(tid) < total) {
        const uint32_t mine = order_key(stg_d[tid]);
        uint32_t below = 0, e = 0;
        auto lt = [&](uint32_t j) -> uint32_t {
          const uint32_t o = order_key(stg_d[j]);
          return uint32_t((o < mine) | ((o == mine) & (j < uint32_t(tid))));
        };
        for (; e + 4 <= total; e += 4) below += lt(e) + lt(e + 1) + lt(e + 2) + lt(e + 3);
        for (; e < total; ++e) below += lt(e);
        if (below + 1 == rank) s_prefix = mine;
      }
      __syncthreads();
      const uint32_t r = s_prefix;
      __syncthreads();
      return r;
    }
    return radix_select(
        [&](auto&& f) {  // every entry's key, warp-uniform calls
          if (staged) {
            for (uint32_t e0 = 0; e0 < total; e0 += kFinishThreads) {
              const uint32_t e = e0 + uint32_t(tid);
              f(e < total ? order_key(stg_d[e]) : 0u, e < total);
            }
          } else {
            for (uint32_t sp = warp; sp < nsplit; sp += nwarps) {
              const uint32_t len = min(lens[sp], a.kp);
              const float* ld = a.part_d + base + size_t(sp) * a.kp;
              for (uint32_t j0 = 0; j0 < len; j0 += 32) {
                const uint32_t j = j0 + uint32_t(lane);
                f(j < len ? order_key(ld[j]) : 0u, j < len);
              }
            }
          }
        },
        rank, 4);
  };
  // keep entries with key <= cut_key (or < when strict); the heads' bound c already left out every
  // entry above it. A staged set no larger than one rerank pass (two with a cluster, whose passes
  // are short) is reranked whole: the exact cut would not save a pass.
  uint32_t cut_key = c_key;
  bool strict = false;
  const bool whole = staged && total <= whole_cap && (c_key != kKeyAll || few);
  if (total > target && !whole) {
    const uint32_t tk = select_key(target);
    cut_key = mg >= 0.f ? order_key(__fadd_ru(key_float(tk), mg)) : tk;
  }
  // Collect the entries the cut keeps (the first kRerankMax of them); more than kRerankMax: keep
  // those strictly below the kRerankMax-th smallest instead (fewer than kRerankMax) and collect
  // again.
  auto collect = [&]() {
    each([&](uint32_t key, float d, uint32_t id) {
      if (strict ? key < cut_key : key <= cut_key) {
        const uint32_t slot = atomicAdd(&s_cnt, 1u);
        if (slot < kRerankMax) {
          cand_d[slot] = d;
          cand_i[slot] = id;
        }
      }
    });
    __syncthreads();
  };
  collect();
  if (s_cnt > kRerankMax) {  // CTA-uniform
    __syncthreads();  // every thread has read the count
    if (tid == 0) s_cnt = 0;
    cut_key = select_key(kRerankMax);
    strict = true;
    collect();
  }
  // the cut's share of the certificate's L: only when it left an entry out
  const uint32_t nc = s_cnt;  // <= kRerankMax
  const bool cut_left_out = nc < all;
  // ---- 3. rerank ----
  if (csize > 1) cluster_sync_all();  // the candidates are ready for the cluster's shares
  rerank_share(nc);
  if (csize > 1) cluster_sync_all();  // every share is in
  __syncthreads();
  // ---- 4. top k by (FP32 dist, id) ----
  // Each candidate's rank among (order key of the distance, id) pairs, counted against all of them
  // (one 8-byte shared load each, the same address across the warp; equal pairs ranked by
  // position, so the ranks are a permutation). The pairs sit in the staging area, free once the
  // candidates are collected (at least kRerankMax x 8 bytes). A NaN distance ranks as +inf (written
  // as a missing result) and -0 as +0: the order is the float order of the distances, then ids.
  // More than kRankAll candidates: an upper bound of the k-th smallest distance key is selected
  // first (one radix round: the end of its bucket), and only the candidates at or below it are
  // ranked, among themselves (every other candidate comes after them); ranking 980 against all
  // took 51 us. (Wide variant: batches up to the SM count.)
  {
    constexpr uint32_t kRankAll = 256, kRankSel = kRerankMax / 2;  // (kRankSel pairs fit cand_d + cand_i)
    unsigned long long* sk = reinterpret_cast<unsigned long long*>(fsm + L.sd);
    for (uint32_t j = tid; j < nc; j += kFinishThreads) {
      float dj = cand_x[j] + 0.f;  // -0 -> +0
      if (dj != dj) dj = __int_as_float(0x7f800000);
      sk[j] = (static_cast<unsigned long long>(order_key(dj)) << 32) | cand_i[j];
    }
    __syncthreads();
    const unsigned long long* rk = sk;
    uint32_t nr = nc;
    // (wide variant only: in the narrow one the selection's registers would spill)
    if (kWide && nc > kRankAll && k < nc) {  // CTA-uniform
      // (one 8-bit round: the end of the bucket holding the k-th key, a few keys above it)
      const uint32_t kd = radix_select(
          [&](auto&& f) {
            for (uint32_t j0 = 0; j0 < nc; j0 += kFinishThreads) {
              const uint32_t j = j0 + uint32_t(tid);
              f(j < nc ? uint32_t(sk[j] >> 32) : 0u, j < nc);
            }
          },
          k, 1);
      unsigned long long* sel = reinterpret_cast<unsigned long long*>(fsm + L.cd);  // cand_d, cand_i: free
      if (tid == 0) s_staged = 0;
      __syncthreads();
      for (uint32_t j = tid; j < nc; j += kFinishThreads)
        if (uint32_t(sk[j] >> 32) <= kd) {
          const uint32_t at = atomicAdd(&s_staged, 1u);
          if (at < kRankSel) sel[at] = sk[j];
        }
      __syncthreads();
      if (s_staged <= kRankSel) {  // (else every candidate is ranked: more ties than that)
        rk = sel;
        nr = s_staged;
      }
      __syncthreads();
    }
    // gs consecutive lanes share one candidate, each counting every gs-th pair (then a butterfly
    // over the group), so few candidates still keep every warp busy: the count is a chain of
    // dependent compares, slow on one warp per scheduler.
    uint32_t gs = 1;
    while (gs < 32 && gs * 2 * nr <= kFinishThreads) gs *= 2;
    const uint32_t part = uint32_t(tid) & (gs - 1);
    for (uint32_t j0 = 0; j0 < nr; j0 += kFinishThreads / gs) {  // CTA-uniform
      const uint32_t j = j0 + uint32_t(tid) / gs;
      const unsigned long long kj = j < nr ? rk[j] : 0ull;
      uint32_t rank = 0;
      if (j < nr) {
        const uint32_t cnt = (nr - part + gs - 1) / gs;  // pairs part, part + gs, ...
#pragma unroll 4
        for (uint32_t i = 0; i < cnt; ++i) {
          const uint32_t t = part + i * gs;
          const unsigned long long kt = rk[t];
          rank += uint32_t(kt < kj) | (uint32_t(kt == kj) & uint32_t(t < j));
        }
      }
      for (uint32_t o = 1; o < gs; o <<= 1) rank += __shfl_xor_sync(kFull, rank, int(o));
      if (j < nr && part == 0) {
        const float dj = key_float(uint32_t(kj >> 32));
        const uint32_t ij = uint32_t(kj);
        if (rank < k) {
          const bool real = ij < a.n && dj != __int_as_float(0x7f800000);
          a.out_d[out_off + rank] = real ? dj : __int_as_float(0x7f800000);
          a.out_i[out_off + rank] = real ? ij : kNone;
        }
        if (rank + 1 == k) s_dk = dj;
      }
    }
  }
  for (uint32_t j = nc + tid; j < k; j += kFinishThreads) {  // fewer than k candidates: pad
    a.out_d[out_off + j] = __int_as_float(0x7f800000);
    a.out_i[out_off + j] = kNone;
  }
  if (!a.fail_count) return;
  __syncthreads();
  // ---- 5. certificate ----
  __shared__ int s_slot;
  if (tid == 0) {
    const float thr0 = a.thr_init ? a.thr_init[q] : __int_as_float(0x7f800000);
    const uint32_t gk = a.gthr ? a.gthr[q] : kKeyNone;
    const float g = gk != kKeyNone ? key_float(gk) : __int_as_float(0x7f800000);
    const float lc = cut_left_out ? key_float(cut_key) : __int_as_float(0x7f800000);
    const float lb = fminf(fminf(thr0, g), lc);
    const bool ok = isinf(lb) || __fsub_rd(lb, a.err[q]) > s_dk;
    s_slot = -1;
    if (!ok) {
      const uint32_t j = atomicAdd(a.fail_count, 1u);
      a.fail_list[j] = q;
      s_slot = int(j);
      if (a.tally) atomicAdd(a.tally, 1ull);
    }
  }
  __syncthreads();
  // An uncertified query takes fallback slot j: its FP32 row (and its filter) go there for the
  // scan kernel that follows.
  const int j = s_slot;
  if (j < 0) return;
  if (a.fq)
    for (uint32_t c = tid; c < a.dp; c += kFinishThreads) a.fq[size_t(j) * a.dp + c] = L.cd > 0 ? qs[c] : qrow[c];
  if (a.fmask)
    for (uint32_t w = tid; w < a.mask_ld; w += kFinishThreads)
      a.fmask[size_t(j) * a.mask_ld + w] = a.qmask[size_t(q) * a.mask_ld + w];
  if (a.fmask_ptrs && tid == 0) a.fmask_ptrs[j] = serving ? a.sq[q].mask : nullptr;
}

// FP32 sample blocks of prepare_queries_kernel (small batches, PrepSample): each block takes
// kPrepRowsPerBlock sampled rows, a warp two of them with both rows' loads issued before any sum
// (so every block's loads are in flight at once); the queries (nq <= 8, padded dim <= 1,024) sit
// in shared memory. Lane l sums chunks l, l + 32, ... of a row against every query, then a
// butterfly.
constexpr uint32_t kPrepRowsPerBlock = 8;
template <bool L2>
__device__ void prep_sample_block(const PrepSample& smp, uint32_t sb, const float* q, uint32_t ldq, uint32_t nq,
                                  uint32_t dim, uint32_t dp) {
  extern __shared__ float4 qsm[];  // nq x dp / 4 (dynamic: only launches with sample blocks have it)
  constexpr int kMaxC = int(kPrepSampleDim / 4 / 32);  // chunk steps a lane takes at most (8)
  const uint32_t n4 = dp / 4, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (uint32_t i = threadIdx.x; i < nq * n4; i += blockDim.x) {
    const uint32_t b = i / n4, c = i % n4;
    const float* src = q + size_t(b) * ldq + 4 * c;
    qsm[i] = make_float4(4 * c < dim ? src[0] : 0.f, 4 * c + 1 < dim ? src[1] : 0.f, 4 * c + 2 < dim ? src[2] : 0.f,
                         4 * c + 3 < dim ? src[3] : 0.f);
  }
  __syncthreads();
  const uint32_t total = smp.ranges * uint32_t(kTcRows);
  const uint32_t rr0 = sb * kPrepRowsPerBlock + warp * 2;
  __shared__ float wmin[kPrepRowsPerBlock / 2][kPrepSampleQueries];  // per warp and query
  if (lane < kPrepSampleQueries) wmin[warp][lane] = __int_as_float(0x7f800000);
  __syncwarp();
  if (rr0 < total) {  // warp-uniform
  float4 xv[2][kMaxC];
  bool valid[2];
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const uint32_t rr = rr0 + uint32_t(h);
    const uint32_t row = (rr / kTcRows) * smp.rps + rr % kTcRows;
    valid[h] = rr < total && row < smp.n;
    const float4* x4 = reinterpret_cast<const float4*>(smp.x + size_t(valid[h] ? row : 0) * dp);
#pragma unroll
    for (int u = 0; u < kMaxC; ++u) {
      const uint32_t c = lane + 32u * uint32_t(u);
      xv[h][u] = c < n4 ? __ldg(x4 + c) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
  }
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const uint32_t rr = rr0 + uint32_t(h);
    if (rr >= total) break;  // warp-uniform
    float acc[kPrepSampleQueries];
#pragma unroll
    for (int b = 0; b < int(kPrepSampleQueries); ++b) acc[b] = 0.f;
#pragma unroll
    for (int u = 0; u < kMaxC; ++u) {
      const uint32_t c = lane + 32u * uint32_t(u);
      if (c >= n4) break;
#pragma unroll
      for (int b = 0; b < int(kPrepSampleQueries); ++b) {
        if (uint32_t(b) >= nq) break;
        const float4 qv = qsm[b * n4 + c];
        const float4 x = xv[h][u];
        if constexpr (L2) {
          float e = qv.x - x.x;
          acc[b] = fmaf(e, e, acc[b]);
          e = qv.y - x.y;
          acc[b] = fmaf(e, e, acc[b]);
          e = qv.z - x.z;
          acc[b] = fmaf(e, e, acc[b]);
          e = qv.w - x.w;
          acc[b] = fmaf(e, e, acc[b]);
        } else {
          acc[b] = fmaf(qv.x, x.x, acc[b]);
          acc[b] = fmaf(qv.y, x.y, acc[b]);
          acc[b] = fmaf(qv.z, x.z, acc[b]);
          acc[b] = fmaf(qv.w, x.w, acc[b]);
        }
      }
    }
#pragma unroll
    for (int b = 0; b < int(kPrepSampleQueries); ++b) {
      if (uint32_t(b) >= nq) break;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc[b] += __shfl_xor_sync(kFull, acc[b], o);
      if (lane == 0 && valid[h]) wmin[warp][b] = fminf(wmin[warp][b], L2 ? acc[b] : 1.f - acc[b]);
    }
  }
  }
  __syncthreads();
  if (threadIdx.x < nq) {
    float m = wmin[0][threadIdx.x];
#pragma unroll
    for (int w = 1; w < int(kPrepRowsPerBlock / 2); ++w) m = fminf(m, wmin[w][threadIdx.x]);
    const uint32_t blocks = (total + kPrepRowsPerBlock - 1) / kPrepRowsPerBlock;
    smp.bmin[size_t(threadIdx.x) * blocks + sb] = m;
  }
}

// The end of every block of a query preparation with an FP32 sample: a ticket, and the last block
// to take one selects each query's threshold from the sample blocks' minima (PrepSample). Up to
// four queries at a time, with the whole block on each (4 minima a thread per query, in
// registers): a min / max pass over the keys, then two 8-bit histogram rounds below their highest
// differing bit (warp q scans query q's histogram); the bucket's largest key bounds the k-th
// smallest from above. Only thread 0 takes the ticket, with an acquire-release atomic after the
// block's barrier (the barrier orders the block's writes before it). Equal bins within a warp are
// added once (a match over the warp): most minima fall into two or three bins, where one shared
// atomic per value serialized for 1.3 us a round.
constexpr int kSelPer = int(kPrepSampleRows / kPrepRowsPerBlock / 128);  // minima a thread holds per query (4)
__device__ void prep_sample_select(const PrepSample& smp, uint32_t nq, uint32_t blocks, const float* margin) {
  __shared__ uint32_t hist[4][256];
  __shared__ uint32_t s_lo[4], s_hi[4], s_prefix[4], s_mask[4], s_rank[4], s_active[4];
  __shared__ int s_shift[4];
  __shared__ uint32_t s_last;
  const uint32_t tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  __syncthreads();  // this block's minima and margins are written
  if (tid == 0) {
    s_last = atomic_add_acq_rel(smp.ticket, 1u) == gridDim.x - 1 ? 1u : 0u;
    if (s_last) *smp.ticket = 0;  // every block has taken its ticket: ready for the next launch
  }
  __syncthreads();
  if (!s_last) return;
  const bool fits = smp.k >= 1 && smp.k <= blocks && blocks <= 128u * kSelPer;  // CTA-uniform
  for (uint32_t q0 = 0; q0 < nq; q0 += 4) {  // CTA-uniform
    const uint32_t nqs = min(nq - q0, 4u);
    uint32_t key[4][kSelPer];  // kKeyNone past the end: never counted
#pragma unroll
    for (int qi = 0; qi < 4; ++qi)
#pragma unroll
      for (int i = 0; i < kSelPer; ++i) {
        const uint32_t j = tid + 128u * uint32_t(i);
        key[qi][i] = (fits && uint32_t(qi) < nqs && j < blocks)
                         ? order_key(__ldcg(smp.bmin + size_t(q0 + uint32_t(qi)) * blocks + j))
                         : kKeyNone;
      }
    if (tid < 4) {
      s_lo[tid] = 0xFFFFFFFFu;
      s_hi[tid] = 0u;
    }
    __syncthreads();
#pragma unroll
    for (int qi = 0; qi < 4; ++qi) {
      uint32_t lo = 0xFFFFFFFFu, hi = 0u;
#pragma unroll
      for (int i = 0; i < kSelPer; ++i)
        if (key[qi][i] != kKeyNone) {
          lo = min(lo, key[qi][i]);
          hi = max(hi, key[qi][i]);
        }
      lo = __reduce_min_sync(kFull, lo);
      hi = __reduce_max_sync(kFull, hi);
      if (lane == 0 && uint32_t(qi) < nqs) {
        atomicMin(&s_lo[qi], lo);
        atomicMax(&s_hi[qi], hi);
      }
    }
    __syncthreads();
    if (tid < nqs) {  // each query's starting prefix: the bits above the highest differing one
      const uint32_t diff = s_lo[tid] ^ s_hi[tid];
      const int top = diff ? 31 - __clz(diff) : 0;
      s_active[tid] = (fits && diff) ? 1u : 0u;
      s_shift[tid] = max(top - 7, 0);
      s_mask[tid] = top == 31 ? 0u : (0xFFFFFFFFu << (top + 1));
      s_prefix[tid] = s_lo[tid] & s_mask[tid];
      s_rank[tid] = smp.k;
    }
    __syncthreads();
    for (int round = 0; round < 2; ++round) {
      for (uint32_t b = tid; b < 4u * 256u; b += blockDim.x) (&hist[0][0])[b] = 0;
      __syncthreads();
#pragma unroll
      for (int qi = 0; qi < 4; ++qi) {
        if (uint32_t(qi) >= nqs || !s_active[qi]) continue;  // CTA-uniform
        const uint32_t mask = s_mask[qi], prefix = s_prefix[qi];
        const int shift = s_shift[qi];
#pragma unroll
        for (int i = 0; i < kSelPer; ++i) {
          const bool in = key[qi][i] != kKeyNone && (key[qi][i] & mask) == prefix;
          const uint32_t bin = in ? (key[qi][i] >> shift) & 255u : 256u;  // 256: not counted
          const unsigned same = __match_any_sync(kFull, bin);
          if (in && lane == uint32_t(__ffs(same) - 1)) atomicAdd(&hist[qi][bin], uint32_t(__popc(same)));
        }
      }
      __syncthreads();
      if (w < nqs && s_active[w]) {  // warp q: the first bucket of query q whose running count reaches its rank
        const uint32_t rank = s_rank[w];
        uint32_t c[8], sum = 0;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          c[i] = hist[w][lane * 8 + i];
          sum += c[i];
        }
        uint32_t incl = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const uint32_t u = __shfl_up_sync(kFull, incl, o);
          if (lane >= uint32_t(o)) incl += u;
        }
        const unsigned reach = __ballot_sync(kFull, incl >= rank);
        const int src = reach ? __ffs(reach) - 1 : 31;
        if (int(lane) == src) {
          uint32_t rr = rank - (incl - sum), bi = 7;
          bool found = false;
#pragma unroll
          for (int i = 0; i < 8; ++i)
            if (!found) {
              if (c[i] >= rr || i == 7) {
                bi = uint32_t(i);
                found = true;
              } else {
                rr -= c[i];
              }
            }
          const int shift = s_shift[w];
          s_prefix[w] |= (lane * 8u + bi) << shift;
          s_mask[w] |= 0xFFu << shift;
          s_rank[w] = rr;
          if (shift == 0) s_active[w] = 0;  // every bit resolved
          s_shift[w] = max(shift - 8, 0);
        }
      }
      __syncthreads();
    }
    if (tid < nqs) {
      const uint32_t diff = s_lo[tid] ^ s_hi[tid];
      // the bucket's largest key (every unresolved bit set); equal keys: the key itself
      const float t = !fits ? __int_as_float(0x7f800000) : key_float(diff ? (s_prefix[tid] | ~s_mask[tid]) : s_lo[tid]);
      smp.thr[q0 + tid] =
          t != t ? __int_as_float(0x7f800000) : margin ? __fadd_ru(t, __ldcg(margin + q0 + tid)) : t;
    }
    __syncthreads();  // the shared state is reused by the next four queries
  }
}

// The queries of the bf16 shortlist path, one warp per query: the bf16 copy (stride dp, padding
// columns zero) and the squared norm, as to_bf16_kernel writes them; the query's shared threshold
// reset to none (gthr); and, with margins, err[q] = E and margin[q] = factor x E (both rounded
// up). A shortlist that keeps every row within the margin m of its k-th best approximate distance
// a_k leaves out only rows at or above a_k + m, so it certifies whenever the k-th FP32 distance is
// below a_k + m - E. That always holds for m > 2 E (the k-th FP32 distance is at most a_k + E); the
// bf16 roundings of real data stay far below their worst case E, so m = 1.3 E already certifies
// nearly every query while keeping about half the rows of 2 E. The first thread also zeroes the
// uncertified-query count.
template <bool L2>
__device__ __forceinline__ void prepare_query_warp(const float* q, uint32_t ldq, uint32_t nq, uint32_t dim,
                                                   uint32_t dp, __nv_bfloat16* qb, float* qnorm, uint32_t* gthr,
                                                   const float* xbound, float factor, float* margin, float* err,
                                                   uint32_t* fails) {
  if (fails && blockIdx.x == 0 && threadIdx.x == 0) *fails = 0;
  const uint32_t qq = blockIdx.x * 4 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (qq >= nq) return;
  const float* s = q + size_t(qq) * ldq;
  __nv_bfloat16* d = qb + size_t(qq) * dp;
  float q2 = 0.f, qb2 = 0.f, r2 = 0.f;
  auto one = [&](float v, uint32_t c) {
    v = c < dim ? v : 0.f;
    const __nv_bfloat16 b = __float2bfloat16_rn(v);
    const float vb = __bfloat162float(b);
    q2 = fmaf(v, v, q2);
    qb2 = fmaf(vb, vb, qb2);
    r2 = fmaf(vb - v, vb - v, r2);
    return b;
  };
  if ((ldq & 3u) == 0 && (reinterpret_cast<uintptr_t>(q) & 15u) == 0 && (dp & 3u) == 0) {
    // 16-byte loads, four chunk steps issued before any is used (a 384-dim query in one round trip)
    const float4* s4 = reinterpret_cast<const float4*>(s);
    const uint32_t n4 = dp / 4;
    for (uint32_t c0 = lane; c0 < n4; c0 += 32u * 4u) {
      float4 v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const uint32_t c = c0 + 32u * u;
        v[u] = c < n4 ? s4[c] : make_float4(0.f, 0.f, 0.f, 0.f);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const uint32_t c = c0 + 32u * u;
        if (c >= n4) break;
        const __nv_bfloat162 lo = __halves2bfloat162(one(v[u].x, 4 * c), one(v[u].y, 4 * c + 1));
        const __nv_bfloat162 hi = __halves2bfloat162(one(v[u].z, 4 * c + 2), one(v[u].w, 4 * c + 3));
        __nv_bfloat162* d2 = reinterpret_cast<__nv_bfloat162*>(d + 4 * c);
        d2[0] = lo;
        d2[1] = hi;
      }
    }
  } else {
    for (uint32_t c = lane; c < dp; c += 32) d[c] = one(c < dim ? s[c] : 0.f, c);
  }
  for (int o = 16; o > 0; o >>= 1) {
    q2 += __shfl_xor_sync(kFull, q2, o);
    qb2 += __shfl_xor_sync(kFull, qb2, o);
    r2 += __shfl_xor_sync(kFull, r2, o);
  }
  if (lane == 0) {
    if (qnorm) qnorm[qq] = q2;
    if (gthr) gthr[qq] = kKeyNone;
    if (margin) {
      const float e = cert_error<L2>(q2, qb2, r2, dp, xbound);
      err[qq] = e;
      margin[qq] = __fmul_ru(factor, e);
    }
  }
}

// The e4m3 form of prepare_query_warp (the certified path over the e4m3 copy): per query its
// scale max |q| / 448 (as to_fp8_kernel takes it), its e4m3 row (stride dpo bytes, padding
// zero), the squared FP32 norm, and with margins E from the sums |q~|^2 and |q~ - q|^2 (q~ = e4m3
// value x scale) and the e4m3 rows' bounds.
template <bool L2>
__device__ __forceinline__ void prepare_query_warp_f8(const float* q, uint32_t ldq, uint32_t nq, uint32_t dim,
                                                      uint32_t dp, uint32_t dpo, uint8_t* q8, float* qscale,
                                                      float* qnorm, uint32_t* gthr, const float* xbound,
                                                      float factor, float* margin, float* err, uint32_t* fails) {
  if (fails && blockIdx.x == 0 && threadIdx.x == 0) *fails = 0;
  const uint32_t qq = blockIdx.x * 4 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (qq >= nq) return;
  const float* s = q + size_t(qq) * ldq;
  // The row in registers, four columns a lane per step (columns 4 (32 u + lane) ..; dims up to
  // 32 x 4 x kF8Steps), loaded in one round trip; the scale needs its maximum before any byte.
  constexpr int kF8Steps = int(kPrepSampleDim / 128);
  float4 v[kF8Steps];
  float mx = 0.f, q2 = 0.f;
#pragma unroll
  for (int u = 0; u < kF8Steps; ++u) {
    const uint32_t c = 4u * (32u * uint32_t(u) + lane);
    v[u] = make_float4(c < dim ? s[c] : 0.f, c + 1 < dim ? s[c + 1] : 0.f, c + 2 < dim ? s[c + 2] : 0.f,
                       c + 3 < dim ? s[c + 3] : 0.f);
  }
#pragma unroll
  for (int u = 0; u < kF8Steps; ++u) {
    mx = fmaxf(fmaxf(mx, fmaxf(fabsf(v[u].x), fabsf(v[u].y))), fmaxf(fabsf(v[u].z), fabsf(v[u].w)));
    q2 = fmaf(v[u].x, v[u].x, fmaf(v[u].y, v[u].y, fmaf(v[u].z, v[u].z, fmaf(v[u].w, v[u].w, q2))));
  }
  for (int o = 16; o > 0; o >>= 1) {
    mx = fmaxf(mx, __shfl_xor_sync(kFull, mx, o));
    q2 += __shfl_xor_sync(kFull, q2, o);
  }
  const float sc = mx > 0.f ? mx / 448.f : 1.f;
  const float inv = 1.f / sc;
  // |q~ - q|^2 and |q~|^2 in FP32: e = fma(b, sc, -q) rounds the exact difference once (relative
  // u), and the sums carry cert_error's (1 + 2 d u) inflation, far above those per-term roundings
  // (FP64 here took the preparation from ~1.5 to 5 us).
  float res = 0.f, accb = 0.f;
  auto one = [&](float x, uint32_t c) -> uint32_t {
    const uint8_t b = c < dim ? uint8_t(__nv_cvt_float_to_fp8(x * inv, __NV_SATFINITE, __NV_E4M3)) : uint8_t(0);
    const float bv = e4m3_value(b);
    const float e = fmaf(bv, sc, -x);
    const float xt = __fmul_ru(fabsf(bv), sc);  // |q~_i| rounded up
    res = fmaf(e, e, res);
    accb = fmaf(xt, xt, accb);
    return b;
  };
#pragma unroll
  for (int u = 0; u < kF8Steps; ++u) {
    const uint32_t c = 4u * (32u * uint32_t(u) + lane);
    if (c >= dpo) break;
    const uint32_t w = one(v[u].x, c) | (one(v[u].y, c + 1) << 8) | (one(v[u].z, c + 2) << 16) | (one(v[u].w, c + 3) << 24);
    *reinterpret_cast<uint32_t*>(q8 + size_t(qq) * dpo + c) = w;  // dpo is a multiple of 16
  }
  for (int o = 16; o > 0; o >>= 1) {
    res += __shfl_xor_sync(kFull, res, o);
    accb += __shfl_xor_sync(kFull, accb, o);
  }
  if (lane == 0) {
    qscale[qq] = sc;
    if (qnorm) qnorm[qq] = q2;
    if (gthr) gthr[qq] = kKeyNone;
    if (margin) {
      // (the difference's single rounding: one more u on each term of |q~ - q|^2)
      const float e = cert_error<L2, true>(q2, accb, __fmul_ru(res, 1.f + 4.f * 5.9604644775390625e-08f), dp, xbound);
      err[qq] = e;
      margin[qq] = __fmul_ru(factor, e);
    }
  }
}

// The query preparation: one warp per query in the first ceil(nq / 4) blocks, the FP32 sample
// (PrepSample, when set) in the blocks after them.
template <bool L2, bool F8>
__global__ void __launch_bounds__(128) prepare_queries_kernel(const float* q, uint32_t ldq, uint32_t nq,
                                                              uint32_t dim, uint32_t dp, void* qout, uint32_t dpo,
                                                              float* qscale, float* qnorm, uint32_t* gthr,
                                                              const float* xbound, float factor, float* margin,
                                                              float* err, uint32_t* fails, PrepSample smp) {
  // The head of a chain of dependent launches: the next kernel may start launching at once, except
  // with an FP32 sample, where it launches when this grid ends. Its CTAs, waiting on this grid on
  // every SM, slowed the sample's threshold select (2.4 to 3.1 us) and the whole batch-1 chain
  // ended 2.4 us later.
  if (!smp.thr) pdl_trigger();
  pdl_wait();
  const uint32_t qblocks = (nq + 3) / 4;
  if (blockIdx.x >= qblocks) {  // FP32 sample blocks (block-uniform)
    prep_sample_block<L2>(smp, blockIdx.x - qblocks, q, ldq, nq, dim, dp);
  } else if constexpr (F8) {
    prepare_query_warp_f8<L2>(q, ldq, nq, dim, dp, dpo, static_cast<uint8_t*>(qout), qscale, qnorm, gthr, xbound,
                              factor, margin, err, fails);
  } else {
    prepare_query_warp<L2>(q, ldq, nq, dim, dp, static_cast<__nv_bfloat16*>(qout), qnorm, gthr, xbound, factor,
                           margin, err, fails);
  }
  if (smp.thr) prep_sample_select(smp, nq, gridDim.x - qblocks, margin);
}

// One CTA per query: an upper bound of the kp-th smallest of `count` values, by radix selection
// on the order key. A first pass finds the keys' minimum and maximum; two 8-bit rounds then
// resolve the 16 bits below their highest differing bit (the bits above are shared), so the
// histograms spread instead of piling into one bin. The result is the largest key of the bucket
// holding the kp-th smallest: at least kp values lie at or below it, within 2^-16 of the range.
__global__ void __launch_bounds__(256) sample_select_kernel(const float* in, uint32_t count, uint32_t nq,
                                                             const uint32_t* kp_per_query, uint32_t kp_all,
                                                             float* thr, const ServeHeader* hdr,
                                                             const ServeQuery* sq, const float* margin) {
  __shared__ uint32_t hist[256];
  __shared__ uint32_t kmin, kmax, sel_prefix, sel_rank;
  pdl_trigger();
  pdl_wait();
  const uint32_t q = blockIdx.x;
  if (hdr) {  // serving mode: the batch shape comes from the header
    nq = hdr->nq;
    count = hdr->nsplit * hdr->sample_tiles * uint32_t(kTcRows);
  }
  if (q >= nq) return;
  const float* v = in + size_t(q) * count;
  // (with margins: the k-th best sampled distance plus the query's margin)
  const uint32_t kp = sq ? (margin ? sq[q].k : sq[q].kp) : kp_per_query ? kp_per_query[q] : kp_all;
  if (kp > count) {  // fewer than kp values: no bound (+inf keeps everything)
    if (threadIdx.x == 0) thr[q] = __int_as_float(0x7f800000);
    return;
  }
  if (threadIdx.x == 0) {
    kmin = 0xFFFFFFFFu;
    kmax = 0u;
    sel_rank = kp;  // 1-based rank still to find inside the current prefix
  }
  __syncthreads();
  // Every value once per pass: float4 loads (count is a multiple of 4 and rows start 16-byte
  // aligned: count = splits x tiles x 256), four independent keys per load.
  // Up to 4,096 values (the small samples) are loaded once and kept in registers for the three
  // passes; more are read again each pass.
  const float4* v4 = reinterpret_cast<const float4*>(v);
  const uint32_t n4 = count / 4;
  constexpr uint32_t kCached = 4;  // float4 values a thread keeps
  const bool cached = n4 <= kCached * blockDim.x;
  float4 held[kCached];
#pragma unroll
  for (uint32_t i = 0; i < kCached; ++i) {
    const uint32_t j = threadIdx.x + i * blockDim.x;
    held[i] = cached && j < n4 ? v4[j] : make_float4(0.f, 0.f, 0.f, 0.f);
  }
  // f(key, valid) for every value.
  auto each_key = [&](auto&& f) {
    auto four = [&](const float4& x, bool ok) {
      f(order_key(x.x), ok);
      f(order_key(x.y), ok);
      f(order_key(x.z), ok);
      f(order_key(x.w), ok);
    };
    if (cached) {
#pragma unroll
      for (uint32_t i = 0; i < kCached; ++i)
        if (i * blockDim.x < n4) four(held[i], threadIdx.x + i * blockDim.x < n4);
    } else {
      const uint32_t rounds = (n4 + blockDim.x - 1) / blockDim.x;
#pragma unroll 4
      for (uint32_t r = 0; r < rounds; ++r) {
        const uint32_t j = threadIdx.x + r * blockDim.x;
        four(j < n4 ? v4[j] : make_float4(0.f, 0.f, 0.f, 0.f), j < n4);
      }
    }
  };
  uint32_t lo = 0xFFFFFFFFu, hi = 0u;
  each_key([&](uint32_t key, bool ok) {
    if (ok) {
      lo = min(lo, key);
      hi = max(hi, key);
    }
  });
  lo = __reduce_min_sync(kFull, lo);
  hi = __reduce_max_sync(kFull, hi);
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&kmin, lo);
    atomicMax(&kmax, hi);
  }
  __syncthreads();
  const uint32_t diff = kmin ^ kmax;
  const int top = diff ? 31 - __clz(diff) : 0;  // highest differing bit
  int shift = max(top - 7, 0);
  // Bits above `top` are the same in every key: they are resolved from the start.
  uint32_t hi_mask = top == 31 ? 0u : (0xFFFFFFFFu << (top + 1));
  uint32_t prefix = kmin & hi_mask;
  if (diff) {
    for (int round = 0; round < 2; ++round) {
      for (int b = threadIdx.x; b < 256; b += blockDim.x) hist[b] = 0;
      __syncthreads();
      each_key([&](uint32_t key, bool ok) {
        if (ok && (key & hi_mask) == prefix) atomicAdd(&hist[(key >> shift) & 255u], 1u);
      });
      __syncthreads();
      if (threadIdx.x < 32) {
        // The first bucket whose running count reaches the rank (bucket 255 if none does): lane
        // l holds buckets 8l .. 8l + 7; a warp scan of their sums finds the lane, the lane its bucket.
        const uint32_t l = threadIdx.x;
        uint32_t c[8], sum = 0;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          c[i] = hist[l * 8 + i];
          sum += c[i];
        }
        uint32_t incl = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const uint32_t t = __shfl_up_sync(kFull, incl, o);
          if (l >= uint32_t(o)) incl += t;
        }
        const uint32_t r = sel_rank;
        const unsigned reach = __ballot_sync(kFull, incl >= r);
        const uint32_t src = reach ? uint32_t(__ffs(reach) - 1) : 31u;
        if (l == src) {
          uint32_t rr = r - (incl - sum), bi = 7;
          bool found = false;
#pragma unroll
          for (int i = 0; i < 8; ++i)
            if (!found) {
              if (c[i] >= rr || i == 7) {
                bi = uint32_t(i);
                found = true;
              } else {
                rr -= c[i];
              }
            }
          sel_prefix = prefix | ((l * 8 + bi) << shift);
          sel_rank = rr;
        }
      }
      __syncthreads();
      prefix = sel_prefix;
      hi_mask |= 0xFFu << shift;  // bits resolved so far
      if (shift == 0) break;
      shift = max(shift - 8, 0);
    }
  }
  if (threadIdx.x == 0) {
    // Upper end of the bucket: every key with this prefix is at most prefix | ~mask. A bucket
    // reaching past +inf (padding entries) gives no bound.
    const float t = key_float(diff ? (prefix | ~hi_mask) : kmin);
    thr[q] = t != t ? __int_as_float(0x7f800000) : margin ? __fadd_ru(t, margin[q]) : t;
  }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static std::once_flag once;
  static EncodeTiledFn fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}

}  // namespace

uint32_t tc_chunks(uint32_t dp, bool fp8) { return (dp + (fp8 ? 127u : 63u)) / (fp8 ? 128u : 64u); }

size_t tc_smem_bytes(uint32_t stages, uint32_t nkc, uint32_t resident) {
  return tc_layout(stages, nkc, resident != 0).total + 1024;
}

uint32_t tc_pick_stages(uint32_t nkc, size_t budget, uint32_t* resident, bool l2, bool fp8) {
  // The kernel's static shared memory comes on top: the work slot, and 1 KB of row norms (L2)
  // and of row scales (e4m3 copies) per epilogue warp.
  // The deepest ring that fits is taken, so a CTA always uses more than half of an SM's shared
  // memory: one CTA per SM, which owns all 512 TMEM columns (a second CTA would wait for them).
  const size_t kStatic = 576 + (l2 ? 8 * kTcRows * 4 : 0) + (fp8 ? 8 * kTcRows * 4 : 0);
  const size_t half = budget / 2 + 1;
  budget = budget > kStatic ? budget - kStatic : 0;
  for (uint32_t s = kMaxTcStages; s >= 3; --s)
    if (tc_smem_bytes(s, nkc, 1) <= budget) {
      *resident = 1;
      return tc_smem_bytes(s, nkc, 1) + kStatic >= half ? s : 0;
    }
  *resident = 0;
  for (uint32_t s = 6; s >= 2; --s)
    if (tc_smem_bytes(s, nkc, 0) <= budget) return tc_smem_bytes(s, nkc, 0) + kStatic >= half ? s : 0;
  return 0;
}

uint32_t tc_buffer_capacity(uint32_t kp) { return tc_capacity(kp); }

uint32_t tc_groups(uint32_t kp) { return uint32_t(tc_groups_cap(tc_capacity(kp))); }

cudaError_t tc_encode_map(CUtensorMap* map, const void* base, uint64_t rows, uint64_t dp, uint32_t box_rows,
                          bool fp8) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return cudaErrorNotSupported;
  if (box_rows == 0 || box_rows > 256u || !base || rows == 0) return cudaErrorInvalidValue;
  const cuuint64_t dims[2] = {dp, rows};
  const cuuint64_t strides[1] = {dp * (fp8 ? 1 : 2)};  // a multiple of 16 bytes
  const cuuint32_t box[2] = {fp8 ? 128u : uint32_t(kTcKChunk), box_rows};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = fn(map, fp8 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2,
                        const_cast<void*>(base), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

// Every instantiation of the shortlist kernel: [fp8][l2][E = 2, 4, 8, 16].
using TcKernel = void (*)(const CUtensorMap, const CUtensorMap, const TcArgs);
const TcKernel kTcKernels[2][2][4] = {
    {{tc_shortlist_kernel<2, false, false>, tc_shortlist_kernel<4, false, false>, tc_shortlist_kernel<8, false, false>,
      tc_shortlist_kernel<16, false, false>},
     {tc_shortlist_kernel<2, true, false>, tc_shortlist_kernel<4, true, false>, tc_shortlist_kernel<8, true, false>,
      tc_shortlist_kernel<16, true, false>}},
    {{tc_shortlist_kernel<2, false, true>, tc_shortlist_kernel<4, false, true>, tc_shortlist_kernel<8, false, true>,
      tc_shortlist_kernel<16, false, true>},
     {tc_shortlist_kernel<2, true, true>, tc_shortlist_kernel<4, true, true>, tc_shortlist_kernel<8, true, true>,
      tc_shortlist_kernel<16, true, true>}}};

cudaError_t tc_prepare(uint32_t stages, uint32_t nkc, uint32_t resident, bool l2, bool fp8) {
  if (stages < 2 || stages > uint32_t(kMaxTcStages) || nkc == 0) return cudaErrorInvalidValue;
  const size_t smem = tc_smem_bytes(stages, nkc, resident);
  static std::mutex mu;
  static size_t configured[64][2][2] = {};  // per device and variant (its static size differs)
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> g(mu);
  if (dev >= 64 || smem > configured[dev][fp8][l2]) {
    for (TcKernel f : kTcKernels[fp8 ? 1 : 0][l2 ? 1 : 0])
      if (e == cudaSuccess)
        e = cudaFuncSetAttribute(reinterpret_cast<const void*>(f), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 int(smem));
    if (e != cudaSuccess) return e;
    if (dev < 64) configured[dev][fp8][l2] = smem;
  }
  return cudaSuccess;
}

cudaError_t launch_tc_shortlist(const CUtensorMap& qmap, const CUtensorMap& xmap, const TcArgs& a, unsigned grid,
                                cudaStream_t stream, bool pdl) {
  if (a.kp == 0 || a.kp > uint32_t(kTcMaxShortlist) || !a.cbuf_d || !a.cbuf_i) return cudaErrorInvalidValue;
  if (a.fp8 && (!a.xscale || !a.qscale)) return cudaErrorInvalidValue;
  const uint32_t nkc = tc_chunks(a.dp, a.fp8 != 0);
  if (a.resident) {  // the resident block's chunks and a ring of at least 3 slots
    if (a.stages < 3) return cudaErrorInvalidValue;
  }
  if (grid == 0) return cudaSuccess;
  cudaError_t e = tc_prepare(a.stages, nkc, a.resident, a.l2 != 0, a.fp8 != 0);
  if (e != cudaSuccess) return e;
  const size_t smem = tc_smem_bytes(a.stages, nkc, a.resident);
  const uint32_t cap = tc_capacity(a.kp);
  const TcKernel fn = kTcKernels[a.fp8 ? 1 : 0][a.l2 ? 1 : 0][cap == 64 ? 0 : cap == 128 ? 1 : cap == 256 ? 2 : 3];
  return launch_kernel(fn, dim3(grid), dim3(unsigned(tc_threads_cap(cap))), smem, stream, pdl, qmap, xmap, a);
}

cudaError_t launch_to_bf16(const float* src, size_t ld_src, size_t rows, uint32_t dim, uint32_t dp, void* dst,
                           float* norms, cudaStream_t stream, float* bounds, size_t tile_row0) {
  if (rows == 0) return cudaSuccess;
  const size_t threads = rows * 32;
  to_bf16_kernel<<<unsigned((threads + 255) / 256), 256, 0, stream>>>(
      src, ld_src, rows, dim, dp, static_cast<__nv_bfloat16*>(dst), norms, bounds, tile_row0);
  return cudaGetLastError();
}

size_t tc_tiled_bytes(size_t rows, uint32_t dp, bool fp8) {
  return (rows + kTcRows - 1) / kTcRows * size_t(tc_chunks(dp, fp8)) * kRowChunkBytes;
}

cudaError_t tc_encode_tiled_map(CUtensorMap* map, const void* base, uint64_t rows, uint32_t dp, uint32_t box_rows,
                                bool fp8) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return cudaErrorNotSupported;
  if (box_rows == 0 || box_rows > uint32_t(kTcRows) || !base || rows == 0) return cudaErrorInvalidValue;
  const cuuint64_t dims[2] = {fp8 ? 128u : uint64_t(kTcKChunk),
                              (rows + kTcRows - 1) / kTcRows * tc_chunks(dp, fp8) * uint64_t(kTcRows)};
  const cuuint64_t strides[1] = {128};  // one 128-byte chunk row after another
  const cuuint32_t box[2] = {fp8 ? 128u : uint32_t(kTcKChunk), box_rows};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = fn(map, fp8 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2,
                        const_cast<void*>(base), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

cudaError_t launch_to_fp8(const float* src, size_t ld_src, size_t rows, uint32_t dim, uint32_t dp8, void* dst,
                          float* scale, float* norms, cudaStream_t stream, size_t tile_row0, float* bounds) {
  if (rows == 0) return cudaSuccess;
  if (dp8 % 16 != 0 || dp8 < dim) return cudaErrorInvalidValue;
  const size_t threads = rows * 32;
  to_fp8_kernel<<<unsigned((threads + 255) / 256), 256, 0, stream>>>(src, ld_src, rows, dim, dp8,
                                                                     static_cast<uint8_t*>(dst), scale, norms,
                                                                     bounds, tile_row0);
  return cudaGetLastError();
}

cudaError_t launch_midpoint_rows(float* dst, const float* src, uint32_t dp, uint32_t n, uint32_t count,
                                 cudaStream_t stream) {
  if (count == 0 || n == 0) return cudaSuccess;
  midpoint_rows_kernel<<<count, 128, 0, stream>>>(dst, src, dp, n, count);
  return cudaGetLastError();
}

cudaError_t launch_serve_scatter(const uint32_t* count, const uint32_t* fail_list, const ServeQuery* sq,
                                 const float* src_d, const uint32_t* src_i, uint32_t kmax, float* out_d,
                                 uint32_t* out_i, unsigned long long* tally, uint32_t max_queries,
                                 cudaStream_t stream) {
  if (max_queries == 0) return cudaSuccess;
  serve_scatter_kernel<<<max_queries, 128, 0, stream>>>(count, fail_list, sq, src_d, src_i, kmax, out_d, out_i,
                                                        tally);
  return cudaGetLastError();
}

cudaError_t launch_sample_select(const float* in, uint32_t count, uint32_t nq, const uint32_t* kp_per_query,
                                 uint32_t kp, float* thr, cudaStream_t stream, const float* margin, bool pdl) {
  if (nq == 0) return cudaSuccess;
  if (count % 4 != 0 || reinterpret_cast<uintptr_t>(in) % 16 != 0) return cudaErrorInvalidValue;  // float4 loads
  return launch_kernel(sample_select_kernel, dim3(nq), dim3(256), 0, stream, pdl, in, count, nq, kp_per_query, kp,
                       thr, static_cast<const ServeHeader*>(nullptr), static_cast<const ServeQuery*>(nullptr),
                       margin);
}

cudaError_t launch_serve_select(const ServeHeader* hdr, const ServeQuery* sq, const float* in, float* thr,
                                uint32_t max_queries, cudaStream_t stream, const float* margin) {
  if (max_queries == 0) return cudaSuccess;
  sample_select_kernel<<<max_queries, 256, 0, stream>>>(in, 0, 0, nullptr, 0, thr, hdr, sq, margin);
  return cudaGetLastError();
}

size_t finish_smem_bytes(uint32_t dp, uint32_t stage_cap) { return finish_smem(dp, stage_cap).total; }

cudaError_t finish_prepare(uint32_t dp, uint32_t stage_cap, bool* cluster16) {
  const size_t smem = finish_smem_bytes(dp, stage_cap);
  static std::mutex mu;
  static size_t configured[64] = {};
  static bool fits16[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> g(mu);
  if (dev >= 64 || smem > configured[dev]) {
    const void* kernels[4] = {reinterpret_cast<const void*>(finish_kernel<false, false>),
                              reinterpret_cast<const void*>(finish_kernel<true, false>),
                              reinterpret_cast<const void*>(finish_kernel<false, true>),
                              reinterpret_cast<const void*>(finish_kernel<true, true>)};
    for (const void* f : kernels)
      if (e == cudaSuccess) e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    // 16-CTA clusters of the wide variants (both metrics alike): allowed, then asked whether one
    // can be resident at this shared memory size
    for (int i = 2; i < 4 && e == cudaSuccess; ++i)
      e = cudaFuncSetAttribute(kernels[i], cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(16);
    cfg.blockDim = dim3(kFinishThreads);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr;
    attr.id = cudaLaunchAttributeClusterDimension;
    attr.val.clusterDim.x = 16;
    attr.val.clusterDim.y = 1;
    attr.val.clusterDim.z = 1;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    int clusters = 0;
    const bool ok16 = cudaOccupancyMaxActiveClusters(&clusters, finish_kernel<false, true>, &cfg) == cudaSuccess &&
                      clusters >= 1;
    (void)cudaGetLastError();  // (a refused query leaves no error behind)
    if (dev < 64) {
      configured[dev] = smem;
      fits16[dev] = ok16;
    }
    if (cluster16) *cluster16 = ok16;
    return cudaSuccess;
  }
  if (cluster16) *cluster16 = dev < 64 && fits16[dev];
  return cudaSuccess;
}

cudaError_t launch_finish(const FinishArgs& a, uint32_t grid, cudaStream_t stream, bool pdl) {
  if (grid == 0) return cudaSuccess;
  if (a.kp == 0 || a.kp > uint32_t(kTcMaxShortlist) || !a.part_n || a.dp % 4 != 0) return cudaErrorInvalidValue;
  if (!a.hdr && (a.k == 0 || a.k > uint32_t(kMaxK))) return cudaErrorInvalidValue;
  if (a.hdr && !a.sq) return cudaErrorInvalidValue;
  if (a.fail_count && (!a.err || !a.fail_list)) return cudaErrorInvalidValue;
  bool fits16 = false;
  cudaError_t e = finish_prepare(a.dp, a.stage_cap, &fits16);
  if (e != cudaSuccess) return e;
  const size_t smem = finish_smem_bytes(a.dp, a.stage_cap);
  int dev = 0, sms = 0;
  e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  const bool wide = grid <= uint32_t(sms);
  auto* kern = a.l2 ? (wide ? finish_kernel<true, true> : finish_kernel<true, false>)
                    : (wide ? finish_kernel<false, true> : finish_kernel<false, false>);
  const uint32_t c = a.cluster > 8 && !fits16 ? 8u : a.cluster;
  if (c > 1 && wide && !a.hdr && c <= 16 && grid * c <= uint32_t(sms))
    return launch_kernel_cluster(kern, dim3(grid * c), dim3(kFinishThreads), smem, stream, pdl, c, a);
  return launch_kernel(kern, dim3(grid), dim3(kFinishThreads), smem, stream, pdl, a);
}

cudaError_t launch_prepare_queries(const PrepSample* sample, const float* q, uint32_t ldq, uint32_t nq, uint32_t dim,
                                   uint32_t dp, void* qb, float* qnorm, uint32_t* gthr, const float* xbound, bool l2,
                                   float factor, float* margin, float* err, uint32_t* fails, cudaStream_t stream,
                                   float* qscale, uint32_t dpo) {
  if (nq == 0) return cudaSuccess;
  if (!q || !qb || ldq < dim || dp < dim || (margin && (!err || !xbound || !(factor >= 0.f))) ||
      (qscale && (dpo < dim || dpo % 16 != 0 || dpo > kPrepSampleDim)))
    return cudaErrorInvalidValue;
  PrepSample smp{};
  unsigned blocks = (nq + 3) / 4;
  size_t smem = 0;
  if (sample) {
    if (nq > kPrepSampleQueries || dp > kPrepSampleDim || dp % 4 != 0 || ldq % 4 != 0 || !sample->x ||
        !sample->bmin || !sample->thr || !sample->ticket || sample->ranges == 0 ||
        sample->ranges * uint32_t(kTcRows) > kPrepSampleRows || sample->rps < uint32_t(kTcRows))
      return cudaErrorInvalidValue;
    smp = *sample;
    blocks += (smp.ranges * uint32_t(kTcRows) + kPrepRowsPerBlock - 1) / kPrepRowsPerBlock;
    smem = size_t(nq) * dp * sizeof(float);  // <= 32 KB
  }
  auto* kern = qscale ? (l2 ? prepare_queries_kernel<true, true> : prepare_queries_kernel<false, true>)
                      : (l2 ? prepare_queries_kernel<true, false> : prepare_queries_kernel<false, false>);
  kern<<<blocks, 128, smem, stream>>>(q, ldq, nq, dim, dp, qb, qscale ? dpo : dp, qscale, qnorm, gthr, xbound, factor,
                                      margin, err, fails, smp);
  return cudaGetLastError();
}


}  // namespace vsg
