// Device-side building blocks shared by the exact k-NN kernels (sm_103a).
//
//  * PTX wrappers for mbarriers and bulk (TMA) global->shared copies. Every
//    wait is bounded by the global timer: a wait that runs past kWaitLimitNs
//    returns false, the kernel records kDevTimeout in its error word and winds
//    down instead of spinning forever.
//  * A warp-owned sorted top-k list in shared memory, ordered by (dist, id):
//    ties go to the lower id, the rule of the reference's final merge
//    (src/brute_force.cpp:152-169) and of its GPU select (src/gpu_brute_force.cu:276).
//  * A warp reduce-scatter: 32 lanes each holding V partial sums end with
//    lane L holding the full sum of value L * V / 32.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace vsg {

constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr int kMaxK = 128;
constexpr unsigned kFull = 0xFFFFFFFFu;
constexpr unsigned long long kWaitLimitNs = 2000000000ull;  // 2 s for any single wait

enum DevStatus : int { kDevOk = 0, kDevTimeout = 1 };

// Programmatic dependent launch. A kernel launched with the programmatic stream serialization
// attribute may start while the kernel before it in the stream still runs. It calls pdl_wait
// before it reads anything a predecessor wrote or writes anything a predecessor may still read;
// the wait returns once the predecessor has completed and its writes are visible (and, since the
// predecessor waited the same way, every earlier kernel of the chain). Every thread of such a
// kernel passes a pdl_wait before it exits, which keeps that ordering transitive. pdl_trigger lets
// the next kernel start launching once every CTA of this one has called it (so all of them are
// resident and a waiting dependent can never hold an SM one of them needs). Both return at once
// in a kernel launched without the attribute.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

__device__ __forceinline__ bool nb_less(float ad, uint32_t ai, float bd, uint32_t bi) {
  return ad < bd || (ad == bd && ai < bi);
}

// Float -> unsigned key with the same order (negative values flipped), and back. A per-query
// threshold published by several CTAs is kept as such a key (atomicMin); kKeyNone = not set.
constexpr uint32_t kKeyNone = 0xFFFFFFFFu;
__device__ __forceinline__ uint32_t order_key(float f) {
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float key_float(uint32_t key) {
  return __uint_as_float((key & 0x80000000u) ? (key & 0x7FFFFFFFu) : ~key);
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// 16-byte global -> shared copies without registers (cp.async, L2 only): `valid` false writes
// zeros and reads nothing. A thread's copies complete in commit groups; cp_async_wait<N> returns
// once at most N of its groups are pending (then a warp or CTA barrier shows them to the others).
__device__ __forceinline__ void cp_async16(void* dst, const void* src, bool valid) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_addr(dst)), "l"(src),
               "r"(valid ? 16 : 0)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Prefetch of `bytes` (a multiple of 16) from a 16-byte aligned global address into L2.
__device__ __forceinline__ void bulk_prefetch_l2(const void* p, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

__device__ __forceinline__ uint32_t atomic_add_acq_rel(uint32_t* p, uint32_t v) {
  uint32_t old;
  asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Waits for the phase with the given parity to complete. False after limit_ns (kWaitLimitNs by
// default; a kernel's waits on other roles take its tunable limit, the waits that drain its own
// copies and MMAs before it exits keep the default).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, unsigned long long limit_ns = kWaitLimitNs) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  for (uint32_t it = 1;; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 63u) == 0 && global_ns() - t0 > limit_ns) return false;
  }
}

// Bulk copy of `bytes` contiguous bytes (multiple of 16, both addresses 16-byte
// aligned) from global to shared memory; completion is signalled on `bar`.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// Same, with an L2 evict-first hint: the base rows are streamed once per search.
__device__ __forceinline__ void bulk_load_stream(void* dst, const void* src, uint32_t bytes, uint64_t* bar,
                                                 uint64_t policy) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], "
      "%4;" ::"r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar)), "l"(policy)
      : "memory");
}

__device__ __forceinline__ uint64_t policy_evict_first() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}

// ---- warp reduce-scatter ------------------------------------------------------------------
// N values per lane, at lane-mask M. After the full recursion (M = 16 .. 1) lane L holds, in
// v[0], the warp-wide sum of value index L / (32 / N) (N <= 32, a power of two).
template <int N, int M>
struct ReduceScatter {
  static __device__ __forceinline__ void run(float* v, int lane) {
    if constexpr (M == 0) {
      return;
    } else if constexpr (N > 1) {
      constexpr int H = N / 2;
      const bool up = (lane & M) != 0;
#pragma unroll
      for (int i = 0; i < H; ++i) {
        const float send = up ? v[i] : v[i + H];
        const float keep = up ? v[i + H] : v[i];
        v[i] = keep + __shfl_xor_sync(kFull, send, M);
      }
      ReduceScatter<H, M / 2>::run(v, lane);
    } else {
      v[0] += __shfl_xor_sync(kFull, v[0], M);
      ReduceScatter<1, M / 2>::run(v, lane);
    }
  }
};

// ---- warp-owned sorted top-k list ------------------------------------------------------------
// ld/li hold k entries sorted by (dist, id), padded with (inf, kNone). Inserts (cd, ci), which
// the caller has checked to be below entry k-1, and drops the last entry. Whole warp, uniform args.
__device__ __forceinline__ void list_insert(float* ld, uint32_t* li, int k, float cd, uint32_t ci, int lane) {
  int pos = 0;
#pragma unroll
  for (int e = 0; e < kMaxK / 32; ++e) {
    if (e * 32 < k) {
      const int j = e * 32 + lane;
      const bool lt = j < k && nb_less(ld[j], li[j], cd, ci);
      pos += __popc(__ballot_sync(kFull, lt));
    }
  }
  float vd[kMaxK / 32];
  uint32_t vi[kMaxK / 32];
#pragma unroll
  for (int e = 0; e < kMaxK / 32; ++e) {
    const int j = e * 32 + lane;
    if (e * 32 < k && j >= pos && j + 1 < k) {
      vd[e] = ld[j];
      vi[e] = li[j];
    }
  }
  __syncwarp();
#pragma unroll
  for (int e = 0; e < kMaxK / 32; ++e) {
    const int j = e * 32 + lane;
    if (e * 32 < k && j >= pos && j + 1 < k) {
      ld[j + 1] = vd[e];
      li[j + 1] = vi[e];
    }
  }
  if (lane == 0) {
    ld[pos] = cd;
    li[pos] = ci;
  }
  __syncwarp();
}

// Merges `len` entries of a list sorted by (dist, id) into the warp's top-k list. Since the
// source is sorted and the list's last entry only decreases, the first rejected entry ends it.
__device__ __forceinline__ void list_merge_sorted(float* ld, uint32_t* li, int k, const float* sd,
                                                  const uint32_t* si, int len, int lane) {
  for (int c0 = 0; c0 < len; c0 += 32) {
    const int j = c0 + lane;
    const bool valid = j < len;
    const float d = valid ? sd[j] : __int_as_float(0x7f800000);
    const uint32_t id = valid ? si[j] : kNone;
    const float td = ld[k - 1];
    const uint32_t ti = li[k - 1];
    const bool pass = valid && nb_less(d, id, td, ti);
    unsigned m = __ballot_sync(kFull, pass);
    const unsigned vmask = __ballot_sync(kFull, valid);
    const bool ended = m != vmask;
    while (m) {
      const int src = __ffs(m) - 1;
      m &= m - 1;
      const float cd = __shfl_sync(kFull, d, src);
      const uint32_t ci = __shfl_sync(kFull, id, src);
      if (nb_less(cd, ci, ld[k - 1], li[k - 1])) list_insert(ld, li, k, cd, ci, lane);
    }
    if (ended) break;
  }
}

// ---- warp top-k held in registers, merged with bitonic networks -----------------------------
// Entry j of a K = 32 * E list lives in register j / 32 of lane j % 32. Merging a sorted list B
// into a sorted list A: C[j] = min(A[j], B[K - 1 - j]) is bitonic and holds the K smallest of
// A and B (Batcher); a bitonic merge network (log2 K compare-exchange stages, across registers
// for strides >= 32 and across lanes by shuffles below) sorts it. Order is (dist, id).
template <int E>
struct WarpTopK {
  float d[E];
  uint32_t i[E];

  __device__ __forceinline__ void clear() {
#pragma unroll
    for (int e = 0; e < E; ++e) {
      d[e] = __int_as_float(0x7f800000);
      i[e] = kNone;
    }
  }
  // Loads len <= 32 * E sorted entries (the rest become (inf, kNone)).
  __device__ __forceinline__ void load(const float* sd, const uint32_t* si, int len, int lane) {
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const int j = e * 32 + lane;
      d[e] = j < len ? sd[j] : __int_as_float(0x7f800000);
      i[e] = j < len ? si[j] : kNone;
    }
  }
  __device__ __forceinline__ void store(float* dd, uint32_t* di, int len, int lane) const {
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const int j = e * 32 + lane;
      if (j < len) {
        dd[j] = d[e];
        di[j] = i[e];
      }
    }
  }
  // Entry j (0 <= j < 32 E), broadcast to the warp. Every register is shuffled and the wanted
  // one selected afterwards: a select over the array itself with a run-time j would make the
  // compiler keep the array in local memory.
  __device__ __forceinline__ void entry(int j, float& od, uint32_t& oi) const {
    const int src = j & 31, reg = j >> 5;
    od = __shfl_sync(kFull, d[0], src);
    oi = __shfl_sync(kFull, i[0], src);
#pragma unroll
    for (int e = 1; e < E; ++e) {
      const float td = __shfl_sync(kFull, d[e], src);
      const uint32_t ti = __shfl_sync(kFull, i[e], src);
      od = reg == e ? td : od;
      oi = reg == e ? ti : oi;
    }
  }
  template <int R>
  __device__ __forceinline__ void cross() {
#pragma unroll
    for (int e = 0; e < E; ++e)
      if (!(e & R) && nb_less(d[e | R], i[e | R], d[e], i[e])) {
        const float td = d[e];
        const uint32_t ti = i[e];
        d[e] = d[e | R];
        i[e] = i[e | R];
        d[e | R] = td;
        i[e | R] = ti;
      }
  }
  // Compare-exchange of entries j and j ^ stride for every j, ascending where (j & size) == 0.
  template <int SIZE, int STRIDE>
  __device__ __forceinline__ void sort_stage(int lane) {
    if constexpr (STRIDE >= 32) {
      constexpr int R = STRIDE / 32;
#pragma unroll
      for (int e = 0; e < E; ++e)
        if (!(e & R)) {
          const bool up = ((e * 32 + lane) & SIZE) == 0;
          if (up == nb_less(d[e | R], i[e | R], d[e], i[e])) {
            const float td = d[e];
            const uint32_t ti = i[e];
            d[e] = d[e | R];
            i[e] = i[e | R];
            d[e | R] = td;
            i[e | R] = ti;
          }
        }
    } else {
#pragma unroll
      for (int e = 0; e < E; ++e) {
        const float od = __shfl_xor_sync(kFull, d[e], STRIDE);
        const uint32_t oi = __shfl_xor_sync(kFull, i[e], STRIDE);
        const bool up = ((e * 32 + lane) & SIZE) == 0;
        const bool lower = (lane & STRIDE) == 0;
        // ascending: the lower index keeps the smaller entry; descending: the larger
        if ((lower == up) == nb_less(od, oi, d[e], i[e])) {
          d[e] = od;
          i[e] = oi;
        }
      }
    }
    if constexpr (STRIDE > 1) sort_stage<SIZE, STRIDE / 2>(lane);
  }
  template <int SIZE>
  __device__ __forceinline__ void sort_from(int lane) {
    sort_stage<SIZE, SIZE / 2>(lane);
    if constexpr (SIZE < 32 * E) sort_from<SIZE * 2>(lane);
  }
  // Bitonic sort of all 32 E entries, ascending by (dist, id). Whole warp.
  __device__ __forceinline__ void sort(int lane) { sort_from<2>(lane); }

  // this = the 32 E smallest of this and b (both sorted). Whole warp.
  __device__ __forceinline__ void merge(const WarpTopK& b, int lane) {
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const float rd = __shfl_sync(kFull, b.d[E - 1 - e], 31 - lane);
      const uint32_t ri = __shfl_sync(kFull, b.i[E - 1 - e], 31 - lane);
      if (nb_less(rd, ri, d[e], i[e])) {
        d[e] = rd;
        i[e] = ri;
      }
    }
    // strides of r * 32 entries: between registers of the same lane
    if constexpr (E >= 4) cross<2>();
    if constexpr (E >= 2) cross<1>();
#pragma unroll
    for (int s = 16; s >= 1; s >>= 1)  // strides below 32: across lanes
#pragma unroll
      for (int e = 0; e < E; ++e) {
        const float od = __shfl_xor_sync(kFull, d[e], s);
        const uint32_t oi = __shfl_xor_sync(kFull, i[e], s);
        const bool lower = (lane & s) == 0;  // the lower index keeps the smaller entry
        if (lower == nb_less(od, oi, d[e], i[e])) {
          d[e] = od;
          i[e] = oi;
        }
      }
  }
};

// Merges `nlists` sorted lists of k entries (list j at sd + j * stride) into acc, skipping a
// list whose best entry does not beat acc's k-th. Whole warp.
template <int E>
__device__ __forceinline__ void warp_merge_lists(WarpTopK<E>& acc, const float* sd, const uint32_t* si,
                                                 int nlists, size_t stride, int k, int lane, int kk = 0,
                                                 float mg = -1.f) {
  float kd;
  uint32_t ki;
  // The bar a list's first entry must beat: the k-th entry so far, or with a margin (mg >= 0)
  // the kk-th entry + mg when that is lower.
  auto bar = [&] {
    acc.entry(k - 1, kd, ki);
    if (mg >= 0.f) {
      float td;
      uint32_t ti;
      acc.entry(kk - 1, td, ti);
      td = __fadd_ru(td, mg);
      if (nb_less(td, kNone, kd, ki)) {
        kd = td;
        ki = kNone;
      }
    }
  };
  bar();
  // The lists' first entries are read 32 at a time (lane l: list base + l), so the reads that
  // decide which lists to skip do not wait on one another.
  for (int base = 0; base < nlists; base += 32) {
    float hd = __int_as_float(0x7f800000);
    uint32_t hi = kNone;
    if (base + lane < nlists) {
      hd = sd[size_t(base + lane) * stride];
      hi = si[size_t(base + lane) * stride];
    }
    unsigned live = __ballot_sync(kFull, nb_less(hd, hi, kd, ki));
    while (live) {
      const int src = __ffs(live) - 1;
      live &= live - 1;
      const float fd = __shfl_sync(kFull, hd, src);
      const uint32_t fi = __shfl_sync(kFull, hi, src);
      if (!nb_less(fd, fi, kd, ki)) continue;  // the bar has moved past this list's best
      WarpTopK<E> b;
      b.load(sd + size_t(base + src) * stride, si + size_t(base + src) * stride, k, lane);
      acc.merge(b, lane);
      bar();
    }
  }
}

// Copies `count` (dist, id) entries from global memory written by other CTAs of the running
// kernel into shared memory with L1-bypassing loads (the caller has fenced after observing
// that the writers are done). Whole CTA.
__device__ __forceinline__ void stage_lists_cg(float* dd, uint32_t* di, const float* sd, const uint32_t* si,
                                               size_t count, int tid, int nthreads) {
  for (size_t j = tid; j < count; j += nthreads) {
    dd[j] = __ldcg(sd + j);
    di[j] = __ldcg(si + j);
  }
}

}  // namespace vsg
