// Large-batch exact scan: register-blocked FP32 distance tiles fused with top-k selection.
//
// Replaces the reference's tiled_kernel (src/gpu_brute_force.cu:142-218), which writes a
// 128 x 128 tile of q.x per CTA into a global distance block, and the select passes that
// read it back (:220-314, :475-482). Here each CTA owns BM queries and a range of rows:
//   * k-slices of 32 dims of the query block and of a 128-row tile are staged in shared
//     memory with 16-byte cp.async copies into a 3-deep ring (rows padded by 4 floats, so
//     the 128-bit shared reads below are free of bank conflicts);
//   * each of 256 threads accumulates a (BM/16) x 8 block of dot products (or squared
//     differences for L2) in registers: queries ty + 16 i, rows tx + 16 j;
//   * after the last k-slice the block is written to a shared score tile as distances, and
//     each warp scans the scores of its queries against the query's current k-th best
//     (dist, id), inserting the few that beat it into the query's sorted list;
//   * at the end each list (kp entries, a few more than k) is written with its length, and a
//     full list publishes its last entry to the query's shared threshold (atomicMin): every
//     row the split left out has a distance at or above it.
// No distance ever reaches global memory. FP32 FMA-bound: 2 * BM * 128 * d flops per tile.
//
// The kernel sums each distance's d products in one FMA chain, a different order from the scan
// kernel's (lane-strided chunks, then a butterfly), so near-ties can order differently. Its lists
// are therefore a shortlist: the finish kernel reranks the rows near each query's k-th best with
// the scan kernel's arithmetic and proves, from a bound E on the difference between the two
// evaluations (launch_prepare_fp32_queries), that no row left out can enter the top k; queries
// it cannot prove run in the scan kernel. The results are the scan kernel's, bit for bit.
#include <mutex>

#include "device_common.cuh"
#include "tiled.cuh"

namespace vsg {

namespace {

constexpr int kBN = 128;       // rows per tile
constexpr int kBK = 32;        // dims per k-slice
constexpr int kPad = 4;        // floats of padding per staged row
constexpr int kLd = kBK + kPad;
constexpr int kThreads = 256;
constexpr int kTN = 8;         // rows per thread
constexpr int kSLd = kBN + 4;  // score tile row stride

__host__ __device__ constexpr size_t al128(size_t v) { return (v + 127) & ~size_t(127); }

struct TiledLayout {
  size_t score_off, ld_off, li_off, total;
};

__host__ __device__ inline TiledLayout tiled_layout(int bm, uint32_t k, int stages) {
  TiledLayout L;
  const size_t stage = size_t(bm + kBN) * kLd * sizeof(float);
  L.score_off = al128(size_t(stages) * stage);
  L.ld_off = L.score_off + al128(size_t(bm) * kSLd * sizeof(float));
  L.li_off = L.ld_off + al128(size_t(bm) * k * sizeof(float));
  L.total = L.li_off + al128(size_t(bm) * k * sizeof(uint32_t));
  return L;
}

template <int BM, bool L2>
__global__ void __launch_bounds__(kThreads, 1) tiled_kernel(const TiledArgs a) {
  constexpr int TM = BM / 16;
  constexpr int kStages = 3;
  extern __shared__ __align__(128) unsigned char smem[];
  const uint32_t dp = a.dp, k = a.kp;
  const TiledLayout L = tiled_layout(BM, k, kStages);
  float* stage_base = reinterpret_cast<float*>(smem);
  float* score = reinterpret_cast<float*>(smem + L.score_off);
  float* lst_d = reinterpret_cast<float*>(smem + L.ld_off);
  uint32_t* lst_i = reinterpret_cast<uint32_t*>(smem + L.li_off);
  constexpr int kStageFloats = (BM + kBN) * kLd;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int ty = tid >> 4, tx = tid & 15;
  const uint32_t qbase = blockIdx.x * BM;
  const uint32_t split = blockIdx.y;
  const uint32_t row_begin = split * a.rows_per_split;
  const uint64_t end64 = uint64_t(row_begin) + a.rows_per_split;  // can pass 2^32 near 2^32 rows
  const uint32_t row_end = end64 < a.n ? uint32_t(end64) : a.n;
  const uint32_t ntiles = row_end > row_begin ? (row_end - row_begin + kBN - 1) / kBN : 0;
  const uint32_t nk = (dp + kBK - 1) / kBK;
  const uint32_t nsteps = ntiles * nk;  // (tile, k-slice) pairs, streamed through one ring

  for (uint32_t i = tid; i < BM * k; i += kThreads) {
    lst_d[i] = __int_as_float(0x7f800000);
    lst_i[i] = kNone;
  }

  // Issues the copies of step t = tile * nk + kslice into ring slot t % kStages.
  auto load_step = [&](uint32_t t) {
    const uint32_t tile = t / nk, k0 = (t % nk) * kBK;
    float* st = stage_base + (t % kStages) * kStageFloats;
    const uint32_t r0 = row_begin + tile * kBN;
    constexpr int kChunks = (BM + kBN) * (kBK / 4);
#pragma unroll
    for (int c = tid; c < kChunks; c += kThreads) {
      const int row = c / (kBK / 4), col = (c % (kBK / 4)) * 4;
      const uint32_t kk = k0 + col;
      if (row < BM) {
        const uint32_t qg = qbase + row;
        const bool ok = qg < a.nq && kk < dp;
        const float* src = ok ? a.q + size_t(qg) * a.ldq + kk : a.q;
        cp_async16(st + row * kLd + col, src, ok);
      } else {
        const uint32_t xr = r0 + (row - BM);
        const bool ok = xr < row_end && kk < dp;
        const float* src = ok ? a.x + size_t(xr) * dp + kk : a.x;
        cp_async16(st + row * kLd + col, src, ok);
      }
    }
  };

#pragma unroll
  for (int s = 0; s < kStages - 1; ++s) {
    if (uint32_t(s) < nsteps) load_step(s);
    cp_async_commit();
  }

  float acc[TM][kTN];
  for (uint32_t t = 0; t < nsteps; ++t) {
    const uint32_t kslice = t % nk;
    if (kslice == 0) {
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < kTN; ++j) acc[i][j] = 0.f;
    }
    cp_async_wait<kStages - 2>();
    __syncthreads();
    // Refill the slot freed at step t - 1 (every thread has passed the barrier above).
    if (t + kStages - 1 < nsteps) load_step(t + kStages - 1);
    cp_async_commit();

    const float* qs = stage_base + (t % kStages) * kStageFloats;
    const float* xs = qs + BM * kLd;
#pragma unroll
    for (int kk = 0; kk < kBK; kk += 4) {
      float4 xv[kTN];
#pragma unroll
      for (int j = 0; j < kTN; ++j) xv[j] = *reinterpret_cast<const float4*>(xs + (tx + 16 * j) * kLd + kk);
#pragma unroll
      for (int i = 0; i < TM; ++i) {
        const float4 qv = *reinterpret_cast<const float4*>(qs + (ty + 16 * i) * kLd + kk);
#pragma unroll
        for (int j = 0; j < kTN; ++j) {
          float s = acc[i][j];
          if constexpr (L2) {
            float e = qv.x - xv[j].x;
            s = fmaf(e, e, s);
            e = qv.y - xv[j].y;
            s = fmaf(e, e, s);
            e = qv.z - xv[j].z;
            s = fmaf(e, e, s);
            e = qv.w - xv[j].w;
            s = fmaf(e, e, s);
          } else {
            s = fmaf(qv.x, xv[j].x, s);
            s = fmaf(qv.y, xv[j].y, s);
            s = fmaf(qv.z, xv[j].z, s);
            s = fmaf(qv.w, xv[j].w, s);
          }
          acc[i][j] = s;
        }
      }
    }

    if (kslice == nk - 1) {
      // Distances of the finished tile into the score tile (+inf for rows past the range).
      const uint32_t r0 = row_begin + (t / nk) * kBN;
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < kTN; ++j) {
          const int n = tx + 16 * j;
          const float d = L2 ? acc[i][j] : 1.0f - acc[i][j];
          score[(ty + 16 * i) * kSLd + n] = r0 + n < row_end ? d : __int_as_float(0x7f800000);
        }
      __syncthreads();
      // Each warp filters its queries' 128 scores against the k-th best and inserts winners.
      for (int m = warp; m < BM; m += kThreads / 32) {
        if (qbase + m >= a.nq) break;
        float* ld = lst_d + size_t(m) * k;
        uint32_t* li = lst_i + size_t(m) * k;
        const float td = ld[k - 1];
        const uint32_t ti = li[k - 1];
        float cd[kBN / 32];
        unsigned any = 0;
#pragma unroll
        for (int c = 0; c < kBN / 32; ++c) {
          cd[c] = score[m * kSLd + c * 32 + lane];
          any |= __ballot_sync(kFull, nb_less(cd[c], r0 + c * 32 + lane, td, ti));
        }
        if (!any) continue;
#pragma unroll
        for (int c = 0; c < kBN / 32; ++c) {
          const uint32_t id = r0 + c * 32 + lane;
          unsigned bal = __ballot_sync(kFull, nb_less(cd[c], id, ld[k - 1], li[k - 1]));
          while (bal) {
            const int src = __ffs(bal) - 1;
            bal &= bal - 1;
            const float v = __shfl_sync(kFull, cd[c], src);
            const uint32_t vid = r0 + c * 32 + src;
            if (nb_less(v, vid, ld[k - 1], li[k - 1])) list_insert(ld, li, int(k), v, vid, lane);
          }
        }
      }
      __syncthreads();  // the score tile is rewritten by the next tile
    }
  }
  cp_async_wait<0>();
  __syncthreads();

  for (int m = warp; m < BM; m += kThreads / 32) {
    const uint32_t qg = qbase + m;
    if (qg >= a.nq) break;
    const size_t o = (size_t(qg) * a.nsplit + split) * k;
    const float* ld = lst_d + size_t(m) * k;
    const uint32_t* li = lst_i + size_t(m) * k;
    uint32_t real = 0;  // the list is sorted: its real entries come first
    for (uint32_t j = lane; j < k; j += 32) {
      a.part_d[o + j] = ld[j];
      a.part_i[o + j] = li[j];
      real += li[j] != kNone ? 1u : 0u;
    }
    real = __reduce_add_sync(kFull, real);
    if (lane == 0) {
      a.part_n[size_t(qg) * a.nsplit + split] = real;
      if (real == k) atomicMin(a.gthr + qg, order_key(ld[k - 1]));
    }
  }
}

// One warp per row (grid-stride): an upper bound of the row's norm, max-reduced into *out.
__global__ void row_norm_max_kernel(const float* __restrict__ x, size_t rows, uint32_t dp, uint32_t* out) {
  const uint32_t lane = threadIdx.x & 31;
  const size_t warps = size_t(gridDim.x) * (blockDim.x >> 5);
  const float u = 5.9604644775390625e-08f;  // 2^-24
  const float infl = __fadd_ru(1.f, __fmul_ru(2.f, __fmul_ru(float(dp), u)));
  float best = 0.f;
  for (size_t r = size_t(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5); r < rows; r += warps) {
    const float* row = x + r * dp;
    float s = 0.f;
    for (uint32_t c = lane; c < dp; c += 32) s = fmaf(row[c], row[c], s);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(kFull, s, o);
    best = fmaxf(best, __fsqrt_ru(__fmul_ru(s, infl)));
  }
  if (lane == 0 && best > 0.f) atomicMax(out, __float_as_uint(best));  // non-negative: bits order as values
}

// |e1 - e2| for two FP32 evaluations of one distance from the same d terms (products for IP,
// squared differences for L2), summed in different orders with FMAs. Any order of d terms is
// within gamma_d sum|terms| of the exact sum, gamma_d = d u / (1 - d u) <= d u (1 + 2 d u) (u =
// 2^-24, d u <= 1/4), so two evaluations differ by at most 2 gamma_d sum|terms|:
//   IP: sum|q_i x_i| <= |q| X (X: the rows' norm bound); the two roundings of 1 - s add at most
//       u (1 + |q| X) each.
//   L2: a difference q_i - x_i is rounded once (relative u), so its square is within 3u of
//       (q_i - x_i)^2; D = sum (q_i - x_i)^2 <= (|q| + X)^2; total 2 (gamma_d + 4u) (|q| + X)^2.
// |q| comes from an FP32 sum of squares inflated by (1 + 2 d u). Every operation rounds up, and
// the result gets a 1.1 margin.
template <bool L2>
__device__ float fp32_pair_error(float sq2, uint32_t dp, float xmax) {
  auto mul = [](float a, float b) { return __fmul_ru(a, b); };
  auto add = [](float a, float b) { return __fadd_ru(a, b); };
  const float u = 5.9604644775390625e-08f;
  const float du = mul(float(dp), u);
  const float infl = add(1.f, mul(2.f, du));
  const float g = mul(du, infl);  // gamma_d
  const float qn = __fsqrt_ru(mul(sq2, infl));
  float e;
  if (L2) {
    const float s = add(qn, xmax);
    e = mul(mul(2.f, add(g, mul(4.f, u))), mul(s, s));
  } else {
    const float qx = mul(qn, xmax);
    e = add(mul(mul(2.f, g), qx), mul(mul(2.f, u), add(1.f, qx)));
  }
  return mul(e, 1.1f);
}

template <bool L2>
__global__ void __launch_bounds__(128) prepare_fp32_queries_kernel(const float* q, uint32_t ldq, uint32_t nq,
                                                                   uint32_t dp, const uint32_t* xmax_bits,
                                                                   float factor, uint32_t* gthr, float* margin,
                                                                   float* err, uint32_t* fails) {
  pdl_trigger();  // the head of a chain: the next kernel may start launching
  if (fails && blockIdx.x == 0 && threadIdx.x == 0) *fails = 0;
  const uint32_t qq = blockIdx.x * 4 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (qq >= nq) return;
  const float* s = q + size_t(qq) * ldq;
  float q2 = 0.f;
  for (uint32_t c = lane; c < dp; c += 32) q2 = fmaf(s[c], s[c], q2);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) q2 += __shfl_xor_sync(kFull, q2, o);
  if (lane == 0) {
    gthr[qq] = kKeyNone;
    const float e = fp32_pair_error<L2>(q2, dp, __uint_as_float(*xmax_bits));
    err[qq] = e;
    margin[qq] = __fmul_ru(factor, e);
  }
}

template <int BM, bool L2>
cudaError_t launch_tiled_one(const TiledArgs& a, dim3 grid, cudaStream_t stream) {
  const size_t smem = tiled_layout(BM, a.kp, 3).total;
  static std::mutex mu;
  static size_t configured[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  {
    std::lock_guard<std::mutex> g(mu);
    if (dev >= 64 || smem > configured[dev]) {
      e = cudaFuncSetAttribute(tiled_kernel<BM, L2>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
      if (e != cudaSuccess) return e;
      if (dev < 64) configured[dev] = smem;
    }
  }
  tiled_kernel<BM, L2><<<grid, kThreads, smem, stream>>>(a);
  return cudaGetLastError();
}

}  // namespace

uint32_t tiled_list_size(uint32_t k) {
  const uint32_t kp = (k + (k / 4 > 8 ? k / 4 : 8) + 7) / 8 * 8;
  return kp < uint32_t(kMaxK) ? kp : uint32_t(kMaxK);
}

int tiled_block_queries(uint32_t kp, uint32_t nq) { return kp <= 48 && nq > 64 ? 128 : 64; }

size_t tiled_smem_bytes(uint32_t kp, uint32_t nq) {
  return tiled_layout(tiled_block_queries(kp, nq), kp, 3).total;
}

cudaError_t launch_row_norm_max(const float* x, size_t rows, uint32_t dp, uint32_t* xmax_bits, cudaStream_t stream) {
  if (rows == 0) return cudaSuccess;
  if (!x || !xmax_bits || dp == 0) return cudaErrorInvalidValue;
  const size_t blocks = (rows + 7) / 8;  // 8 warps a block
  row_norm_max_kernel<<<unsigned(blocks < 4096 ? blocks : 4096), 256, 0, stream>>>(x, rows, dp, xmax_bits);
  return cudaGetLastError();
}

cudaError_t launch_prepare_fp32_queries(const float* q, uint32_t ldq, uint32_t nq, uint32_t dp, bool l2,
                                        const uint32_t* xmax_bits, float factor, uint32_t* gthr, float* margin,
                                        float* err, uint32_t* fails, cudaStream_t stream) {
  if (nq == 0) return cudaSuccess;
  if (!q || !xmax_bits || !gthr || !margin || !err || ldq < dp || !(factor >= 0.f)) return cudaErrorInvalidValue;
  const unsigned blocks = (nq + 3) / 4;
  if (l2)
    prepare_fp32_queries_kernel<true><<<blocks, 128, 0, stream>>>(q, ldq, nq, dp, xmax_bits, factor, gthr, margin,
                                                                  err, fails);
  else
    prepare_fp32_queries_kernel<false><<<blocks, 128, 0, stream>>>(q, ldq, nq, dp, xmax_bits, factor, gthr, margin,
                                                                   err, fails);
  return cudaGetLastError();
}

cudaError_t launch_tiled(const TiledArgs& a, bool l2, dim3 grid, cudaStream_t stream) {
  if (!a.part_n || !a.gthr || a.kp == 0 || a.kp > uint32_t(kMaxK)) return cudaErrorInvalidValue;
  if (tiled_block_queries(a.kp, a.nq) == 128)
    return l2 ? launch_tiled_one<128, true>(a, grid, stream) : launch_tiled_one<128, false>(a, grid, stream);
  return l2 ? launch_tiled_one<64, true>(a, grid, stream) : launch_tiled_one<64, false>(a, grid, stream);
}

}  // namespace vsg
