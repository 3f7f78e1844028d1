// Launch interface of the large-batch tiled FP32 kernel and its certificate helpers (host side).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace vsg {

struct TiledArgs {
  const float* x;      // base rows, n x dp floats
  const float* q;      // queries, row stride ldq floats (16-byte aligned rows)
  float* part_d;       // [nq][nsplit][kp]: each split's best kp by the kernel's FP32 distance
  uint32_t* part_i;
  uint32_t* part_n;    // [nq][nsplit]: real entries of each list
  // Per-query order key (atomicMin): the kp-th entry of every full split list. Every row left out
  // of a split's list has a distance (this kernel's arithmetic) at or above it.
  uint32_t* gthr;
  uint32_t n, dp, ldq, nq, kp;
  uint32_t rows_per_split, nsplit;
};

// Per-split list length for a top-k: k plus max(8, k / 4), rounded up to 8, at most 128. The rows
// past the k-th give the certificate its room: a full list's last entry bounds what it left out.
uint32_t tiled_list_size(uint32_t k);
// Queries per CTA: 128 when the lists hold at most 48 entries and the batch has more than 64
// queries, else 64 (the per-query lists fit, and small batches waste less of the tile).
int tiled_block_queries(uint32_t kp, uint32_t nq);
size_t tiled_smem_bytes(uint32_t kp, uint32_t nq);
cudaError_t launch_tiled(const TiledArgs& a, bool l2, dim3 grid, cudaStream_t stream);

// Raises *xmax_bits (a non-negative float's bits, atomicMax) to an upper bound of the Euclidean
// norm of rows [0, rows) of x (stride dp): each row's FP32 sum of squares inflated by (1 + 2 dp u)
// and its square root rounded up.
cudaError_t launch_row_norm_max(const float* x, size_t rows, uint32_t dp, uint32_t* xmax_bits, cudaStream_t stream);

// The tiled path's queries, one warp per query: gthr[q] reset to none, and err[q] = E, a bound on
// the difference between two FP32 evaluations of one (query, row) distance that sum the same
// products (squared differences for L2) in different orders (the tiled kernel's and the scan
// kernel's), from |q| and the rows' norm bound *xmax_bits; margin[q] = factor x E (both rounded
// up). The first thread zeroes *fails. Launched at the head of a chain (not as a dependent).
cudaError_t launch_prepare_fp32_queries(const float* q, uint32_t ldq, uint32_t nq, uint32_t dp, bool l2,
                                        const uint32_t* xmax_bits, float factor, uint32_t* gthr, float* margin,
                                        float* err, uint32_t* fails, cudaStream_t stream);

}  // namespace vsg
