// Launch interface of the large-batch tiled FP32 kernel (host side).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace vsg {

struct TiledArgs {
  const float* x;      // base rows, n x dp floats
  const float* q;      // queries, row stride ldq floats (16-byte aligned rows)
  float* part_d;       // [nq][nsplit][k]
  uint32_t* part_i;
  uint32_t n, dp, ldq, nq, k;
  uint32_t rows_per_split, nsplit;
};

// Queries per CTA: 128 for k <= 32 and batches above 64, else 64 (the per-query lists fit,
// and small batches waste less of the tile).
int tiled_block_queries(uint32_t k, uint32_t nq);
size_t tiled_smem_bytes(uint32_t k, uint32_t nq);
cudaError_t launch_tiled(const TiledArgs& a, bool l2, dim3 grid, cudaStream_t stream);

}  // namespace vsg
