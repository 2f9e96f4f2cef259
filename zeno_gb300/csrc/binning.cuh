// Binning of one particle into its 4^3 block (MPMPipeline.cu:73-84), shared
// by the bin kernel and the G2P epilogue that bins the new positions for the
// next partition.
#pragma once

#include <cuda_runtime.h>

#include "zsmpm_internal.cuh"

namespace zsmpm {

// base = floor(x / dx - 0.5) per axis (MPMPipeline.cu:78-82), computed as
// one rounded multiply by 1/dx and one rounded subtraction so that no FMA
// contraction changes a key.
__device__ __forceinline__ int particle_base(float x, float inv_dx) {
  return __float2int_rd(__fsub_rn(__fmul_rn(x, inv_dx), 0.5f));
}

// Cell id of a particle inside its 4^3 block, the order of particles within
// a block: z-major, (l2 << 4) | (l0 << 2) | l1, so that the block's 16 cell
// columns (l0, l1) interleave along the sorted order and every contiguous
// chunk of a block's particles spans all 16 columns.
__device__ __forceinline__ int sort_cell(int l0, int l1, int l2) {
  return (l2 << 4) | (l0 << 2) | l1;
}

// key = (global directory index << 6) | cell, or -1 (status bit set) for a
// non-finite position or one outside the interior of the scene's directory
__device__ __forceinline__ int bin_key(const SceneParams &S, float x0, float x1, float x2,
                                       int *status) {
  if (!(isfinite(x0) && isfinite(x1) && isfinite(x2))) {
    atomicOr(status, ST_NAN);
    return -1;
  }
  const int b0 = particle_base(x0, S.inv_dx), b1 = particle_base(x1, S.inv_dx),
            b2 = particle_base(x2, S.inv_dx);
  const int c0 = (b0 >> 2) - S.block_lo[0], c1 = (b1 >> 2) - S.block_lo[1],
            c2 = (b2 >> 2) - S.block_lo[2];
  const int dy = S.block_dims[1], dz = S.block_dims[2];
  if (c0 < 1 || c0 > S.block_dims[0] - 2 || c1 < 1 || c1 > dy - 2 || c2 < 1 || c2 > dz - 2) {
    atomicOr(status, ST_OUT_OF_DOMAIN);
    return -1;
  }
  const int dd = S.dir_off + (c0 * dy + c1) * dz + c2;
  return (dd << 6) | sort_cell(b0 & 3, b1 & 3, b2 & 3);
}

// Warp-aggregated count of `key` into its block; the first particle of a
// block marks the block and its 26 neighbours as grid blocks (the 1-ring
// halo of ExpandZSPartition, MPMPipeline.cu:131-199).  Every lane of `mask`
// must call this together; lanes of one call may belong to different scenes
// (the leader of a block marks with its own scene's strides).
__device__ __forceinline__ void bin_count(const DevPtrs &d, const SceneParams &S, int key,
                                          unsigned mask) {
  const int dd = key >> 6;  // -1 for invalid
  const unsigned peers = __match_any_sync(mask, dd);
  const int leader = __ffs(peers) - 1;
  if (key >= 0 && (int)(threadIdx.x & 31) == leader) {
    const int old = atomicAdd(&d.dir_count[dd], __popc(peers));
    if (old == 0) {
      const int dy = S.block_dims[1], dz = S.block_dims[2];
      for (int a = -1; a <= 1; ++a)
        for (int b = -1; b <= 1; ++b)
          for (int c = -1; c <= 1; ++c) d.dir_flag[dd + (a * dy + b) * dz + c] = 1;
    }
  }
}

}  // namespace zsmpm
