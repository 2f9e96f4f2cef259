// Block helpers shared by the transfer kernels: the node origin and the
// 2x2x2 grid-block neighbourhood of a particle block, and the launch
// metadata the G2P pipelines stage in shared memory.
#pragma once

#include <cuda_runtime.h>

#include "zsmpm_internal.cuh"

namespace zsmpm {

// node index of the first node of the particle block at (scene-local)
// directory index `ldir`
__device__ __forceinline__ void bucket_origin(const SceneParams &S, int ldir, int (&K)[3]) {
  const int dz = S.block_dims[2], dy = S.block_dims[1];
  const int c2 = ldir % dz, c1 = (ldir / dz) % dy, c0 = ldir / (dz * dy);
  K[0] = (c0 + S.block_lo[0]) * 4;
  K[1] = (c1 + S.block_lo[1]) * 4;
  K[2] = (c2 + S.block_lo[2]) * 4;
}

// grid block of each of the 2x2x2 blocks around the particle block at
// (global) directory index `dir`
__device__ __forceinline__ int neighbour_gb(const DevPtrs &d, const SceneParams &S, int dir,
                                            int t) {
  const int dz = S.block_dims[2], dy = S.block_dims[1];
  return d.dir_gb[dir + ((t >> 2) * dy + ((t >> 1) & 1)) * dz + (t & 1)];
}

// G2P launch metadata of one particle block, held in shared memory for the
// blocks a CTA owns so that the G2P software pipelines need no dependent
// global loads to find their next chunk.
struct G2PMeta {
  int start, cnt, dir, scene;
  int gb[8];  // grid blocks of the 2x2x2 block neighbourhood (-1: absent)
  int K[3];   // node index of the block's first node
  int pad;
};

__device__ __forceinline__ G2PMeta g2p_load_meta(const DevPtrs &d, long long n, int b) {
  G2PMeta m;
  m.dir = d.bk_dir[b];
  m.scene = scene_of_dir(d, m.dir);
  m.start = d.bk_start[b];
  m.cnt = (int)max(0ll, min((long long)d.bk_count[b], n - m.start));
  const SceneParams &S = d.scn[m.scene];
#pragma unroll
  for (int t = 0; t < 8; ++t) m.gb[t] = neighbour_gb(d, S, m.dir, t);
  bucket_origin(S, m.dir - S.dir_off, m.K);
  m.pad = 0;
  return m;
}

}  // namespace zsmpm
