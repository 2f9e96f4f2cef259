// The cloth's P2G tiles (one per cloth block: the sums of its 6^3 nodes)
// added into the grid the particles were gathered into.  Node (l0, l1, l2)
// of grid block G lies in the tile of cloth block G - o (o in {0, 1}^3, in
// blocks) at tile coordinate l + 4 o when that is < 6; the <= 8 tiles add in
// the fixed order o = (0,0,0), (0,0,1), ..., so the sums are reproducible.
// Used by the stage path's k_cloth_grid_add and, fused with the update, by
// the grid updates of the whole substep (mode bit kGridAddCloth).
#pragma once

#include <cuda_runtime.h>

#include "zsmpm_internal.cuh"

namespace zsmpm {

constexpr int kGridAddCloth = 4;  // grid-update mode bit: add the cloth's tiles first

// lane k < 8: the cloth block of source o = k of the grid block at global
// directory entry gdir (local block coordinates c0, c1, c2), or -1
__device__ __forceinline__ int cloth_source(const ClothDev &cl, const SceneParams &S, int gdir,
                                            int c0, int c1, int c2, int lane) {
  if (lane >= 8) return -1;
  const int o0 = lane >> 2, o1 = (lane >> 1) & 1, o2 = lane & 1;
  if (c0 < o0 || c1 < o1 || c2 < o2) return -1;
  const int bk = cl.cdir_bk[gdir - (o0 * S.block_dims[1] + o1) * S.block_dims[2] - o2];
  return bk >= 0 && bk < cl.cap_cblocks ? bk : -1;
}

// the tiles covering node `cell` (sources src) into g (mass, momentum) and,
// on FLIP-style grids, h (vstar); true when some tile covers the node
__device__ __forceinline__ bool add_cloth_tiles(const ClothDev &cl, const int (&src)[8], int cell,
                                                bool flip_style, float4 &g, float4 &h) {
  const int l0 = cell >> 4, l1 = (cell >> 2) & 3, l2 = cell & 3;
  float4 s = make_float4(0.f, 0.f, 0.f, 0.f), u2 = make_float4(0.f, 0.f, 0.f, 0.f);
  bool any = false;
#pragma unroll
  for (int o = 0; o < 8; ++o) {
    const int o0 = o >> 2, o1 = (o >> 1) & 1, o2 = o & 1;
    if ((o0 && l0 >= 2) || (o1 && l1 >= 2) || (o2 && l2 >= 2) || src[o] < 0) continue;
    const long long ti =
        (long long)src[o] * kTileNodes + ((l0 + 4 * o0) * 6 + (l1 + 4 * o1)) * 6 + (l2 + 4 * o2);
    const float4 t = cl.ctile[ti];
    s.x += t.x;
    s.y += t.y;
    s.z += t.z;
    s.w += t.w;
    if (flip_style) {
      const float4 u = cl.ctile2[ti];
      u2.x += u.x;
      u2.y += u.y;
      u2.z += u.z;
    }
    any = true;
  }
  if (!any) return false;
  g.x += s.x;
  g.y += s.y;
  g.z += s.z;
  g.w += s.w;
  if (flip_style) {
    h.x += u2.x;
    h.y += u2.y;
    h.z += u2.z;
  }
  return true;
}

}  // namespace zsmpm
