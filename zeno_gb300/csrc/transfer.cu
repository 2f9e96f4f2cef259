// Particle-to-grid, grid update + boundary, grid-to-particle.
//
// One CTA owns one particle block at a time (particles sorted by block and
// cell, see partition.cu).  A block's quadratic stencils all fall in the 6^3
// nodes [K, K+6) of its block key K, which lie in the 2x2x2 grid blocks
// K + {0,4}^3:
//  * P2G (Transfer.cu:849-889) sums the block's particle contributions per
//    node in shared memory (one warp per cell, one lane per stencil node) and
//    stores the 216 node sums of the block as a tile; the grid gather then
//    adds, per grid node, the <= 8 tiles that cover it in a fixed order and
//    applies the grid update and boundary.  The reference's 27 x 4 global
//    float atomics per particle become plain stores, the grid needs no clear,
//    and the grid sums do not depend on scheduling.
//  * G2P (Transfer.cu:1139-1173) stages the 216 node velocities in shared
//    memory and gathers from there; it writes the particle's new state into
//    the other particle buffer at its sorted position, so storage follows
//    the block order from one substep to the next.  It ends with the return
//    mapping (ZSReturnMapping) and the Kirchhoff stress of the new F, stored
//    as S = vol * tau for the next P2G, so that the Drucker-Prager projection
//    and the StVK-Hencky stress share one eigen-decomposition.
#include <cuda_runtime.h>

#include <algorithm>

#include "binning.cuh"
#include "blocks.cuh"
#include "cloth_grid.cuh"
#include "colliders.cuh"
#include "cp_async.cuh"
#include "mpm_math.cuh"
#include "tile_scatter.cuh"
#include "transfer_stages.cuh"
#include "zsmpm_internal.cuh"

namespace zsmpm {
namespace {

// the stages as their own kernels (transfer_stages.cuh holds their bodies)
template <int kColThreads, int kColChunk>
__global__ void __launch_bounds__(kColThreads, kColThreads == 192 ? 4 : 3)
    k_p2g(DevPtrs d, const float *__restrict__ pin, const int32_t *__restrict__ iin) {
  extern __shared__ __align__(16) unsigned char p2g_smem[];
  stage_p2g<kColThreads, kColChunk>(d, pin, iin, p2g_smem, blockIdx.x, gridDim.x);
}

template <int kGatherBlocks>
__global__ void __launch_bounds__(64 * kGatherBlocks) k_grid_gather(DevPtrs d, int mode) {
  stage_grid_gather<kGatherBlocks>(d, mode, blockIdx.x, gridDim.x);
}

template <bool kFuseRM, bool kFuseBin, int NT, bool kHencky>
__global__ void __launch_bounds__(NT, 768 / NT)
    k_g2p(DevPtrs d, const float *__restrict__ pin, const int32_t *__restrict__ iin,
          float *__restrict__ pout, int32_t *__restrict__ iout) {
  extern __shared__ __align__(16) unsigned char g2p_smem[];
  stage_g2p<kFuseRM, kFuseBin, NT, kHencky>(d, pin, iin, pout, iout, g2p_smem, blockIdx.x,
                                            gridDim.x);
}

__global__ void k_grid_update(DevPtrs d, int mode) {
  if (ZSMPM_HALTED(d)) return;
  const SimParams &P = *d.prm;
  const long long n = (long long)min(d.cnt->n_gblocks, d.cap_gblocks) * 64;
  float vmax = 0.0f;
  if (mode & kGridAddCloth) {
    // the cloth's tiles first (one context, one scene): a warp per grid
    // block, two nodes per lane
    const SceneParams &S = d.scn[0];
    const int dy = S.block_dims[1], dz = S.block_dims[2], lane = threadIdx.x & 31;
    const int warps = gridDim.x * (blockDim.x >> 5);
    for (int gb = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); gb < (int)(n >> 6);
         gb += warps) {
      const int gdir = d.gb_dir[gb], ldir = gdir - S.dir_off;
      const int bk =
          cloth_source(d.cloth, S, gdir, ldir / (dz * dy), (ldir / dz) % dy, ldir % dz, lane);
      const bool covered = __any_sync(0xffffffffu, bk >= 0);
      int src[8];
#pragma unroll
      for (int o = 0; o < 8; ++o) src[o] = __shfl_sync(0xffffffffu, bk, o);
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int cell = lane + 32 * h;
        const long long idx = (long long)gb * 64 + cell;
        float4 g = d.grid[idx], unused;
        const bool added = covered && add_cloth_tiles(d.cloth, src, cell, false, g, unused);
        if (g.x != 0.0f) update_node(d, 0, S, P.dt, mode, ldir, cell, g, vmax);
        if (g.x != 0.0f || added) d.grid[idx] = g;
      }
    }
  } else {
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
         idx += (long long)gridDim.x * blockDim.x) {
      float4 g = d.grid[idx];
      if (g.x == 0.0f) continue;
      const int gdir = d.gb_dir[idx >> 6];
      const int sc = scene_of_dir(d, gdir);
      const SceneParams &S = d.scn[sc];
      update_node(d, sc, S, P.dt, mode, gdir - S.dir_off, (int)(idx & 63), g, vmax);
      d.grid[idx] = g;
    }
  }
  if (mode & 1) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
    if ((threadIdx.x & 31) == 0 && vmax > 0.0f)
      atomicMax(&d.cnt->max_vel_sqr_bits, __float_as_uint(vmax));
  }
}

__device__ __forceinline__ void store_stress(float *__restrict__ pb, long long p, float vol,
                                             const Sym3 &t) {
  pb[pidx((CH_S + 0), p)] = vol * t.xx;
  pb[pidx((CH_S + 1), p)] = vol * t.yy;
  pb[pidx((CH_S + 2), p)] = vol * t.zz;
  pb[pidx((CH_S + 3), p)] = vol * t.xy;
  pb[pidx((CH_S + 4), p)] = vol * t.xz;
  pb[pidx((CH_S + 5), p)] = vol * t.yz;
}

// ZSReturnMapping as its own pass (in place, storage order); refreshes the
// stored stress of every projected particle.
__global__ void k_return_mapping(DevPtrs d, float *__restrict__ pbuf,
                                 const int32_t *__restrict__ ibuf) {
  const SimParams &P = *d.prm;
  const long long n = P.n;
  const bool lame = P.has_lame != 0;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    const MatParams mp = d.mats[min(max(ibuf[iidx(IC_MAT, p)], 0), kMaxMaterials - 1)];
    if (mp.type == MPM_EOS || mp.plastic == MPM_PLASTIC_NONE) continue;
    float F[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) F[k] = pbuf[pidx((CH_F + k), p)];
    float mu = mp.mu, lam = mp.lam;
    if (lame) {
      mu = pbuf[pidx(CH_MU, p)];
      lam = pbuf[pidx(CH_LAM, p)];
    }
    Sym3 tau;
    float jch = pbuf[pidx(CH_J, p)];  // log(Jp) of a Cam-Clay particle
    const int r = return_mapping(mp, mu, lam, F, jch, tau);
    if (r < 0) atomicOr(&d.cnt->status, ST_NAN);
    if (r > 0) {
#pragma unroll
      for (int k = 0; k < 9; ++k) pbuf[pidx((CH_F + k), p)] = F[k];
      pbuf[pidx(CH_J, p)] = mp.plastic == MPM_PLASTIC_NACC ? jch : det3(F);
      // the FLIP P2G takes the material's Lame parameters (Transfer.cu:897-907)
      if (lame && d.transfer == MPM_TRANSFER_FLIP &&
          !kirchhoff(mp.type, mp.mu, mp.lam, mp.bulk, mp.gamma, F, 1.0f, tau))
        atomicOr(&d.cnt->status, ST_NAN);
      store_stress(pbuf, p, pbuf[pidx(CH_VOL, p)], tau);
    }
  }
}

// S = vol * tau of every particle from its current F (or J): the stress P2G
// reads, recomputed after an upload or a change of materials.
__global__ void k_stress(DevPtrs d, float *__restrict__ pbuf, const int32_t *__restrict__ ibuf,
                         long long b0, long long b1) {
  const SimParams &P = *d.prm;
  const long long n = b1 < 0 ? P.n : b1;
  const bool lame = P.has_lame != 0;
  for (long long p = b0 + blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    const MatParams mp = d.mats[min(max(ibuf[iidx(IC_MAT, p)], 0), kMaxMaterials - 1)];
    float F[9];
    float J = 1.0f;
    if (mp.type == MPM_EOS) {
      J = pbuf[pidx(CH_J, p)];
#pragma unroll
      for (int k = 0; k < 9; ++k) F[k] = (k % 4 == 0) ? 1.0f : 0.0f;
    } else {
#pragma unroll
      for (int k = 0; k < 9; ++k) F[k] = pbuf[pidx((CH_F + k), p)];
    }
    float mu = mp.mu, lam = mp.lam;
    if (lame && d.transfer != MPM_TRANSFER_FLIP) {  // FLIP: Transfer.cu:897-907
      mu = pbuf[pidx(CH_MU, p)];
      lam = pbuf[pidx(CH_LAM, p)];
    }
    Sym3 tau;
    if (!kirchhoff(mp.type, mu, lam, mp.bulk, mp.gamma, F, J, tau))
      atomicOr(&d.cnt->status, ST_NAN);
    store_stress(pbuf, p, pbuf[pidx(CH_VOL, p)], tau);
  }
}

}  // namespace

int g2p_occupancy() {
  constexpr int NT = 128;
  constexpr int smem = g2p_smem_bytes<NT>();
  cudaFuncSetAttribute(k_g2p<true, true, NT, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       smem);
  cudaFuncSetAttribute(k_g2p<true, false, NT, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       smem);
  cudaFuncSetAttribute(k_g2p<false, false, NT, false>,
                       cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  cudaFuncSetAttribute(k_g2p<true, true, NT, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       smem);
  cudaFuncSetAttribute(k_g2p<true, false, NT, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       smem);
  int b = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_g2p<true, true, NT, false>, NT, smem);
  return b > 0 ? b : 1;
}

// the P2G tile shapes the launch knobs can pick: (threads, chunk)
template <int NT, int CH> int p2g_occupancy() {
  constexpr int smem = ColLayout<NT, CH>::smem;
  cudaFuncSetAttribute(k_p2g<NT, CH>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  int a = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_p2g<NT, CH>, NT, smem);
  return a > 0 ? a : 1;
}

int p2g_shape_occupancy(int shape) {
  switch (shape) {
    case 1: return p2g_occupancy<192, 192>();
    case 2: return p2g_occupancy<192, 96>();
    case 3: return p2g_occupancy<256, 128>();
    case 4: return p2g_occupancy<256, 256>();
    default: return p2g_occupancy<192, 128>();
  }
}

void configure_launches(DevPtrs &d) {
  const int a = p2g_shape_occupancy(d.launch.p2g_shape);
  const LaunchConfig &L = d.launch;
  const int gt = 128;
  const int g = g2p_occupancy();
  d.grid_p2g = d.num_sms * (L.p2g_ctas_per_sm > 0 ? std::min(L.p2g_ctas_per_sm, a) : a);
  d.grid_g2p = d.num_sms * (L.g2p_ctas_per_sm > 0 ? std::min(L.g2p_ctas_per_sm, g) : g);
  d.grid_sort = d.num_sms * (L.sort_ctas_per_sm > 0 ? L.sort_ctas_per_sm : 8);
  d.grid_stream = d.num_sms * (L.stream_ctas_per_sm > 0 ? L.stream_ctas_per_sm : 8);
  d.g2p_threads = gt;
  d.grid_persist = persistent_grid(d);
  configure_adjoint();
  configure_cloth();
}

template <int NT, int CH> void launch_p2g_shape(const DevPtrs &d, int cur, cudaStream_t s) {
  k_p2g<NT, CH><<<d.grid_p2g, NT, ColLayout<NT, CH>::smem, s>>>(d, d.pbuf[cur], d.ibuf[cur]);
}

void launch_p2g(const DevPtrs &d, int cur, cudaStream_t s) {
  if (d.transfer != MPM_TRANSFER_APIC) return launch_p2g_flip(d, cur, s);
  switch (d.launch.p2g_shape) {
    case 1: return launch_p2g_shape<192, 192>(d, cur, s);
    case 2: return launch_p2g_shape<192, 96>(d, cur, s);
    case 3: return launch_p2g_shape<256, 128>(d, cur, s);
    case 4: return launch_p2g_shape<256, 256>(d, cur, s);
    default: return launch_p2g_shape<192, 128>(d, cur, s);
  }
}

void launch_grid_gather(const DevPtrs &d, int mode, cudaStream_t s) {
  if (d.transfer != MPM_TRANSFER_APIC) return launch_grid_gather_flip(d, mode, s);
  switch (d.launch.gather_blocks) {
    case 2: k_grid_gather<2><<<d.grid_stream * 2, 128, 0, s>>>(d, mode); return;
    case 8: k_grid_gather<8><<<(d.grid_stream + 1) / 2, 512, 0, s>>>(d, mode); return;
    default: k_grid_gather<4><<<d.grid_stream, 256, 0, s>>>(d, mode); return;
  }
}

__global__ void k_apply_colliders(DevPtrs d, int id, int listed) {
  stage_apply_colliders(d, id, listed, blockIdx.x, gridDim.x);
}

void launch_apply_colliders(const DevPtrs &d, int id, cudaStream_t s) {
  k_apply_colliders<<<d.grid_stream, 256, 0, s>>>(d, id, 0);
}

void launch_apply_colliders_listed(const DevPtrs &d, cudaStream_t s) {
  k_apply_colliders<<<d.num_sms * 4, 256, 0, s>>>(d, -1, 1);
}

// StepZSBoundary on collider `id` (-1: every collider)
__global__ void k_step_colliders(DevPtrs d, int id, float dt) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  const int nc = d.prm->n_colliders;
  for (int k = 0; k < nc; ++k) {
    if (id >= 0 && k != id) continue;
    ColliderDev &c = d.colliders[k];
    for (int a = 0; a < 3; ++a) c.b[a] += c.db[a] * dt;
    c.s += c.ds * dt;
    collider_world_box(c);
  }
}

void launch_step_colliders(const DevPtrs &d, int id, float dt, cudaStream_t s) {
  k_step_colliders<<<1, 32, 0, s>>>(d, id, dt);
}

void launch_grid_update(const DevPtrs &d, int mode, cudaStream_t s) {
  if (d.transfer != MPM_TRANSFER_APIC) return launch_grid_update_flip(d, mode, s);
  k_grid_update<<<d.num_sms * 8, 256, 0, s>>>(d, mode);
}

void launch_g2p(const DevPtrs &d, int cur, int fuse_rm, int fuse_bin, cudaStream_t s) {
  if (d.transfer != MPM_TRANSFER_APIC) return launch_g2p_flip(d, cur, fuse_rm, fuse_bin, s);
  constexpr int NT = 128;
  const int grid = d.grid_g2p;
  constexpr int smem = g2p_smem_bytes<NT>();
  float *pi = d.pbuf[cur], *po = d.pbuf[1 - cur];
  int32_t *ii = d.ibuf[cur], *io = d.ibuf[1 - cur];
  if (fuse_rm && d.hencky) {
    if (fuse_bin)
      k_g2p<true, true, NT, true><<<grid, NT, smem, s>>>(d, pi, ii, po, io);
    else
      k_g2p<true, false, NT, true><<<grid, NT, smem, s>>>(d, pi, ii, po, io);
  } else if (fuse_rm && fuse_bin) {
    k_g2p<true, true, NT, false><<<grid, NT, smem, s>>>(d, pi, ii, po, io);
  } else if (fuse_rm) {
    k_g2p<true, false, NT, false><<<grid, NT, smem, s>>>(d, pi, ii, po, io);
  } else {
    k_g2p<false, false, NT, false><<<grid, NT, smem, s>>>(d, pi, ii, po, io);
  }
}

void launch_return_mapping(const DevPtrs &d, int cur, cudaStream_t s) {
  k_return_mapping<<<d.num_sms * 8, 256, 0, s>>>(d, d.pbuf[cur], d.ibuf[cur]);
}

void launch_stress(const DevPtrs &d, int cur, cudaStream_t s, long long b0, long long b1) {
  k_stress<<<d.num_sms * 8, 256, 0, s>>>(d, d.pbuf[cur], d.ibuf[cur], b0, b1);
}

}  // namespace zsmpm
