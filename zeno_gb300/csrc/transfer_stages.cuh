// The transfer stages as device functions of (CTA `cta` of `ncta`), shared
// by their own kernels (transfer.cu) and by the persistent substep kernel
// (persistent.cu): P2G (column scatter into per-block tiles), the grid
// gather with the grid update and walls, the level-set colliders and G2P
// with the return mapping, the stress and the next binning.
#pragma once

#include <cuda_runtime.h>

#include "binning.cuh"
#include "blocks.cuh"
#include "colliders.cuh"
#include "cp_async.cuh"
#include "mpm_math.cuh"
#include "tile_scatter.cuh"
#include "zsmpm_internal.cuh"

namespace zsmpm {
namespace {

// P2G of one particle block (ZSParticleToZSGrid::p2g_apic, Transfer.cu:849-889):
// per particle the affine matrix A = m C - dt Dinv S (S = vol tau from the
// previous G2P); the momentum of stencil node o is W (m v + A (o - f) dx) =
// W (b + a o) with a = dx A and b = m v - dx A f.
//
// Column scatter: the block's 16 cell columns (cx, cy) each belong to one
// 9-lane slot of a warp (6 warps, 3 slots each); lane (oi, oj) of the slot
// keeps the 6 nodes (cx + oi, cy + oj, 0..5) of its column in registers and
// adds, cell by cell (cz = 0..3, nodes cz..cz+2), every particle of the
// column in sorted order, over all chunks of the block.  At the end each
// lane writes its 6 node sums as a record, and the 216 tile nodes are the
// sums of the <= 9 records that cover them, added in a fixed (oi, oj) order:
// no atomics, no shared-memory read-modify-write, and a reproducible tile.
//
// Particles of a block are sorted by the z-major cell id (l2, l0, l1), so a
// chunk of the block holds cells of every column.  A CTA walks its blocks in
// chunks of kColChunk particles (thread j < kColChunk <-> particle j): each
// thread converts its own particle's raw channels into a scatter record, and
// as soon as the records are published it issues the cp.async copies of its
// particle of the next chunk into the raw buffer, so that those loads are in
// flight while the current chunk scatters; the permutation entries of the
// chunk after that load into registers.  A chunk is one cell layer of a
// block at the nominal 8 particles per cell (16 cells x 8), so the 16
// columns scatter equal shares before the chunk's barrier (a chunk of 192,
// one and a half layers, gave half the columns twice the work: 7 % slower).
constexpr int kColRaw = 23;            // x3 v3 C9 S6 m key
constexpr int kColRecs = 16 * 9 * 6;  // float4 records: (column, oi oj, z)
constexpr int kColMeta = 64;           // blocks per CTA whose metadata is staged
// per-block launch metadata staged in shared memory (32 bytes)
struct ColMeta {
  int start, cnt, dir, scene;
  int K[3];  // node index of the block's first node
  int pad;
};
// Shared-memory layout of k_p2g<NT, CH> (NT threads, chunks of CH <= NT
// particles): raw[23][CH] floats; spd[4][CH] float4 (b0 b1 a00 a10),
// (a01 a11 a02 a12), (b2 m a20 a21), (a22 wz0 wz1 wz2), laid out so that
// the pairs the scatter combines with packed FP32x2 instructions are the
// halves of one float4; sw[CH][6] wx0..2 wy0..2; the records; the chunk's
// cells; block metadata
template <int NT, int CH>
struct ColLayout {
  static_assert(CH <= NT && NT % 32 == 0 && NT >= 192, "a chunk is at most one particle per "
                "thread, and 16 columns need 6 warps of three 9-lane slots");
  static constexpr int off_spd = kColRaw * CH * 4;
  static constexpr int off_w = off_spd + 4 * CH * 16;
  static constexpr int off_rec = off_w + CH * 6 * 4;
  static constexpr int off_cell = off_rec + kColRecs * 16;
  static constexpr int off_meta = off_cell + ((CH + 15) & ~15);
  static constexpr int smem = off_meta + kColMeta * (int)sizeof(ColMeta);
  static_assert(off_spd % 16 == 0 && off_rec % 16 == 0 && off_meta % 16 == 0,
                "float4 / int4 regions must be 16-byte aligned");
};
// raw channel slots
constexpr int RC_X = 0, RC_V = 3, RC_C = 6, RC_S = 15, RC_M = 21, RC_KEY = 22;

template <int kColThreads, int kColChunk>
__device__ __forceinline__ void stage_p2g(const DevPtrs &d, const float *__restrict__ pin,
                                          const int32_t *__restrict__ iin,
                                          unsigned char *p2g_smem, int cta, int ncta) {
  using Lay = ColLayout<kColThreads, kColChunk>;
  if (ZSMPM_HALTED(d)) return;
  float(*raw)[kColChunk] = reinterpret_cast<float(*)[kColChunk]>(p2g_smem);
  float4(*spd)[kColChunk] = reinterpret_cast<float4(*)[kColChunk]>(p2g_smem + Lay::off_spd);
  float(*sw)[6] = reinterpret_cast<float(*)[6]>(p2g_smem + Lay::off_w);
  float4 *rec = reinterpret_cast<float4 *>(p2g_smem + Lay::off_rec);
  unsigned char *scell = p2g_smem + Lay::off_cell;
  ColMeta *meta = reinterpret_cast<ColMeta *>(p2g_smem + Lay::off_meta);
  const SimParams &P = *d.prm;
  const long long n = P.n;
  const float dt = P.dt;
  const int nb = d.cnt->n_buckets;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // lane constants: slot, column, stencil offsets (oi, oj)
  const int slot = lane / 9, oij = lane % 9;
  const int col = 3 * warp + slot;
  const bool has_col = lane < 27 && col < 16;
  const float foi = (float)(oij / 3), foj = (float)(oij % 3);
  const int wxo = oij / 3, wyo = 3 + oij % 3;

  const int nblk = nb > (int)cta ? (nb - 1 - (int)cta) / (int)ncta + 1 : 0;
  auto load_meta = [&](int k) {
    const int b = cta + k * ncta;
    const int dir = d.bk_dir[b], start = d.bk_start[b];
    const int cnt = (int)max(0ll, min((long long)d.bk_count[b], n - start));
    ColMeta m;
    m.start = start;
    m.cnt = cnt;
    m.dir = dir;
    m.scene = scene_of_dir(d, dir);
    const SceneParams &S = d.scn[m.scene];
    bucket_origin(S, dir - S.dir_off, m.K);
    m.pad = 0;
    return m;
  };
  for (int k = tid; k < min(nblk, kColMeta); k += kColThreads) meta[k] = load_meta(k);
  __syncthreads();
  auto meta_of = [&](int k) { return k < kColMeta ? meta[k] : load_meta(k); };

  struct Item {
    int k, c0;
  };
  auto skip_empty = [&](Item it) {
    while (it.k < nblk && meta_of(it.k).cnt == 0) ++it.k;
    return it;
  };
  auto advance = [&](Item it) {
    if (it.k >= nblk) return it;
    it.c0 += kColChunk;
    if (it.c0 >= meta_of(it.k).cnt) {
      ++it.k;
      it.c0 = 0;
      it = skip_empty(it);
    }
    return it;
  };
  auto perm_of = [&](const Item &it) {
    if (it.k >= nblk) return -1;
    const ColMeta m = meta_of(it.k);
    return tid < kColChunk && tid < m.cnt - it.c0 ? d.perm[m.start + it.c0 + tid] : -1;
  };
  auto issue = [&](int p) {
    if (p < 0) return;
    float(*q)[kColChunk] = raw;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      cp_async4(&q[RC_X + c][tid], &pin[pidx((CH_X + c), p)]);
      cp_async4(&q[RC_V + c][tid], &pin[pidx((CH_V + c), p)]);
    }
#pragma unroll
    for (int c = 0; c < 9; ++c) cp_async4(&q[RC_C + c][tid], &pin[pidx((CH_C + c), p)]);
#pragma unroll
    for (int c = 0; c < 6; ++c) cp_async4(&q[RC_S + c][tid], &pin[pidx((CH_S + c), p)]);
    cp_async4(&q[RC_M][tid], &pin[pidx(CH_M, p)]);
    cp_async4(&q[RC_KEY][tid], &d.pkey[p]);
  };

  // node sums of the lane's 6 column nodes: (mom0, mom1) and (mom2, mass)
  float2 accP[6], accQ[6];
#pragma unroll
  for (int z = 0; z < 6; ++z) accP[z] = accQ[z] = make_float2(0.f, 0.f);
  const float2 oi2 = make_float2(foi, foi), oj2 = make_float2(foj, foj);
  Item cur = skip_empty(Item{0, 0});
  Item nxt = advance(cur);
  Item nn = advance(nxt);
  int p_nxt = perm_of(nxt);
  issue(perm_of(cur));
  cp_async_commit();
  while (cur.k < nblk) {
    const int p_nn = perm_of(nn);
    const ColMeta m = meta_of(cur.k);
    const SceneParams &S = d.scn[m.scene];
    const float dx = S.dx, inv_dx = S.inv_dx, Dinv = S.Dinv;
    const int K[3] = {m.K[0], m.K[1], m.K[2]};
    const int nc = min(kColChunk, m.cnt - cur.c0);
    cp_async_wait<0>();  // this thread's particle of chunk `cur` has landed
    // convert particle tid of the chunk into its scatter record
    if (tid < nc) {
      const float(*q)[kColChunk] = raw;
      float x[3], v[3], C[9], Sv[6];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        x[k] = q[RC_X + k][tid];
        v[k] = q[RC_V + k][tid];
      }
#pragma unroll
      for (int k = 0; k < 9; ++k) C[k] = q[RC_C + k][tid];
#pragma unroll
      for (int k = 0; k < 6; ++k) Sv[k] = q[RC_S + k][tid];
      float mass = q[RC_M][tid];
      const int cell = __float_as_int(q[RC_KEY][tid]) & 63;
      // A = m C - dt Dinv vol tau (contrib of Transfer.cu:868 is -dt Dinv vol P F^T)
      const float kk = -dt * Dinv;
      float A[9];
      A[0] = mass * C[0] + kk * Sv[0];
      A[1] = mass * C[1] + kk * Sv[3];
      A[2] = mass * C[2] + kk * Sv[4];
      A[3] = mass * C[3] + kk * Sv[3];
      A[4] = mass * C[4] + kk * Sv[1];
      A[5] = mass * C[5] + kk * Sv[5];
      A[6] = mass * C[6] + kk * Sv[4];
      A[7] = mass * C[7] + kk * Sv[5];
      A[8] = mass * C[8] + kk * Sv[2];
      const Stencil1 s0 = stencil1(x[0], inv_dx), s1 = stencil1(x[1], inv_dx),
                     s2 = stencil1(x[2], inv_dx);
      const int l0 = s0.base - K[0], l1 = s1.base - K[1], l2 = s2.base - K[2];
      if ((unsigned)l0 > 3u || (unsigned)l1 > 3u || (unsigned)l2 > 3u ||
          sort_cell(l0, l1, l2) != cell) {
        atomicOr(&d.cnt->status, ST_STENCIL);
        mass = 0.0f;
#pragma unroll
        for (int k = 0; k < 9; ++k) A[k] = 0.0f;
        v[0] = v[1] = v[2] = 0.0f;
      }
      const float fdx0 = s0.f * dx, fdx1 = s1.f * dx, fdx2 = s2.f * dx;
      const float b0 = mass * v[0] - (A[0] * fdx0 + A[1] * fdx1 + A[2] * fdx2);
      const float b1 = mass * v[1] - (A[3] * fdx0 + A[4] * fdx1 + A[5] * fdx2);
      const float b2 = mass * v[2] - (A[6] * fdx0 + A[7] * fdx1 + A[8] * fdx2);
      // a_kc = dx A[k][c]: momentum component k, axis c
      spd[0][tid] = make_float4(b0, b1, dx * A[0], dx * A[3]);
      spd[1][tid] = make_float4(dx * A[1], dx * A[4], dx * A[2], dx * A[5]);
      spd[2][tid] = make_float4(b2, mass, dx * A[6], dx * A[7]);
      spd[3][tid] = make_float4(dx * A[8], s2.w[0], s2.w[1], s2.w[2]);
      sw[tid][0] = s0.w[0];
      sw[tid][1] = s0.w[1];
      sw[tid][2] = s0.w[2];
      sw[tid][3] = s1.w[0];
      sw[tid][4] = s1.w[1];
      sw[tid][5] = s1.w[2];
      scell[tid] = (unsigned char)cell;
    }
    __syncthreads();  // records published, raw free
    issue(p_nxt);     // next chunk's particle of this thread
    cp_async_commit();
    // the slot's 8 range bounds: lane k < 8 finds the first chunk index with
    // cell >= cz * 16 + col + (k & 1) for cz = k >> 1 (cells sorted)
    int bnd;
    {
      const int k = oij < 8 ? oij : 0;
      const int c = (k >> 1) * 16 + col + (k & 1);
      int lo = 0, hi = nc;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (scell[mid] < c)
          lo = mid + 1;
        else
          hi = mid;
      }
      bnd = lo;
    }
    int qb[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) qb[k] = __shfl_sync(0xffffffffu, bnd, (slot * 9 + k) & 31);
    if (has_col) {
#pragma unroll
      for (int cz = 0; cz < 4; ++cz) {
        const int q1 = qb[2 * cz + 1];
        for (int q = qb[2 * cz]; q < q1; ++q) {
          const float4 u0 = spd[0][q], u1 = spd[1][q], u2 = spd[2][q], u3 = spd[3][q];
          const float wij = sw[q][wxo] * sw[q][wyo];
          // node values b + a (oi, oj, oz): (k = 0, 1) as one pair, k = 2 and
          // the mass as the other; the z steps are r = a_k2
          float2 s01 = __ffma2_rn(make_float2(u1.x, u1.y), oj2,
                                  __ffma2_rn(make_float2(u0.z, u0.w), oi2,
                                             make_float2(u0.x, u0.y)));
          float2 s2m = make_float2(fmaf(u2.w, foj, fmaf(u2.z, foi, u2.x)), u2.y);
          const float2 r01 = make_float2(u1.z, u1.w);
          const float r2 = u3.x;
          const float wz[3] = {u3.y, u3.z, u3.w};
#pragma unroll
          for (int oz = 0; oz < 3; ++oz) {
            const float W = wij * wz[oz];
            const float2 W2 = make_float2(W, W);
            accP[cz + oz] = __ffma2_rn(W2, s01, accP[cz + oz]);
            accQ[cz + oz] = __ffma2_rn(W2, s2m, accQ[cz + oz]);
            if (oz < 2) {
              s01 = __fadd2_rn(s01, r01);
              s2m.x += r2;
            }
          }
        }
      }
    }
    if (nxt.k != cur.k) {  // last chunk of the block: records, then the tile
      if (has_col) {
#pragma unroll
        for (int z = 0; z < 6; ++z)
          rec[(col * 9 + oij) * 6 + z] = make_float4(accQ[z].y, accP[z].x, accP[z].y, accQ[z].x);
      }
#pragma unroll
      for (int z = 0; z < 6; ++z) accP[z] = accQ[z] = make_float2(0.f, 0.f);
      __syncthreads();
      float4 *tile = d.ptile + (long long)(cta + cur.k * ncta) * kTileNodes;
      for (int nd = tid; nd < kTileNodes; nd += kColThreads) {
        const int I = nd / 36, J = (nd / 6) % 6, Kz = nd % 6;
        float4 g = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int oi = 0; oi < 3; ++oi) {
          const int cx = I - oi;
          if (cx < 0 || cx > 3) continue;
#pragma unroll
          for (int oj = 0; oj < 3; ++oj) {
            const int cy = J - oj;
            if (cy < 0 || cy > 3) continue;
            const float4 r = rec[((cx * 4 + cy) * 9 + oi * 3 + oj) * 6 + Kz];
            g.x += r.x;
            g.y += r.y;
            g.z += r.z;
            g.w += r.w;
          }
        }
        tile[nd] = g;
      }
    }
    __syncthreads();  // spd, sw, scell and records free
    cur = nxt;
    nxt = nn;
    nn = advance(nn);
    p_nxt = p_nn;
  }
  cp_async_wait<0>();
}

// Grid node sums from the P2G tiles: node (l0, l1, l2) of grid block G lies
// in the tile of particle block G - o (o in {0, 1}^3, in blocks) at tile
// coordinate l + 4 o when that is < 6.  The <= 8 tiles are added in the fixed
// order o = (0,0,0), (0,0,1), ..., so the sums are reproducible.  mode bit 1
// applies UpdateZSGrid and bit 2 ApplyBoundaryOnZSGrid to the sum.
__device__ __forceinline__ void update_node(const DevPtrs &d, int scene, const SceneParams &S,
                                            float dt, int mode, int ldir, int cell, float4 &g,
                                            float &vmax);
__device__ __forceinline__ void update_node_at(const DevPtrs &d, int scene, const SceneParams &S,
                                               float dt, int mode, const int (&I)[3], float4 &g,
                                               float &vmax);

// One 64-thread group per grid block, kGatherBlocks (2, 4 or 8) blocks per
// CTA, a launch knob: the group fetches its
// block's scene, node origin and the (particle block) tiles of the 8 blocks
// whose tiles can cover it once into shared memory; each thread then sums
// its node's <= 8 tile entries and applies the update.
template <int kGatherBlocks>
__device__ __forceinline__ void stage_grid_gather(const DevPtrs &d, int mode, int cta, int ncta) {
  if (ZSMPM_HALTED(d)) return;
  __shared__ int sbk[kGatherBlocks][8];
  __shared__ int sorg[kGatherBlocks][4];  // node origin, scene
  const SimParams &P = *d.prm;
  const int ng = min(d.cnt->n_gblocks, d.cap_gblocks);
  const int grp = threadIdx.x >> 6, cell = threadIdx.x & 63;
  const int l0 = cell >> 4, l1 = (cell >> 2) & 3, l2 = cell & 3;
  float vmax = 0.0f;
  for (int g0 = cta * kGatherBlocks; g0 < ng; g0 += ncta * kGatherBlocks) {
    const int gb = g0 + grp;
    if (cell < 8 && gb < ng) {
      const int gdir = d.gb_dir[gb];
      const int sc = scene_of_dir(d, gdir);
      const SceneParams &S = d.scn[sc];
      const int dy = S.block_dims[1], dz = S.block_dims[2];
      const int ldir = gdir - S.dir_off;
      const int c0 = ldir / (dz * dy), c1 = (ldir / dz) % dy, c2 = ldir % dz;
      const int o0 = cell >> 2, o1 = (cell >> 1) & 1, o2 = cell & 1;
      int bk = -1;
      if (!((o0 && c0 < 1) || (o1 && c1 < 1) || (o2 && c2 < 1)))
        bk = d.dir_bk[gdir - (o0 * dy + o1) * dz - o2];
      sbk[grp][cell] = bk;
      if (cell == 0) {
        const int I0[3] = {(c0 + S.block_lo[0]) * 4, (c1 + S.block_lo[1]) * 4,
                           (c2 + S.block_lo[2]) * 4};
        sorg[grp][0] = I0[0];
        sorg[grp][1] = I0[1];
        sorg[grp][2] = I0[2];
        sorg[grp][3] = sc;
        if (mode & 2) note_near_block(d, P.n_colliders, sc, I0, S.dx, gb);
      }
    }
    __syncthreads();
    if (gb < ng) {
      float4 g = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int o = 0; o < 8; ++o) {
        const int o0 = o >> 2, o1 = (o >> 1) & 1, o2 = o & 1;
        if ((o0 && l0 >= 2) || (o1 && l1 >= 2) || (o2 && l2 >= 2)) continue;
        const int bk = sbk[grp][o];
        if (bk < 0) continue;
        const float4 t = d.ptile[(long long)bk * kTileNodes +
                                 ((l0 + 4 * o0) * 6 + (l1 + 4 * o1)) * 6 + (l2 + 4 * o2)];
        g.x += t.x;
        g.y += t.y;
        g.z += t.z;
        g.w += t.w;
      }
      if (g.x != 0.0f) {
        const int I[3] = {sorg[grp][0] + l0, sorg[grp][1] + l1, sorg[grp][2] + l2};
        update_node_at(d, sorg[grp][3], d.scn[sorg[grp][3]], P.dt, mode, I, g, vmax);
      }
      d.grid[(long long)gb * 64 + cell] = g;
    }
    __syncthreads();  // shared entries reused
  }
  if (mode & 1) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
    if ((threadIdx.x & 31) == 0 && vmax > 0.0f)
      atomicMax(&d.cnt->max_vel_sqr_bits, __float_as_uint(vmax));
  }
}

// UpdateZSGrid (MPMPipeline.cu:852-877): v = mv / m + g dt where m != 0,
// running max of |v|^2; then ApplyBoundaryOnZSGrid (Boundary.cu:105-116) with
// the analytic box walls (apply_walls).
__device__ __forceinline__ void update_node(const DevPtrs &d, int scene, const SceneParams &S,
                                            float dt, int mode, int ldir, int cell, float4 &g,
                                            float &vmax) {
  const int dz = S.block_dims[2], dy = S.block_dims[1];
  const int I[3] = {((ldir / (dz * dy)) + S.block_lo[0]) * 4 + (cell >> 4),
                    (((ldir / dz) % dy) + S.block_lo[1]) * 4 + ((cell >> 2) & 3),
                    ((ldir % dz) + S.block_lo[2]) * 4 + (cell & 3)};
  update_node_at(d, scene, S, dt, mode, I, g, vmax);
}

// the same at the node's global index I
__device__ __forceinline__ void update_node_at(const DevPtrs &d, int scene, const SceneParams &S,
                                               float dt, int mode, const int (&I)[3], float4 &g,
                                               float &vmax) {
  if (mode & 1) {
    const float r = 1.0f / g.x;
    g.y = g.y * r + S.gravity[0] * dt;
    g.z = g.z * r + S.gravity[1] * dt;
    g.w = g.w * r + S.gravity[2] * dt;
    vmax = fmaxf(vmax, g.y * g.y + g.z * g.z + g.w * g.w);
  }
  if ((mode & 2) && S.bc_type != MPM_BC_NONE) {
    float vel[3] = {g.y, g.z, g.w};
    apply_walls(S, I, vel);
    g.y = vel[0];
    g.z = vel[1];
    g.w = vel[2];
  }
}

constexpr int kG2PCh = 19;     // staged particle channels
constexpr int kG2PMeta = 64;   // blocks per CTA whose metadata is staged
// staged channel slots
constexpr int GC_X = 0, GC_F = 3, GC_J = 12, GC_M = 13, GC_VOL = 14, GC_MU = 15, GC_LAM = 16,
              GC_MAT = 17, GC_ID = 18;

template <int NT>
constexpr int g2p_smem_bytes() {
  return 2 * kNodes * 16 + 2 * kG2PCh * NT * 4 + kG2PMeta * (int)sizeof(G2PMeta);
}


// G2P (ZSGridToZSParticle, Transfer.cu:1139-1173) with the return mapping and
// the stress of the new F fused in.  A CTA walks the particle blocks it owns
// in chunks of NT particles (thread j <-> particle j of the chunk) through a
// two-stage pipeline: while chunk i computes, the node velocities of chunk
// i+1's block (216 float4) and chunk i+1's particle channels are in flight
// as cp.async copies into the other half of double-buffered shared memory,
// and the permutation entries of chunk i+2 are loading into registers.
// kHencky: the von Mises / Cam-Clay return mappings are compiled in (only for
// contexts whose materials use them: their extra registers would otherwise
// make every G2P spill)
template <bool kFuseRM, bool kFuseBin, int NT, bool kHencky>
__device__ __forceinline__ void stage_g2p(const DevPtrs &d, const float *__restrict__ pin,
                                          const int32_t *__restrict__ iin,
                                          float *__restrict__ pout, int32_t *__restrict__ iout,
                                          unsigned char *g2p_smem, int cta, int ncta) {
  if (ZSMPM_HALTED(d)) return;
  float4(*gsm)[kNodes] = reinterpret_cast<float4(*)[kNodes]>(g2p_smem);
  float(*psm)[kG2PCh][NT] =
      reinterpret_cast<float(*)[kG2PCh][NT]>(g2p_smem + 2 * kNodes * 16);
  G2PMeta *meta =
      reinterpret_cast<G2PMeta *>(g2p_smem + 2 * kNodes * 16 + 2 * kG2PCh * NT * 4);
  const SimParams &P = *d.prm;
  const long long n = P.n;
  const float dt = P.dt;
  const int nb = d.cnt->n_buckets;
  const bool lame = P.has_lame != 0;
  const int tid = threadIdx.x;
  const int nblk = nb > (int)cta ? (nb - 1 - (int)cta) / (int)ncta + 1 : 0;
  for (int k = tid; k < min(nblk, kG2PMeta); k += NT)
    meta[k] = g2p_load_meta(d, n, cta + k * ncta);
  __syncthreads();

  // chunk iterator over (k = this CTA's k-th block, c0 = first particle);
  // `ord` counts blocks, selecting the grid buffer
  struct Item {
    int k, c0, ord;
  };
  auto cnt_of = [&](int k) {
    return k < kG2PMeta ? meta[k].cnt : g2p_load_meta(d, n, cta + k * ncta).cnt;
  };
  auto meta_of = [&](int k) {
    return k < kG2PMeta ? meta[k] : g2p_load_meta(d, n, cta + k * ncta);
  };
  auto skip_empty = [&](Item it) {
    while (it.k < nblk && cnt_of(it.k) == 0) ++it.k;
    return it;
  };
  auto advance = [&](Item it) {
    if (it.k >= nblk) return it;
    it.c0 += NT;
    if (it.c0 >= cnt_of(it.k)) {
      ++it.k;
      it.c0 = 0;
      ++it.ord;
      it = skip_empty(it);
    }
    return it;
  };
  auto perm_of = [&](const Item &it) {
    if (it.k >= nblk) return -1;
    const G2PMeta m = meta_of(it.k);
    return tid < m.cnt - it.c0 ? d.perm[m.start + it.c0 + tid] : -1;
  };
  // issue the copies of chunk `it` into particle buffer `pb`
  auto issue = [&](const Item &it, int pb, int p) {
    if (it.c0 == 0) {
      float4 *g = gsm[it.ord & 1];
      const bool staged = it.k < kG2PMeta;
      int dir = 0, scene = 0;
      if (!staged) {
        dir = d.bk_dir[cta + it.k * ncta];
        scene = scene_of_dir(d, dir);
      }
      for (int nd = tid; nd < kNodes; nd += NT) {
        const int lx = nd / 36, ly = (nd / 6) % 6, lz = nd % 6;
        const int t = ((lx >> 2) << 2) | ((ly >> 2) << 1) | (lz >> 2);
        const int gb = staged ? meta[it.k].gb[t] : neighbour_gb(d, d.scn[scene], dir, t);
        const int cell = ((lx & 3) << 4) | ((ly & 3) << 2) | (lz & 3);
        if (gb >= 0)
          cp_async16(&g[nd], &d.grid[(long long)gb * 64 + cell]);
        else
          g[nd] = make_float4(0.f, 0.f, 0.f, 0.f);
      }
    }
    if (p >= 0) {
      float(*q)[NT] = psm[pb];
#pragma unroll
      for (int c = 0; c < 3; ++c) cp_async4(&q[GC_X + c][tid], &pin[pidx((CH_X + c), p)]);
#pragma unroll
      for (int c = 0; c < 9; ++c) cp_async4(&q[GC_F + c][tid], &pin[pidx((CH_F + c), p)]);
      cp_async4(&q[GC_J][tid], &pin[pidx(CH_J, p)]);
      cp_async4(&q[GC_M][tid], &pin[pidx(CH_M, p)]);
      cp_async4(&q[GC_VOL][tid], &pin[pidx(CH_VOL, p)]);
      if (lame) {
        cp_async4(&q[GC_MU][tid], &pin[pidx(CH_MU, p)]);
        cp_async4(&q[GC_LAM][tid], &pin[pidx(CH_LAM, p)]);
      }
      cp_async4(&q[GC_MAT][tid], &iin[iidx(IC_MAT, p)]);
      cp_async4(&q[GC_ID][tid], &iin[iidx(IC_ID, p)]);
    }
  };

  Item cur = skip_empty(Item{0, 0, 0});
  Item nxt = advance(cur);
  Item nn = advance(nxt);
  int p_cur = perm_of(cur), p_nxt = perm_of(nxt);
  if (cur.k < nblk) issue(cur, 0, p_cur);
  cp_async_commit();
  int buf = 0;
  while (cur.k < nblk) {
    const int p_nn = perm_of(nn);  // consumed two iterations from now
    if (nxt.k < nblk) issue(nxt, buf ^ 1, p_nxt);
    cp_async_commit();
    cp_async_wait<1>();  // chunk `cur` has landed
    __syncthreads();

    const G2PMeta m = meta_of(cur.k);
    const SceneParams &S = d.scn[m.scene];
    const float dx = S.dx, inv_dx = S.inv_dx, Dinv = S.Dinv;
    const int K[3] = {m.K[0], m.K[1], m.K[2]};
    const float4 *gv = gsm[cur.ord & 1];
    const float(*q)[NT] = psm[buf];
    const bool live = tid < m.cnt - cur.c0;
    const unsigned mask = __ballot_sync(0xffffffffu, live);
    if (live) {
      const int s = m.start + cur.c0 + tid;
      const int p = p_cur;
      const int mid = min(max(__float_as_int(q[GC_MAT][tid]), 0), kMaxMaterials - 1);
      const MatParams mp = d.mats[mid];
      float x[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) x[k] = q[GC_X + k][tid];
      const Stencil1 s0 = stencil1(x[0], inv_dx), s1 = stencil1(x[1], inv_dx),
                     s2 = stencil1(x[2], inv_dx);
      const int l0 = s0.base - K[0], l1 = s1.base - K[1], l2 = s2.base - K[2];
      float vel[3] = {0.f, 0.f, 0.f}, Cn[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      if ((unsigned)l0 > 3u || (unsigned)l1 > 3u || (unsigned)l2 > 3u) {
        atomicOr(&d.cnt->status, ST_STENCIL);
      } else {
        // v = sum W g and C = Dinv sum W g (x_i - x_p)^T over the 27 nodes,
        // summed k-innermost so each weight product is formed once per level:
        // with W = w_i w_j w_k and x_i - x_p = (xi, xj, xk),
        //   t = sum_k w_k g, tk = sum_k w_k xk g; S = sum_j w_j t,
        //   Sj = sum_j w_j xj t, Sk = sum_j w_j tk; then over i.
        float xi[3], xj[3], xk[3], wxk[3], wyj[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          xi[c] = ((float)c - s0.f) * dx;
          xj[c] = ((float)c - s1.f) * dx;
          xk[c] = ((float)c - s2.f) * dx;
          wxk[c] = s2.w[c] * xk[c];
          wyj[c] = s1.w[c] * xj[c];
        }
        float cx[3] = {0.f, 0.f, 0.f}, cy[3] = {0.f, 0.f, 0.f}, cz[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          float Sa[3] = {0.f, 0.f, 0.f}, Sj[3] = {0.f, 0.f, 0.f}, Sk[3] = {0.f, 0.f, 0.f};
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            const int row = ((l0 + i) * 6 + (l1 + j)) * 6 + l2;
            float t[3] = {0.f, 0.f, 0.f}, tk[3] = {0.f, 0.f, 0.f};
#pragma unroll
            for (int kk = 0; kk < 3; ++kk) {
              const float4 g4 = gv[row + kk];
              const float g[3] = {g4.y, g4.z, g4.w};
#pragma unroll
              for (int a = 0; a < 3; ++a) {
                t[a] = fmaf(s2.w[kk], g[a], t[a]);
                tk[a] = fmaf(wxk[kk], g[a], tk[a]);
              }
            }
#pragma unroll
            for (int a = 0; a < 3; ++a) {
              Sa[a] = fmaf(s1.w[j], t[a], Sa[a]);
              Sj[a] = fmaf(wyj[j], t[a], Sj[a]);
              Sk[a] = fmaf(s1.w[j], tk[a], Sk[a]);
            }
          }
          const float wxi = s0.w[i] * xi[i];
#pragma unroll
          for (int a = 0; a < 3; ++a) {
            vel[a] = fmaf(s0.w[i], Sa[a], vel[a]);
            cx[a] = fmaf(wxi, Sa[a], cx[a]);
            cy[a] = fmaf(s0.w[i], Sj[a], cy[a]);
            cz[a] = fmaf(s0.w[i], Sk[a], cz[a]);
          }
        }
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          Cn[a * 3 + 0] = cx[a];
          Cn[a * 3 + 1] = cy[a];
          Cn[a * 3 + 2] = cz[a];
        }
      }
#pragma unroll
      for (int k = 0; k < 9; ++k) Cn[k] *= Dinv;
#pragma unroll
      for (int k = 0; k < 3; ++k) x[k] += vel[k] * dt;
      float F[9], J;
      Sym3 tau;
      bool ok_state = true;
      float mu = mp.mu, lam = mp.lam;
      if (lame) {
        mu = q[GC_MU][tid];
        lam = q[GC_LAM][tid];
      }
      if (mp.type == MPM_EOS) {
        J = q[GC_J][tid] * (1.0f + dt * (Cn[0] + Cn[4] + Cn[8]));
        const float c = cbrtf(J);
#pragma unroll
        for (int k = 0; k < 9; ++k) F[k] = (k % 4 == 0) ? c : 0.0f;
        ok_state = kirchhoff(MPM_EOS, mu, lam, mp.bulk, mp.gamma, F, J, tau);
      } else {
        float Fo[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) Fo[k] = q[GC_F + k][tid];
        // F <- (I + dt C) F
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int c = 0; c < 3; ++c)
            F[r * 3 + c] = Fo[r * 3 + c] + dt * (Cn[r * 3 + 0] * Fo[c] + Cn[r * 3 + 1] * Fo[3 + c] +
                                                 Cn[r * 3 + 2] * Fo[6 + c]);
        float jch = q[GC_J][tid];  // log(Jp) of a Cam-Clay particle
        if (kFuseRM && mp.plastic == MPM_PLASTIC_NADP)
          ok_state = project_dp(mu, lam, mp.alpha, F, tau) >= 0;
        else if (kHencky && kFuseRM && mp.plastic != MPM_PLASTIC_NONE)
          ok_state = project_hencky(mp, mu, lam, F, jch, tau) >= 0;
        else
          ok_state = kirchhoff(mp.type, mu, lam, mp.bulk, mp.gamma, F, 1.0f, tau);
        J = mp.plastic == MPM_PLASTIC_NACC ? jch : det3(F);
      }
      if (!ok_state) atomicOr(&d.cnt->status, ST_NAN);
      const float vol = q[GC_VOL][tid];
      bool finite = isfinite(x[0]) && isfinite(x[1]) && isfinite(x[2]) && isfinite(J);
#pragma unroll
      for (int k = 0; k < 9; ++k) finite = finite && isfinite(F[k]);
      if (!finite) atomicOr(&d.cnt->status, ST_NAN);
      // next buffer: the particle's sorted position
      const int so = s;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        pout[pidx((CH_X + k), so)] = x[k];
        pout[pidx((CH_V + k), so)] = vel[k];
      }
#pragma unroll
      for (int k = 0; k < 9; ++k) {
        pout[pidx((CH_C + k), so)] = Cn[k];
        pout[pidx((CH_F + k), so)] = F[k];
      }
      pout[pidx(CH_J, so)] = J;
      pout[pidx(CH_M, so)] = q[GC_M][tid];
      pout[pidx(CH_VOL, so)] = vol;
      pout[pidx((CH_S + 0), so)] = vol * tau.xx;
      pout[pidx((CH_S + 1), so)] = vol * tau.yy;
      pout[pidx((CH_S + 2), so)] = vol * tau.zz;
      pout[pidx((CH_S + 3), so)] = vol * tau.xy;
      pout[pidx((CH_S + 4), so)] = vol * tau.xz;
      pout[pidx((CH_S + 5), so)] = vol * tau.yz;
      if (lame) {
        pout[pidx(CH_MU, so)] = mu;
        pout[pidx(CH_LAM, so)] = lam;
      }
      iout[iidx(IC_MAT, so)] = mid;
      iout[iidx(IC_ID, so)] = __float_as_int(q[GC_ID][tid]);
      if (kFuseBin) {
        // key of the new position for the next partition (storage slot so)
        const int key = bin_key(S, x[0], x[1], x[2], &d.cnt->status);
        d.pkey[so] = key;
        bin_count(d, S, key, mask);
      }
    }
    __syncthreads();  // buffers of `cur` free for the chunk after `nxt`
    cur = nxt;
    nxt = nn;
    nn = advance(nn);
    p_cur = p_nxt;
    p_nxt = p_nn;
    buf ^= 1;
  }
  cp_async_wait<0>();
}

// ApplyBoundaryOnZSGrid with level sets: collider `id` (-1: every collider,
// in id order) on the active nodes, after the box walls; its own pass,
// launched only when colliders exist.  One warp per grid block, two nodes
// per lane.  Listed form (the fused substep): the blocks the gather noted
// as near a collider.  Full form (the stage path, whose colliders may move
// between gather and boundary): every block, skipped by the warp unless its
// node box meets the world box of a collider.
__device__ __forceinline__ void stage_apply_colliders(const DevPtrs &d, int id, int listed,
                                                      int cta, int ncta) {
  if (ZSMPM_HALTED(d)) return;
  const int nc = d.prm->n_colliders;
  const int k0 = id < 0 ? 0 : id, k1 = id < 0 ? nc : min(id + 1, nc);
  const int ng = listed ? min(d.cnt->n_near, d.cap_gblocks) : min(d.cnt->n_gblocks, d.cap_gblocks);
  const int lane = threadIdx.x & 31;
  const int nw = ncta * (blockDim.x >> 5);
  for (int w = cta * (blockDim.x >> 5) + (threadIdx.x >> 5); w < ng; w += nw) {
    const int gb = listed ? d.near_gb[w] : w;
    const int gdir = d.gb_dir[gb];
    const int sc = scene_of_dir(d, gdir);
    const SceneParams &S = d.scn[sc];
    const int dz = S.block_dims[2], dy = S.block_dims[1];
    const int ldir = gdir - S.dir_off;
    const int I0[3] = {((ldir / (dz * dy)) + S.block_lo[0]) * 4, (((ldir / dz) % dy) + S.block_lo[1]) * 4,
                       ((ldir % dz) + S.block_lo[2]) * 4};
    if (!listed && !block_near_colliders(d, k0, k1, sc, I0, S.dx)) continue;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int cell = lane + 32 * h;
      const long long idx = (long long)gb * 64 + cell;
      if (d.grid[idx].x == 0.0f) continue;
      const float p[3] = {(float)(I0[0] + (cell >> 4)) * S.dx, (float)(I0[1] + ((cell >> 2) & 3)) * S.dx,
                          (float)(I0[2] + (cell & 3)) * S.dx};
      if (d.transfer == MPM_TRANSFER_APIC) {
        float4 g = d.grid[idx];
        float vel[3] = {g.y, g.z, g.w};
        apply_colliders(d, k0, k1, sc, p, vel);
        g.y = vel[0];
        g.z = vel[1];
        g.w = vel[2];
        d.grid[idx] = g;
      } else {  // the FLIP grids resolve collisions on vstar (Boundary.cu:90-101)
        float4 h4 = d.grid2[idx];
        float vel[3] = {h4.x, h4.y, h4.z};
        apply_colliders(d, k0, k1, sc, p, vel);
        d.grid2[idx] = make_float4(vel[0], vel[1], vel[2], h4.w);
      }
    }
  }
}

}  // namespace
}  // namespace zsmpm
