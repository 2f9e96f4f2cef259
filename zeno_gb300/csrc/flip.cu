// The FLIP and affine-FLIP transfers (MakeZSGrid transfer = "flip" |
// "aflip"): P2G, grid gather + update + walls, and G2P with the return
// mapping, on the same partition, tiles and launch shapes as the APIC path.
//
// The grid carries a second velocity, vstar (Generation.cu:1495-1500):
//  * P2G (Transfer.cu:891-984): the mass and the transferred momentum go to
//    (m, mv) as in APIC (FLIP: W m v_p; AFLIP: W m (v_p + C (x_i - x_p))),
//    the grid force impulse to vstar (FLIP: W contrib grad W with contrib =
//    -dt vol P F^T -- the reference weights this term by W as well; AFLIP:
//    W contrib (x_i - x_p) with contrib = -dt Dinv vol P F^T);
//  * grid update (MPMPipeline.cu:878-897): v = mv / m, vstar = vstar / m + v
//    + g dt, MaxVelSqr of vstar; walls and colliders act on vstar
//    (Boundary.cu:90-101);
//  * G2P (Transfer.cu:1174-1257): vel = sum W v_i, vs = sum W vstar_i,
//    v_p <- vs + 0.99 (v_p - vel); AFLIP C = Dinv sum W vstar_i (x_i - x_p)^T,
//    x += dt (vs + beta 0.99 (v_p - vel)); FLIP x += dt vs, F <- (I + dt
//    sum vstar_i grad W_i^T) F and C is carried unchanged.
// grad W is the derivative of the weight with respect to the particle
// position (the quadratic B-spline's w_o'(f) times the other two weights, /dx).
#include <cuda_runtime.h>

#include <algorithm>

#include "binning.cuh"
#include "blocks.cuh"
#include "cloth_grid.cuh"
#include "colliders.cuh"
#include "cp_async.cuh"
#include "mpm_math.cuh"
#include "tile_scatter.cuh"
#include "zsmpm_internal.cuh"

namespace zsmpm {
namespace {

// ---------------------------------------------------------------- P2G ----
//
// The column scatter of the APIC P2G with seven node channels: each of the
// block's 16 cell columns belongs to a 9-lane slot, lane (oi, oj) keeps the
// 6 z-nodes of its column (m, mv, vstar) in registers over the block's
// particles in sorted order, and the 216 tile nodes are the fixed-order sums
// of the <= 9 lane records that cover them (no atomics, reproducible).
//
// Per particle, the momentum part is affine in the stencil offset o (APIC
// form b + a o with b = m v - dx A f, a = dx A; A = m C for AFLIP, 0 for
// FLIP), and the vstar part is, per z-node k, alpha_k U + beta_k V with lane
// vectors U, V:
//   AFLIP  U = wij (bs + as0 oi + as1 oj), V = wij as2, alpha_k = wz_k,
//          beta_k = wz_k k (bs, as* from contrib as b, a from A);
//   FLIP   W grad W = (ax_i By_j Bz_k, Bx_i ay_j Bz_k, Bx_i By_j az_k) with
//          B = w^2, a = w w' / dx per axis, so U = ax_i By_j c0 + Bx_i ay_j c1,
//          V = Bx_i By_j c2 (c* the columns of contrib), alpha_k = Bz_k,
//          beta_k = az_k.
constexpr int kFThreads = 192;
constexpr int kFChunk = kFThreads;
constexpr int kFMeta = 64;
constexpr int kFRecs = 16 * 9 * 6;  // lane records: (column, oi oj, z)
// raw channel slots (AFLIP: x v C S m key; FLIP: x v S m key)
template <bool kAffine> struct FRaw {
  static constexpr int X = 0, V = 3, C = 6, S = kAffine ? 15 : 6, M = S + 6, KEY = M + 1,
                       N = KEY + 1;
};
// shared memory: raw[N][chunk]; per-particle records rec4[7][chunk] float4 +
// sw[chunk][6] (wx, wy) + sa[chunk][6] (FLIP: ax, ay), aliased at the end of
// a block by the lane records (recA: m mv, recB: vstar) once every warp has
// finished the block's scatter; cells; block metadata
struct FMeta {
  int start, cnt, dir, scene;
  int K[3];
  int pad;
};
template <bool kAffine> struct FLayout {
  static constexpr int raw = 0;
  static constexpr int rec4 = FRaw<kAffine>::N * kFChunk * 4;
  static constexpr int sw = rec4 + 7 * kFChunk * 16;
  static constexpr int sa = sw + kFChunk * 6 * 4;
  static constexpr int region_end = sa + kFChunk * 6 * 4 > rec4 + 2 * kFRecs * 16
                                        ? sa + kFChunk * 6 * 4
                                        : rec4 + 2 * kFRecs * 16;
  static constexpr int recA = rec4;
  static constexpr int recB = recA + kFRecs * 16;
  static constexpr int cell = region_end;
  static constexpr int meta = cell + ((kFChunk + 15) & ~15);
  static constexpr int bytes = meta + kFMeta * (int)sizeof(FMeta);
  static_assert(recB + kFRecs * 16 <= region_end, "lane records must fit the particle records");
  static_assert(rec4 % 16 == 0 && meta % 16 == 0, "float4 regions must be 16-byte aligned");
};

// CTAs per SM: FLIP fits 4 at 80 registers; AFLIP's affine records would
// spill there, so it keeps 3
template <bool kAffine>
__global__ void __launch_bounds__(kFThreads, kAffine ? 3 : 4)
    k_p2g_flip(DevPtrs d, const float *__restrict__ pin) {
  if (ZSMPM_HALTED(d)) return;
  using RC = FRaw<kAffine>;
  using L = FLayout<kAffine>;
  extern __shared__ __align__(16) unsigned char fsm[];
  float(*raw)[kFChunk] = reinterpret_cast<float(*)[kFChunk]>(fsm + L::raw);
  float4(*rec4)[kFChunk] = reinterpret_cast<float4(*)[kFChunk]>(fsm + L::rec4);
  float(*sw)[6] = reinterpret_cast<float(*)[6]>(fsm + L::sw);
  float(*sa)[6] = reinterpret_cast<float(*)[6]>(fsm + L::sa);
  float4 *recA = reinterpret_cast<float4 *>(fsm + L::recA);
  float4 *recB = reinterpret_cast<float4 *>(fsm + L::recB);
  unsigned char *scell = fsm + L::cell;
  FMeta *meta = reinterpret_cast<FMeta *>(fsm + L::meta);
  const SimParams &P = *d.prm;
  const long long n = P.n;
  const float dt = P.dt;
  const int nb = d.cnt->n_buckets;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int slot = lane / 9, oij = lane % 9;
  const int col = 3 * warp + slot;
  const bool has_col = lane < 27 && col < 16;
  const float foi = (float)(oij / 3), foj = (float)(oij % 3);
  const int wxo = oij / 3, wyo = 3 + oij % 3;

  const int nblk = nb > (int)blockIdx.x ? (nb - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
  auto load_meta = [&](int k) {
    const int b = blockIdx.x + k * gridDim.x;
    const int dir = d.bk_dir[b], start = d.bk_start[b];
    FMeta m;
    m.start = start;
    m.cnt = (int)max(0ll, min((long long)d.bk_count[b], n - start));
    m.dir = dir;
    m.scene = scene_of_dir(d, dir);
    const SceneParams &S = d.scn[m.scene];
    bucket_origin(S, dir - S.dir_off, m.K);
    m.pad = 0;
    return m;
  };
  for (int k = tid; k < min(nblk, kFMeta); k += kFThreads) meta[k] = load_meta(k);
  __syncthreads();
  auto meta_of = [&](int k) { return k < kFMeta ? meta[k] : load_meta(k); };

  struct Item {
    int k, c0;
  };
  auto skip_empty = [&](Item it) {
    while (it.k < nblk && meta_of(it.k).cnt == 0) ++it.k;
    return it;
  };
  auto advance = [&](Item it) {
    if (it.k >= nblk) return it;
    it.c0 += kFChunk;
    if (it.c0 >= meta_of(it.k).cnt) {
      ++it.k;
      it.c0 = 0;
      it = skip_empty(it);
    }
    return it;
  };
  auto perm_of = [&](const Item &it) {
    if (it.k >= nblk) return -1;
    const FMeta m = meta_of(it.k);
    return tid < kFChunk && tid < m.cnt - it.c0 ? d.perm[m.start + it.c0 + tid] : -1;
  };
  auto issue = [&](int p) {
    if (p < 0) return;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      cp_async4(&raw[RC::X + c][tid], &pin[pidx((CH_X + c), p)]);
      cp_async4(&raw[RC::V + c][tid], &pin[pidx((CH_V + c), p)]);
    }
    if (kAffine) {
#pragma unroll
      for (int c = 0; c < 9; ++c) cp_async4(&raw[RC::C + c][tid], &pin[pidx((CH_C + c), p)]);
    }
#pragma unroll
    for (int c = 0; c < 6; ++c) cp_async4(&raw[RC::S + c][tid], &pin[pidx((CH_S + c), p)]);
    cp_async4(&raw[RC::M][tid], &pin[pidx(CH_M, p)]);
    cp_async4(&raw[RC::KEY][tid], &d.pkey[p]);
  };

  // node sums of the lane's 6 column nodes
  float accM[6], accV[6][3], accS[6][3];
#pragma unroll
  for (int z = 0; z < 6; ++z) {
    accM[z] = 0.f;
#pragma unroll
    for (int a = 0; a < 3; ++a) accV[z][a] = accS[z][a] = 0.f;
  }
  Item cur = skip_empty(Item{0, 0});
  Item nxt = advance(cur);
  Item nn = advance(nxt);
  int p_nxt = perm_of(nxt);
  issue(perm_of(cur));
  cp_async_commit();
  while (cur.k < nblk) {
    const int p_nn = perm_of(nn);
    const FMeta m = meta_of(cur.k);
    const SceneParams &S = d.scn[m.scene];
    const float dx = S.dx, inv_dx = S.inv_dx, Dinv = S.Dinv;
    const int nc = min(kFChunk, m.cnt - cur.c0);
    cp_async_wait<0>();
    if (tid < nc) {
      float x[3], v[3], Sv[6], C[9];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        x[k] = raw[RC::X + k][tid];
        v[k] = raw[RC::V + k][tid];
      }
#pragma unroll
      for (int k = 0; k < 6; ++k) Sv[k] = raw[RC::S + k][tid];
#pragma unroll
      for (int k = 0; k < 9; ++k) C[k] = kAffine ? raw[RC::C + k][tid] : 0.0f;
      float mass = raw[RC::M][tid];
      const int cell = __float_as_int(raw[RC::KEY][tid]) & 63;
      const Stencil1 s0 = stencil1(x[0], inv_dx), s1 = stencil1(x[1], inv_dx),
                     s2 = stencil1(x[2], inv_dx);
      const int l0 = s0.base - m.K[0], l1 = s1.base - m.K[1], l2 = s2.base - m.K[2];
      // contrib = kc S (S = vol tau, symmetric, xx yy zz xy xz yz)
      const float kc = kAffine ? -dt * Dinv : -dt;
      float G[9] = {kc * Sv[0], kc * Sv[3], kc * Sv[4], kc * Sv[3], kc * Sv[1],
                    kc * Sv[5], kc * Sv[4], kc * Sv[5], kc * Sv[2]};
      if ((unsigned)l0 > 3u || (unsigned)l1 > 3u || (unsigned)l2 > 3u ||
          sort_cell(l0, l1, l2) != cell) {
        atomicOr(&d.cnt->status, ST_STENCIL);
        mass = 0.0f;
#pragma unroll
        for (int k = 0; k < 9; ++k) G[k] = C[k] = 0.0f;
        v[0] = v[1] = v[2] = 0.0f;
      }
      const float fdx[3] = {s0.f * dx, s1.f * dx, s2.f * dx};
      if (kAffine) {
        // momentum: A = m C; vstar: A_s = contrib (row r, column c = axis)
        float bv[3], bs[3];
#pragma unroll
        for (int r = 0; r < 3; ++r) {
          const float a0 = mass * C[r * 3 + 0], a1 = mass * C[r * 3 + 1], a2 = mass * C[r * 3 + 2];
          bv[r] = mass * v[r] - (a0 * fdx[0] + a1 * fdx[1] + a2 * fdx[2]);
          bs[r] = -(G[r * 3 + 0] * fdx[0] + G[r * 3 + 1] * fdx[1] + G[r * 3 + 2] * fdx[2]);
        }
        // a_c = dx (A[0][c], A[1][c], A[2][c])
        const float av0x = dx * mass * C[0], av0y = dx * mass * C[3], av0z = dx * mass * C[6];
        const float av1x = dx * mass * C[1], av1y = dx * mass * C[4], av1z = dx * mass * C[7];
        const float av2x = dx * mass * C[2], av2y = dx * mass * C[5], av2z = dx * mass * C[8];
        rec4[0][tid] = make_float4(bv[0], bv[1], bv[2], mass);
        rec4[1][tid] = make_float4(av0x, av0y, av0z, av1x);
        rec4[2][tid] = make_float4(av1y, av1z, av2x, av2y);
        rec4[3][tid] = make_float4(av2z, bs[0], bs[1], bs[2]);
        rec4[4][tid] = make_float4(dx * G[0], dx * G[3], dx * G[6], dx * G[1]);
        rec4[5][tid] = make_float4(dx * G[4], dx * G[7], dx * G[2], dx * G[5]);
        rec4[6][tid] = make_float4(dx * G[8], s2.w[0], s2.w[1], s2.w[2]);
      } else {
        // w' of the three nodes per axis: -(1.5 - f), -2 (f - 1), f - 0.5
        auto wgrad = [&](const Stencil1 &st, int o) {
          return o == 0 ? st.f - 1.5f : (o == 1 ? -2.0f * (st.f - 1.0f) : st.f - 0.5f);
        };
        rec4[0][tid] = make_float4(mass * v[0], mass * v[1], mass * v[2], mass);
        // columns of contrib: c_c = (G[0][c], G[1][c], G[2][c])
        rec4[1][tid] = make_float4(G[0], G[3], G[6], G[1]);
        rec4[2][tid] = make_float4(G[4], G[7], G[2], G[5]);
        rec4[3][tid] = make_float4(G[8], s2.w[0], s2.w[1], s2.w[2]);
        rec4[4][tid] = make_float4(s2.w[0] * wgrad(s2, 0) * inv_dx, s2.w[1] * wgrad(s2, 1) * inv_dx,
                                   s2.w[2] * wgrad(s2, 2) * inv_dx, 0.0f);
#pragma unroll
        for (int o = 0; o < 3; ++o) {
          sa[tid][o] = s0.w[o] * wgrad(s0, o) * inv_dx;
          sa[tid][3 + o] = s1.w[o] * wgrad(s1, o) * inv_dx;
        }
      }
#pragma unroll
      for (int o = 0; o < 3; ++o) {
        sw[tid][o] = s0.w[o];
        sw[tid][3 + o] = s1.w[o];
      }
      scell[tid] = (unsigned char)cell;
    }
    __syncthreads();  // records published, raw free
    issue(p_nxt);
    cp_async_commit();
    // the slot's 8 range bounds (cells sorted): first index with cell >=
    // cz * 16 + col + (k & 1) for cz = k >> 1
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
          const float4 u0 = rec4[0][q], u1 = rec4[1][q], u2 = rec4[2][q], u3 = rec4[3][q];
          const float wx = sw[q][wxo], wy = sw[q][wyo];
          const float wij = wx * wy;
          const float mq = u0.w;
          float sv[3], rv[3], U[3], V[3], wz[3], al[3], be[3];
          if (kAffine) {
            const float4 u4 = rec4[4][q], u5 = rec4[5][q], u6 = rec4[6][q];
            sv[0] = fmaf(u1.w, foj, fmaf(u1.x, foi, u0.x));
            sv[1] = fmaf(u2.x, foj, fmaf(u1.y, foi, u0.y));
            sv[2] = fmaf(u2.y, foj, fmaf(u1.z, foi, u0.z));
            rv[0] = u2.z;
            rv[1] = u2.w;
            rv[2] = u3.x;
            U[0] = wij * fmaf(u4.w, foj, fmaf(u4.x, foi, u3.y));
            U[1] = wij * fmaf(u5.x, foj, fmaf(u4.y, foi, u3.z));
            U[2] = wij * fmaf(u5.y, foj, fmaf(u4.z, foi, u3.w));
            V[0] = wij * u5.z;
            V[1] = wij * u5.w;
            V[2] = wij * u6.x;
            wz[0] = u6.y;
            wz[1] = u6.z;
            wz[2] = u6.w;
#pragma unroll
            for (int o = 0; o < 3; ++o) {
              al[o] = wz[o];
              be[o] = wz[o] * (float)o;
            }
          } else {
            const float4 u4 = rec4[4][q];
            const float ax = sa[q][wxo], ay = sa[q][wyo];
            const float l1 = ax * (wy * wy), l2 = (wx * wx) * ay, l4 = (wx * wx) * (wy * wy);
            U[0] = fmaf(l2, u1.w, l1 * u1.x);
            U[1] = fmaf(l2, u2.x, l1 * u1.y);
            U[2] = fmaf(l2, u2.y, l1 * u1.z);
            V[0] = l4 * u2.z;
            V[1] = l4 * u2.w;
            V[2] = l4 * u3.x;
            sv[0] = u0.x;
            sv[1] = u0.y;
            sv[2] = u0.z;
            rv[0] = rv[1] = rv[2] = 0.0f;
            wz[0] = u3.y;
            wz[1] = u3.z;
            wz[2] = u3.w;
            al[0] = wz[0] * wz[0];
            al[1] = wz[1] * wz[1];
            al[2] = wz[2] * wz[2];
            be[0] = u4.x;
            be[1] = u4.y;
            be[2] = u4.z;
          }
#pragma unroll
          for (int oz = 0; oz < 3; ++oz) {
            const float W = wij * wz[oz];
            accM[cz + oz] = fmaf(W, mq, accM[cz + oz]);
#pragma unroll
            for (int a = 0; a < 3; ++a) {
              accV[cz + oz][a] = fmaf(W, sv[a], accV[cz + oz][a]);
              accS[cz + oz][a] = fmaf(al[oz], U[a], fmaf(be[oz], V[a], accS[cz + oz][a]));
              if (kAffine && oz < 2) sv[a] += rv[a];
            }
          }
        }
      }
    }
    if (nxt.k != cur.k) {  // last chunk of the block: lane records, then the tile
      __syncthreads();       // every warp is done with the particle records
      if (has_col) {
#pragma unroll
        for (int z = 0; z < 6; ++z) {
          recA[(col * 9 + oij) * 6 + z] = make_float4(accM[z], accV[z][0], accV[z][1], accV[z][2]);
          recB[(col * 9 + oij) * 6 + z] = make_float4(accS[z][0], accS[z][1], accS[z][2], 0.0f);
        }
      }
#pragma unroll
      for (int z = 0; z < 6; ++z) {
        accM[z] = 0.f;
#pragma unroll
        for (int a = 0; a < 3; ++a) accV[z][a] = accS[z][a] = 0.f;
      }
      __syncthreads();
      const long long tb = (long long)(blockIdx.x + cur.k * gridDim.x) * kTileNodes;
      for (int nd = tid; nd < kTileNodes; nd += kFThreads) {
        const int I = nd / 36, J = (nd / 6) % 6, Kz = nd % 6;
        float4 ga = make_float4(0.f, 0.f, 0.f, 0.f), gb = ga;
#pragma unroll
        for (int oi = 0; oi < 3; ++oi) {
          const int cx = I - oi;
          if (cx < 0 || cx > 3) continue;
#pragma unroll
          for (int oj = 0; oj < 3; ++oj) {
            const int cy = J - oj;
            if (cy < 0 || cy > 3) continue;
            const int r = ((cx * 4 + cy) * 9 + oi * 3 + oj) * 6 + Kz;
            const float4 a = recA[r], b = recB[r];
            ga.x += a.x;
            ga.y += a.y;
            ga.z += a.z;
            ga.w += a.w;
            gb.x += b.x;
            gb.y += b.y;
            gb.z += b.z;
          }
        }
        d.ptile[tb + nd] = ga;
        d.ptile2[tb + nd] = gb;
      }
    }
    __syncthreads();  // particle records, cells and lane records free
    cur = nxt;
    nxt = nn;
    nn = advance(nn);
    p_nxt = p_nn;
  }
  cp_async_wait<0>();
}

// ------------------------------------------------------- grid gather ----
//
// As the APIC gather (one 64-thread group per grid block, the <= 8 covering
// tiles added in a fixed order), summing both tiles.  mode bit 1: the FLIP
// grid update (v = mv / m, vstar = vstar / m + v + g dt, running max of
// |vstar|^2), bit 2: the walls on vstar.  Mode 0 leaves (m, mv) and the raw
// vstar sums, as after the reference P2G.
constexpr int kFGatherBlocks = 4;

__device__ __forceinline__ void flip_update_node(const SceneParams &S, float dt, int mode,
                                                 const int (&I)[3], float4 &g, float4 &h,
                                                 float &vmax) {
  if (mode & 1) {
    const float r = 1.0f / g.x;
    g.y *= r;
    g.z *= r;
    g.w *= r;
    h.x = h.x * r + g.y + S.gravity[0] * dt;
    h.y = h.y * r + g.z + S.gravity[1] * dt;
    h.z = h.z * r + g.w + S.gravity[2] * dt;
    vmax = fmaxf(vmax, h.x * h.x + h.y * h.y + h.z * h.z);
  }
  if (mode & 2) {
    float vs[3] = {h.x, h.y, h.z};
    apply_walls(S, I, vs);
    h.x = vs[0];
    h.y = vs[1];
    h.z = vs[2];
  }
}

__global__ void __launch_bounds__(64 * kFGatherBlocks) k_grid_gather_flip(DevPtrs d, int mode) {
  if (ZSMPM_HALTED(d)) return;
  __shared__ int sbk[kFGatherBlocks][8];
  __shared__ int sorg[kFGatherBlocks][4];
  const SimParams &P = *d.prm;
  const int ng = min(d.cnt->n_gblocks, d.cap_gblocks);
  const int grp = threadIdx.x >> 6, cell = threadIdx.x & 63;
  const int l0 = cell >> 4, l1 = (cell >> 2) & 3, l2 = cell & 3;
  float vmax = 0.0f;
  for (int g0 = blockIdx.x * kFGatherBlocks; g0 < ng; g0 += gridDim.x * kFGatherBlocks) {
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
      float4 g = make_float4(0.f, 0.f, 0.f, 0.f), h = g;
#pragma unroll
      for (int o = 0; o < 8; ++o) {
        const int o0 = o >> 2, o1 = (o >> 1) & 1, o2 = o & 1;
        if ((o0 && l0 >= 2) || (o1 && l1 >= 2) || (o2 && l2 >= 2)) continue;
        const int bk = sbk[grp][o];
        if (bk < 0) continue;
        const long long t = (long long)bk * kTileNodes +
                            ((l0 + 4 * o0) * 6 + (l1 + 4 * o1)) * 6 + (l2 + 4 * o2);
        const float4 a = d.ptile[t], b = d.ptile2[t];
        g.x += a.x;
        g.y += a.y;
        g.z += a.z;
        g.w += a.w;
        h.x += b.x;
        h.y += b.y;
        h.z += b.z;
      }
      if (g.x != 0.0f) {
        const int I[3] = {sorg[grp][0] + l0, sorg[grp][1] + l1, sorg[grp][2] + l2};
        flip_update_node(d.scn[sorg[grp][3]], P.dt, mode, I, g, h, vmax);
      }
      d.grid[(long long)gb * 64 + cell] = g;
      d.grid2[(long long)gb * 64 + cell] = h;
    }
    __syncthreads();
  }
  if (mode & 1) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
    if ((threadIdx.x & 31) == 0 && vmax > 0.0f)
      atomicMax(&d.cnt->max_vel_sqr_bits, __float_as_uint(vmax));
  }
}

// the stage path's UpdateZSGrid / walls on a gathered FLIP grid
__global__ void k_grid_update_flip(DevPtrs d, int mode) {
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
      const int c0 = ldir / (dz * dy), c1 = (ldir / dz) % dy, c2 = ldir % dz;
      const int bk = cloth_source(d.cloth, S, gdir, c0, c1, c2, lane);
      const bool covered = __any_sync(0xffffffffu, bk >= 0);
      int src[8];
#pragma unroll
      for (int o = 0; o < 8; ++o) src[o] = __shfl_sync(0xffffffffu, bk, o);
#pragma unroll
      for (int hh = 0; hh < 2; ++hh) {
        const int cell = lane + 32 * hh;
        const long long idx = (long long)gb * 64 + cell;
        float4 g = d.grid[idx], h = d.grid2[idx];
        const bool added = covered && add_cloth_tiles(d.cloth, src, cell, true, g, h);
        if (g.x != 0.0f) {
          const int I[3] = {(c0 + S.block_lo[0]) * 4 + (cell >> 4),
                            (c1 + S.block_lo[1]) * 4 + ((cell >> 2) & 3),
                            (c2 + S.block_lo[2]) * 4 + (cell & 3)};
          flip_update_node(S, P.dt, mode, I, g, h, vmax);
        }
        if (g.x != 0.0f || added) {
          d.grid[idx] = g;
          d.grid2[idx] = h;
        }
      }
    }
  } else {
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
         idx += (long long)gridDim.x * blockDim.x) {
      float4 g = d.grid[idx];
      if (g.x == 0.0f) continue;
      float4 h = d.grid2[idx];
      const int gdir = d.gb_dir[idx >> 6];
      const int sc = scene_of_dir(d, gdir);
      const SceneParams &S = d.scn[sc];
      const int dz = S.block_dims[2], dy = S.block_dims[1];
      const int ldir = gdir - S.dir_off, cell = (int)(idx & 63);
      const int I[3] = {((ldir / (dz * dy)) + S.block_lo[0]) * 4 + (cell >> 4),
                        (((ldir / dz) % dy) + S.block_lo[1]) * 4 + ((cell >> 2) & 3),
                        ((ldir % dz) + S.block_lo[2]) * 4 + (cell & 3)};
      flip_update_node(S, P.dt, mode, I, g, h, vmax);
      d.grid[idx] = g;
      d.grid2[idx] = h;
    }
  }
  if (mode & 1) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
    if ((threadIdx.x & 31) == 0 && vmax > 0.0f)
      atomicMax(&d.cnt->max_vel_sqr_bits, __float_as_uint(vmax));
  }
}

// ---------------------------------------------------------------- G2P ----
//
// The pipelined G2P of the APIC path (chunks of 128 particles, node values
// and particle channels of the next chunk in flight as cp.async copies into
// double-buffered shared memory), gathering both grids.  The vstar moments
// use per-axis weight pairs (w, q): q = w (o - f) dx for the AFLIP affine
// velocity C = Dinv sum W vstar (x_i - x_p)^T, q = w' for the FLIP velocity
// gradient sum vstar grad W^T (then / dx).
constexpr int kFG2PThreads = 128;
constexpr int kG2PMetaFlip = 32;  // blocks per CTA whose metadata is staged
template <bool kAffine> struct FG2PCh {
  // x F J m vol mu lam mat id v (+ C for FLIP, which carries it unchanged)
  static constexpr int X = 0, F = 3, J = 12, M = 13, VOL = 14, MU = 15, LAM = 16, MAT = 17,
                       ID = 18, V = 19, C = 22, N = kAffine ? 22 : 31;
};
template <bool kAffine> constexpr int fg2p_smem_bytes() {
  return 2 * 2 * kNodes * 16 + 2 * FG2PCh<kAffine>::N * kFG2PThreads * 4 +
         kG2PMetaFlip * (int)sizeof(G2PMeta);
}

// kHencky: the von Mises / Cam-Clay return mappings are compiled in (only
// for contexts whose materials use them; Drucker-Prager alone keeps the
// register count down)
// CTAs per SM: AFLIP fits 5 (96 registers); FLIP's staged C holds it at 4
template <bool kAffine, bool kFuseRM, bool kFuseBin, bool kHencky>
__global__ void __launch_bounds__(kFG2PThreads, kAffine ? 5 : 4)
    k_g2p_flip(DevPtrs d, const float *__restrict__ pin, const int32_t *__restrict__ iin,
               float *__restrict__ pout, int32_t *__restrict__ iout) {
  if (ZSMPM_HALTED(d)) return;
  constexpr int NT = kFG2PThreads;
  using GC = FG2PCh<kAffine>;
  extern __shared__ __align__(16) unsigned char fg_smem[];
  float4(*gsm)[2 * kNodes] = reinterpret_cast<float4(*)[2 * kNodes]>(fg_smem);
  float(*psm)[GC::N][NT] = reinterpret_cast<float(*)[GC::N][NT]>(fg_smem + 2 * 2 * kNodes * 16);
  G2PMeta *meta =
      reinterpret_cast<G2PMeta *>(fg_smem + 2 * 2 * kNodes * 16 + 2 * GC::N * NT * 4);
  const SimParams &P = *d.prm;
  const long long n = P.n;
  const float dt = P.dt;
  const int nb = d.cnt->n_buckets;
  const bool lame = P.has_lame != 0;
  const int tid = threadIdx.x;
  const int nblk = nb > (int)blockIdx.x ? (nb - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
  for (int k = tid; k < min(nblk, kG2PMetaFlip); k += NT)
    meta[k] = g2p_load_meta(d, n, blockIdx.x + k * gridDim.x);
  __syncthreads();

  struct Item {
    int k, c0, ord;
  };
  auto meta_of = [&](int k) {
    return k < kG2PMetaFlip ? meta[k] : g2p_load_meta(d, n, blockIdx.x + k * gridDim.x);
  };
  auto cnt_of = [&](int k) { return meta_of(k).cnt; };
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
  auto issue = [&](const Item &it, int pb, int p) {
    if (it.c0 == 0) {
      float4 *g = gsm[it.ord & 1];
      const bool staged = it.k < kG2PMetaFlip;
      int dir = 0, scene = 0;
      if (!staged) {
        dir = d.bk_dir[blockIdx.x + it.k * gridDim.x];
        scene = scene_of_dir(d, dir);
      }
      for (int nd = tid; nd < kNodes; nd += NT) {
        const int lx = nd / 36, ly = (nd / 6) % 6, lz = nd % 6;
        const int t = ((lx >> 2) << 2) | ((ly >> 2) << 1) | (lz >> 2);
        const int gb = staged ? meta[it.k].gb[t] : neighbour_gb(d, d.scn[scene], dir, t);
        const int cell = ((lx & 3) << 4) | ((ly & 3) << 2) | (lz & 3);
        if (gb >= 0) {
          cp_async16(&g[nd], &d.grid[(long long)gb * 64 + cell]);
          cp_async16(&g[kNodes + nd], &d.grid2[(long long)gb * 64 + cell]);
        } else {
          g[nd] = g[kNodes + nd] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
      }
    }
    if (p >= 0) {
      float(*q)[NT] = psm[pb];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        cp_async4(&q[GC::X + c][tid], &pin[pidx((CH_X + c), p)]);
        cp_async4(&q[GC::V + c][tid], &pin[pidx((CH_V + c), p)]);
      }
#pragma unroll
      for (int c = 0; c < 9; ++c) cp_async4(&q[GC::F + c][tid], &pin[pidx((CH_F + c), p)]);
      if (!kAffine) {
#pragma unroll
        for (int c = 0; c < 9; ++c) cp_async4(&q[GC::C + c][tid], &pin[pidx((CH_C + c), p)]);
      }
      cp_async4(&q[GC::J][tid], &pin[pidx(CH_J, p)]);
      cp_async4(&q[GC::M][tid], &pin[pidx(CH_M, p)]);
      cp_async4(&q[GC::VOL][tid], &pin[pidx(CH_VOL, p)]);
      if (lame) {
        cp_async4(&q[GC::MU][tid], &pin[pidx(CH_MU, p)]);
        cp_async4(&q[GC::LAM][tid], &pin[pidx(CH_LAM, p)]);
      }
      cp_async4(&q[GC::MAT][tid], &iin[iidx(IC_MAT, p)]);
      cp_async4(&q[GC::ID][tid], &iin[iidx(IC_ID, p)]);
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
    const int p_nn = perm_of(nn);
    if (nxt.k < nblk) issue(nxt, buf ^ 1, p_nxt);
    cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();

    const G2PMeta m = meta_of(cur.k);
    const SceneParams &S = d.scn[m.scene];
    const float dx = S.dx, inv_dx = S.inv_dx, Dinv = S.Dinv;
    const float4 *gv = gsm[cur.ord & 1];
    const float4 *gs = gv + kNodes;
    const float(*q)[NT] = psm[buf];
    const bool live = tid < m.cnt - cur.c0;
    const unsigned mask = __ballot_sync(0xffffffffu, live);
    if (live) {
      const int s = m.start + cur.c0 + tid;
      const int p = p_cur;
      const int mid = min(max(__float_as_int(q[GC::MAT][tid]), 0), kMaxMaterials - 1);
      const MatParams mp = d.mats[mid];
      const int id = __float_as_int(q[GC::ID][tid]);
      float x[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) x[k] = q[GC::X + k][tid];
      const Stencil1 s0 = stencil1(x[0], inv_dx), s1 = stencil1(x[1], inv_dx),
                     s2 = stencil1(x[2], inv_dx);
      const int l0 = s0.base - m.K[0], l1 = s1.base - m.K[1], l2 = s2.base - m.K[2];
      float vel[3] = {0.f, 0.f, 0.f}, vs[3] = {0.f, 0.f, 0.f};
      float Mx[3] = {0.f, 0.f, 0.f}, My[3] = {0.f, 0.f, 0.f}, Mz[3] = {0.f, 0.f, 0.f};
      if ((unsigned)l0 > 3u || (unsigned)l1 > 3u || (unsigned)l2 > 3u) {
        atomicOr(&d.cnt->status, ST_STENCIL);
      } else {
        // per-axis second weights: AFLIP w (o - f) dx, FLIP w'
        float qx[3], qy[3], qz[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          if (kAffine) {
            qx[c] = s0.w[c] * (((float)c - s0.f) * dx);
            qy[c] = s1.w[c] * (((float)c - s1.f) * dx);
            qz[c] = s2.w[c] * (((float)c - s2.f) * dx);
          } else {
            qx[c] = c == 0 ? s0.f - 1.5f : (c == 1 ? -2.0f * (s0.f - 1.0f) : s0.f - 0.5f);
            qy[c] = c == 0 ? s1.f - 1.5f : (c == 1 ? -2.0f * (s1.f - 1.0f) : s1.f - 0.5f);
            qz[c] = c == 0 ? s2.f - 1.5f : (c == 1 ? -2.0f * (s2.f - 1.0f) : s2.f - 0.5f);
          }
        }
        // k innermost: t = sum_k wz v, u = sum_k wz vs, uz = sum_k qz vs;
        // then over j and i (each product of weights formed once per level)
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          float Sv[3] = {0.f, 0.f, 0.f}, Su[3] = {0.f, 0.f, 0.f}, Sy[3] = {0.f, 0.f, 0.f},
                Sz[3] = {0.f, 0.f, 0.f};
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            const int row = ((l0 + i) * 6 + (l1 + j)) * 6 + l2;
            float t[3] = {0.f, 0.f, 0.f}, u[3] = {0.f, 0.f, 0.f}, uz[3] = {0.f, 0.f, 0.f};
#pragma unroll
            for (int kk = 0; kk < 3; ++kk) {
              const float4 a = gv[row + kk], b = gs[row + kk];
              const float va[3] = {a.y, a.z, a.w}, vb[3] = {b.x, b.y, b.z};
#pragma unroll
              for (int c = 0; c < 3; ++c) {
                t[c] = fmaf(s2.w[kk], va[c], t[c]);
                u[c] = fmaf(s2.w[kk], vb[c], u[c]);
                uz[c] = fmaf(qz[kk], vb[c], uz[c]);
              }
            }
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              Sv[c] = fmaf(s1.w[j], t[c], Sv[c]);
              Su[c] = fmaf(s1.w[j], u[c], Su[c]);
              Sy[c] = fmaf(qy[j], u[c], Sy[c]);
              Sz[c] = fmaf(s1.w[j], uz[c], Sz[c]);
            }
          }
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            vel[c] = fmaf(s0.w[i], Sv[c], vel[c]);
            vs[c] = fmaf(s0.w[i], Su[c], vs[c]);
            Mx[c] = fmaf(qx[i], Su[c], Mx[c]);
            My[c] = fmaf(s0.w[i], Sy[c], My[c]);
            Mz[c] = fmaf(s0.w[i], Sz[c], Mz[c]);
          }
        }
      }
      // X = the velocity gradient that updates F: AFLIP Dinv M (also the new
      // C), FLIP M / dx
      const float sc = kAffine ? Dinv : inv_dx;
      float X[9];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        X[a * 3 + 0] = Mx[a] * sc;
        X[a * 3 + 1] = My[a] * sc;
        X[a * 3 + 2] = Mz[a] * sc;
      }
      constexpr float kFlip = 0.99f;
      const float beta = kAffine ? d.beta[id] : 0.0f;
      float vn[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const float d0 = q[GC::V + k][tid] - vel[k];
        vn[k] = vs[k] + kFlip * d0;
        x[k] += kAffine ? dt * (vs[k] + beta * kFlip * d0) : vs[k] * dt;
      }
      float F[9], J;
      Sym3 tau;
      bool ok_state = true;
      float mu = mp.mu, lam = mp.lam;
      if (lame) {
        mu = q[GC::MU][tid];
        lam = q[GC::LAM][tid];
      }
      // the FLIP P2G takes the material's Lame parameters (Transfer.cu:897-907)
      const float mu_s = kAffine ? mu : mp.mu, lam_s = kAffine ? lam : mp.lam;
      if (mp.type == MPM_EOS) {
        J = q[GC::J][tid] * (1.0f + dt * (X[0] + X[4] + X[8]));
        const float c = cbrtf(J);
#pragma unroll
        for (int k = 0; k < 9; ++k) F[k] = (k % 4 == 0) ? c : 0.0f;
        ok_state = kirchhoff(MPM_EOS, mu_s, lam_s, mp.bulk, mp.gamma, F, J, tau);
      } else {
        float Fo[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) Fo[k] = q[GC::F + k][tid];
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int c = 0; c < 3; ++c)
            F[r * 3 + c] = Fo[r * 3 + c] + dt * (X[r * 3 + 0] * Fo[c] + X[r * 3 + 1] * Fo[3 + c] +
                                                 X[r * 3 + 2] * Fo[6 + c]);
        float jch = q[GC::J][tid];  // log(Jp) of a Cam-Clay particle
        if (kFuseRM && mp.plastic != MPM_PLASTIC_NONE &&
            (kHencky || mp.plastic == MPM_PLASTIC_NADP)) {
          ok_state = (kHencky ? return_mapping(mp, mu, lam, F, jch, tau)
                              : project_dp(mu, lam, mp.alpha, F, tau)) >= 0;
          if (!kAffine && lame)  // the stress of the projected F with the material's mu, lam
            ok_state = kirchhoff(mp.type, mu_s, lam_s, mp.bulk, mp.gamma, F, 1.0f, tau) && ok_state;
        } else {
          ok_state = kirchhoff(mp.type, mu_s, lam_s, mp.bulk, mp.gamma, F, 1.0f, tau);
        }
        J = mp.plastic == MPM_PLASTIC_NACC ? jch : det3(F);
      }
      if (!ok_state) atomicOr(&d.cnt->status, ST_NAN);
      const float vol = q[GC::VOL][tid];
      bool finite = isfinite(x[0]) && isfinite(x[1]) && isfinite(x[2]) && isfinite(J);
#pragma unroll
      for (int k = 0; k < 9; ++k) finite = finite && isfinite(F[k]);
      if (!finite) atomicOr(&d.cnt->status, ST_NAN);
      const int so = s;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        pout[pidx((CH_X + k), so)] = x[k];
        pout[pidx((CH_V + k), so)] = vn[k];
      }
#pragma unroll
      for (int k = 0; k < 9; ++k) {
        pout[pidx((CH_C + k), so)] = kAffine ? X[k] : q[GC::C + k][tid];
        pout[pidx((CH_F + k), so)] = F[k];
      }
      pout[pidx(CH_J, so)] = J;
      pout[pidx(CH_M, so)] = q[GC::M][tid];
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
      iout[iidx(IC_ID, so)] = id;
      if (kFuseBin) {
        const int key = bin_key(S, x[0], x[1], x[2], &d.cnt->status);
        d.pkey[so] = key;
        bin_count(d, S, key, mask);
      }
    }
    __syncthreads();
    cur = nxt;
    nxt = nn;
    nn = advance(nn);
    p_cur = p_nxt;
    p_nxt = p_nn;
    buf ^= 1;
  }
  cp_async_wait<0>();
}

// ComputeParticleBeta (Boundary.cu:172-516) on the current store: the
// boundary-grid form (collider -2, :172-222) or the level-set form
// (determine_beta_sdf, :285-315) first -- at x + dt v, a
// particle inside the collider moving into it, (v - v_obj) . n < 0, gets
// beta 0 -- then the volume criterion beta = 0.5 where J > Jp_critical = 1
// (J = det F, or the fluid's J), else 0.  beta is stored by upload index.
__global__ void k_particle_beta(DevPtrs d, const float *__restrict__ pb,
                                const int32_t *__restrict__ ib, float dt, int collider) {
  const long long n = d.prm->n;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    const int id = ib[iidx(IC_ID, p)];
    if (id < 0 || id >= n) continue;
    const MatParams mp = d.mats[min(max(ib[iidx(IC_MAT, p)], 0), kMaxMaterials - 1)];
    float v[3], x[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      v[a] = pb[pidx((CH_V + a), p)];
      x[a] = pb[pidx((CH_X + a), p)] + dt * v[a];
    }
    if (collider == -2) {
      // the boundary grid (Boundary.cu:172-222): a node of the linear
      // stencil at x + dt v with boundary mass where (v - v_b) . nrm_b < 0
      const SceneParams &S = d.scn[0];
      int base[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) base[a] = __float2int_rd(__fmul_rn(x[a], S.inv_dx));
      bool in = false;
      for (int o = 0; o < 8 && !in; ++o) {
        const int I[3] = {base[0] + (o >> 2), base[1] + ((o >> 1) & 1), base[2] + (o & 1)};
        int c[3];
        bool inside = true;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          c[a] = (I[a] >> 2) - S.block_lo[a];
          inside = inside && c[a] >= 0 && c[a] < S.block_dims[a];
        }
        if (!inside) continue;
        const int bb = d.bnd_map[S.dir_off + ((long long)c[0] * S.block_dims[1] + c[1]) * S.block_dims[2] + c[2]];
        if (bb < 0) continue;
        const int cell = ((I[0] & 3) << 4) | ((I[1] & 3) << 2) | (I[2] & 3);
        const float4 bmv = d.bnd_grid[2 * ((long long)bb * 64 + cell)];
        if (bmv.x == 0.0f) continue;
        const float4 bn = d.bnd_grid[2 * ((long long)bb * 64 + cell) + 1];
        in = (v[0] - bmv.y) * bn.x + (v[1] - bmv.z) * bn.y + (v[2] - bmv.w) * bn.z < 0.0f;
      }
      if (in) {
        d.beta[id] = 0.0f;
        continue;
      }
    }
    if (collider >= 0) {
      float nrm[3], vo[3];
      if (collider_hit(d.colliders[collider], x, nrm, vo) &&
          (v[0] - vo[0]) * nrm[0] + (v[1] - vo[1]) * nrm[1] + (v[2] - vo[2]) * nrm[2] < 0.0f) {
        d.beta[id] = 0.0f;
        continue;
      }
    }
    double J;
    if (mp.type == MPM_EOS) {
      J = pb[pidx(CH_J, p)];
    } else {
      double F[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) F[k] = pb[pidx((CH_F + k), p)];
      // det F in double, compared in double (Boundary.cu:206-208)
      J = F[0] * (F[4] * F[8] - F[5] * F[7]) - F[1] * (F[3] * F[8] - F[5] * F[6]) +
          F[2] * (F[3] * F[7] - F[4] * F[6]);
    }
    d.beta[id] = J > 1.0 ? 0.5f : 0.0f;
  }
}

}  // namespace

template <class K> static int occupancy(K kernel, int threads, int smem) {
  cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  int b = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kernel, threads, smem);
  return b > 0 ? b : 1;
}

void configure_flip_launches(DevPtrs &d) {
  const int pa = occupancy(k_p2g_flip<true>, kFThreads, FLayout<true>::bytes),
            pf = occupancy(k_p2g_flip<false>, kFThreads, FLayout<false>::bytes);
  // the G2P grids: as many CTAs as every instance of the transfer holds
  int ga = occupancy(k_g2p_flip<true, true, true, false>, kFG2PThreads, fg2p_smem_bytes<true>());
  ga = std::min(ga, occupancy(k_g2p_flip<true, true, true, true>, kFG2PThreads,
                              fg2p_smem_bytes<true>()));
  ga = std::min(ga, occupancy(k_g2p_flip<true, false, false, false>, kFG2PThreads,
                              fg2p_smem_bytes<true>()));
  int gf = occupancy(k_g2p_flip<false, true, true, false>, kFG2PThreads, fg2p_smem_bytes<false>());
  gf = std::min(gf, occupancy(k_g2p_flip<false, true, true, true>, kFG2PThreads,
                              fg2p_smem_bytes<false>()));
  gf = std::min(gf, occupancy(k_g2p_flip<false, false, false, false>, kFG2PThreads,
                              fg2p_smem_bytes<false>()));
  d.grid_p2g_flip = d.num_sms * pf;
  d.grid_p2g_aflip = d.num_sms * pa;
  d.grid_g2p_flip = d.num_sms * gf;
  d.grid_g2p_aflip = d.num_sms * ga;
}

void launch_p2g_flip(const DevPtrs &d, int cur, cudaStream_t s) {
  if (d.transfer == MPM_TRANSFER_AFLIP)
    k_p2g_flip<true><<<d.grid_p2g_aflip, kFThreads, FLayout<true>::bytes, s>>>(d, d.pbuf[cur]);
  else
    k_p2g_flip<false><<<d.grid_p2g_flip, kFThreads, FLayout<false>::bytes, s>>>(d, d.pbuf[cur]);
}

void launch_grid_gather_flip(const DevPtrs &d, int mode, cudaStream_t s) {
  k_grid_gather_flip<<<d.grid_stream, 64 * kFGatherBlocks, 0, s>>>(d, mode);
}

void launch_grid_update_flip(const DevPtrs &d, int mode, cudaStream_t s) {
  k_grid_update_flip<<<d.num_sms * 8, 256, 0, s>>>(d, mode);
}

void launch_g2p_flip(const DevPtrs &d, int cur, int fuse_rm, int fuse_bin, cudaStream_t s) {
  float *pi = d.pbuf[cur], *po = d.pbuf[1 - cur];
  int32_t *ii = d.ibuf[cur], *io = d.ibuf[1 - cur];
  const int grid = d.transfer == MPM_TRANSFER_AFLIP ? d.grid_g2p_aflip : d.grid_g2p_flip;
  if (d.transfer == MPM_TRANSFER_AFLIP) {
    constexpr int smem = fg2p_smem_bytes<true>();
    if (fuse_rm && fuse_bin && d.hencky)
      k_g2p_flip<true, true, true, true><<<grid, kFG2PThreads, smem, s>>>(d, pi, ii, po, io);
    else if (fuse_rm && fuse_bin)
      k_g2p_flip<true, true, true, false><<<grid, kFG2PThreads, smem, s>>>(d, pi, ii, po, io);
    else
      k_g2p_flip<true, false, false, false><<<grid, kFG2PThreads, smem, s>>>(d, pi, ii, po, io);
  } else {
    constexpr int smem = fg2p_smem_bytes<false>();
    if (fuse_rm && fuse_bin && d.hencky)
      k_g2p_flip<false, true, true, true><<<grid, kFG2PThreads, smem, s>>>(d, pi, ii, po, io);
    else if (fuse_rm && fuse_bin)
      k_g2p_flip<false, true, true, false><<<grid, kFG2PThreads, smem, s>>>(d, pi, ii, po, io);
    else
      k_g2p_flip<false, false, false, false><<<grid, kFG2PThreads, smem, s>>>(d, pi, ii, po, io);
  }
}

void launch_particle_beta(const DevPtrs &d, int cur, float dt, int collider, cudaStream_t s) {
  k_particle_beta<<<d.num_sms * 8, 256, 0, s>>>(d, d.pbuf[cur], d.ibuf[cur], dt, collider);
}

}  // namespace zsmpm
