// Adjoint of one substep (the differentiable form; the reference has none).
//
// Forward substep n (particles x, v, C, F; grid nodes i):
//   P2G   m_i = sum_p W m_p,  mv_i = sum_p W (m_p v_p + A_p (x_i - x_p)),
//         A_p = m_p C_p - dt Dinv vol_p tau(F_p)
//   grid  v_i = BC(mv_i / m_i + g dt)
//   G2P   v' = sum_i W v_i,  C' = Dinv sum_i W v_i (x_i - x_p)^T,
//         x' = x + dt v',  F' = (I + dt C') F
// Given the adjoints (x', v', C', F')-bar of the next state, the three
// kernels here produce the adjoints of this state and of mu, lam:
//   k_g2p_adjoint_particles  per particle: recomputes G2P's C', takes F'b back
//                   through the Drucker-Prager projection (sand), forms
//                   Cb = C'b + dt F'b F^T, vb = v'b + dt x'b, F-bar = (I + dt C')^T F'b,
//                   x-bar through the weights (stencil moments), and writes
//                   the record of its node adjoint W (vb + Dinv Cb (x_i - x_p))
//   k_g2p_adjoint_scatter    per particle block: the records into tiles
//                   (tile_scatter: deterministic, no atomics)
//   k_grid_adjoint  per node: the tiles' sum, the boundary's transpose, then
//                   mv_i-bar = v-bar / m_i, m_i-bar = -v-bar . mv_i / m_i^2
//   k_p2g_adjoint   per particle block: gathers (m-bar, mv-bar) of the 216
//                   nodes: v-bar = m sum W mv-bar, A-bar = sum W mv-bar (x_i - x_p)^T,
//                   C-bar = m A-bar, tau-bar = -dt Dinv vol A-bar through the
//                   stress adjoint, x-bar through the weights and (x_i - x_p)
// Every state is in its own slot order (the forward sorts the store by block
// each substep): a particle at slot p of state n sits at its sorted position
// sp of state n+1, so the G2P adjoint reads the next adjoint at sp and
// writes this one at p; the mu / lam gradients go by upload index.
#include <cuda_runtime.h>

#include <algorithm>

#include "adj_moments.cuh"
#include "binning.cuh"
#include "colliders.cuh"
#include "mpm_math.cuh"
#include "tile_scatter.cuh"
#include "zsmpm_internal.cuh"

namespace zsmpm {
namespace {

// adjoint planes (n each): x 3, v 3, C 9, F 9, J 1
enum : int { AJ_X = 0, AJ_V = 3, AJ_C = 6, AJ_F = 15, AJ_J = 24, NAJ = 25 };

__device__ __forceinline__ void origin_of(const SceneParams &S, int ldir, int (&K)[3]) {
  const int dz = S.block_dims[2], dy = S.block_dims[1];
  K[0] = ((ldir / (dz * dy)) + S.block_lo[0]) * 4;
  K[1] = (((ldir / dz) % dy) + S.block_lo[1]) * 4;
  K[2] = ((ldir % dz) + S.block_lo[2]) * 4;
}

__device__ __forceinline__ int gb_of(const DevPtrs &d, const SceneParams &S, int dir, int t) {
  const int dz = S.block_dims[2], dy = S.block_dims[1];
  return d.dir_gb[dir + ((t >> 2) * dy + ((t >> 1) & 1)) * dz + (t & 1)];
}

// Scatter records of the G2P adjoint, one per particle at its sorted
// position: b (3), A (9, row-major), f (3) as in tile_stage, then the cell
// (int32 bits): the node adjoint of stencil node o is W (b + A o dx).
constexpr int kAdjRec = 16;

// Per-particle part of the G2P adjoint.  A CTA takes particle blocks
// (grid-stride over the partition), stages the block's 216 node velocities,
// and gives one particle to each thread: the node sums it needs are stencil
// moments (adj_moments), the forward C' among them; then the Drucker-Prager
// projection's adjoint (sand), Cb, F-bar, x-bar, and the scatter record.
constexpr int kAdjPThreads = 128;

__global__ void __launch_bounds__(kAdjPThreads, 4)
    k_g2p_adjoint_particles(DevPtrs d, const float *__restrict__ pin,
                            const int32_t *__restrict__ iin, const float *__restrict__ an,
                            float *__restrict__ ap, float *__restrict__ gmu,
                            float *__restrict__ glam, float *__restrict__ rec, long long n,
                            int kc) {
  __shared__ float4 sg[kNodes];
  __shared__ int sgb[8];
  const SimParams &P = *d.prm;
  const float dt = P.dt;
  const int nb = d.cnt->n_buckets;
  const int tid = threadIdx.x;
  const bool lame = P.has_lame != 0;
  const long long cap = d.cap;
  // work item w: chunk w % kc of particle block w / kc (kc CTAs share a
  // block when the scene has few blocks)
  for (int w = blockIdx.x; w < nb * kc; w += gridDim.x) {
    const int b = w / kc, chunk = w - b * kc;
    const int dir = d.bk_dir[b];
    const SceneParams &S = d.scn[scene_of_dir(d, dir)];
    const float dx = S.dx, inv_dx = S.inv_dx, Dinv = S.Dinv;
    if (tid < 8) sgb[tid] = gb_of(d, S, dir, tid);
    int K[3];
    origin_of(S, dir - S.dir_off, K);
    __syncthreads();
    for (int nd = tid; nd < kNodes; nd += kAdjPThreads) {
      const int lx = nd / 36, ly = (nd / 6) % 6, lz = nd % 6;
      const int gb = sgb[((lx >> 2) << 2) | ((ly >> 2) << 1) | (lz >> 2)];
      const int cell = ((lx & 3) << 4) | ((ly & 3) << 2) | (lz & 3);
      sg[nd] = gb >= 0 ? d.grid[(long long)gb * 64 + cell] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncthreads();
    const int start = d.bk_start[b];
    const int cnt = (int)max(0ll, min((long long)d.bk_count[b], P.n - start));
    for (int j = chunk * kAdjPThreads + tid; j < cnt; j += kc * kAdjPThreads) {
      // the particle's slot p in this state and its slot sp in the next
      // (the forward G2P writes it at its sorted position)
      const int sp = start + j;
      const int p = d.perm[sp];
      const int id = iin[iidx(IC_ID, p)];
      float x[3], F[9], xb[3], vb[3], Cb[9], Fb[9];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        x[k] = pin[pidx((CH_X + k), p)];
        xb[k] = an[(AJ_X + k) * n + sp];
        vb[k] = an[(AJ_V + k) * n + sp] + dt * xb[k];
      }
#pragma unroll
      for (int k = 0; k < 9; ++k) {
        F[k] = pin[pidx((CH_F + k), p)];
        Fb[k] = an[(AJ_F + k) * n + sp];
        Cb[k] = an[(AJ_C + k) * n + sp];
      }
      const Stencil1 s0 = stencil1(x[0], inv_dx), s1 = stencil1(x[1], inv_dx),
                     s2 = stencil1(x[2], inv_dx);
      const int l0 = s0.base - K[0], l1 = s1.base - K[1], l2 = s2.base - K[2];
      const bool inside = (unsigned)l0 <= 3u && (unsigned)l1 <= 3u && (unsigned)l2 <= 3u;
      if (!inside) atomicOr(&d.cnt->status, ST_STENCIL);
      AdjMoments M;
      const AxisFactors A0 = axis_factors(s0, dx, inv_dx), A1 = axis_factors(s1, dx, inv_dx),
                        A2 = axis_factors(s2, dx, inv_dx);
      if (inside) {
        adj_moments<false>(sg, l0, l1, l2, A0, A1, A2, M);
      } else {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          M.W[c] = 0.f;
#pragma unroll
          for (int a = 0; a < 3; ++a) {
            M.X[a][c] = M.D[a][c] = 0.f;
#pragma unroll
            for (int bb = 0; bb < 3; ++bb) M.DX[a][bb][c] = 0.f;
          }
        }
      }
      // forward C' (times 1/Dinv) of this substep: Cn[c][b] = sum W g_c xx_b
      float Cn[9];
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int bb = 0; bb < 3; ++bb) Cn[c * 3 + bb] = M.X[bb][c];
      // Drucker-Prager return mapping: F'b is the adjoint of the projected
      // F; take it back to the trial F = (I + dt C') F
      const MatParams mp = d.mats[min(max(iin[iidx(IC_MAT, p)], 0), kMaxMaterials - 1)];
      if (mp.type != MPM_EOS && mp.plastic == MPM_PLASTIC_NADP) {
        float Ft[9];
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int c = 0; c < 3; ++c)
            Ft[r * 3 + c] = F[r * 3 + c] + dt * Dinv *
                                               (Cn[r * 3 + 0] * F[0 * 3 + c] +
                                                Cn[r * 3 + 1] * F[1 * 3 + c] +
                                                Cn[r * 3 + 2] * F[2 * 3 + c]);
        const float mu = lame ? pin[pidx(CH_MU, p)] : mp.mu;
        const float lam = lame ? pin[pidx(CH_LAM, p)] : mp.lam;
        float mub = 0.f, lamb = 0.f;
        dp_projection_vjp(mu, lam, mp.alpha, Ft, Fb, mub, lamb);
        gmu[id] += mub;
        glam[id] += lamb;
      }
      // C'b += dt F'b F^T
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
          Cb[r * 3 + c] += dt * (Fb[r * 3] * F[c * 3] + Fb[r * 3 + 1] * F[c * 3 + 1] +
                                 Fb[r * 3 + 2] * F[c * 3 + 2]);
      // x-bar through the weights: with s_n = g_n . vb + Dinv g_n . (Cb xx_n),
      //   gx_a = sum dW_a s_n - Dinv sum W (Cb^T g_n)_a
      //        = vb . D[a] + Dinv sum_bc Cb_cb DX[a][b][c] - Dinv sum_c Cb_ca W[c]
      float gx[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        float t = 0.f, u = 0.f;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          t = fmaf(vb[c], M.D[a][c], t);
          u = fmaf(-Cb[c * 3 + a], M.W[c], u);
#pragma unroll
          for (int bb = 0; bb < 3; ++bb) u = fmaf(Cb[c * 3 + bb], M.DX[a][bb][c], u);
        }
        gx[a] = fmaf(Dinv, u, t);
      }
      // F-bar = (I + dt C')^T F'b
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
          ap[(AJ_F + r * 3 + c) * n + p] =
              Fb[r * 3 + c] + dt * Dinv *
                                  (Cn[0 * 3 + r] * Fb[0 * 3 + c] + Cn[1 * 3 + r] * Fb[1 * 3 + c] +
                                   Cn[2 * 3 + r] * Fb[2 * 3 + c]);
#pragma unroll
      for (int k = 0; k < 3; ++k) ap[(AJ_X + k) * n + p] = xb[k] + gx[k];
      // the scatter record of W (vb + Dinv Cb (x_i - x_p)): b = vb - dx A f, A = Dinv Cb
      const float f[3] = {s0.f, s1.f, s2.f};
      float A[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) A[k] = inside ? Dinv * Cb[k] : 0.0f;
#pragma unroll
      for (int a = 0; a < 3; ++a)
        rec[a * cap + sp] = inside ? vb[a] - dx * (A[a * 3] * f[0] + A[a * 3 + 1] * f[1] +
                                                   A[a * 3 + 2] * f[2])
                                   : 0.0f;
#pragma unroll
      for (int k = 0; k < 9; ++k) rec[(3 + k) * cap + sp] = A[k];
#pragma unroll
      for (int k = 0; k < 3; ++k) rec[(12 + k) * cap + sp] = f[k];
      // the cell of the particle's key, from its position as the binning
      // forms it (the key store itself holds the next state's keys by now)
      rec[15 * cap + sp] = __int_as_float(sort_cell(s0.base & 3, s1.base & 3, s2.base & 3));
    }
    __syncthreads();  // sg reused by the next block
  }
}

// Scatter part of the G2P adjoint: per particle block, its records (read
// in sorted order) into the block's tile of node adjoints (tile_scatter:
// deterministic, no atomics).
__global__ void __launch_bounds__(kP2GThreads)
    k_g2p_adjoint_scatter(DevPtrs d, const float *__restrict__ rec) {
  extern __shared__ __align__(16) unsigned char adj_smem[];
  const TileSmem ts = tile_smem(adj_smem);
  const SimParams &P = *d.prm;
  const int nb = d.cnt->n_buckets;
  const int tid = threadIdx.x;
  const long long cap = d.cap;
  for (int b = blockIdx.x; b < nb; b += gridDim.x) {
    tile_zero(ts);
    const int dir = d.bk_dir[b];
    const SceneParams &S = d.scn[scene_of_dir(d, dir)];
    const int start = d.bk_start[b];
    const int cnt = (int)max(0ll, min((long long)d.bk_count[b], P.n - start));
    for (int c0 = 0; c0 < cnt; c0 += kP2GChunk) {
      const int nc = min(kP2GChunk, cnt - c0);
      __syncthreads();
      for (int j = tid; j < nc; j += kP2GThreads) {
        const long long sp = start + c0 + j;
        float bv[3], A[9], f[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) bv[k] = rec[k * cap + sp];
#pragma unroll
        for (int k = 0; k < 9; ++k) A[k] = rec[(3 + k) * cap + sp];
#pragma unroll
        for (int k = 0; k < 3; ++k) f[k] = rec[(12 + k) * cap + sp];
        tile_stage(ts, j, 0.0f, bv, A, f, __float_as_int(rec[15 * cap + sp]));
      }
      __syncthreads();
      tile_cell_ranges(ts, nc);
      __syncthreads();
      tile_scatter(ts, S.dx);
    }
    __syncthreads();
    tile_store(ts, d.ptile_adj + (long long)b * kTileNodes);
    __syncthreads();
  }
}

// per grid node: v-bar from the adjoint tiles; m, mv from the forward tiles
__global__ void k_grid_adjoint(DevPtrs d) {
  const SimParams &P = *d.prm;
  const long long nn = (long long)min(d.cnt->n_gblocks, d.cap_gblocks) * 64;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < nn;
       idx += (long long)gridDim.x * blockDim.x) {
    const int gb = (int)(idx >> 6), cell = (int)(idx & 63);
    const int gdir = d.gb_dir[gb];
    const SceneParams &S = d.scn[scene_of_dir(d, gdir)];
    const int dy = S.block_dims[1], dz = S.block_dims[2];
    const int ldir = gdir - S.dir_off;
    const int c0 = ldir / (dz * dy), c1 = (ldir / dz) % dy, c2 = ldir % dz;
    const int l0 = cell >> 4, l1 = (cell >> 2) & 3, l2 = cell & 3;
    float4 fw = make_float4(0.f, 0.f, 0.f, 0.f), ad = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int o = 0; o < 8; ++o) {
      const int o0 = o >> 2, o1 = (o >> 1) & 1, o2 = o & 1;
      if ((o0 && (l0 >= 2 || c0 < 1)) || (o1 && (l1 >= 2 || c1 < 1)) ||
          (o2 && (l2 >= 2 || c2 < 1)))
        continue;
      const int bk = d.dir_bk[gdir - (o0 * dy + o1) * dz - o2];
      if (bk < 0) continue;
      const long long t = (long long)bk * kTileNodes +
                          ((l0 + 4 * o0) * 6 + (l1 + 4 * o1)) * 6 + (l2 + 4 * o2);
      const float4 a = d.ptile[t], c = d.ptile_adj[t];
      fw.x += a.x;
      fw.y += a.y;
      fw.z += a.z;
      fw.w += a.w;
      ad.y += c.y;
      ad.z += c.z;
      ad.w += c.w;
    }
    float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
    if (fw.x != 0.0f) {
      const float r = 1.0f / fw.x;
      const float vp[3] = {fw.y * r + S.gravity[0] * P.dt, fw.z * r + S.gravity[1] * P.dt,
                           fw.w * r + S.gravity[2] * P.dt};
      float vb[3] = {ad.y, ad.z, ad.w};
      const int scene = scene_of_dir(d, gdir);
      const int nc = P.n_colliders;
      if (nc > 0) {
        // the colliders act after the walls: their transpose comes first
        const int I[3] = {(c0 + S.block_lo[0]) * 4 + l0, (c1 + S.block_lo[1]) * 4 + l1,
                          (c2 + S.block_lo[2]) * 4 + l2};
        float vw[3] = {vp[0], vp[1], vp[2]};
        if (S.bc_type != MPM_BC_NONE) {
          bool any = false;
          const int th = S.bc_thickness;
          for (int a = 0; a < 3; ++a) {
            const bool lower = I[a] < S.bc_lo[a] + th, upper = I[a] > S.bc_hi[a] - th;
            if (!(lower || upper)) continue;
            any = true;
            if (S.bc_type == MPM_BC_SLIP) vw[a] = 0.0f;
            if (S.bc_type == MPM_BC_SEPARATE && ((lower && vw[a] < 0.0f) || (upper && vw[a] > 0.0f)))
              vw[a] = 0.0f;
          }
          if (any && S.bc_type == MPM_BC_STICKY) vw[0] = vw[1] = vw[2] = 0.0f;
        }
        const float p[3] = {(float)I[0] * S.dx, (float)I[1] * S.dx, (float)I[2] * S.dx};
        apply_colliders_adjoint(d, nc, scene, p, vw, vb);
      }
      if (S.bc_type != MPM_BC_NONE) {
        const int I[3] = {(c0 + S.block_lo[0]) * 4 + l0, (c1 + S.block_lo[1]) * 4 + l1,
                          (c2 + S.block_lo[2]) * 4 + l2};
        bool any = false;
        const int th = S.bc_thickness;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          const bool lower = I[a] < S.bc_lo[a] + th, upper = I[a] > S.bc_hi[a] - th;
          if (!(lower || upper)) continue;
          any = true;
          if (S.bc_type == MPM_BC_SLIP) vb[a] = 0.0f;
          if (S.bc_type == MPM_BC_SEPARATE && ((lower && vp[a] < 0.0f) || (upper && vp[a] > 0.0f)))
            vb[a] = 0.0f;
        }
        if (any && S.bc_type == MPM_BC_STICKY) vb[0] = vb[1] = vb[2] = 0.0f;
      }
      out.y = vb[0] * r;
      out.z = vb[1] * r;
      out.w = vb[2] * r;
      out.x = -(vb[0] * fw.y + vb[1] * fw.z + vb[2] * fw.w) * r * r;
    }
    d.grid[idx] = out;  // (m-bar, mv-bar)
  }
}

constexpr int kP2GAdjThreads = 128;

__global__ void __launch_bounds__(kP2GAdjThreads, 4)
    k_p2g_adjoint(DevPtrs d, const float *__restrict__ pin, const int32_t *__restrict__ iin,
                  float *__restrict__ ap, float *__restrict__ gmu, float *__restrict__ glam,
                  long long n, int kc) {
  __shared__ float4 sg[kNodes];
  __shared__ int sgb[8];
  const SimParams &P = *d.prm;
  const float dt = P.dt;
  const int nb = d.cnt->n_buckets;
  const bool lame = P.has_lame != 0;
  for (int w = blockIdx.x; w < nb * kc; w += gridDim.x) {  // chunk w % kc of block w / kc
    const int b = w / kc, chunk = w - b * kc;
    const int dir = d.bk_dir[b];
    const SceneParams &S = d.scn[scene_of_dir(d, dir)];
    const float dx = S.dx, inv_dx = S.inv_dx, Dinv = S.Dinv;
    if (threadIdx.x < 8) sgb[threadIdx.x] = gb_of(d, S, dir, threadIdx.x);
    int K[3];
    origin_of(S, dir - S.dir_off, K);
    __syncthreads();
    for (int nd = threadIdx.x; nd < kNodes; nd += kP2GAdjThreads) {
      const int lx = nd / 36, ly = (nd / 6) % 6, lz = nd % 6;
      const int gb = sgb[((lx >> 2) << 2) | ((ly >> 2) << 1) | (lz >> 2)];
      const int cell = ((lx & 3) << 4) | ((ly & 3) << 2) | (lz & 3);
      sg[nd] = gb >= 0 ? d.grid[(long long)gb * 64 + cell] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncthreads();
    const int start = d.bk_start[b];
    const int cnt = (int)max(0ll, min((long long)d.bk_count[b], P.n - start));
    for (int s = start + chunk * kP2GAdjThreads + threadIdx.x; s < start + cnt;
         s += kc * kP2GAdjThreads) {
      const int p = d.perm[s];
      const MatParams mp = d.mats[min(max(iin[iidx(IC_MAT, p)], 0), kMaxMaterials - 1)];
      float x[3], v[3], C[9], F[9], Sv[6];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        x[k] = pin[pidx((CH_X + k), p)];
        v[k] = pin[pidx((CH_V + k), p)];
      }
#pragma unroll
      for (int k = 0; k < 9; ++k) {
        C[k] = pin[pidx((CH_C + k), p)];
        F[k] = pin[pidx((CH_F + k), p)];
      }
#pragma unroll
      for (int k = 0; k < 6; ++k) Sv[k] = pin[pidx((CH_S + k), p)];
      const float mass = pin[pidx(CH_M, p)], vol = pin[pidx(CH_VOL, p)];
      float mu = mp.mu, lam = mp.lam;
      if (lame) {
        mu = pin[pidx(CH_MU, p)];
        lam = pin[pidx(CH_LAM, p)];
      }
      const float kk = -dt * Dinv;
      const float A[9] = {mass * C[0] + kk * Sv[0], mass * C[1] + kk * Sv[3],
                          mass * C[2] + kk * Sv[4], mass * C[3] + kk * Sv[3],
                          mass * C[4] + kk * Sv[1], mass * C[5] + kk * Sv[5],
                          mass * C[6] + kk * Sv[4], mass * C[7] + kk * Sv[5],
                          mass * C[8] + kk * Sv[2]};
      const Stencil1 s0 = stencil1(x[0], inv_dx), s1 = stencil1(x[1], inv_dx),
                     s2 = stencil1(x[2], inv_dx);
      const int l0 = s0.base - K[0], l1 = s1.base - K[1], l2 = s2.base - K[2];
      float vbar[3] = {0.f, 0.f, 0.f}, Ab[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      float gx[3] = {0.f, 0.f, 0.f};
      if ((unsigned)l0 > 3u || (unsigned)l1 > 3u || (unsigned)l2 > 3u) {
        atomicOr(&d.cnt->status, ST_STENCIL);
      } else {
        // node sums as stencil moments of (m-bar, mv-bar): with
        //   u_n = m-bar_n m + mv-bar_n . (m v + A xx_n),
        // v-bar_a = sum W mv-bar_a, A-bar_ab = sum W mv-bar_a xx_b and
        // x-bar_a = sum dW_a u_n - sum W (A^T mv-bar_n)_a
        AdjMoments M;
        const AxisFactors A0 = axis_factors(s0, dx, inv_dx), A1 = axis_factors(s1, dx, inv_dx),
                          A2 = axis_factors(s2, dx, inv_dx);
        adj_moments<true>(sg, l0, l1, l2, A0, A1, A2, M);
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          vbar[a] = M.W[a];
#pragma unroll
          for (int bb = 0; bb < 3; ++bb) Ab[a * 3 + bb] = M.X[bb][a];
        }
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          float t = mass * M.Dm[a];
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            t = fmaf(mass * v[c], M.D[a][c], t);
            t = fmaf(-A[c * 3 + a], M.W[c], t);
#pragma unroll
            for (int bb = 0; bb < 3; ++bb) t = fmaf(A[c * 3 + bb], M.DX[a][bb][c], t);
          }
          gx[a] = t;
        }
      }
      // tau-bar = -dt Dinv vol A-bar; stress adjoint
      float tb[9], Fb[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) {
        tb[k] = -dt * Dinv * vol * Ab[k];
        Fb[k] = ap[(AJ_F + k) * n + p];
      }
      float mub = 0.f, lamb = 0.f;
      if (mp.type == MPM_FCR)
        fcr_vjp(mu, lam, F, tb, Fb, mub, lamb);
      else if (mp.type == MPM_NHK)
        nhk_vjp(mu, lam, F, tb, Fb, mub, lamb);
      else if (mp.type == MPM_STVK)
        hencky_vjp(mu, lam, F, tb, Fb, mub, lamb);
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        ap[(AJ_X + k) * n + p] += gx[k];
        ap[(AJ_V + k) * n + p] = mass * vbar[k];
      }
#pragma unroll
      for (int k = 0; k < 9; ++k) {
        ap[(AJ_C + k) * n + p] = mass * Ab[k];
        ap[(AJ_F + k) * n + p] = Fb[k];
      }
      ap[AJ_J * n + p] = 0.0f;
      const int id = iin[iidx(IC_ID, p)];
      gmu[id] += mub;
      glam[id] += lamb;
    }
    __syncthreads();
  }
}

// CTAs per particle block of the per-particle adjoint kernels: a scene of
// few blocks (about 400 particles each) spreads each block over several CTAs
// so that the launch's CTAs all have work; the results do not depend on it.
int adjoint_chunks(const DevPtrs &d, long long n) {
  const long long want = (long long)d.num_sms * 4 * 384;
  return (int)std::min<long long>(8, std::max<long long>(1, (want + n - 1) / std::max(n, 1ll)));
}

}  // namespace

void launch_g2p_adjoint(const DevPtrs &d, int cur, const float *an, float *ap, float *gmu,
                        float *glam, long long n, cudaStream_t s) {
  k_g2p_adjoint_particles<<<d.num_sms * 4, kAdjPThreads, 0, s>>>(
      d, d.pbuf[cur], d.ibuf[cur], an, ap, gmu, glam, d.adj_rec, n, adjoint_chunks(d, n));
  k_g2p_adjoint_scatter<<<d.num_sms * 4, kP2GThreads, kP2GSmem, s>>>(d, d.adj_rec);
}

void configure_adjoint() {
  cudaFuncSetAttribute(k_g2p_adjoint_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       kP2GSmem);
}

void launch_grid_adjoint(const DevPtrs &d, cudaStream_t s) {
  k_grid_adjoint<<<d.num_sms * 8, 256, 0, s>>>(d);
}

void launch_p2g_adjoint(const DevPtrs &d, int cur, float *ap, float *gmu, float *glam, long long n,
                        cudaStream_t s) {
  k_p2g_adjoint<<<d.num_sms * 4, kP2GAdjThreads, 0, s>>>(d, d.pbuf[cur], d.ibuf[cur], ap, gmu,
                                                        glam, n, adjoint_chunks(d, n));
}

}  // namespace zsmpm
