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
#include "mpm_math.cuh"
#include "tile_scatter.cuh"
#include "zsmpm_internal.cuh"

namespace zsmpm {
namespace {


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

// P2G of one particle block (ZSParticleToZSGrid::p2g_apic, Transfer.cu:849-889):
// per particle the affine matrix A = m C - dt Dinv S (S = vol tau from the
// previous G2P); the momentum of stencil node o is W (m v + A (o - f) dx) =
// W (b + A o dx) with b = m v - dx A f.  The block's particles are staged and
// scattered into its 216-node tile by tile_scatter (tile_scatter.cuh).
__global__ void __launch_bounds__(kP2GThreads) k_p2g(DevPtrs d, const float *__restrict__ pin,
                                                     const int32_t *__restrict__ iin) {
  extern __shared__ __align__(16) unsigned char p2g_smem[];
  const TileSmem ts = tile_smem(p2g_smem);
  const SimParams &P = *d.prm;
  const long long cap = d.cap;
  const float dt = P.dt;
  const int nb = d.cnt->n_buckets;
  const int tid = threadIdx.x;

  for (int b = blockIdx.x; b < nb; b += gridDim.x) {
    tile_zero(ts);
    const int dir = d.bk_dir[b];
    const SceneParams &S = d.scn[scene_of_dir(d, dir)];
    const float dx = S.dx, inv_dx = S.inv_dx, Dinv = S.Dinv;
    int K[3];
    bucket_origin(S, dir - S.dir_off, K);
    const int start = d.bk_start[b];
    const int cnt = (int)max(0ll, min((long long)d.bk_count[b], P.n - start));
    for (int c0 = 0; c0 < cnt; c0 += kP2GChunk) {
      const int nc = min(kP2GChunk, cnt - c0);
      __syncthreads();  // the previous chunk consumed
      for (int j = tid; j < nc; j += kP2GThreads) {
        const int p = d.perm[start + c0 + j];
        float x[3], v[3], C[9], Sv[6];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          x[k] = pin[(CH_X + k) * cap + p];
          v[k] = pin[(CH_V + k) * cap + p];
        }
#pragma unroll
        for (int k = 0; k < 9; ++k) C[k] = pin[(CH_C + k) * cap + p];
#pragma unroll
        for (int k = 0; k < 6; ++k) Sv[k] = pin[(CH_S + k) * cap + p];
        float mass = pin[CH_M * cap + p];
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
        const int cell = d.pkey[p] & 63;
        if ((unsigned)l0 > 3u || (unsigned)l1 > 3u || (unsigned)l2 > 3u ||
            ((l0 << 4) | (l1 << 2) | l2) != cell) {
          atomicOr(&d.cnt->status, ST_STENCIL);
          mass = 0.0f;
#pragma unroll
          for (int k = 0; k < 9; ++k) A[k] = 0.0f;
          v[0] = v[1] = v[2] = 0.0f;
        }
        const float f[3] = {s0.f, s1.f, s2.f};
        const float fdx0 = s0.f * dx, fdx1 = s1.f * dx, fdx2 = s2.f * dx;
        const float bv[3] = {mass * v[0] - (A[0] * fdx0 + A[1] * fdx1 + A[2] * fdx2),
                             mass * v[1] - (A[3] * fdx0 + A[4] * fdx1 + A[5] * fdx2),
                             mass * v[2] - (A[6] * fdx0 + A[7] * fdx1 + A[8] * fdx2)};
        tile_stage(ts, j, mass, bv, A, f, cell);
      }
      __syncthreads();
      tile_cell_ranges(ts, nc);
      __syncthreads();
      tile_scatter(ts, dx);
    }
    __syncthreads();
    tile_store(ts, d.ptile + (long long)b * kTileNodes);
    __syncthreads();
  }
}

// Grid node sums from the P2G tiles: node (l0, l1, l2) of grid block G lies
// in the tile of particle block G - o (o in {0, 1}^3, in blocks) at tile
// coordinate l + 4 o when that is < 6.  The <= 8 tiles are added in the fixed
// order o = (0,0,0), (0,0,1), ..., so the sums are reproducible.  mode bit 1
// applies UpdateZSGrid and bit 2 ApplyBoundaryOnZSGrid to the sum.
__device__ __forceinline__ void update_node(const SceneParams &S, float dt, int mode, int ldir,
                                            int cell, float4 &g, float &vmax);

__global__ void k_grid_gather(DevPtrs d, int mode) {
  const SimParams &P = *d.prm;
  const long long n = (long long)min(d.cnt->n_gblocks, d.cap_gblocks) * 64;
  float vmax = 0.0f;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
       idx += (long long)gridDim.x * blockDim.x) {
    const int gb = (int)(idx >> 6), cell = (int)(idx & 63);
    const int gdir = d.gb_dir[gb];
    const SceneParams &S = d.scn[scene_of_dir(d, gdir)];
    const int dy = S.block_dims[1], dz = S.block_dims[2];
    const int ldir = gdir - S.dir_off;
    const int c0 = ldir / (dz * dy), c1 = (ldir / dz) % dy, c2 = ldir % dz;
    const int l0 = cell >> 4, l1 = (cell >> 2) & 3, l2 = cell & 3;
    float4 g = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int o = 0; o < 8; ++o) {
      const int o0 = o >> 2, o1 = (o >> 1) & 1, o2 = o & 1;
      if ((o0 && (l0 >= 2 || c0 < 1)) || (o1 && (l1 >= 2 || c1 < 1)) ||
          (o2 && (l2 >= 2 || c2 < 1)))
        continue;
      const int bk = d.dir_bk[gdir - (o0 * dy + o1) * dz - o2];
      if (bk < 0) continue;
      const float4 t = d.ptile[(long long)bk * kTileNodes +
                               ((l0 + 4 * o0) * 6 + (l1 + 4 * o1)) * 6 + (l2 + 4 * o2)];
      g.x += t.x;
      g.y += t.y;
      g.z += t.z;
      g.w += t.w;
    }
    if (g.x != 0.0f) update_node(S, P.dt, mode, ldir, cell, g, vmax);
    d.grid[idx] = g;
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
// the analytic box walls: a node is in the lower wall of axis a when
// I_a < lo_a + thickness and in the upper wall when I_a > hi_a - thickness;
// sticky sets v = 0, slip removes the wall-normal component, separate removes
// it only when it points into the wall (collider velocity 0).
__device__ __forceinline__ void update_node(const SceneParams &S, float dt, int mode, int ldir,
                                            int cell, float4 &g, float &vmax) {
  if (mode & 1) {
    const float r = 1.0f / g.x;
    g.y = g.y * r + S.gravity[0] * dt;
    g.z = g.z * r + S.gravity[1] * dt;
    g.w = g.w * r + S.gravity[2] * dt;
    vmax = fmaxf(vmax, g.y * g.y + g.z * g.z + g.w * g.w);
  }
  if ((mode & 2) && S.bc_type != MPM_BC_NONE) {
    const int dz = S.block_dims[2], dy = S.block_dims[1];
    const int I[3] = {((ldir / (dz * dy)) + S.block_lo[0]) * 4 + (cell >> 4),
                      (((ldir / dz) % dy) + S.block_lo[1]) * 4 + ((cell >> 2) & 3),
                      ((ldir % dz) + S.block_lo[2]) * 4 + (cell & 3)};
    float vel[3] = {g.y, g.z, g.w};
    bool any = false;
    const int t = S.bc_thickness;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const bool lower = I[a] < S.bc_lo[a] + t, upper = I[a] > S.bc_hi[a] - t;
      if (!(lower || upper)) continue;
      any = true;
      if (S.bc_type == MPM_BC_SLIP) vel[a] = 0.0f;
      if (S.bc_type == MPM_BC_SEPARATE) {
        if (lower && vel[a] < 0.0f) vel[a] = 0.0f;
        if (upper && vel[a] > 0.0f) vel[a] = 0.0f;
      }
    }
    if (any && S.bc_type == MPM_BC_STICKY) vel[0] = vel[1] = vel[2] = 0.0f;
    g.y = vel[0];
    g.z = vel[1];
    g.w = vel[2];
  }
}

__global__ void k_grid_update(DevPtrs d, int mode) {
  const SimParams &P = *d.prm;
  const long long n = (long long)min(d.cnt->n_gblocks, d.cap_gblocks) * 64;
  float vmax = 0.0f;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
       idx += (long long)gridDim.x * blockDim.x) {
    float4 g = d.grid[idx];
    if (g.x == 0.0f) continue;
    const int gdir = d.gb_dir[idx >> 6];
    const SceneParams &S = d.scn[scene_of_dir(d, gdir)];
    update_node(S, P.dt, mode, gdir - S.dir_off, (int)(idx & 63), g, vmax);
    d.grid[idx] = g;
  }
  if (mode & 1) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
    if ((threadIdx.x & 31) == 0 && vmax > 0.0f)
      atomicMax(&d.cnt->max_vel_sqr_bits, __float_as_uint(vmax));
  }
}

template <bool kFuseRM, bool kFuseBin, int NT>
__global__ void __launch_bounds__(NT)
    k_g2p(DevPtrs d, const float *__restrict__ pin, const int32_t *__restrict__ iin,
          float *__restrict__ pout, int32_t *__restrict__ iout) {
  __shared__ float sv[3][kNodes];
  __shared__ int sgb[8];
  const SimParams &P = *d.prm;
  const long long cap = d.cap;
  const float dt = P.dt;
  const int nb = d.cnt->n_buckets;
  const bool lame = P.has_lame != 0;
  for (int b = blockIdx.x; b < nb; b += gridDim.x) {
    const int dir = d.bk_dir[b];
    const SceneParams &S = d.scn[scene_of_dir(d, dir)];
    const float dx = S.dx, inv_dx = S.inv_dx, Dinv = S.Dinv;
    if (threadIdx.x < 8) sgb[threadIdx.x] = neighbour_gb(d, S, dir, threadIdx.x);
    int K[3];
    bucket_origin(S, dir - S.dir_off, K);
    __syncthreads();
    for (int nd = threadIdx.x; nd < kNodes; nd += NT) {
      const int lx = nd / 36, ly = (nd / 6) % 6, lz = nd % 6;
      const int gb = sgb[((lx >> 2) << 2) | ((ly >> 2) << 1) | (lz >> 2)];
      const int cell = ((lx & 3) << 4) | ((ly & 3) << 2) | (lz & 3);
      const float4 g =
          gb >= 0 ? d.grid[(long long)gb * 64 + cell] : make_float4(0.f, 0.f, 0.f, 0.f);
      sv[0][nd] = g.y;
      sv[1][nd] = g.z;
      sv[2][nd] = g.w;
    }
    __syncthreads();
    const int start = d.bk_start[b];
    const int cnt = (int)max(0ll, min((long long)d.bk_count[b], P.n - start));
    // warp-uniform trip count: the fused binning below is a warp collective
    for (int sbase = start; sbase < start + cnt; sbase += NT) {
      const int s = sbase + (int)threadIdx.x;
      const bool live = s < start + cnt;
      const unsigned mask = __ballot_sync(0xffffffffu, live);
      if (!mask) continue;
      if (!live) continue;  // live lanes are exactly `mask`
      const int p = d.perm[s];
      const int mid = min(max(iin[IC_MAT * cap + p], 0), kMaxMaterials - 1);
      const MatParams mp = d.mats[mid];
      float x[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) x[k] = pin[(CH_X + k) * cap + p];
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
        for (int q = 0; q < 3; ++q) {
          xi[q] = ((float)q - s0.f) * dx;
          xj[q] = ((float)q - s1.f) * dx;
          xk[q] = ((float)q - s2.f) * dx;
          wxk[q] = s2.w[q] * xk[q];
          wyj[q] = s1.w[q] * xj[q];
        }
        float cx[3] = {0.f, 0.f, 0.f}, cy[3] = {0.f, 0.f, 0.f}, cz[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          float S[3] = {0.f, 0.f, 0.f}, Sj[3] = {0.f, 0.f, 0.f}, Sk[3] = {0.f, 0.f, 0.f};
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            const int row = ((l0 + i) * 6 + (l1 + j)) * 6 + l2;
            float t[3] = {0.f, 0.f, 0.f}, tk[3] = {0.f, 0.f, 0.f};
#pragma unroll
            for (int kk = 0; kk < 3; ++kk) {
              const int nd = row + kk;
              const float g[3] = {sv[0][nd], sv[1][nd], sv[2][nd]};
#pragma unroll
              for (int a = 0; a < 3; ++a) {
                t[a] = fmaf(s2.w[kk], g[a], t[a]);
                tk[a] = fmaf(wxk[kk], g[a], tk[a]);
              }
            }
#pragma unroll
            for (int a = 0; a < 3; ++a) {
              S[a] = fmaf(s1.w[j], t[a], S[a]);
              Sj[a] = fmaf(wyj[j], t[a], Sj[a]);
              Sk[a] = fmaf(s1.w[j], tk[a], Sk[a]);
            }
          }
          const float wxi = s0.w[i] * xi[i];
#pragma unroll
          for (int a = 0; a < 3; ++a) {
            vel[a] = fmaf(s0.w[i], S[a], vel[a]);
            cx[a] = fmaf(wxi, S[a], cx[a]);
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
        mu = pin[CH_MU * cap + p];
        lam = pin[CH_LAM * cap + p];
      }
      if (mp.type == MPM_EOS) {
        J = pin[CH_J * cap + p] * (1.0f + dt * (Cn[0] + Cn[4] + Cn[8]));
        const float c = cbrtf(J);
#pragma unroll
        for (int k = 0; k < 9; ++k) F[k] = (k % 4 == 0) ? c : 0.0f;
        ok_state = kirchhoff(MPM_EOS, mu, lam, mp.bulk, mp.gamma, F, J, tau);
      } else {
        float Fo[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) Fo[k] = pin[(CH_F + k) * cap + p];
        // F <- (I + dt C) F
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int c = 0; c < 3; ++c)
            F[r * 3 + c] = Fo[r * 3 + c] + dt * (Cn[r * 3 + 0] * Fo[c] + Cn[r * 3 + 1] * Fo[3 + c] +
                                                 Cn[r * 3 + 2] * Fo[6 + c]);
        if (kFuseRM && mp.plastic == MPM_PLASTIC_NADP)
          ok_state = project_dp(mu, lam, mp.alpha, F, tau) >= 0;
        else
          ok_state = kirchhoff(mp.type, mu, lam, mp.bulk, mp.gamma, F, 1.0f, tau);
        J = det3(F);
      }
      if (!ok_state) atomicOr(&d.cnt->status, ST_NAN);
      const float vol = pin[CH_VOL * cap + p];
      bool finite = isfinite(x[0]) && isfinite(x[1]) && isfinite(x[2]) && isfinite(J);
#pragma unroll
      for (int k = 0; k < 9; ++k) finite = finite && isfinite(F[k]);
      if (!finite) atomicOr(&d.cnt->status, ST_NAN);
      // next buffer: sorted position s, or the particle's own slot p in the
      // differentiable mode (every state then shares the upload order)
      const int so = d.keep_order ? p : s;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        pout[(CH_X + k) * cap + so] = x[k];
        pout[(CH_V + k) * cap + so] = vel[k];
      }
#pragma unroll
      for (int k = 0; k < 9; ++k) {
        pout[(CH_C + k) * cap + so] = Cn[k];
        pout[(CH_F + k) * cap + so] = F[k];
      }
      pout[CH_J * cap + so] = J;
      pout[CH_M * cap + so] = pin[CH_M * cap + p];
      pout[CH_VOL * cap + so] = vol;
      pout[(CH_S + 0) * cap + so] = vol * tau.xx;
      pout[(CH_S + 1) * cap + so] = vol * tau.yy;
      pout[(CH_S + 2) * cap + so] = vol * tau.zz;
      pout[(CH_S + 3) * cap + so] = vol * tau.xy;
      pout[(CH_S + 4) * cap + so] = vol * tau.xz;
      pout[(CH_S + 5) * cap + so] = vol * tau.yz;
      if (lame) {
        pout[CH_MU * cap + so] = pin[CH_MU * cap + p];
        pout[CH_LAM * cap + so] = pin[CH_LAM * cap + p];
      }
      iout[IC_MAT * cap + so] = mid;
      iout[IC_ID * cap + so] = iin[IC_ID * cap + p];
      if (kFuseBin) {
        // key of the new position for the next partition (storage slot s)
        const int key = bin_key(S, x[0], x[1], x[2], &d.cnt->status);
        d.pkey[so] = key;
        bin_count(d, S, key, mask);
      }
    }
    __syncthreads();
  }
}

__device__ __forceinline__ void store_stress(float *__restrict__ pb, long long cap, long long p,
                                             float vol, const Sym3 &t) {
  pb[(CH_S + 0) * cap + p] = vol * t.xx;
  pb[(CH_S + 1) * cap + p] = vol * t.yy;
  pb[(CH_S + 2) * cap + p] = vol * t.zz;
  pb[(CH_S + 3) * cap + p] = vol * t.xy;
  pb[(CH_S + 4) * cap + p] = vol * t.xz;
  pb[(CH_S + 5) * cap + p] = vol * t.yz;
}

// ZSReturnMapping as its own pass (in place, storage order); refreshes the
// stored stress of every projected particle.
__global__ void k_return_mapping(DevPtrs d, float *__restrict__ pbuf,
                                 const int32_t *__restrict__ ibuf) {
  const SimParams &P = *d.prm;
  const long long cap = d.cap, n = P.n;
  const bool lame = P.has_lame != 0;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    const MatParams mp = d.mats[min(max(ibuf[IC_MAT * cap + p], 0), kMaxMaterials - 1)];
    if (mp.type == MPM_EOS || mp.plastic != MPM_PLASTIC_NADP) continue;
    float F[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) F[k] = pbuf[(CH_F + k) * cap + p];
    float mu = mp.mu, lam = mp.lam;
    if (lame) {
      mu = pbuf[CH_MU * cap + p];
      lam = pbuf[CH_LAM * cap + p];
    }
    Sym3 tau;
    const int r = project_dp(mu, lam, mp.alpha, F, tau);
    if (r < 0) atomicOr(&d.cnt->status, ST_NAN);
    if (r > 0) {
#pragma unroll
      for (int k = 0; k < 9; ++k) pbuf[(CH_F + k) * cap + p] = F[k];
      pbuf[CH_J * cap + p] = det3(F);
      store_stress(pbuf, cap, p, pbuf[CH_VOL * cap + p], tau);
    }
  }
}

// S = vol * tau of every particle from its current F (or J): the stress P2G
// reads, recomputed after an upload or a change of materials.
__global__ void k_stress(DevPtrs d, float *__restrict__ pbuf, const int32_t *__restrict__ ibuf) {
  const SimParams &P = *d.prm;
  const long long cap = d.cap, n = P.n;
  const bool lame = P.has_lame != 0;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    const MatParams mp = d.mats[min(max(ibuf[IC_MAT * cap + p], 0), kMaxMaterials - 1)];
    float F[9];
    float J = 1.0f;
    if (mp.type == MPM_EOS) {
      J = pbuf[CH_J * cap + p];
#pragma unroll
      for (int k = 0; k < 9; ++k) F[k] = (k % 4 == 0) ? 1.0f : 0.0f;
    } else {
#pragma unroll
      for (int k = 0; k < 9; ++k) F[k] = pbuf[(CH_F + k) * cap + p];
    }
    float mu = mp.mu, lam = mp.lam;
    if (lame) {
      mu = pbuf[CH_MU * cap + p];
      lam = pbuf[CH_LAM * cap + p];
    }
    Sym3 tau;
    if (!kirchhoff(mp.type, mu, lam, mp.bulk, mp.gamma, F, J, tau))
      atomicOr(&d.cnt->status, ST_NAN);
    store_stress(pbuf, cap, p, pbuf[CH_VOL * cap + p], tau);
  }
}

}  // namespace

template <int NT> int g2p_occupancy() {
  int b = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_g2p<true, true, NT>, NT, 0);
  return b > 0 ? b : 1;
}

void configure_launches(DevPtrs &d) {
  int a = 0;
  cudaFuncSetAttribute(k_p2g, cudaFuncAttributeMaxDynamicSharedMemorySize, kP2GSmem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_p2g, kP2GThreads, kP2GSmem);
  a = a > 0 ? a : 1;
  const LaunchConfig &L = d.launch;
  const int gt = L.g2p_threads == 256 ? 256 : 128;
  const int g = gt == 256 ? g2p_occupancy<256>() : g2p_occupancy<128>();
  d.grid_p2g = d.num_sms * (L.p2g_ctas_per_sm > 0 ? std::min(L.p2g_ctas_per_sm, a) : a);
  d.grid_g2p = d.num_sms * (L.g2p_ctas_per_sm > 0 ? std::min(L.g2p_ctas_per_sm, g) : g);
  d.grid_sort = d.num_sms * (L.sort_ctas_per_sm > 0 ? L.sort_ctas_per_sm : 8);
  d.grid_stream = d.num_sms * (L.stream_ctas_per_sm > 0 ? L.stream_ctas_per_sm : 8);
  d.g2p_threads = gt;
}

void launch_p2g(const DevPtrs &d, int cur, cudaStream_t s) {
  k_p2g<<<d.grid_p2g, kP2GThreads, kP2GSmem, s>>>(d, d.pbuf[cur], d.ibuf[cur]);
}

void launch_grid_gather(const DevPtrs &d, int mode, cudaStream_t s) {
  k_grid_gather<<<d.grid_stream, 256, 0, s>>>(d, mode);
}

void launch_grid_update(const DevPtrs &d, int mode, cudaStream_t s) {
  k_grid_update<<<d.num_sms * 8, 256, 0, s>>>(d, mode);
}

template <int NT>
void launch_g2p_nt(const DevPtrs &d, int cur, int fuse_rm, int fuse_bin, cudaStream_t s) {
  const int grid = d.grid_g2p;
  float *pi = d.pbuf[cur], *po = d.pbuf[1 - cur];
  int32_t *ii = d.ibuf[cur], *io = d.ibuf[1 - cur];
  if (fuse_rm && fuse_bin)
    k_g2p<true, true, NT><<<grid, NT, 0, s>>>(d, pi, ii, po, io);
  else if (fuse_rm)
    k_g2p<true, false, NT><<<grid, NT, 0, s>>>(d, pi, ii, po, io);
  else
    k_g2p<false, false, NT><<<grid, NT, 0, s>>>(d, pi, ii, po, io);
}

void launch_g2p(const DevPtrs &d, int cur, int fuse_rm, int fuse_bin, cudaStream_t s) {
  if (d.g2p_threads == 256)
    launch_g2p_nt<256>(d, cur, fuse_rm, fuse_bin, s);
  else
    launch_g2p_nt<128>(d, cur, fuse_rm, fuse_bin, s);
}

void launch_return_mapping(const DevPtrs &d, int cur, cudaStream_t s) {
  k_return_mapping<<<d.num_sms * 8, 256, 0, s>>>(d, d.pbuf[cur], d.ibuf[cur]);
}

void launch_stress(const DevPtrs &d, int cur, cudaStream_t s) {
  k_stress<<<d.num_sms * 8, 256, 0, s>>>(d, d.pbuf[cur], d.ibuf[cur]);
}

}  // namespace zsmpm
