// Particle-to-grid, grid update + boundary, grid-to-particle.
//
// One CTA owns one particle block at a time (particles sorted by block, see
// partition.cu).  A block's quadratic stencils all fall in the 6^3 nodes
// [K, K+6) of its block key K, which lie in the 2x2x2 grid blocks K + {0,4}^3:
//  * P2G (Transfer.cu:849-889) accumulates the 27-node APIC scatter of the
//    block's particles into those 216 nodes in shared memory and flushes
//    each node once with a vector float4 atomic, instead of the reference's
//    27 x 4 global float atomics per particle.
//  * G2P (Transfer.cu:1139-1173) stages the 216 node velocities in shared
//    memory and gathers from there; it writes the particle's new state into
//    the other particle buffer at its sorted position, so storage follows
//    the block order from one substep to the next.
#include <cuda_runtime.h>

#include "mpm_math.cuh"
#include "zsmpm_internal.cuh"

namespace zsmpm {
namespace {

constexpr int kP2GThreads = 128;
constexpr int kG2PThreads = 128;
constexpr int kNodes = 216;  // 6^3

__device__ __forceinline__ void bucket_origin(const SimParams &P, int dir, int (&K)[3]) {
  const int dz = P.block_dims[2], dy = P.block_dims[1];
  const int c2 = dir % dz, c1 = (dir / dz) % dy, c0 = dir / (dz * dy);
  K[0] = (c0 + P.block_lo[0]) * 4;
  K[1] = (c1 + P.block_lo[1]) * 4;
  K[2] = (c2 + P.block_lo[2]) * 4;
}

// grid block of each of the 2x2x2 blocks around particle block `dir`
__device__ __forceinline__ int neighbour_gb(const DevPtrs &d, const SimParams &P, int dir,
                                            int t) {
  const int dz = P.block_dims[2], dy = P.block_dims[1];
  return d.dir_gb[dir + ((t >> 2) * dy + ((t >> 1) & 1)) * dz + (t & 1)];
}

__global__ void __launch_bounds__(kP2GThreads) k_p2g(DevPtrs d, const float *__restrict__ pin,
                                                     const int32_t *__restrict__ iin) {
  __shared__ float sm[4][kNodes];
  __shared__ int sgb[8];
  const SimParams &P = *d.prm;
  const long long cap = d.cap;
  const float dt = P.dt, dx = P.dx, inv_dx = P.inv_dx, Dinv = P.Dinv;
  const int nb = d.cnt->n_buckets;
  const bool lame = P.has_lame != 0;
  for (int b = blockIdx.x; b < nb; b += gridDim.x) {
    for (int i = threadIdx.x; i < 4 * kNodes; i += kP2GThreads) (&sm[0][0])[i] = 0.0f;
    const int dir = d.bk_dir[b];
    if (threadIdx.x < 8) sgb[threadIdx.x] = neighbour_gb(d, P, dir, threadIdx.x);
    int K[3];
    bucket_origin(P, dir, K);
    __syncthreads();
    const int start = d.bk_start[b];
    const int cnt = (int)max(0ll, min((long long)d.bk_count[b], P.n - start));
    for (int s = start + threadIdx.x; s < start + cnt; s += kP2GThreads) {
      const int p = d.perm[s];
      const int mid = min(max(iin[IC_MAT * cap + p], 0), kMaxMaterials - 1);
      const MatParams mp = d.mats[mid];
      float x[3], v[3], C[9], F[9];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        x[k] = pin[(CH_X + k) * cap + p];
        v[k] = pin[(CH_V + k) * cap + p];
      }
#pragma unroll
      for (int k = 0; k < 9; ++k) C[k] = pin[(CH_C + k) * cap + p];
      const float mass = pin[CH_M * cap + p], vol = pin[CH_VOL * cap + p];
      float Jeos = 1.0f;
      if (mp.type == MPM_EOS) {
        Jeos = pin[CH_J * cap + p];
#pragma unroll
        for (int k = 0; k < 9; ++k) F[k] = (k % 4 == 0) ? 1.0f : 0.0f;
      } else {
#pragma unroll
        for (int k = 0; k < 9; ++k) F[k] = pin[(CH_F + k) * cap + p];
      }
      float mu = mp.mu, lam = mp.lam;
      if (lame) {
        mu = pin[CH_MU * cap + p];
        lam = pin[CH_LAM * cap + p];
      }
      Sym3 tau;
      if (!kirchhoff(mp.type, mu, lam, mp.bulk, mp.gamma, F, Jeos, tau))
        atomicOr(&d.cnt->status, ST_NAN);
      // A = m C - dt Dinv vol tau: momentum of node i is W (m v + A (x_i - x_p))
      const float k = -dt * Dinv * vol;
      float A[9];
      A[0] = mass * C[0] + k * tau.xx;
      A[1] = mass * C[1] + k * tau.xy;
      A[2] = mass * C[2] + k * tau.xz;
      A[3] = mass * C[3] + k * tau.xy;
      A[4] = mass * C[4] + k * tau.yy;
      A[5] = mass * C[5] + k * tau.yz;
      A[6] = mass * C[6] + k * tau.xz;
      A[7] = mass * C[7] + k * tau.yz;
      A[8] = mass * C[8] + k * tau.zz;
      const Stencil1 s0 = stencil1(x[0], inv_dx), s1 = stencil1(x[1], inv_dx),
                     s2 = stencil1(x[2], inv_dx);
      const int l0 = s0.base - K[0], l1 = s1.base - K[1], l2 = s2.base - K[2];
      if ((unsigned)l0 > 3u || (unsigned)l1 > 3u || (unsigned)l2 > 3u) {
        atomicOr(&d.cnt->status, ST_STENCIL);
        continue;
      }
      const float mv0 = mass * v[0], mv1 = mass * v[1], mv2 = mass * v[2];
      // Particles are sorted by cell, so ~8 neighbouring lanes share one
      // stencil.  Each lane walks the 27 nodes in its own rotated order
      // (axis offsets shifted by the base-3 digits of lane % 27), so lanes of
      // one cell update different nodes at every step instead of serialising
      // on the same shared-memory word.
      const int rot = (threadIdx.x & 31) % 27;
      int o0[3], o1[3], o2[3];
      float w0[3], w1[3], w2[3];
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        o0[q] = (q + rot % 3) % 3;
        o1[q] = (q + (rot / 3) % 3) % 3;
        o2[q] = (q + rot / 9) % 3;
        w0[q] = o0[q] == 0 ? s0.w[0] : (o0[q] == 1 ? s0.w[1] : s0.w[2]);
        w1[q] = o1[q] == 0 ? s1.w[0] : (o1[q] == 1 ? s1.w[1] : s1.w[2]);
        w2[q] = o2[q] == 0 ? s2.w[0] : (o2[q] == 1 ? s2.w[1] : s2.w[2]);
      }
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const float xi = ((float)o0[i] - s0.f) * dx;
        const float a0 = mv0 + A[0] * xi, a1 = mv1 + A[3] * xi, a2 = mv2 + A[6] * xi;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const float xj = ((float)o1[j] - s1.f) * dx;
          const float b0 = a0 + A[1] * xj, b1 = a1 + A[4] * xj, b2 = a2 + A[7] * xj;
          const float wij = w0[i] * w1[j];
          const int row = ((l0 + o0[i]) * 6 + (l1 + o1[j])) * 6 + l2;
#pragma unroll
          for (int kk = 0; kk < 3; ++kk) {
            const float xk = ((float)o2[kk] - s2.f) * dx;
            const float W = wij * w2[kk];
            const int nd = row + o2[kk];
            atomicAdd(&sm[0][nd], W * mass);
            atomicAdd(&sm[1][nd], W * (b0 + A[2] * xk));
            atomicAdd(&sm[2][nd], W * (b1 + A[5] * xk));
            atomicAdd(&sm[3][nd], W * (b2 + A[8] * xk));
          }
        }
      }
    }
    __syncthreads();
    for (int nd = threadIdx.x; nd < kNodes; nd += kP2GThreads) {
      const float4 val = make_float4(sm[0][nd], sm[1][nd], sm[2][nd], sm[3][nd]);
      if (val.x != 0.0f || val.y != 0.0f || val.z != 0.0f || val.w != 0.0f) {
        const int lx = nd / 36, ly = (nd / 6) % 6, lz = nd % 6;
        const int gb = sgb[((lx >> 2) << 2) | ((ly >> 2) << 1) | (lz >> 2)];
        const int cell = ((lx & 3) << 4) | ((ly & 3) << 2) | (lz & 3);
        if (gb >= 0) atomicAdd(&d.grid[(long long)gb * 64 + cell], val);
      }
    }
    __syncthreads();
  }
}

// UpdateZSGrid (MPMPipeline.cu:852-877): v = mv / m + g dt where m != 0,
// running max of |v|^2; then ApplyBoundaryOnZSGrid (Boundary.cu:105-116) with
// the analytic box walls (see the oracle's apply_bc for the same rule).
__global__ void k_grid_update(DevPtrs d, int mode) {
  const SimParams &P = *d.prm;
  const long long n = (long long)min(d.cnt->n_gblocks, d.cap_gblocks) * 64;
  const float dt = P.dt;
  float vmax = 0.0f;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
       idx += (long long)gridDim.x * blockDim.x) {
    float4 g = d.grid[idx];
    if (g.x == 0.0f) continue;
    if (mode & 1) {
      const float r = 1.0f / g.x;
      g.y = g.y * r + P.gravity[0] * dt;
      g.z = g.z * r + P.gravity[1] * dt;
      g.w = g.w * r + P.gravity[2] * dt;
      vmax = fmaxf(vmax, g.y * g.y + g.z * g.z + g.w * g.w);
    }
    if ((mode & 2) && P.bc_type != MPM_BC_NONE) {
      const int gb = (int)(idx >> 6), cell = (int)(idx & 63);
      const int dir = d.gb_dir[gb];
      const int dz = P.block_dims[2], dy = P.block_dims[1];
      const int I[3] = {((dir / (dz * dy)) + P.block_lo[0]) * 4 + (cell >> 4),
                        (((dir / dz) % dy) + P.block_lo[1]) * 4 + ((cell >> 2) & 3),
                        ((dir % dz) + P.block_lo[2]) * 4 + (cell & 3)};
      float vel[3] = {g.y, g.z, g.w};
      bool any = false;
      const int t = P.bc_thickness;
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const bool lower = I[a] < P.bc_lo[a] + t, upper = I[a] > P.bc_hi[a] - t;
        if (!(lower || upper)) continue;
        any = true;
        if (P.bc_type == MPM_BC_SLIP) vel[a] = 0.0f;
        if (P.bc_type == MPM_BC_SEPARATE) {
          if (lower && vel[a] < 0.0f) vel[a] = 0.0f;
          if (upper && vel[a] > 0.0f) vel[a] = 0.0f;
        }
      }
      if (any && P.bc_type == MPM_BC_STICKY) vel[0] = vel[1] = vel[2] = 0.0f;
      g.y = vel[0];
      g.z = vel[1];
      g.w = vel[2];
    }
    d.grid[idx] = g;
  }
  if (mode & 1) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
    if ((threadIdx.x & 31) == 0 && vmax > 0.0f)
      atomicMax(&d.cnt->max_vel_sqr_bits, __float_as_uint(vmax));
  }
}

template <bool kFuseRM>
__global__ void __launch_bounds__(kG2PThreads)
    k_g2p(DevPtrs d, const float *__restrict__ pin, const int32_t *__restrict__ iin,
          float *__restrict__ pout, int32_t *__restrict__ iout) {
  __shared__ float sv[3][kNodes];
  __shared__ int sgb[8];
  const SimParams &P = *d.prm;
  const long long cap = d.cap;
  const float dt = P.dt, dx = P.dx, inv_dx = P.inv_dx, Dinv = P.Dinv;
  const int nb = d.cnt->n_buckets;
  const bool lame = P.has_lame != 0;
  for (int b = blockIdx.x; b < nb; b += gridDim.x) {
    const int dir = d.bk_dir[b];
    if (threadIdx.x < 8) sgb[threadIdx.x] = neighbour_gb(d, P, dir, threadIdx.x);
    int K[3];
    bucket_origin(P, dir, K);
    __syncthreads();
    for (int nd = threadIdx.x; nd < kNodes; nd += kG2PThreads) {
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
    for (int s = start + threadIdx.x; s < start + cnt; s += kG2PThreads) {
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
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          const float xi = ((float)i - s0.f) * dx;
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            const float xj = ((float)j - s1.f) * dx;
            const float wij = s0.w[i] * s1.w[j];
            const int row = ((l0 + i) * 6 + (l1 + j)) * 6 + l2;
#pragma unroll
            for (int kk = 0; kk < 3; ++kk) {
              const float xk = ((float)kk - s2.f) * dx;
              const float W = wij * s2.w[kk];
              const int nd = row + kk;
              const float g0 = sv[0][nd], g1 = sv[1][nd], g2 = sv[2][nd];
              vel[0] += W * g0;
              vel[1] += W * g1;
              vel[2] += W * g2;
              const float w0 = W * g0, w1 = W * g1, w2 = W * g2;
              Cn[0] += w0 * xi;
              Cn[1] += w0 * xj;
              Cn[2] += w0 * xk;
              Cn[3] += w1 * xi;
              Cn[4] += w1 * xj;
              Cn[5] += w1 * xk;
              Cn[6] += w2 * xi;
              Cn[7] += w2 * xj;
              Cn[8] += w2 * xk;
            }
          }
        }
      }
#pragma unroll
      for (int k = 0; k < 9; ++k) Cn[k] *= Dinv;
#pragma unroll
      for (int k = 0; k < 3; ++k) x[k] += vel[k] * dt;
      float F[9], J;
      if (mp.type == MPM_EOS) {
        J = pin[CH_J * cap + p] * (1.0f + dt * (Cn[0] + Cn[4] + Cn[8]));
        const float c = cbrtf(J);
#pragma unroll
        for (int k = 0; k < 9; ++k) F[k] = (k % 4 == 0) ? c : 0.0f;
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
        if (kFuseRM && mp.plastic == MPM_PLASTIC_NADP) {
          float mu = mp.mu, lam = mp.lam;
          if (lame) {
            mu = pin[CH_MU * cap + p];
            lam = pin[CH_LAM * cap + p];
          }
          if (project_dp(mu, lam, mp.alpha, F) < 0) atomicOr(&d.cnt->status, ST_NAN);
        }
        J = det3(F);
      }
      bool finite = isfinite(x[0]) && isfinite(x[1]) && isfinite(x[2]) && isfinite(J);
#pragma unroll
      for (int k = 0; k < 9; ++k) finite = finite && isfinite(F[k]);
      if (!finite) atomicOr(&d.cnt->status, ST_NAN);
      // next buffer, sorted position s
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        pout[(CH_X + k) * cap + s] = x[k];
        pout[(CH_V + k) * cap + s] = vel[k];
      }
#pragma unroll
      for (int k = 0; k < 9; ++k) {
        pout[(CH_C + k) * cap + s] = Cn[k];
        pout[(CH_F + k) * cap + s] = F[k];
      }
      pout[CH_J * cap + s] = J;
      pout[CH_M * cap + s] = pin[CH_M * cap + p];
      pout[CH_VOL * cap + s] = pin[CH_VOL * cap + p];
      if (lame) {
        pout[CH_MU * cap + s] = pin[CH_MU * cap + p];
        pout[CH_LAM * cap + s] = pin[CH_LAM * cap + p];
      }
      iout[IC_MAT * cap + s] = mid;
      iout[IC_ID * cap + s] = iin[IC_ID * cap + p];
    }
    __syncthreads();
  }
}

// ZSReturnMapping as its own pass (in place, storage order).
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
    const int r = project_dp(mu, lam, mp.alpha, F);
    if (r < 0) atomicOr(&d.cnt->status, ST_NAN);
    if (r > 0) {
#pragma unroll
      for (int k = 0; k < 9; ++k) pbuf[(CH_F + k) * cap + p] = F[k];
      pbuf[CH_J * cap + p] = det3(F);
    }
  }
}

}  // namespace

void launch_p2g(const DevPtrs &d, int cur, cudaStream_t s) {
  k_p2g<<<d.num_sms * 8, kP2GThreads, 0, s>>>(d, d.pbuf[cur], d.ibuf[cur]);
}

void launch_grid_update(const DevPtrs &d, int mode, cudaStream_t s) {
  k_grid_update<<<d.num_sms * 8, 256, 0, s>>>(d, mode);
}

void launch_g2p(const DevPtrs &d, int cur, int fuse_rm, cudaStream_t s) {
  if (fuse_rm)
    k_g2p<true><<<d.num_sms * 8, kG2PThreads, 0, s>>>(d, d.pbuf[cur], d.ibuf[cur],
                                                      d.pbuf[1 - cur], d.ibuf[1 - cur]);
  else
    k_g2p<false><<<d.num_sms * 8, kG2PThreads, 0, s>>>(d, d.pbuf[cur], d.ibuf[cur],
                                                       d.pbuf[1 - cur], d.ibuf[1 - cur]);
}

void launch_return_mapping(const DevPtrs &d, int cur, cudaStream_t s) {
  k_return_mapping<<<d.num_sms * 8, 256, 0, s>>>(d, d.pbuf[cur], d.ibuf[cur]);
}

}  // namespace zsmpm
