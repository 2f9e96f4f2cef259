// Boundary grids: MakeZSGrid transfer="boundary" (Generation.cu:1490-1506)
// filled from the points of a boundary mesh by ZSBoundaryPrimitiveToZSGrid
// (Transfer.cu:1532-1623) and normalised by UpdateZSGrid's boundary branch
// (MPMPipeline.cu:899-911), then applied to the simulation grid's velocities
// by ApplyGridBoundaryOnZSGrid (Boundary.cu:18-69).
//
// The boundary grid shares the context's block directory: bnd_map gives each
// directory entry its boundary block (or -1), and a boundary block holds its
// 64 nodes as (m, v) and (unit normal, 0).  It is built once per mesh (the
// points do not move with the substeps): the points' linear stencils mark
// their blocks, the marked entries are numbered, and the points add
// W m, W m v and (triangle rows) W m nrm into FP64 accumulators, which the
// last pass turns into v = mv / m and nrm = unit(m nrm).  A node that no
// triangle reached keeps a zero normal, so slip and separate leave it alone.
#include <cuda_runtime.h>

#include <algorithm>

#include "zsmpm_internal.cuh"

namespace zsmpm {
namespace {

constexpr int kBndThreads = 256;

// linear kernel: nodes base .. base + 1 per axis, base = floor(x / dx)
__device__ __forceinline__ void linear_stencil(const SceneParams &S, const float *x, int *base,
                                               double (*w)[2]) {
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float c = __fmul_rn(x[a], S.inv_dx);
    base[a] = __float2int_rd(c);
    const double f = (double)c - (double)base[a];
    w[a][0] = 1.0 - f;
    w[a][1] = f;
  }
}

// directory entry of the block of node I, or -1 outside the directory
__device__ __forceinline__ long long node_dir(const SceneParams &S, const int *I) {
  int c[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    c[a] = (I[a] >> 2) - S.block_lo[a];
    if (c[a] < 0 || c[a] >= S.block_dims[a]) return -1;
  }
  return S.dir_off + ((long long)c[0] * S.block_dims[1] + c[1]) * S.block_dims[2] + c[2];
}

__global__ void k_bnd_mark(DevPtrs d, SceneParams S, const float *__restrict__ x, long long n) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    const float xp[3] = {x[3 * p], x[3 * p + 1], x[3 * p + 2]};
    if (!(isfinite(xp[0]) && isfinite(xp[1]) && isfinite(xp[2]))) continue;
    int base[3];
    double w[3][2];
    linear_stencil(S, xp, base, w);
    for (int o = 0; o < 8; ++o) {
      const int I[3] = {base[0] + (o >> 2), base[1] + ((o >> 1) & 1), base[2] + (o & 1)};
      const long long dd = node_dir(S, I);
      if (dd >= 0) d.bnd_map[dd] = -2;
    }
  }
}

__global__ void k_bnd_index(DevPtrs d, int32_t *n_blocks) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < d.ndir;
       i += (long long)gridDim.x * blockDim.x)
    if (d.bnd_map[i] == -2) d.bnd_map[i] = atomicAdd(n_blocks, 1);
}

__global__ void k_bnd_accumulate(DevPtrs d, SceneParams S, const float *__restrict__ x,
                                 const float *__restrict__ v, const float *__restrict__ m,
                                 const float *__restrict__ nrm, long long n_verts, long long n,
                                 double *__restrict__ acc) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    const float xp[3] = {x[3 * p], x[3 * p + 1], x[3 * p + 2]};
    if (!(isfinite(xp[0]) && isfinite(xp[1]) && isfinite(xp[2]))) continue;
    int base[3];
    double w[3][2];
    linear_stencil(S, xp, base, w);
    const double mp = m[p];
    const double vp[3] = {v[3 * p], v[3 * p + 1], v[3 * p + 2]};
    const bool with_n = p >= n_verts;
    const double np_[3] = {with_n ? nrm[3 * p] : 0.0, with_n ? nrm[3 * p + 1] : 0.0,
                           with_n ? nrm[3 * p + 2] : 0.0};
    for (int o = 0; o < 8; ++o) {
      const int I[3] = {base[0] + (o >> 2), base[1] + ((o >> 1) & 1), base[2] + (o & 1)};
      const long long dd = node_dir(S, I);
      if (dd < 0) continue;
      const int bb = d.bnd_map[dd];
      const int cell = ((I[0] & 3) << 4) | ((I[1] & 3) << 2) | (I[2] & 3);
      double *a = acc + ((long long)bb * 64 + cell) * 7;
      const double W = w[0][o >> 2] * w[1][(o >> 1) & 1] * w[2][o & 1] * mp;
      atomicAdd(&a[0], W);
#pragma unroll
      for (int k = 0; k < 3; ++k) atomicAdd(&a[1 + k], W * vp[k]);
      if (with_n)
#pragma unroll
        for (int k = 0; k < 3; ++k) atomicAdd(&a[4 + k], W * np_[k]);
    }
  }
}

__global__ void k_bnd_finalize(DevPtrs d, const double *__restrict__ acc, long long nodes) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nodes;
       i += (long long)gridDim.x * blockDim.x) {
    const double *a = acc + i * 7;
    float4 mv = make_float4(0.f, 0.f, 0.f, 0.f), nn = make_float4(0.f, 0.f, 0.f, 0.f);
    if (a[0] != 0.0) {
      mv = make_float4((float)a[0], (float)(a[1] / a[0]), (float)(a[2] / a[0]), (float)(a[3] / a[0]));
      const double l = sqrt(a[4] * a[4] + a[5] * a[5] + a[6] * a[6]);
      if (l > 0.0) nn = make_float4((float)(a[4] / l), (float)(a[5] / l), (float)(a[6] / l), 0.f);
    }
    d.bnd_grid[2 * i] = mv;
    d.bnd_grid[2 * i + 1] = nn;
  }
}

// One thread per node of the active grid blocks; the node must carry mass in
// both grids.  FLIP-style grids take the boundary on vstar (Boundary.cu:36).
__global__ void k_apply_grid_boundary(DevPtrs d) {
  if (ZSMPM_HALTED(d)) return;
  const long long nn = (long long)min(d.cnt->n_gblocks, d.cap_gblocks) * 64;
  const bool apic = d.transfer == MPM_TRANSFER_APIC;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < nn;
       idx += (long long)gridDim.x * blockDim.x) {
    const int gb = (int)(idx >> 6), cell = (int)(idx & 63);
    const int bb = d.bnd_map[d.gb_dir[gb]];
    if (bb < 0) continue;
    const float4 bmv = d.bnd_grid[2 * ((long long)bb * 64 + cell)];
    if (bmv.x == 0.0f) continue;
    float4 g = d.grid[idx];
    if (g.x == 0.0f) continue;
    float4 t = apic ? g : d.grid2[idx];
    float u[3] = {apic ? t.y : t.x, apic ? t.z : t.y, apic ? t.w : t.z};
    const float bv[3] = {bmv.y, bmv.z, bmv.w};
    if (d.bnd_type == MPM_BC_STICKY) {
#pragma unroll
      for (int a = 0; a < 3; ++a) u[a] = bv[a];
    } else {
      const float4 bn = d.bnd_grid[2 * ((long long)bb * 64 + cell) + 1];
      const float nv[3] = {bn.x, bn.y, bn.z};
#pragma unroll
      for (int a = 0; a < 3; ++a) u[a] -= bv[a];
      const float proj = nv[0] * u[0] + nv[1] * u[1] + nv[2] * u[2];
      if ((d.bnd_type == MPM_BC_SEPARATE && proj < 0.0f) || d.bnd_type == MPM_BC_SLIP)
#pragma unroll
        for (int a = 0; a < 3; ++a) u[a] -= proj * nv[a];
#pragma unroll
      for (int a = 0; a < 3; ++a) u[a] += bv[a];
    }
    if (apic) {
      d.grid[idx] = make_float4(g.x, u[0], u[1], u[2]);
    } else {
      d.grid2[idx] = make_float4(u[0], u[1], u[2], t.w);
    }
  }
}

inline int grid_for(long long work, const DevPtrs &d) {
  return (int)std::max<long long>(1, std::min<long long>((work + kBndThreads - 1) / kBndThreads,
                                                         (long long)d.num_sms * 8));
}

}  // namespace

void launch_bnd_mark(const DevPtrs &d, const SceneParams &S, const float *x, long long n,
                     cudaStream_t s) {
  if (n > 0) k_bnd_mark<<<grid_for(n, d), kBndThreads, 0, s>>>(d, S, x, n);
}

void launch_bnd_index(const DevPtrs &d, int32_t *n_blocks, cudaStream_t s) {
  k_bnd_index<<<grid_for(d.ndir, d), kBndThreads, 0, s>>>(d, n_blocks);
}

void launch_bnd_accumulate(const DevPtrs &d, const SceneParams &S, const float *x, const float *v,
                           const float *m, const float *nrm, long long n_verts, long long n,
                           double *acc, cudaStream_t s) {
  if (n > 0)
    k_bnd_accumulate<<<grid_for(n, d), kBndThreads, 0, s>>>(d, S, x, v, m, nrm, n_verts, n, acc);
}

void launch_bnd_finalize(const DevPtrs &d, const double *acc, int n_blocks, cudaStream_t s) {
  const long long nodes = (long long)n_blocks * 64;
  if (nodes > 0) k_bnd_finalize<<<grid_for(nodes, d), kBndThreads, 0, s>>>(d, acc, nodes);
}

void launch_apply_grid_boundary(const DevPtrs &d, cudaStream_t s) {
  if (!d.bnd_map) return;
  k_apply_grid_boundary<<<d.num_sms * 8, kBndThreads, 0, s>>>(d);
}

}  // namespace zsmpm
