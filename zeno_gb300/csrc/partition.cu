// Particle binning and block-key sort: the GB300 form of
// ZSPartitionForZSParticles + ExpandZSPartition
// (projects/CuLagrange/mpm/MPMPipeline.cu:21-231).
//
// The reference inserts every particle's block key into a hash table with
// CAS and expands the table on the host in several synchronised passes.
// Here a dense block directory stands in for the hash table (O(1) lookup,
// no probing, 1-8 MB for the domains in use), and one substep's partition is
// four device kernels with no host read:
//   bin     per particle: key = (block << 6) | cell, warp-aggregated count;
//           the first particle of a block marks its 27-block neighbourhood
//           (the 1-ring halo).  In the fused substep G2P does this for the
//           positions it writes, so the kernel only runs after an upload.
//   scan    two passes over the directory: grid block index of each marked
//           block, start of each non-empty particle block; the second pass
//           rewrites every directory entry it reads (grid block / particle
//           block index or -1) and zeroes the counts for the next binning,
//           so no separate reset is needed
//   scatter placement of particle indices into their block, one global
//           atomic per (CTA, block) after a shared-memory count
//   sort    per block, counting sort by cell and a rank by storage index
//           inside each cell: the canonical (block, cell, index) order,
//           independent of atomic timing
#include <cuda_runtime.h>

#include <algorithm>

#include "binning.cuh"
#include "colliders.cuh"
#include "partition_stages.cuh"
#include "zsmpm_internal.cuh"

namespace zsmpm {
namespace {

__global__ void k_full_dir_clear(DevPtrs d) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < d.ndir;
       i += (long long)gridDim.x * blockDim.x) {
    d.dir_count[i] = 0;
    d.dir_fill[i] = 0;
    d.dir_gb[i] = -1;
    d.dir_bk[i] = -1;
    d.dir_flag[i] = 0;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    d.cnt->n_gblocks = 0;
    d.cnt->n_buckets = 0;
  }
}

// Binning of particles in upload order (after an upload the storage slot is
// the upload index, which gives the scene).
__global__ void k_bin(DevPtrs d, const float *__restrict__ pin) {
  const SimParams &P = *d.prm;
  const long long n = P.n;
  const long long cap = d.cap;
  const int lane = threadIdx.x & 31;
  const long long warp0 = (blockIdx.x * (long long)blockDim.x + threadIdx.x) - lane;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long w = warp0; w < n; w += stride) {
    const long long i = w + lane;
    int key = -1;
    int scene = 0;
    if (i < n) {
      scene = scene_of_particle(d, i);
      float x[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) x[k] = d.planar_x ? pin[k * cap + i] : pin[pidx(CH_X + k, i)];
      key = bin_key(d.scn[scene], x[0], x[1], x[2], &d.cnt->status);
      d.pkey[i] = key;
    }
    bin_count(d, d.scn[scene], key, 0xffffffffu);
  }
}

__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(DevPtrs d) {
  stage_scan_reduce(d, blockIdx.x, gridDim.x);
}

__global__ void __launch_bounds__(kScanThreads) k_scan_apply(DevPtrs d) {
  stage_scan_apply(d, blockIdx.x, gridDim.x);
}

__global__ void __launch_bounds__(kScatterThreads) k_scatter(DevPtrs d) {
  stage_scatter(d, blockIdx.x, gridDim.x);
}

__global__ void __launch_bounds__(kSortThreads) k_bucket_sort(DevPtrs d) {
  stage_bucket_sort(d, blockIdx.x, gridDim.x);
}

__global__ void k_grid_clear(DevPtrs d) {
  const long long n = (long long)min(d.cnt->n_gblocks, d.cap_gblocks) * 64;
  const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    d.grid[i] = z;
}

// The gate of one fused substep: a particle that left the directory (bit
// set by the previous substep's binning) halts this and every later queued
// substep; otherwise the substep is counted as started.
__global__ void k_substep_gate(DevPtrs d) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  Counters *c = d.cnt;
  if (c->status & ST_OUT_OF_DOMAIN) c->halt = 1;
  if (!c->halt) c->n_started += 1;
}

// float -> unsigned with the order of the floats (for atomicMin / atomicMax)
__device__ __forceinline__ unsigned ordered_bits(float f) {
  const unsigned u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__global__ void k_bbox(DevPtrs d, const float *__restrict__ pin) {
  unsigned lo[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, hi[3] = {0u, 0u, 0u};
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  auto take = [&](float x0, float x1, float x2) {
    const float x[3] = {x0, x1, x2};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      if (!isfinite(x[a])) continue;
      const unsigned b = ordered_bits(x[a]);
      lo[a] = min(lo[a], b);
      hi[a] = max(hi[a], b);
    }
  };
  for (long long i = t0; i < d.prm->n; i += stride)
    take(pin[pidx(CH_X, i)], pin[pidx(CH_X + 1, i)], pin[pidx(CH_X + 2, i)]);
  for (long long i = t0; i < d.cloth.n_verts; i += stride)
    take(d.cloth.vx[3 * i], d.cloth.vx[3 * i + 1], d.cloth.vx[3 * i + 2]);
  for (long long i = t0; i < d.n_trackers; i += stride)
    take(d.tx[3 * i], d.tx[3 * i + 1], d.tx[3 * i + 2]);
#pragma unroll
  for (int a = 0; a < 3; ++a) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      lo[a] = min(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
      hi[a] = max(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
    }
  }
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      atomicMin(&d.cnt->bbox[a], lo[a]);
      atomicMax(&d.cnt->bbox[3 + a], hi[a]);
    }
  }
}

inline int grid_for(const DevPtrs &d, int per_sm) { return d.num_sms * per_sm; }

}  // namespace

void launch_full_dir_clear(const DevPtrs &d, cudaStream_t s) {
  k_full_dir_clear<<<grid_for(d, 8), 256, 0, s>>>(d);
}

void launch_bin(const DevPtrs &d, int cur, cudaStream_t s) {
  k_bin<<<d.grid_stream > 0 ? d.grid_stream : grid_for(d, 8), 256, 0, s>>>(d, d.pbuf[cur]);
}

void launch_scan(const DevPtrs &d, cudaStream_t s) {
  k_scan_reduce<<<d.ntiles, kScanThreads, 0, s>>>(d);
  k_scan_apply<<<d.ntiles, kScanThreads, 0, s>>>(d);
}

// one chunk per CTA up to the capacity (fixed for graph capture)
void launch_scatter(const DevPtrs &d, cudaStream_t s) {
  const long long g = (d.cap + kScatterPerCta - 1) / kScatterPerCta;
  k_scatter<<<(int)std::min<long long>(std::max<long long>(g, 1), 1 << 30), kScatterThreads, 0,
              s>>>(d);
}

void launch_bucket_sort(const DevPtrs &d, cudaStream_t s) {
  k_bucket_sort<<<d.grid_sort > 0 ? d.grid_sort : grid_for(d, 8), kSortThreads, 0, s>>>(d);
}

void launch_grid_clear(const DevPtrs &d, cudaStream_t s) {
  k_grid_clear<<<grid_for(d, 8), 256, 0, s>>>(d);
}

void launch_substep_gate(const DevPtrs &d, cudaStream_t s) { k_substep_gate<<<1, 32, 0, s>>>(d); }

// the caller sets bbox to (all ones) x 3, (zeros) x 3 first
void launch_bbox(const DevPtrs &d, int cur, cudaStream_t s) {
  k_bbox<<<grid_for(d, 4), 256, 0, s>>>(d, d.pbuf[cur]);
}

}  // namespace zsmpm
