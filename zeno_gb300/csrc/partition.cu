// Particle binning and block-key sort: the GB300 form of
// ZSPartitionForZSParticles + ExpandZSPartition
// (projects/CuLagrange/mpm/MPMPipeline.cu:21-231).
//
// The reference inserts every particle's block key into a hash table with
// CAS and expands the table on the host in several synchronised passes.
// Here a dense block directory stands in for the hash table (O(1) lookup,
// no probing, 1-8 MB for the domains in use), and one substep's partition is
// six device kernels with no host read:
//   reset   clear the directory entries the previous partition touched
//   bin     per particle: key = (block << 6) | cell, warp-aggregated count;
//           the first particle of a block marks its 27-block neighbourhood
//           (the 1-ring halo of ExpandZSPartition)
//   scan    two-pass scan over the directory: grid block index of each
//           marked block, start of each non-empty particle block
//   scatter warp-aggregated placement of particle indices into their block
//   sort    per block, bitonic sort on chip by (cell, index): the canonical
//           (block, cell, index) order, independent of atomic timing
//   clear   zero the grid blocks (ZSGridFromZSPartition, :256-262)
#include <cuda_runtime.h>

#include "zsmpm_internal.cuh"

namespace zsmpm {
namespace {

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__global__ void k_reset(DevPtrs d) {
  const int n = min(d.cnt->n_gblocks, d.cap_gblocks);
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < n; g += gridDim.x * blockDim.x) {
    const int dd = d.gb_dir[g];
    d.dir_count[dd] = 0;
    d.dir_fill[dd] = 0;
    d.dir_gb[dd] = -1;
    d.dir_flag[dd] = 0;
  }
}

__global__ void k_full_dir_clear(DevPtrs d) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < d.ndir;
       i += (long long)gridDim.x * blockDim.x) {
    d.dir_count[i] = 0;
    d.dir_fill[i] = 0;
    d.dir_gb[i] = -1;
    d.dir_flag[i] = 0;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    d.cnt->n_gblocks = 0;
    d.cnt->n_buckets = 0;
  }
}

// Block of a particle: base = floor(x / dx - 0.5) per axis
// (MPMPipeline.cu:78-82), computed as one rounded multiply by 1/dx and one
// rounded subtraction so that no FMA contraction changes a key.
__device__ __forceinline__ int particle_base(float x, float inv_dx) {
  return __float2int_rd(__fsub_rn(__fmul_rn(x, inv_dx), 0.5f));
}

__global__ void k_bin(DevPtrs d, const float *__restrict__ pin) {
  const SimParams &P = *d.prm;
  const long long n = P.n;
  const long long cap = d.cap;
  if (blockIdx.x == 0 && threadIdx.x == 0) d.cnt->max_vel_sqr_bits = 0u;
  const int lane = threadIdx.x & 31;
  const long long warp0 = (blockIdx.x * (long long)blockDim.x + threadIdx.x) - lane;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const int dy = P.block_dims[1], dz = P.block_dims[2];
  for (long long w = warp0; w < n; w += stride) {
    const long long i = w + lane;
    int key = -1;
    if (i < n) {
      const float x0 = pin[CH_X * cap + i], x1 = pin[(CH_X + 1) * cap + i],
                  x2 = pin[(CH_X + 2) * cap + i];
      if (isfinite(x0) && isfinite(x1) && isfinite(x2)) {
        const int b0 = particle_base(x0, P.inv_dx), b1 = particle_base(x1, P.inv_dx),
                  b2 = particle_base(x2, P.inv_dx);
        const int c0 = (b0 >> 2) - P.block_lo[0], c1 = (b1 >> 2) - P.block_lo[1],
                  c2 = (b2 >> 2) - P.block_lo[2];
        if (c0 >= 1 && c0 <= P.block_dims[0] - 2 && c1 >= 1 && c1 <= dy - 2 && c2 >= 1 &&
            c2 <= dz - 2) {
          const int dd = (c0 * dy + c1) * dz + c2;
          key = (dd << 6) | ((b0 & 3) << 4) | ((b1 & 3) << 2) | (b2 & 3);
        } else {
          atomicOr(&d.cnt->status, ST_OUT_OF_DOMAIN);
        }
      } else {
        atomicOr(&d.cnt->status, ST_NAN);
      }
      d.pkey[i] = key;
    }
    const int dd = key >> 6;  // -1 for invalid
    const unsigned peers = __match_any_sync(0xffffffffu, dd);
    const int leader = __ffs(peers) - 1;
    if (key >= 0 && lane == leader) {
      const int old = atomicAdd(&d.dir_count[dd], __popc(peers));
      if (old == 0) {
        // first particle of the block: mark the block and its 26 neighbours
        for (int a = -1; a <= 1; ++a)
          for (int b = -1; b <= 1; ++b)
            for (int c = -1; c <= 1; ++c) d.dir_flag[dd + (a * dy + b) * dz + c] = 1;
      }
    }
  }
}

// Pass 1 of the directory scan: per tile sums of (grid block flag, particle
// count, non-empty flag).
__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(DevPtrs d) {
  const long long base = (long long)blockIdx.x * kScanTile + threadIdx.x * 16;
  int f = 0, c = 0, e = 0;
  if (base < d.ndir) {
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      const long long i = base + k;
      if (i < d.ndir) {
        const int cc = d.dir_count[i];
        f += d.dir_flag[i];
        c += cc;
        e += cc > 0;
      }
    }
  }
  __shared__ int red[3][kScanThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    f += __shfl_xor_sync(0xffffffffu, f, o);
    c += __shfl_xor_sync(0xffffffffu, c, o);
    e += __shfl_xor_sync(0xffffffffu, e, o);
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    red[0][warp] = f;
    red[1][warp] = c;
    red[2][warp] = e;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    int s = 0;
    for (int w = 0; w < kScanThreads / 32; ++w) s += red[threadIdx.x][w];
    d.tile_sums[3 * blockIdx.x + threadIdx.x] = s;
  }
}

// Pass 2: exclusive prefix of the tile sums, local scan, and the outputs.
__global__ void __launch_bounds__(kScanThreads) k_scan_apply(DevPtrs d) {
  __shared__ int red[3][kScanThreads / 32];
  __shared__ int tile_prefix[3];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // prefix over previous tiles
  int pf = 0, pc = 0, pe = 0;
  for (int t = tid; t < (int)blockIdx.x; t += kScanThreads) {
    pf += d.tile_sums[3 * t];
    pc += d.tile_sums[3 * t + 1];
    pe += d.tile_sums[3 * t + 2];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    pf += __shfl_xor_sync(0xffffffffu, pf, o);
    pc += __shfl_xor_sync(0xffffffffu, pc, o);
    pe += __shfl_xor_sync(0xffffffffu, pe, o);
  }
  if (lane == 0) {
    red[0][warp] = pf;
    red[1][warp] = pc;
    red[2][warp] = pe;
  }
  __syncthreads();
  if (tid < 3) {
    int s = 0;
    for (int w = 0; w < kScanThreads / 32; ++w) s += red[tid][w];
    tile_prefix[tid] = s;
  }
  __syncthreads();

  // thread-local values
  const long long base = (long long)blockIdx.x * kScanTile + tid * 16;
  int fl[16], ct[16];
  int f = 0, c = 0, e = 0;
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    const long long i = base + k;
    fl[k] = 0;
    ct[k] = 0;
    if (i < d.ndir) {
      fl[k] = d.dir_flag[i];
      ct[k] = d.dir_count[i];
    }
    f += fl[k];
    c += ct[k];
    e += ct[k] > 0;
  }
  // block exclusive scan of (f, c, e)
  int sf = f, sc = c, se = e;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int a = __shfl_up_sync(0xffffffffu, sf, o), b = __shfl_up_sync(0xffffffffu, sc, o),
              g = __shfl_up_sync(0xffffffffu, se, o);
    if (lane >= o) {
      sf += a;
      sc += b;
      se += g;
    }
  }
  __syncthreads();  // red reused
  if (lane == 31) {
    red[0][warp] = sf;
    red[1][warp] = sc;
    red[2][warp] = se;
  }
  __syncthreads();
  int wf = 0, wc = 0, we = 0;
  for (int w = 0; w < warp; ++w) {
    wf += red[0][w];
    wc += red[1][w];
    we += red[2][w];
  }
  int gpos = tile_prefix[0] + wf + sf - f;
  int ppos = tile_prefix[1] + wc + sc - c;
  int bpos = tile_prefix[2] + we + se - e;
  const int cap = d.cap_gblocks;
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    const long long i = base + k;
    if (fl[k]) {
      if (gpos < cap) {
        d.gb_dir[gpos] = (int)i;
        d.dir_gb[i] = gpos;
      } else {
        atomicOr(&d.cnt->status, ST_CAPACITY);
      }
      ++gpos;
    }
    if (ct[k] > 0) {
      if (bpos < cap) {
        d.bk_dir[bpos] = (int)i;
        d.bk_start[bpos] = ppos;
        d.bk_count[bpos] = ct[k];
      }
      d.dir_fill[i] = ppos;
      ++bpos;
      ppos += ct[k];
    }
  }
  if (blockIdx.x == gridDim.x - 1 && tid == kScanThreads - 1) {
    d.cnt->n_gblocks = min(gpos, cap);
    d.cnt->n_buckets = min(bpos, cap);
    d.cnt->n_binned = ppos;
    if (gpos > cap) atomicOr(&d.cnt->status, ST_CAPACITY);
  }
}

__global__ void k_scatter(DevPtrs d) {
  const long long n = d.prm->n;
  const int lane = threadIdx.x & 31;
  const long long warp0 = (blockIdx.x * (long long)blockDim.x + threadIdx.x) - lane;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long w = warp0; w < n; w += stride) {
    const long long i = w + lane;
    const int key = (i < n) ? d.pkey[i] : -1;
    const int dd = key >> 6;
    const unsigned peers = __match_any_sync(0xffffffffu, dd);
    const int leader = __ffs(peers) - 1;
    int base = 0;
    if (key >= 0 && lane == leader) base = atomicAdd(&d.dir_fill[dd], __popc(peers));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (key >= 0) {
      const long long pos = (long long)base + __popc(peers & lanemask_lt());
      if (pos < n)
        d.perm[pos] = (int)i;
      else  // stale directory counts after an earlier overflow
        atomicOr(&d.cnt->status, ST_CAPACITY);
    }
  }
}

// Canonical order inside each particle block: bitonic sort of
// (cell << 32 | storage index) in shared memory.
constexpr int kSortThreads = 512;

__global__ void __launch_bounds__(kSortThreads) k_bucket_sort(DevPtrs d) {
  extern __shared__ unsigned long long skeys[];
  const int nb = d.cnt->n_buckets;
  for (int b = blockIdx.x; b < nb; b += gridDim.x) {
    const int start = d.bk_start[b];
    const int cnt = (int)min((long long)d.bk_count[b], d.prm->n - start);
    if (cnt <= 1) continue;
    if (cnt > kMaxSortBucket) {
      if (threadIdx.x == 0) atomicOr(&d.cnt->status, ST_BUCKET_OVERSIZE);
      continue;
    }
    int N = 2;
    while (N < cnt) N <<= 1;
    for (int j = threadIdx.x; j < N; j += kSortThreads) {
      unsigned long long k = ~0ull;
      if (j < cnt) {
        const int p = d.perm[start + j];
        k = ((unsigned long long)(d.pkey[p] & 63) << 32) | (unsigned)p;
      }
      skeys[j] = k;
    }
    __syncthreads();
    for (int k = 2; k <= N; k <<= 1) {
      for (int j = k >> 1; j > 0; j >>= 1) {
        for (int i = threadIdx.x; i < N; i += kSortThreads) {
          const int ixj = i ^ j;
          if (ixj > i) {
            const unsigned long long a = skeys[i], c = skeys[ixj];
            const bool up = (i & k) == 0;
            if ((a > c) == up) {
              skeys[i] = c;
              skeys[ixj] = a;
            }
          }
        }
        __syncthreads();
      }
    }
    for (int j = threadIdx.x; j < cnt; j += kSortThreads)
      d.perm[start + j] = (int)(skeys[j] & 0xffffffffull);
    __syncthreads();
  }
}

__global__ void k_grid_clear(DevPtrs d) {
  const long long n = (long long)min(d.cnt->n_gblocks, d.cap_gblocks) * 64;
  const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    d.grid[i] = z;
}

inline int grid_for(const DevPtrs &d, int per_sm) { return d.num_sms * per_sm; }

}  // namespace

void launch_reset(const DevPtrs &d, cudaStream_t s) {
  k_reset<<<grid_for(d, 4), 256, 0, s>>>(d);
}

void launch_full_dir_clear(const DevPtrs &d, cudaStream_t s) {
  k_full_dir_clear<<<grid_for(d, 8), 256, 0, s>>>(d);
}

void launch_bin(const DevPtrs &d, int cur, cudaStream_t s) {
  k_bin<<<grid_for(d, 8), 256, 0, s>>>(d, d.pbuf[cur]);
}

void launch_scan(const DevPtrs &d, cudaStream_t s) {
  k_scan_reduce<<<d.ntiles, kScanThreads, 0, s>>>(d);
  k_scan_apply<<<d.ntiles, kScanThreads, 0, s>>>(d);
}

void launch_scatter(const DevPtrs &d, cudaStream_t s) {
  k_scatter<<<grid_for(d, 8), 256, 0, s>>>(d);
}

void launch_bucket_sort(const DevPtrs &d, cudaStream_t s) {
  k_bucket_sort<<<grid_for(d, 4), kSortThreads, kMaxSortBucket * sizeof(unsigned long long), s>>>(
      d);
}

void launch_grid_clear(const DevPtrs &d, cudaStream_t s) {
  k_grid_clear<<<grid_for(d, 8), 256, 0, s>>>(d);
}

}  // namespace zsmpm
