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

// Pass 1 of the directory scan: per tile sums of (grid block flag, particle
// count, non-empty flag).
__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(DevPtrs d) {
  if (ZSMPM_HALTED(d)) return;
  // a particle left the directory (binned with key -1): the partition of
  // these positions is incomplete, so this and the queued stages stop here
  // and the state stays the last complete one (with a growing directory the
  // host then grows it and replays them; otherwise the status is the error)
  if (d.cnt->status & ST_OUT_OF_DOMAIN) {
    if (blockIdx.x == 0 && threadIdx.x == 0) d.cnt->halt = 1;
    return;
  }
  const long long base = (long long)blockIdx.x * kScanTile + threadIdx.x * kScanPerThread;
  int f = 0, c = 0, e = 0;
#pragma unroll
  for (int k = 0; k < kScanPerThread; ++k) {
    const long long i = base + k;
    if (i < d.ndir) {
      const int cc = d.dir_count[i];
      f += d.dir_flag[i];
      c += cc;
      e += cc > 0;
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
// Every entry of the tile is rewritten: grid block index or -1, particle
// block index or -1, count and flag back to 0 for the next binning.
__global__ void __launch_bounds__(kScanThreads) k_scan_apply(DevPtrs d) {
  if (ZSMPM_HALTED(d)) return;
  __shared__ int red[3][kScanThreads / 32];
  __shared__ int tile_prefix[3];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (blockIdx.x == 0 && tid == 0) {
    d.cnt->max_vel_sqr_bits = 0u;
    d.cnt->n_near = 0;
    // the fused substep moves the colliders to this substep's time
    if (d.prm->auto_step) step_colliders(d, d.prm->n_colliders, d.prm->dt);
  }
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

  const long long base = (long long)blockIdx.x * kScanTile + tid * kScanPerThread;
  int fl[kScanPerThread], ct[kScanPerThread];
  int f = 0, c = 0, e = 0;
#pragma unroll
  for (int k = 0; k < kScanPerThread; ++k) {
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
  for (int k = 0; k < kScanPerThread; ++k) {
    const long long i = base + k;
    if (i >= d.ndir) break;
    int gb = -1, bk = -1;
    if (fl[k]) {
      if (gpos < cap) {
        d.gb_dir[gpos] = (int)i;
        gb = gpos;
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
        bk = bpos;
      }
      d.dir_fill[i] = ppos;
      ++bpos;
      ppos += ct[k];
    }
    d.dir_gb[i] = gb;
    d.dir_bk[i] = bk;
    if (fl[k]) d.dir_flag[i] = 0;
    if (ct[k]) d.dir_count[i] = 0;
  }
  if (blockIdx.x == gridDim.x - 1 && tid == kScanThreads - 1) {
    d.cnt->n_gblocks = min(gpos, cap);
    d.cnt->n_buckets = min(bpos, cap);
    d.cnt->n_binned = ppos;
    if (gpos > cap) atomicOr(&d.cnt->status, ST_CAPACITY);
  }
}

// Placement of particle indices into their block's range.  A CTA takes
// kScatterPerCta consecutive storage slots, which (storage following the
// previous partition) hold few distinct blocks: it counts them in a small
// shared-memory table, reserves each block's share with one global atomic,
// and places its particles from there.  A key that finds no table slot is
// placed with its own global atomic.  The order inside a block is left to
// the bucket sort.
constexpr int kScatterThreads = 256;
constexpr int kScatterPer = 4;
constexpr int kScatterPerCta = kScatterThreads * kScatterPer;
constexpr int kScatterSlots = 64;

__global__ void __launch_bounds__(kScatterThreads) k_scatter(DevPtrs d) {
  if (ZSMPM_HALTED(d)) return;
  __shared__ int tkey[kScatterSlots], tcount[kScatterSlots], tbase[kScatterSlots];
  const long long n = d.prm->n;
  const int tid = threadIdx.x;
  for (long long c0 = (long long)blockIdx.x * kScatterPerCta; c0 < n;
       c0 += (long long)gridDim.x * kScatterPerCta) {
    if (tid < kScatterSlots) {
      tkey[tid] = -1;
      tcount[tid] = 0;
    }
    __syncthreads();
    int slot[kScatterPer], rank[kScatterPer], dd[kScatterPer];
    const int lane = tid & 31;
#pragma unroll
    for (int k = 0; k < kScatterPer; ++k) {
      const long long i = c0 + k * kScatterThreads + tid;
      const int key = i < n ? d.pkey[i] : -1;
      dd[k] = key >> 6;
      // warp aggregation first: the leader of each key's peers takes the
      // table entry and the peers' share of its count
      const unsigned peers = __match_any_sync(0xffffffffu, dd[k]);
      const int leader = __ffs(peers) - 1;
      int t_slot = -1, base = 0;
      if (key >= 0 && lane == leader) {
        const int h = (int)(((unsigned)dd[k] * 2654435761u) >> 26);  // 6-bit hash
        for (int probe = 0; probe < kScatterSlots; ++probe) {
          const int t = (h + probe) & (kScatterSlots - 1);
          const int old = atomicCAS(&tkey[t], -1, dd[k]);
          if (old == -1 || old == dd[k]) {
            t_slot = t;
            base = atomicAdd(&tcount[t], __popc(peers));
            break;
          }
        }
        if (t_slot < 0) base = atomicAdd(&d.dir_fill[dd[k]], __popc(peers));  // table full
      }
      slot[k] = __shfl_sync(0xffffffffu, t_slot, leader);
      rank[k] = __shfl_sync(0xffffffffu, base, leader) + __popc(peers & ((1u << lane) - 1u));
    }
    __syncthreads();
    if (tid < kScatterSlots && tkey[tid] >= 0)
      tbase[tid] = atomicAdd(&d.dir_fill[tkey[tid]], tcount[tid]);
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kScatterPer; ++k) {
      const long long i = c0 + k * kScatterThreads + tid;
      if (i >= n || dd[k] < 0) continue;
      const long long pos = slot[k] >= 0 ? (long long)tbase[slot[k]] + rank[k] : rank[k];
      if (pos < n)
        d.perm[pos] = (int)i;
      else  // stale directory counts after an earlier overflow
        atomicOr(&d.cnt->status, ST_CAPACITY);
    }
    __syncthreads();  // table reused
  }
}

// Canonical order inside each particle block: (cell, storage index).
// A counting sort by cell id (64 bins, integer shared-memory atomics) puts
// each cell's particles in a contiguous range in arbitrary order; each
// particle's final slot is then the start of its cell plus the number of the
// cell's particles with a smaller storage index, all ranks computed at once.
// A cell with more than kCellSortMax particles sends the block to an on-chip
// bitonic sort; a block with more than kSortCap particles is sorted through
// global scratch (slower; flagged with the informational ST_BUCKET_OVERSIZE
// bit).
constexpr int kSortThreads = 256;
constexpr int kSortCap = 2048;
constexpr int kCellSortMax = 256;

__device__ __forceinline__ void warp_exclusive_scan64(const int *in, int *out) {
  // one warp: 64 values, two per lane
  const int lane = threadIdx.x & 31;
  const int a = in[2 * lane], b = in[2 * lane + 1];
  int s = a + b;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, s, o);
    if (lane >= o) s += t;
  }
  const int excl = s - a - b;
  out[2 * lane] = excl;
  out[2 * lane + 1] = excl + a;
  if (lane == 31) out[64] = s;
}

__global__ void __launch_bounds__(kSortThreads) k_bucket_sort(DevPtrs d) {
  if (ZSMPM_HALTED(d)) return;
  __shared__ __align__(16) int sbuf[2 * kSortCap];
  int *sp = sbuf, *op = sbuf + kSortCap;
  __shared__ unsigned char sc[kSortCap], oc[kSortCap];
  __shared__ int ccount[64], cstart[65], cfill[64];
  __shared__ int big_cell;
  const int nb = d.cnt->n_buckets;
  const long long n = d.prm->n;
  const int tid = threadIdx.x;
  for (int b = blockIdx.x; b < nb; b += gridDim.x) {
    const int start = d.bk_start[b];
    const int cnt = (int)min((long long)d.bk_count[b], n - start);
    if (cnt <= 1) continue;
    if (tid < 64) {
      ccount[tid] = 0;
      cfill[tid] = 0;
    }
    if (tid == 0) big_cell = 0;
    __syncthreads();
    if (cnt <= kSortCap) {
      for (int j = tid; j < cnt; j += kSortThreads) {
        const int p = d.perm[start + j];
        const int c = d.pkey[p] & 63;
        sp[j] = p;
        sc[j] = (unsigned char)c;
        atomicAdd(&ccount[c], 1);
      }
      __syncthreads();
      if (tid < 32) warp_exclusive_scan64(ccount, cstart);
      if (tid < 64 && ccount[tid] > kCellSortMax) big_cell = 1;
      __syncthreads();
      if (!big_cell) {
        for (int j = tid; j < cnt; j += kSortThreads) {
          const int c = sc[j];
          const int o = cstart[c] + atomicAdd(&cfill[c], 1);
          op[o] = sp[j];
          oc[o] = (unsigned char)c;
        }
        __syncthreads();
        for (int j = tid; j < cnt; j += kSortThreads) {
          const int c = oc[j], v = op[j];
          const int lo = cstart[c], hi = cstart[c + 1];
          int r = lo;
          for (int i = lo; i < hi; ++i) r += op[i] < v;
          d.perm[start + r] = v;
        }
      } else {
        // bitonic sort of (cell << 32 | index) over the whole block
        unsigned long long *key = reinterpret_cast<unsigned long long *>(sbuf);  // 16 KB
        int N = 2;
        while (N < cnt) N <<= 1;
        __syncthreads();
        for (int j = tid; j < N; j += kSortThreads) {
          unsigned long long k = ~0ull;
          if (j < cnt) {
            const int p = d.perm[start + j];
            k = ((unsigned long long)(d.pkey[p] & 63) << 32) | (unsigned)p;
          }
          key[j] = k;
        }
        __syncthreads();
        for (int k = 2; k <= N; k <<= 1) {
          for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = tid; i < N; i += kSortThreads) {
              const int ixj = i ^ j;
              if (ixj > i) {
                const unsigned long long a = key[i], c = key[ixj];
                if ((a > c) == ((i & k) == 0)) {
                  key[i] = c;
                  key[ixj] = a;
                }
              }
            }
            __syncthreads();
          }
        }
        for (int j = tid; j < cnt; j += kSortThreads)
          d.perm[start + j] = (int)(key[j] & 0xffffffffull);
      }
    } else {
      // oversize block: counting sort by cell through global scratch
      for (int j = tid; j < cnt; j += kSortThreads)
        atomicAdd(&ccount[d.pkey[d.perm[start + j]] & 63], 1);
      __syncthreads();
      if (tid < 32) warp_exclusive_scan64(ccount, cstart);
      __syncthreads();
      for (int j = tid; j < cnt; j += kSortThreads) {
        const int p = d.perm[start + j];
        const int c = d.pkey[p] & 63;
        d.perm_tmp[start + cstart[c] + atomicAdd(&cfill[c], 1)] = p;
      }
      __syncthreads();
      // canonical order inside each cell (insertion sort in global scratch)
      if (tid < 64) {
        int *q = d.perm_tmp + start;
        const int lo = cstart[tid], hi = cstart[tid + 1];
        for (int i = lo + 1; i < hi; ++i) {
          const int v = q[i];
          int k = i - 1;
          while (k >= lo && q[k] > v) {
            q[k + 1] = q[k];
            --k;
          }
          q[k + 1] = v;
        }
      }
      __syncthreads();
      for (int j = tid; j < cnt; j += kSortThreads) d.perm[start + j] = d.perm_tmp[start + j];
      if (tid == 0) atomicOr(&d.cnt->status, ST_BUCKET_OVERSIZE);
    }
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
