// The partition's stages as device functions of (CTA `bid` of `nblk`), shared
// by their own kernels (partition.cu) and by the persistent substep kernel
// (persistent.cu): the directory scan (two passes), the placement of
// particles into their blocks, and the canonical sort inside each block.
#pragma once

#include <cuda_runtime.h>

#include "binning.cuh"
#include "colliders.cuh"
#include "zsmpm_internal.cuh"

namespace zsmpm {
namespace {

// Pass 1 of the directory scan: per tile sums of (grid block flag, particle
// count, non-empty flag); CTA `bid` of `nblk` takes tiles bid, bid + nblk, ...
__device__ __forceinline__ void stage_scan_reduce(const DevPtrs &d, int bid, int nblk) {
  if (ZSMPM_HALTED(d)) return;
  for (int tile = bid; tile < d.ntiles; tile += nblk) {
    // a particle left the directory (binned with key -1): the partition of
    // these positions is incomplete, so this and the queued stages stop here
    // and the state stays the last complete one (with a growing directory the
    // host then grows it and replays them; otherwise the status is the error)
    if (d.cnt->status & ST_OUT_OF_DOMAIN) {
      if (tile == 0 && threadIdx.x == 0) d.cnt->halt = 1;
      return;
    }
    const long long base = (long long)tile * kScanTile + threadIdx.x * kScanPerThread;
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
      d.tile_sums[3 * tile + threadIdx.x] = s;
    }
    __syncthreads();  // red reused by the next tile
  }
}

// Pass 2: exclusive prefix of the tile sums, local scan, and the outputs.
// Every entry of the tile is rewritten: grid block index or -1, particle
// block index or -1, count and flag back to 0 for the next binning.
__device__ __forceinline__ void stage_scan_apply(const DevPtrs &d, int bid, int nblk) {
  if (ZSMPM_HALTED(d)) return;
  for (int tile = bid; tile < d.ntiles; tile += nblk) {
    __shared__ int red[3][kScanThreads / 32];
    __shared__ int tile_prefix[3];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tile == 0 && tid == 0) {
      d.cnt->max_vel_sqr_bits = 0u;
      d.cnt->n_near = 0;
      // the fused substep moves the colliders to this substep's time
      if (d.prm->auto_step) step_colliders(d, d.prm->n_colliders, d.prm->dt);
    }
    int pf = 0, pc = 0, pe = 0;
    for (int t = tid; t < tile; t += kScanThreads) {
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

    const long long base = (long long)tile * kScanTile + tid * kScanPerThread;
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
    if (tile == d.ntiles - 1 && tid == kScanThreads - 1) {
      d.cnt->n_gblocks = min(gpos, cap);
      d.cnt->n_buckets = min(bpos, cap);
      d.cnt->n_binned = ppos;
      atomicMax(&d.cnt->max_gblocks, gpos);
      atomicMax(&d.cnt->max_buckets, bpos);
      if (gpos > cap) atomicOr(&d.cnt->status, ST_CAPACITY);
    }
    __syncthreads();  // shared entries reused by the next tile
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

__device__ __forceinline__ void stage_scatter(const DevPtrs &d, int bid, int nblk) {
  if (ZSMPM_HALTED(d)) return;
  __shared__ int tkey[kScatterSlots], tcount[kScatterSlots], tbase[kScatterSlots];
  const long long n = d.prm->n;
  const int tid = threadIdx.x;
  for (long long c0 = (long long)bid * kScatterPerCta; c0 < n;
       c0 += (long long)nblk * kScatterPerCta) {
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

__device__ __forceinline__ void stage_bucket_sort(const DevPtrs &d, int bid, int nblk) {
  if (ZSMPM_HALTED(d)) return;
  __shared__ __align__(16) int sbuf[2 * kSortCap];
  int *sp = sbuf, *op = sbuf + kSortCap;
  __shared__ unsigned char sc[kSortCap], oc[kSortCap];
  __shared__ int ccount[64], cstart[65], cfill[64];
  __shared__ int big_cell;
  const int nb = d.cnt->n_buckets;
  const long long n = d.prm->n;
  const int tid = threadIdx.x;
  for (int b = bid; b < nb; b += nblk) {
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

}  // namespace
}  // namespace zsmpm
