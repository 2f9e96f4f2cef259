// The fused substep as one persistent kernel per substep.
//
// A cooperative launch of as many CTAs of 256 threads as the SMs hold at
// once runs the seven stages of a substep in order -- the two directory scan
// passes, the placement of particles into their blocks, the canonical sort,
// P2G (tile shape 256 x 128), the grid gather with the grid update and walls
// (then the level-set colliders, if any) and G2P with the return mapping,
// the stress and the next binning -- each a grid-stride loop over its work,
// separated by grid-wide barriers.  The stages are the same device functions
// the per-stage kernels run (partition_stages.cuh, transfer_stages.cuh), so
// the results are those of the graph of seven kernels.  The context captures
// the launch (with the reset of the barrier counter) in its CUDA graph.
//
// The barrier is bounded: a CTA that has waited `barrier_limit` spins sets
// ST_TIMEOUT and the halt flag and returns, and so does every CTA at the next
// barrier it cannot pass, so the kernel ends, the substeps queued behind it
// do nothing, and the host reads MPM_ERR_TIMEOUT.  No stage starts before
// every CTA has finished the one before it, so a timeout leaves an
// incomplete substep but no stage reading incomplete inputs.  The
// cooperative launch guarantees that all CTAs are resident, so in a correct
// run every barrier completes.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>

#include "partition_stages.cuh"
#include "transfer_stages.cuh"
#include "zsmpm_internal.cuh"

namespace zsmpm {
namespace {

constexpr int kPersistThreads = 256;
constexpr int kPersistP2GChunk = 128;
constexpr int kPersistSmem = ColLayout<kPersistThreads, kPersistP2GChunk>::smem >
                                     g2p_smem_bytes<kPersistThreads>()
                                 ? ColLayout<kPersistThreads, kPersistP2GChunk>::smem
                                 : g2p_smem_bytes<kPersistThreads>();

// Grid-wide barrier of `ncta` CTAs (sense by generation): each CTA arrives
// once; the last arrival resets the count and publishes the next
// generation, the others spin on it with a bound.  Every thread fences
// after the barrier, so the writes of every CTA before it are seen by every
// load after it.  Returns false (ST_TIMEOUT set) if this CTA gave up.
__device__ __forceinline__ bool grid_barrier(const DevPtrs &d, unsigned &gen, unsigned ncta,
                                             unsigned long long limit) {
  __shared__ int passed;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    const unsigned target = gen + 1;
    __threadfence();  // this CTA's writes before its arrival
    if (atomicAdd(&d.cnt->bar_count, 1u) + 1u == ncta) {
      atomicExch(&d.cnt->bar_count, 0u);
      __threadfence();
      atomicExch(&d.cnt->bar_gen, target);
    } else {
      const volatile unsigned *g = &d.cnt->bar_gen;
      unsigned long long it = 0;
      while (*g != target) {
        if (++it > limit) {
          atomicOr(&d.cnt->status, ST_TIMEOUT);
          atomicExch(&d.cnt->halt, 1);  // the queued substeps leave the state alone
          ok = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    passed = ok;
  }
  __syncthreads();
  __threadfence();  // every thread: the other CTAs' writes before the barrier
  gen += 1;
  return passed != 0;
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// CTA 0 notes when it passed barrier `i` (all CTAs had finished stage i)
__device__ __forceinline__ void stamp(const DevPtrs &d, int i) {
  if (blockIdx.x == 0 && threadIdx.x == 0) d.cnt->stage_t[i] = global_ns();
}

template <bool kHencky, bool kColliders>
__global__ void __launch_bounds__(kPersistThreads, 3)
    k_substep_persistent(DevPtrs d, const float *__restrict__ pin,
                         const int32_t *__restrict__ iin, float *__restrict__ pout,
                         int32_t *__restrict__ iout) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int cta = blockIdx.x, ncta = gridDim.x;
  // no CTA passes the first barrier before every CTA has read this
  unsigned gen = *(const volatile unsigned *)&d.cnt->bar_gen;
  const unsigned long long limit = d.prm->barrier_limit;
  stamp(d, 0);
  stage_scan_reduce(d, cta, ncta);
  if (!grid_barrier(d, gen, ncta, limit)) return;
  stamp(d, 1);
  stage_scan_apply(d, cta, ncta);
  if (!grid_barrier(d, gen, ncta, limit)) return;
  stamp(d, 2);
  stage_scatter(d, cta, ncta);
  if (!grid_barrier(d, gen, ncta, limit)) return;
  stamp(d, 3);
  stage_bucket_sort(d, cta, ncta);
  if (!grid_barrier(d, gen, ncta, limit)) return;
  stamp(d, 4);
  stage_p2g<kPersistThreads, kPersistP2GChunk>(d, pin, iin, smem, cta, ncta);
  if (!grid_barrier(d, gen, ncta, limit)) return;
  stamp(d, 5);
  stage_grid_gather<kPersistThreads / 64>(d, 3, cta, ncta);
  if (!grid_barrier(d, gen, ncta, limit)) return;
  if (kColliders) {
    stage_apply_colliders(d, -1, 1, cta, ncta);
    if (!grid_barrier(d, gen, ncta, limit)) return;
  }
  stamp(d, 6);
  stage_g2p<true, true, kPersistThreads, kHencky>(d, pin, iin, pout, iout, smem, cta, ncta);
  // the last CTA to finish notes the end (and resets the count)
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&d.cnt->bar_done, 1u) + 1u == (unsigned)ncta) {
      d.cnt->stage_t[7] = global_ns();
      atomicExch(&d.cnt->bar_done, 0u);
    }
  }
}

// A barrier that expects one CTA more than the grid has: nobody completes it.
__global__ void k_barrier_selftest(DevPtrs d, unsigned long long limit) {
  unsigned gen = *(const volatile unsigned *)&d.cnt->bar_gen;
  grid_barrier(d, gen, gridDim.x + 1, limit);
}

template <bool kHencky, bool kColliders> int occupancy() {
  auto k = k_substep_persistent<kHencky, kColliders>;
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, kPersistSmem);
  int b = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k, kPersistThreads, kPersistSmem) !=
      cudaSuccess)
    return 0;
  return b;
}

template <bool kHencky, bool kColliders>
cudaError_t launch(const DevPtrs &d, int cur, int grid, cudaStream_t s) {
  const float *pin = d.pbuf[cur];
  const int32_t *iin = d.ibuf[cur];
  float *pout = d.pbuf[1 - cur];
  int32_t *iout = d.ibuf[1 - cur];
  DevPtrs dd = d;
  void *args[] = {&dd, &pin, &iin, &pout, &iout};
  return cudaLaunchCooperativeKernel((const void *)k_substep_persistent<kHencky, kColliders>,
                                     dim3(grid), dim3(kPersistThreads), args, kPersistSmem, s);
}

}  // namespace

// Fewer CTAs make each barrier cheaper (one arrival each); a small
// context's stages have little work to spread: a CTA per 256 particle
// slots of capacity (and per directory scan tile), at least one per SM.
int persistent_grid(const DevPtrs &d) {
  int occ = occupancy<false, false>();
  occ = std::min(occ, occupancy<false, true>());
  occ = std::min(occ, occupancy<true, false>());
  occ = std::min(occ, occupancy<true, true>());
  if (occ <= 0) return 0;
  const long long want = std::max<long long>((d.cap + 255) / 256, d.ntiles);
  return (int)std::min<long long>(std::max<long long>(want, d.num_sms), (long long)occ * d.num_sms);
}

cudaError_t launch_substep_persistent(const DevPtrs &d, int cur, bool col, cudaStream_t s) {
  const int grid = d.grid_persist;
  if (grid <= 0) return cudaErrorCooperativeLaunchTooLarge;
  // the arrival counts (a launch that timed out may have left them set)
  static_assert(offsetof(Counters, bar_done) == offsetof(Counters, bar_count) + sizeof(unsigned),
                "bar_count, bar_done adjacent");
  cudaError_t e = cudaMemsetAsync(&d.cnt->bar_count, 0, 2 * sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  if (d.hencky)
    return col ? launch<true, true>(d, cur, grid, s) : launch<true, false>(d, cur, grid, s);
  return col ? launch<false, true>(d, cur, grid, s) : launch<false, false>(d, cur, grid, s);
}

cudaError_t launch_barrier_selftest(const DevPtrs &d, unsigned long long limit, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(&d.cnt->bar_count, 0, sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  DevPtrs dd = d;
  void *args[] = {&dd, &limit};
  const int grid = d.num_sms;  // one CTA per SM: all resident
  e = cudaLaunchCooperativeKernel((const void *)k_barrier_selftest, dim3(grid), dim3(32), args, 0,
                                  s);
  if (e != cudaSuccess) return e;
  return cudaMemsetAsync(&d.cnt->bar_count, 0, sizeof(unsigned), s);
}

}  // namespace zsmpm
