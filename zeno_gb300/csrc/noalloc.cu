// mpm_partition_noalloc: the particle partition (binning into 4^3 blocks and
// the canonical sort) for callers that cannot allocate device memory.
//
// Some hosts own every byte of device memory through their own allocator or
// a fixed budget -- a renderer or game engine plugin, a framework with a
// caching allocator that a stray cudaMalloc would fragment, code that runs
// between the frames of a real-time loop where cudaMalloc / cudaFree would
// synchronise the device.  They pass in their positions and output buffers;
// everything else this entry point needs lives in one file-scope device
// array, `g_noalloc_scratch`, of kNoAllocScratchBytes (32 MiB), which every
// GPU that loads the library holds until the process exits.
//
// Set-up: the first call on a device (with that device current) looks up
// the device address of the array with cudaGetSymbolAddress -- host code
// cannot use the symbol itself, which names a host-side stand-in -- and
// caches it per device.  Make that first call before any stream capture.
// The cached address belongs to the device's primary context: after
// cudaDeviceReset (or any teardown of that context) it is stale, so a process
// that resets a device must not call this entry point on it again.
//
// Every call shares the one array and leaves its contents behind; each call
// clears the parts that must start at zero.  Calls that overlap on the GPU
// (two streams, or two host threads) race on the array: serialise them.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>

#include "zsmpm_internal.cuh"

namespace zsmpm {
namespace {

constexpr long long kNoAllocMaxParticles = ZSMPM_NOALLOC_MAX_PARTICLES;
constexpr long long kNoAllocMaxBlocks = ZSMPM_NOALLOC_MAX_BLOCKS;
constexpr int kNoAllocMaxTiles = (int)((kNoAllocMaxBlocks + kScanTile - 1) / kScanTile);

// scratch layout (byte offsets, each 256-byte aligned)
constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t kOffCounters = 0;
constexpr size_t kOffParams = align256(kOffCounters + sizeof(Counters));
constexpr size_t kOffScene = align256(kOffParams + sizeof(SimParams));
constexpr size_t kOffKeys = align256(kOffScene + sizeof(SceneParams));
constexpr size_t kOffPermTmp = align256(kOffKeys + 4 * kNoAllocMaxParticles);
constexpr size_t kOffDirCount = align256(kOffPermTmp + 4 * kNoAllocMaxParticles);
constexpr size_t kOffDirFill = align256(kOffDirCount + 4 * kNoAllocMaxBlocks);
constexpr size_t kOffDirGb = align256(kOffDirFill + 4 * kNoAllocMaxBlocks);
constexpr size_t kOffDirBk = align256(kOffDirGb + 4 * kNoAllocMaxBlocks);
constexpr size_t kOffDirFlag = align256(kOffDirBk + 4 * kNoAllocMaxBlocks);
constexpr size_t kOffGbDir = align256(kOffDirFlag + kNoAllocMaxBlocks);
constexpr size_t kOffBkDir = align256(kOffGbDir + 4 * kNoAllocMaxBlocks);
constexpr size_t kOffBkStart = align256(kOffBkDir + 4 * kNoAllocMaxBlocks);
constexpr size_t kOffBkCount = align256(kOffBkStart + 4 * kNoAllocMaxBlocks);
constexpr size_t kOffTiles = align256(kOffBkCount + 4 * kNoAllocMaxBlocks);
constexpr size_t kNoAllocUsed = align256(kOffTiles + 12 * (size_t)kNoAllocMaxTiles);
constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;
static_assert(kNoAllocUsed <= kNoAllocScratchBytes, "scratch layout exceeds the array");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// zero what the partition expects to start at zero: counters and the
// directory entries of this call's domain
__global__ void k_noalloc_clear(unsigned char *base, long long ndir) {
  int32_t *count = reinterpret_cast<int32_t *>(base + kOffDirCount);
  int32_t *fill = reinterpret_cast<int32_t *>(base + kOffDirFill);
  uint8_t *flag = base + kOffDirFlag;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ndir;
       i += (long long)gridDim.x * blockDim.x) {
    count[i] = 0;
    fill[i] = 0;
    flag[i] = 0;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    Counters *c = reinterpret_cast<Counters *>(base + kOffCounters);
    c->n_gblocks = 0;
    c->n_buckets = 0;
    c->status = 0;
    c->max_vel_sqr_bits = 0u;
    c->n_binned = 0;
    c->halt = 0;
  }
}

struct DeviceScratch {
  unsigned char *ptr = nullptr;
  int num_sms = 0;
};

std::mutex g_setup_mutex;
DeviceScratch g_setup[64];

int32_t fail(int32_t code, const std::string &msg) {
  set_last_error(msg);  // read back with mpm_last_error()
  return code;
}

// Once per device, with the device current: the device address of the
// scratch array (the symbol itself is a host-side stand-in).
int32_t scratch_for_current_device(DeviceScratch &out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(MPM_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= 64) return fail(MPM_ERR_INVALID, "device ordinal above 63");
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  DeviceScratch &s = g_setup[dev];
  if (!s.ptr) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess)
      return fail(MPM_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess)
      return fail(MPM_ERR_CUDA, std::string("cudaDeviceGetAttribute: ") + cudaGetErrorString(e));
    s.ptr = static_cast<unsigned char *>(p);
    s.num_sms = sms;
  }
  out = s;
  return MPM_OK;
}

}  // namespace
}  // namespace zsmpm

using namespace zsmpm;

extern "C" int32_t mpm_partition_noalloc(const float *x_planes, int64_t n, float dx,
                                         const int32_t block_lo[3], const int32_t block_dims[3],
                                         int32_t *perm, int32_t *pb_dir, int32_t *pb_count,
                                         int64_t cap_pb, int32_t *n_pb, void *stream) {
  if (n < 0 || (n > 0 && (!x_planes || !perm)) || !block_lo || !block_dims || !n_pb ||
      !(dx > 0.0f) || (cap_pb > 0 && (!pb_dir || !pb_count)))
    return fail(MPM_ERR_INVALID, "invalid argument");
  if (n > kNoAllocMaxParticles)
    return fail(MPM_ERR_CAPACITY, "mpm_partition_noalloc takes at most " +
                                      std::to_string(kNoAllocMaxParticles) + " particles");
  // each factor and each partial product is bounded before the next
  // multiplication, so the directory size cannot wrap around
  long long ndir = 1;
  for (int k = 0; k < 3; ++k) {
    if (block_dims[k] < 3) return fail(MPM_ERR_INVALID, "block_dims must be >= 3");
    if (block_lo[k] < -kMaxBlockCoord || block_lo[k] > kMaxBlockCoord - block_dims[k])
      return fail(MPM_ERR_INVALID, "block_lo + block_dims outside +-2^27 blocks");
    ndir *= block_dims[k];
    if (ndir > kNoAllocMaxBlocks)
      return fail(MPM_ERR_CAPACITY, "mpm_partition_noalloc takes a block directory of at most " +
                                        std::to_string(kNoAllocMaxBlocks) + " blocks");
  }
  DeviceScratch sc;
  int32_t rc = scratch_for_current_device(sc);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned char *base = sc.ptr;

  SimParams P{};
  P.dt = 1.0f;
  P.n = n;
  SceneParams S{};
  S.dx = dx;
  S.inv_dx = 1.0f / dx;
  S.Dinv = 4.0f * S.inv_dx * S.inv_dx;
  for (int k = 0; k < 3; ++k) {
    S.block_lo[k] = block_lo[k];
    S.block_dims[k] = block_dims[k];
  }

  DevPtrs d{};
  d.pbuf[0] = const_cast<float *>(x_planes);  // planes x[0..n), y[n..2n), z[2n..3n)
  d.planar_x = 1;
  d.cap = n > 0 ? n : 1;
  d.pkey = reinterpret_cast<int32_t *>(base + kOffKeys);
  d.perm = perm;
  d.perm_tmp = reinterpret_cast<int32_t *>(base + kOffPermTmp);
  d.dir_count = reinterpret_cast<int32_t *>(base + kOffDirCount);
  d.dir_fill = reinterpret_cast<int32_t *>(base + kOffDirFill);
  d.dir_gb = reinterpret_cast<int32_t *>(base + kOffDirGb);
  d.dir_bk = reinterpret_cast<int32_t *>(base + kOffDirBk);
  d.dir_flag = base + kOffDirFlag;
  d.ndir = ndir;
  d.gb_dir = reinterpret_cast<int32_t *>(base + kOffGbDir);
  d.bk_dir = reinterpret_cast<int32_t *>(base + kOffBkDir);
  d.bk_start = reinterpret_cast<int32_t *>(base + kOffBkStart);
  d.bk_count = reinterpret_cast<int32_t *>(base + kOffBkCount);
  d.cap_gblocks = (int)ndir;
  d.tile_sums = reinterpret_cast<int32_t *>(base + kOffTiles);
  d.ntiles = (int)((ndir + kScanTile - 1) / kScanTile);
  d.cnt = reinterpret_cast<Counters *>(base + kOffCounters);
  d.prm = reinterpret_cast<SimParams *>(base + kOffParams);
  d.scn = reinterpret_cast<SceneParams *>(base + kOffScene);
  d.n_scenes = 1;
  d.num_sms = sc.num_sms;

  cudaError_t e = cudaMemcpyAsync(d.prm, &P, sizeof(SimParams), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d.scn, &S, sizeof(SceneParams), cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return fail(MPM_ERR_CUDA, std::string("parameters: ") + cudaGetErrorString(e));
  k_noalloc_clear<<<sc.num_sms * 4, 256, 0, s>>>(base, ndir);
  launch_bin(d, 0, s);
  launch_scan(d, s);
  launch_scatter(d, s);
  launch_bucket_sort(d, s);
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(MPM_ERR_CUDA, std::string("partition: ") + cudaGetErrorString(e));
  Counters h{};
  e = cudaMemcpyAsync(&h, d.cnt, sizeof(Counters), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail(MPM_ERR_CUDA, std::string("partition: ") + cudaGetErrorString(e));
  *n_pb = h.n_buckets;
  if (h.status & ST_NAN) return fail(MPM_ERR_NAN, "non-finite particle position");
  if (h.status & ST_OUT_OF_DOMAIN) return fail(MPM_ERR_OUT_OF_DOMAIN, "a particle lies outside the block directory");
  if (h.n_buckets > cap_pb)
    return fail(MPM_ERR_CAPACITY, "cap_pb is smaller than the number of particle blocks (" +
                                      std::to_string(h.n_buckets) + ")");
  if (h.n_buckets > 0) {
    e = cudaMemcpyAsync(pb_dir, d.bk_dir, h.n_buckets * sizeof(int32_t), cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(pb_count, d.bk_count, h.n_buckets * sizeof(int32_t),
                          cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(MPM_ERR_CUDA, std::string("outputs: ") + cudaGetErrorString(e));
  }
  return MPM_OK;
}
