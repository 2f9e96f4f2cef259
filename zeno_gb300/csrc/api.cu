// C ABI of the GB300 MLS-MPM substep (declared in include/zsmpm.h).
//
// A context owns every device buffer of one scene (allocated once at
// creation; no allocation on the substep path), one CUDA stream, and two
// instantiated CUDA graphs of a whole substep, one per particle buffer
// parity.  Kernel parameters that change between calls (dt, gravity,
// boundary, material count) live in a small device struct that the host
// refreshes with one copy before launching, so a captured graph stays valid
// when dt changes (SubstepDt, zeno/src/nodes/ControlNodes.cpp:251-320).
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstddef>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "cloth_grid.cuh"
#include "zsmpm_internal.cuh"

using namespace zsmpm;

// An NVTX range around a C-ABI call: the call's name on a profiler's
// timeline (NVTX v3 is header-only; with no tool attached a push is a check
// of one function pointer).
struct NvtxRange {
  explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange &) = delete;
  NvtxRange &operator=(const NvtxRange &) = delete;
};
#define ZS_RANGE(name) NvtxRange zs_nvtx_range_(name)

namespace {

thread_local std::string g_last_error;

int32_t fail(int32_t code, const std::string &msg) {
  g_last_error = msg;
  return code;
}

#define ZS_CUDA(expr)                                                                   \
  do {                                                                                  \
    cudaError_t e_ = (expr);                                                            \
    if (e_ != cudaSuccess)                                                              \
      return fail(MPM_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
  } while (0)

}  // namespace

void zsmpm::set_last_error(const std::string &msg) { g_last_error = msg; }

constexpr int kUploadChunks = 4;  // pieces of a large upload, pipelined

struct mpm_ctx {
  int device = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  DevPtrs d{};
  SimParams prm{};
  bool prm_dirty = true;
  int cur = 0;
  bool partition_valid = false;
  long long cloth_capb_want = 0;  // the cloth's block capacity before the directory's bound
  bool needs_full_clear = false;
  bool binned = false;  // directory counts describe the current positions
  int64_t substeps = 0;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  Counters *h_cnt = nullptr;  // pinned
  std::vector<void *> allocs;
  std::vector<void *> collider_allocs;  // sample grids of the level-set colliders
  std::vector<ColliderDev> colliders;   // host copy (positions as set)
  cudaEvent_t events[MPM_NUM_STAGES + 1] = {};
  std::vector<SceneParams> scenes;
  int n_materials = 0;
  bool differentiable = false;  // every material has an adjoint
  // pipelined upload: host-to-device copies on their own stream
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t copy_ev[kUploadChunks + 1] = {};
  // asynchronous frame output: device snapshot, copy stream, events
  float *frame_buf = nullptr;
  cudaStream_t frame_stream = nullptr;
  cudaEvent_t frame_ready = nullptr, frame_done = nullptr;
  bool frame_pending = false;
  // growing directory (mpm_set_auto_regrow): the fused substeps queued since
  // the last synchronisation, as (dt, count) batches, and the device's
  // started-substep count at that synchronisation
  bool auto_regrow = false;
  std::vector<std::pair<float, int32_t>> pending;
  int64_t pending_total = 0;
  int64_t started_base = 0;
  int32_t regrows = 0;
  int32_t max_grid_blocks_req = 0;  // as given at creation (0: the default rule)
  // mpm_set_persistent: the fused substep as one cooperative kernel
  bool persistent = false;
  // boundary grid (mpm_set_grid_boundary): its points as given (the grid is
  // built again when the directory grows)
  std::vector<float> bnd_pts;  // x 3, v 3, m, nrm 3 per point
  int64_t bnd_n = 0, bnd_n_verts = 0;
  // differentiable rollout: the partition and grid of each recomputed
  // substep of a segment, kept for its adjoint (PartSet below), `pset_cap`
  // blocks each; n_gblocks, n_buckets of each (device, 2 per set)
  std::vector<zsmpm::PartSet> psets;
  int pset_cap = 0;
  int32_t *pset_cnt = nullptr;
  // the last segment of the latest rollout forward, kept in seg_states and
  // psets for the backward with the same arguments
  struct {
    bool valid = false;
    float dt = 0.0f;
    int32_t n = 0, every = 0;
    const float *ckpts = nullptr;
    const float *seg = nullptr;
  } tail;
};

namespace {

// A capacity overflow drops particle or grid blocks, so whatever the next
// substeps flag (stale slots binned out of the domain, non-finite values) is
// its consequence: it is reported first.
int32_t map_status(int bits) {
  if (bits & ST_CAPACITY) return MPM_ERR_CAPACITY;
  if (bits & ST_NAN) return MPM_ERR_NAN;
  if (bits & ST_OUT_OF_DOMAIN) return MPM_ERR_OUT_OF_DOMAIN;
  if (bits & ST_TIMEOUT) return MPM_ERR_TIMEOUT;
  if (bits & ST_STENCIL) return MPM_ERR_CFL;
  if (bits & ST_MATERIAL) return MPM_ERR_INVALID;
  return MPM_OK;  // ST_BUCKET_OVERSIZE only affects the in-block order
}

const char *status_text(int32_t st) {
  switch (st) {
    case MPM_ERR_NAN: return "non-finite particle state or inverted element";
    case MPM_ERR_OUT_OF_DOMAIN: return "a particle left the block directory";
    case MPM_ERR_CAPACITY: return "more grid blocks than the context's capacity";
    case MPM_ERR_TIMEOUT: return "a bounded device-side wait gave up";
    case MPM_ERR_CFL: return "a particle moved out of its block's stencil window";
    case MPM_ERR_INVALID: return "material id out of range in an asynchronous upload";
    default: return "";
  }
}

template <class T> int32_t dalloc(mpm_ctx *c, T **p, size_t count) {
  void *q = nullptr;
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc(&q, count * sizeof(T));
  if (e != cudaSuccess)
    return fail(MPM_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  c->allocs.push_back(q);
  *p = static_cast<T *>(q);
  return MPM_OK;
}

int32_t push_params(mpm_ctx *c) {
  if (!c->prm_dirty) return MPM_OK;
  ZS_CUDA(cudaMemcpyAsync(c->d.prm, &c->prm, sizeof(SimParams), cudaMemcpyHostToDevice,
                          c->stream));
  ZS_CUDA(cudaMemcpyAsync(c->d.scn, c->scenes.data(), sizeof(SceneParams) * c->scenes.size(),
                          cudaMemcpyHostToDevice, c->stream));
  c->prm_dirty = false;
  return MPM_OK;
}

int32_t set_dt(mpm_ctx *c, float dt) {
  if (!(dt > 0.0f) || !std::isfinite(dt)) return fail(MPM_ERR_INVALID, "dt must be positive");
  if (c->prm.dt != dt) {
    c->prm.dt = dt;
    c->prm_dirty = true;
  }
  return push_params(c);
}

void set_auto_step(mpm_ctx *c, int v) {
  if (c->prm.auto_step != v) {
    c->prm.auto_step = v;
    c->prm_dirty = true;
  }
}

int32_t check(mpm_ctx *c) {
  if (!c) return fail(MPM_ERR_INVALID, "null context");
  cudaError_t e = cudaSetDevice(c->device);
  if (e != cudaSuccess) return fail(MPM_ERR_CUDA, cudaGetErrorString(e));
  return MPM_OK;
}

int32_t launch_check(const char *what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(MPM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  return MPM_OK;
}

// Binning of the current positions into the directory counts (only when
// they do not already describe them: after an upload or a stage G2P).
void enqueue_bin_if_needed(mpm_ctx *c) {
  if (!c->binned) {
    launch_bin(c->d, c->cur, c->stream);
    c->binned = true;
  }
}

void enqueue_sort(mpm_ctx *c) {
  launch_scan(c->d, c->stream);  // consumes (zeroes) the counts
  launch_scatter(c->d, c->stream);
  launch_bucket_sort(c->d, c->stream);
  c->binned = false;
}

// mpm_set_persistent applies: the fused substep is one cooperative kernel
bool uses_persistent(const mpm_ctx *c) {
  return c->persistent && c->d.cloth.n_verts == 0 && c->d.n_trackers == 0 &&
         c->d.transfer == MPM_TRANSFER_APIC && !c->d.bnd_map;
}

// One substep of the fused path; the counts of the current positions must be
// binned already, and the G2P epilogue bins the new positions, so a graph of
// this sequence can be replayed back to back.  With `ev` set, event i is
// recorded before stage i and event MPM_NUM_STAGES after the last one.
void enqueue_substep(mpm_ctx *c, int cur, cudaEvent_t *ev = nullptr) {
  auto mark = [&](int i) {
    if (ev) cudaEventRecord(ev[i], c->stream);
  };
  const bool cloth = c->d.cloth.n_verts > 0, trackers = c->d.n_trackers > 0;
  mark(MPM_STAGE_SCAN);
  if (uses_persistent(c)) {
    if (c->auto_regrow) launch_substep_gate(c->d, c->stream);
    launch_substep_persistent(c->d, cur, !c->colliders.empty(), c->stream);
    for (int i = MPM_STAGE_SCATTER; i <= MPM_NUM_STAGES; ++i) mark(i);
    return;
  }
  if (cloth) launch_cloth_mark(c->d, c->stream);  // the cloth's grid blocks
  if (trackers) launch_tracker_mark(c->d, c->stream);
  // a growing directory: this substep and the queued ones halt if a
  // particle, cloth vertex or tracker left the directory
  if (c->auto_regrow) launch_substep_gate(c->d, c->stream);
  launch_scan(c->d, c->stream);
  mark(MPM_STAGE_SCATTER);
  launch_scatter(c->d, c->stream);
  mark(MPM_STAGE_SORT);
  launch_bucket_sort(c->d, c->stream);
  mark(MPM_STAGE_P2G);
  launch_p2g(c->d, cur, c->stream);
  mark(MPM_STAGE_GRID_UPDATE);
  if (cloth) {  // particle sums, the cloth's scatter, then its tiles and the update
    launch_grid_gather(c->d, 0, c->stream);
    launch_cloth_p2g(c->d, false, c->stream);
    launch_grid_update(c->d, 3 | kGridAddCloth, c->stream);
    if (!c->colliders.empty()) launch_apply_colliders(c->d, -1, c->stream);
  } else {
    launch_grid_gather(c->d, 3, c->stream);
    if (!c->colliders.empty()) launch_apply_colliders_listed(c->d, c->stream);
  }
  launch_apply_grid_boundary(c->d, c->stream);  // a boundary grid, if set
  mark(MPM_STAGE_G2P);
  launch_g2p(c->d, cur, 1, 1, c->stream);
  if (cloth) launch_cloth_g2p(c->d, c->stream);
  if (trackers) launch_tracker_g2p(c->d, c->stream);
  mark(MPM_NUM_STAGES);
}

bool graphs_enabled() {
  const char *e = std::getenv("ZSMPM_NO_GRAPH");
  return !(e && e[0] == '1');
}

int32_t ensure_graph(mpm_ctx *c, int cur) {
  if (c->graph[cur]) return MPM_OK;
  cudaGraph_t g = nullptr;
  ZS_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  enqueue_substep(c, cur);
  cudaError_t e = cudaStreamEndCapture(c->stream, &g);
  if (e != cudaSuccess) return fail(MPM_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(e));
  e = cudaGraphInstantiate(&c->graph[cur], g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess)
    return fail(MPM_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
  return MPM_OK;
}

int32_t prepare_partition(mpm_ctx *c) {
  if (c->needs_full_clear) {
    launch_full_dir_clear(c->d, c->stream);
    c->needs_full_clear = false;
    c->binned = false;
  }
  return MPM_OK;
}

void drop_graphs(mpm_ctx *c) {
  for (int k = 0; k < 2; ++k)
    if (c->graph[k]) {
      cudaGraphExecDestroy(c->graph[k]);
      c->graph[k] = nullptr;
    }
}

// replays of one synchronisation after which the directory has grown
constexpr int kMaxRegrowRounds = 8;

}  // namespace
extern "C" int32_t mpm_sync(mpm_ctx *c);
namespace {

// With a growing directory, the calls that read or change the particle state
// first let the queued substeps finish (growing the directory and replaying
// them if a particle left it), so that they see the state after all of them.
int32_t settle(mpm_ctx *c) {
  if (!c->auto_regrow || c->pending_total == 0) return MPM_OK;
  return mpm_sync(c);
}

// frees a buffer of the context and forgets it
void dfree(mpm_ctx *c, void *p) {
  if (!p) return;
  auto it = std::find(c->allocs.begin(), c->allocs.end(), p);
  if (it != c->allocs.end()) c->allocs.erase(it);
  cudaFree(p);
}

template <class T> int32_t drealloc(mpm_ctx *c, T **p, size_t count) {
  dfree(c, *p);
  *p = nullptr;
  return dalloc(c, p, count);
}

// ordered bits (k_bbox) -> float
float from_ordered_bits(unsigned u) {
  const unsigned b = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
  float f;
  std::memcpy(&f, &b, sizeof(f));
  return f;
}

// Grows the directory of a one-scene context around its current particles
// (and cloth vertices, trackers): the box of their blocks plus a margin of a
// quarter of its extent (at least 2 blocks) on every side.  The directory
// and, if the new box allows more grid blocks than the context holds, the
// grid-sized buffers are reallocated; the counters, graphs and partition
// start afresh, and the next substep bins the current positions.
int32_t build_grid_boundary(mpm_ctx *c);

// frees a rollout's kept partition sets (PartSet)
void drop_psets(mpm_ctx *c) {
  for (PartSet &p : c->psets) {
    for (void *q : {(void *)p.perm, (void *)p.dir_gb, (void *)p.dir_bk, (void *)p.gb_dir,
                    (void *)p.bk_dir, (void *)p.bk_start, (void *)p.bk_count, (void *)p.grid,
                    (void *)p.ptile})
      dfree(c, q);
  }
  c->psets.clear();
  dfree(c, c->pset_cnt);
  c->pset_cnt = nullptr;
  c->pset_cap = 0;
}

int32_t regrow(mpm_ctx *c) {
  DevPtrs &d = c->d;
  if (c->scenes.size() != 1) return fail(MPM_ERR_OUT_OF_DOMAIN, "a particle left the block directory");
  const unsigned init[6] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u};
  ZS_CUDA(cudaMemcpyAsync(d.cnt->bbox, init, sizeof(init), cudaMemcpyHostToDevice, c->stream));
  launch_bbox(d, c->cur, c->stream);
  ZS_CUDA(cudaMemcpyAsync(c->h_cnt, d.cnt, sizeof(Counters), cudaMemcpyDeviceToHost, c->stream));
  ZS_CUDA(cudaStreamSynchronize(c->stream));
  SceneParams &S = c->scenes[0];
  int lo[3], dims[3];
  long long ndir = 1;
  for (int a = 0; a < 3; ++a) {
    if (c->h_cnt->bbox[a] > c->h_cnt->bbox[3 + a]) {  // nothing to place
      lo[a] = S.block_lo[a];
      dims[a] = S.block_dims[a];
    } else {
      const double xl = from_ordered_bits(c->h_cnt->bbox[a]);
      const double xh = from_ordered_bits(c->h_cnt->bbox[3 + a]);
      const double bl = std::floor(std::floor(xl * S.inv_dx - 0.5) / 4.0);
      const double bh = std::floor(std::floor(xh * S.inv_dx - 0.5) / 4.0);
      const double ext = bh - bl + 1.0, margin = std::max(2.0, std::floor(ext / 4.0));
      const double l = bl - margin, dm = ext + 2.0 * margin;
      if (l < -kMaxBlockCoord || l + dm > kMaxBlockCoord || dm > (double)kMaxDirBlocks)
        return fail(MPM_ERR_OUT_OF_DOMAIN, "particles spread beyond the largest block directory");
      lo[a] = (int)l;
      dims[a] = std::max(3, (int)dm);
    }
    ndir *= dims[a];
    if (ndir >= kMaxDirBlocks)
      return fail(MPM_ERR_OUT_OF_DOMAIN,
                  "particles spread beyond the largest block directory (2^25 blocks)");
  }
  int32_t rc;
  const int ntiles = (int)((ndir + kScanTile - 1) / kScanTile);
  if ((rc = drealloc(c, &d.dir_count, ndir)) || (rc = drealloc(c, &d.dir_fill, ndir)) ||
      (rc = drealloc(c, &d.dir_gb, ndir)) || (rc = drealloc(c, &d.dir_bk, ndir)) ||
      (rc = drealloc(c, &d.dir_flag, ndir)) || (rc = drealloc(c, &d.tile_sums, (size_t)3 * ntiles)))
    return rc;
  long long capg = c->max_grid_blocks_req > 0 ? c->max_grid_blocks_req
                                               : std::max<long long>(16384, d.cap / 4);
  capg = std::min<long long>(capg, ndir);
  if (capg > d.cap_gblocks) {
    if ((rc = drealloc(c, &d.ptile, (size_t)capg * kTileNodes)) ||
        (rc = drealloc(c, &d.gb_dir, capg)) || (rc = drealloc(c, &d.bk_dir, capg)) ||
        (rc = drealloc(c, &d.bk_start, capg)) || (rc = drealloc(c, &d.bk_count, capg)) ||
        (rc = drealloc(c, &d.grid, (size_t)capg * 64)) || (rc = drealloc(c, &d.near_gb, capg)))
      return rc;
    if (d.grid2 && (rc = drealloc(c, &d.grid2, (size_t)capg * 64))) return rc;
    if (d.ptile2 && (rc = drealloc(c, &d.ptile2, (size_t)capg * kTileNodes))) return rc;
    if (d.ptile_adj && (rc = drealloc(c, &d.ptile_adj, (size_t)capg * kTileNodes))) return rc;
    d.cap_gblocks = (int)capg;
  }
  ZS_CUDA(cudaMemsetAsync(d.dir_count, 0, ndir * sizeof(int32_t), c->stream));
  ZS_CUDA(cudaMemsetAsync(d.dir_fill, 0, ndir * sizeof(int32_t), c->stream));
  ZS_CUDA(cudaMemsetAsync(d.dir_gb, 0xff, ndir * sizeof(int32_t), c->stream));
  ZS_CUDA(cudaMemsetAsync(d.dir_bk, 0xff, ndir * sizeof(int32_t), c->stream));
  ZS_CUDA(cudaMemsetAsync(d.dir_flag, 0, ndir, c->stream));
  ZS_CUDA(cudaMemsetAsync(d.cnt, 0, sizeof(Counters), c->stream));
  ClothDev &cl = d.cloth;
  if (cl.n_verts > 0) {  // the cloth's own partition runs on the same directory
    if ((rc = drealloc(c, &cl.cdir_count, ndir)) || (rc = drealloc(c, &cl.cdir_fill, ndir)) ||
        (rc = drealloc(c, &cl.cdir_gb, ndir)) || (rc = drealloc(c, &cl.cdir_bk, ndir)) ||
        (rc = drealloc(c, &cl.cdir_flag, ndir)) ||
        (rc = drealloc(c, &cl.ctile_sums, (size_t)3 * ntiles)))
      return rc;
    ZS_CUDA(cudaMemsetAsync(cl.cdir_count, 0, ndir * sizeof(int32_t), c->stream));
    ZS_CUDA(cudaMemsetAsync(cl.cdir_flag, 0, ndir, c->stream));
    ZS_CUDA(cudaMemsetAsync(cl.ccnt, 0, sizeof(Counters), c->stream));
    const long long capb =
        std::min<long long>({ndir, cl.n_verts + cl.n_eles, c->cloth_capb_want});
    if (capb > cl.cap_cblocks) {  // the old directory bounded the cloth's blocks
      if ((rc = drealloc(c, &cl.cgb_dir, capb)) || (rc = drealloc(c, &cl.cbk_dir, capb)) ||
          (rc = drealloc(c, &cl.cbk_start, capb)) || (rc = drealloc(c, &cl.cbk_count, capb)) ||
          (rc = drealloc(c, &cl.ctile, (size_t)capb * kTileNodes)) ||
          (rc = drealloc(c, &cl.ctile2, (size_t)capb * kTileNodes)))
        return rc;
      cl.cap_cblocks = (int)capb;
    }
  }
  for (int a = 0; a < 3; ++a) {
    S.block_lo[a] = lo[a];
    S.block_dims[a] = dims[a];
  }
  S.dir_off = 0;
  d.ndir = ndir;
  d.ntiles = ntiles;
  d.grid_persist = persistent_grid(d);
  c->prm_dirty = true;
  if ((rc = push_params(c))) return rc;
  drop_graphs(c);
  c->started_base = 0;
  c->needs_full_clear = false;
  c->binned = false;
  c->partition_valid = false;
  c->regrows += 1;
  // a rollout's kept partition sets index the old directory
  drop_psets(c);
  c->tail.valid = false;
  if (c->bnd_n > 0) {  // the boundary grid on the new directory
    dfree(c, d.bnd_map);
    d.bnd_map = nullptr;
    if ((rc = build_grid_boundary(c))) return rc;
  }
  return MPM_OK;
}

}  // namespace

extern "C" {

int32_t mpm_abi_version(void) { return ZSMPM_ABI_VERSION; }

const char *mpm_last_error(void) { return g_last_error.c_str(); }

}  // extern "C"

namespace {

SceneParams scene_from(const mpm_scene_desc &sd) {
  SceneParams S{};
  S.dx = sd.dx;
  S.inv_dx = 1.0f / sd.dx;
  S.Dinv = 4.0f * S.inv_dx * S.inv_dx;
  for (int k = 0; k < 3; ++k) {
    S.gravity[k] = sd.gravity[k];
    S.block_lo[k] = sd.block_lo[k];
    S.block_dims[k] = sd.block_dims[k];
    S.bc_lo[k] = sd.boundary.lo[k];
    S.bc_hi[k] = sd.boundary.hi[k];
  }
  S.bc_type = sd.boundary.type;
  S.bc_thickness = sd.boundary.thickness;
  return S;
}

int32_t create_context(int32_t device, const mpm_scene_desc *scenes, int32_t n_scenes,
                       int64_t max_particles, int32_t max_grid_blocks, mpm_ctx **out) {
  if (!scenes || !out || n_scenes <= 0) return fail(MPM_ERR_INVALID, "null argument");
  *out = nullptr;
  if (n_scenes > kMaxScenes)
    return fail(MPM_ERR_INVALID, "at most " + std::to_string(kMaxScenes) + " scenes");
  if (max_particles <= 0 || max_particles >= (int64_t(1) << 31))
    return fail(MPM_ERR_INVALID, "max_particles must be in [1, 2^31)");
  long long ndir = 0;
  std::vector<SceneParams> sp(n_scenes);
  for (int s = 0; s < n_scenes; ++s) {
    const mpm_scene_desc &sd = scenes[s];
    if (!(sd.dx > 0.0f)) return fail(MPM_ERR_INVALID, "dx must be positive");
    if (sd.boundary.type < MPM_BC_NONE || sd.boundary.type > MPM_BC_SEPARATE ||
        sd.boundary.thickness < 0)
      return fail(MPM_ERR_INVALID, "bad boundary");
    // each factor and each partial product is bounded before the next
    // multiplication, so the directory size cannot wrap around
    long long nd = 1;
    for (int k = 0; k < 3; ++k) {
      if (sd.block_dims[k] < 3) return fail(MPM_ERR_INVALID, "block_dims must be >= 3");
      if (sd.block_lo[k] < -kMaxBlockCoord || sd.block_lo[k] > kMaxBlockCoord - sd.block_dims[k])
        return fail(MPM_ERR_INVALID, "block_lo + block_dims outside +-2^27 blocks");
      nd *= sd.block_dims[k];
      if (nd >= kMaxDirBlocks)
        return fail(MPM_ERR_INVALID, "block directory larger than 2^25 blocks");
    }
    sp[s] = scene_from(sd);
    sp[s].dir_off = (int)std::min<long long>(ndir, 1ll << 30);
    ndir += nd;
    if (ndir >= kMaxDirBlocks) return fail(MPM_ERR_INVALID, "block directory larger than 2^25 blocks");
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0)
    return fail(MPM_ERR_NO_DEVICE, "no CUDA device");
  if (device == -1 && cudaGetDevice(&device) != cudaSuccess)
    return fail(MPM_ERR_CUDA, "cudaGetDevice");
  if (device < 0 || device >= ndev) return fail(MPM_ERR_INVALID, "bad device ordinal");
  int major = 0, minor = 0, sms = 0;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, device);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (major * 10 + minor != 103)
    return fail(MPM_ERR_NO_DEVICE, "zsmpm is built for sm_103a (GB300) only; device is sm_" +
                                       std::to_string(major * 10 + minor));

  mpm_ctx *c = new mpm_ctx();
  c->device = device;
  int32_t rc = MPM_OK;
  auto bail = [&](int32_t r) {
    mpm_ctx_destroy(c);
    return r;
  };
  if (cudaSetDevice(c->device) != cudaSuccess) return bail(fail(MPM_ERR_CUDA, "cudaSetDevice"));
  if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(fail(MPM_ERR_CUDA, "cudaStreamCreate"));
  c->stream = c->own_stream;

  const long long cap = max_particles;
  long long capg = max_grid_blocks > 0 ? max_grid_blocks : std::max<long long>(16384, cap / 4);
  capg = std::min<long long>(capg, ndir);
  DevPtrs &d = c->d;
  c->max_grid_blocks_req = max_grid_blocks;
  d.cap = cap;
  d.ndir = ndir;
  d.cap_gblocks = (int)capg;
  d.num_sms = sms;
  d.ntiles = (int)((ndir + kScanTile - 1) / kScanTile);
  d.n_scenes = n_scenes;
  configure_launches(d);
  for (int k = 0; k < 2; ++k) {
    if ((rc = dalloc(c, &d.pbuf[k], (size_t)tiled_elems(cap, NCH)))) return bail(rc);
    if ((rc = dalloc(c, &d.ibuf[k], (size_t)tiled_elems(cap, NICH)))) return bail(rc);
  }
  if ((rc = dalloc(c, &d.pkey, cap)) || (rc = dalloc(c, &d.perm, cap)) ||
      (rc = dalloc(c, &d.perm_tmp, cap)) ||
      (rc = dalloc(c, &d.dir_count, ndir)) || (rc = dalloc(c, &d.dir_fill, ndir)) ||
      (rc = dalloc(c, &d.dir_gb, ndir)) || (rc = dalloc(c, &d.dir_flag, ndir)) ||
      (rc = dalloc(c, &d.dir_bk, ndir)) || (rc = dalloc(c, &d.ptile, (size_t)capg * kTileNodes)) ||
      (rc = dalloc(c, &d.gb_dir, capg)) || (rc = dalloc(c, &d.bk_dir, capg)) ||
      (rc = dalloc(c, &d.bk_start, capg)) || (rc = dalloc(c, &d.bk_count, capg)) ||
      (rc = dalloc(c, &d.grid, (size_t)capg * 64)) ||
      (rc = dalloc(c, &d.tile_sums, (size_t)3 * d.ntiles)) || (rc = dalloc(c, &d.cnt, 1)) ||
      (rc = dalloc(c, &d.prm, 1)) || (rc = dalloc(c, &d.scn, n_scenes)) ||
      (rc = dalloc(c, &d.mats, kMaxMaterials)) || (rc = dalloc(c, &d.colliders, kMaxColliders)) ||
      (rc = dalloc(c, &d.beta, cap)) || (rc = dalloc(c, &d.vms, cap)) ||
      (rc = dalloc(c, &d.near_gb, capg)))
    return bail(rc);
  if (cudaMallocHost(&c->h_cnt, sizeof(Counters)) != cudaSuccess)
    return bail(fail(MPM_ERR_CUDA, "cudaMallocHost"));
  // every slot of the particle-indexed buffers starts as a valid index / id
  for (int k = 0; k < 2; ++k) {
    cudaMemsetAsync(d.pbuf[k], 0, (size_t)tiled_elems(cap, NCH) * sizeof(float), c->stream);
    cudaMemsetAsync(d.ibuf[k], 0, (size_t)tiled_elems(cap, NICH) * sizeof(int32_t), c->stream);
  }
  cudaMemsetAsync(d.perm, 0, (size_t)cap * sizeof(int32_t), c->stream);
  cudaMemsetAsync(d.pkey, 0, (size_t)cap * sizeof(int32_t), c->stream);
  cudaMemsetAsync(d.beta, 0, (size_t)cap * sizeof(float), c->stream);
  cudaMemsetAsync(d.vms, 0, (size_t)cap * sizeof(float), c->stream);
  cudaMemsetAsync(d.dir_count, 0, ndir * sizeof(int32_t), c->stream);
  cudaMemsetAsync(d.dir_fill, 0, ndir * sizeof(int32_t), c->stream);
  cudaMemsetAsync(d.dir_gb, 0xff, ndir * sizeof(int32_t), c->stream);
  cudaMemsetAsync(d.dir_bk, 0xff, ndir * sizeof(int32_t), c->stream);
  cudaMemsetAsync(d.dir_flag, 0, ndir, c->stream);
  cudaMemsetAsync(d.cnt, 0, sizeof(Counters), c->stream);
  cudaMemsetAsync(d.mats, 0, kMaxMaterials * sizeof(MatParams), c->stream);

  c->scenes = sp;
  SimParams &P = c->prm;
  P.dt = 1e-4f;
  P.has_lame = 0;
  P.n = 0;
  c->prm_dirty = true;
  if ((rc = push_params(c))) return bail(rc);
  if (cudaStreamSynchronize(c->stream) != cudaSuccess)
    return bail(fail(MPM_ERR_CUDA, "context initialisation failed"));
  *out = c;
  return MPM_OK;
}

}  // namespace

extern "C" {

int32_t mpm_ctx_create(const mpm_ctx_desc *desc, mpm_ctx **out) {
  if (!desc || !out) return fail(MPM_ERR_INVALID, "null argument");
  mpm_scene_desc sd{};
  sd.dx = desc->dx;
  for (int k = 0; k < 3; ++k) {
    sd.block_lo[k] = desc->block_lo[k];
    sd.block_dims[k] = desc->block_dims[k];
  }
  sd.gravity[1] = -9.8f;  // UpdateZSGrid "gravity" default (MPMPipeline.cu:946-951)
  sd.boundary.type = MPM_BC_NONE;
  return create_context(desc->device, &sd, 1, desc->max_particles, desc->max_grid_blocks, out);
}

int32_t mpm_batch_create(int32_t device, const mpm_scene_desc *scenes, int32_t n_scenes,
                         int64_t max_particles, int32_t max_grid_blocks, mpm_ctx **out) {
  return create_context(device, scenes, n_scenes, max_particles, max_grid_blocks, out);
}

int32_t mpm_ctx_destroy(mpm_ctx *c) {
  if (!c) return MPM_OK;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (int k = 0; k < 2; ++k)
    if (c->graph[k]) cudaGraphExecDestroy(c->graph[k]);
  for (cudaEvent_t e : c->events)
    if (e) cudaEventDestroy(e);
  if (c->frame_stream) {
    cudaStreamSynchronize(c->frame_stream);
    cudaStreamDestroy(c->frame_stream);
  }
  if (c->frame_ready) cudaEventDestroy(c->frame_ready);
  if (c->copy_stream) {
    cudaStreamSynchronize(c->copy_stream);
    cudaStreamDestroy(c->copy_stream);
  }
  for (cudaEvent_t e : c->copy_ev)
    if (e) cudaEventDestroy(e);
  if (c->frame_done) cudaEventDestroy(c->frame_done);
  for (void *p : c->allocs) cudaFree(p);
  for (void *p : c->collider_allocs) cudaFree(p);
  if (c->h_cnt) cudaFreeHost(c->h_cnt);
  if (c->own_stream) cudaStreamDestroy(c->own_stream);
  delete c;
  return MPM_OK;
}

int32_t mpm_set_stream(mpm_ctx *c, void *stream) {
  int32_t rc = check(c);
  if (rc) return rc;
  c->stream = stream ? static_cast<cudaStream_t>(stream) : c->own_stream;
  c->prm_dirty = true;
  return push_params(c);
}

int32_t mpm_set_materials(mpm_ctx *c, const mpm_material *mats, int32_t n) {
  int32_t rc = check(c);
  if (rc) return rc;
  if ((rc = settle(c))) return rc;
  if (!mats || n <= 0 || n > kMaxMaterials)
    return fail(MPM_ERR_INVALID, "need 1.." + std::to_string(kMaxMaterials) + " materials");
  std::vector<MatParams> h(kMaxMaterials);
  for (int i = 0; i < n; ++i) {
    const mpm_material &m = mats[i];
    if (m.type < MPM_FCR || m.type > MPM_SNHK) return fail(MPM_ERR_INVALID, "unknown material type");
    if (m.plasticity < MPM_PLASTIC_NONE || m.plasticity > MPM_PLASTIC_NACC)
      return fail(MPM_ERR_INVALID, "unknown plasticity");
    if (m.plasticity != MPM_PLASTIC_NONE && m.type != MPM_STVK)
      return fail(MPM_ERR_INVALID,
                  "plasticity runs on the StVK-Hencky model (Generation.cu:66-84)");
    if (m.plasticity == MPM_PLASTIC_NAVM && !(m.yield_stress > 0.0f))
      return fail(MPM_ERR_INVALID, "von Mises plasticity needs a positive yield stress");
    if (m.plasticity == MPM_PLASTIC_NACC && !(m.cc_beta >= 0.0f && m.cc_xi >= 0.0f))
      return fail(MPM_ERR_INVALID, "Cam-Clay needs beta >= 0 and xi >= 0");
    MatParams &p = h[i];
    p.type = m.type;
    p.plastic = m.plasticity;
    // Lame parameters (standard relations, zs::lame_parameters at Temp.cu:47)
    p.mu = m.E / (2.0f * (1.0f + m.nu));
    p.lam = m.E * m.nu / ((1.0f + m.nu) * (1.0f - 2.0f * m.nu));
    const double phi = (double)m.friction_angle_deg * 3.14159265358979323846 / 180.0;
    const double s = std::sin(phi);
    p.alpha = (float)(std::sqrt(2.0 / 3.0) * 2.0 * s / (3.0 - s));
    p.bulk = m.bulk;
    p.gamma = m.gamma;
    p.yield = m.yield_stress;
    // Cam-Clay critical-state slope from the friction angle (the
    // Mohr-Coulomb compression match M = 6 sin(phi) / (3 - sin(phi)))
    p.cc_M = (float)(6.0 * s / (3.0 - s));
    p.cc_beta = m.cc_beta;
    p.cc_xi = m.cc_xi;
    p.pad = 0.0f;
  }
  ZS_CUDA(cudaMemcpyAsync(c->d.mats, h.data(), sizeof(MatParams) * kMaxMaterials,
                          cudaMemcpyHostToDevice, c->stream));
  ZS_CUDA(cudaStreamSynchronize(c->stream));
  c->n_materials = n;
  int hencky = 0;
  for (int i = 0; i < n; ++i)
    hencky |= mats[i].plasticity == MPM_PLASTIC_NAVM || mats[i].plasticity == MPM_PLASTIC_NACC;
  if (hencky != c->d.hencky) {
    c->d.hencky = hencky;
    drop_graphs(c);  // the graphs hold the G2P variant
  }
  // adjoints exist for the elastic models and for sand (StVK-Hencky with or
  // without the Drucker-Prager projection); not for the equation-of-state fluid
  c->differentiable = true;
  for (int i = 0; i < n; ++i)
    if (mats[i].type == MPM_EOS || mats[i].type == MPM_SNHK ||
        mats[i].plasticity == MPM_PLASTIC_NAVM || mats[i].plasticity == MPM_PLASTIC_NACC)
      c->differentiable = false;
  c->prm_dirty = true;
  if ((rc = push_params(c))) return rc;
  if (c->prm.n > 0) {  // stored stresses follow the new parameters
    launch_stress(c->d, c->cur, c->stream);
    if ((rc = launch_check("stress"))) return rc;
  }
  return MPM_OK;
}

int32_t mpm_set_boundary(mpm_ctx *c, const mpm_boundary *bc) {
  int32_t rc = check(c);
  if (rc) return rc;
  if (!bc || bc->type < MPM_BC_NONE || bc->type > MPM_BC_SEPARATE || bc->thickness < 0)
    return fail(MPM_ERR_INVALID, "bad boundary");
  for (SceneParams &S : c->scenes) {
    S.bc_type = bc->type;
    S.bc_thickness = bc->thickness;
    for (int k = 0; k < 3; ++k) {
      S.bc_lo[k] = bc->lo[k];
      S.bc_hi[k] = bc->hi[k];
    }
  }
  c->prm_dirty = true;
  return push_params(c);
}

// R = Ry(yaw) Rx(pitch) Rz(roll), angles in degrees
static void ypr_rotation(const float ypr_deg[3], float R[9]) {
  const double k = 3.14159265358979323846 / 180.0;
  const double cy = std::cos(ypr_deg[0] * k), sy = std::sin(ypr_deg[0] * k);
  const double cp = std::cos(ypr_deg[1] * k), sp = std::sin(ypr_deg[1] * k);
  const double cr = std::cos(ypr_deg[2] * k), sr = std::sin(ypr_deg[2] * k);
  const double Ry[9] = {cy, 0, sy, 0, 1, 0, -sy, 0, cy};
  const double Rx[9] = {1, 0, 0, 0, cp, -sp, 0, sp, cp};
  const double Rz[9] = {cr, -sr, 0, sr, cr, 0, 0, 0, 1};
  double A[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      A[i * 3 + j] = 0;
      for (int l = 0; l < 3; ++l) A[i * 3 + j] += Ry[i * 3 + l] * Rx[l * 3 + j];
    }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double v = 0;
      for (int l = 0; l < 3; ++l) v += A[i * 3 + l] * Rz[l * 3 + j];
      R[i * 3 + j] = (float)v;
    }
}

// the captured substep graphs contain the collider pass or not


int32_t mpm_add_collider(mpm_ctx *c, const mpm_collider_desc *desc, int32_t *id) {
  int32_t rc = check(c);
  if (rc) return rc;
  if (!desc || !desc->sdf) return fail(MPM_ERR_INVALID, "null collider or signed distance grid");
  if (desc->type != MPM_BC_STICKY && desc->type != MPM_BC_SLIP && desc->type != MPM_BC_SEPARATE)
    return fail(MPM_ERR_INVALID, "collider type must be sticky, slip or separate");
  if (desc->scene < -1 || desc->scene >= (int)c->scenes.size())
    return fail(MPM_ERR_INVALID, "collider scene out of range");
  long long cells = 1;
  for (int a = 0; a < 3; ++a) {
    if (desc->dims[a] < 2) return fail(MPM_ERR_INVALID, "collider grid needs >= 2 samples per axis");
    cells *= desc->dims[a];
  }
  if (!(desc->spacing > 0.0f) || !(desc->scale > 0.0f))
    return fail(MPM_ERR_INVALID, "collider spacing and scale must be positive");
  if ((int)c->colliders.size() >= kMaxColliders)
    return fail(MPM_ERR_CAPACITY, "at most MPM_MAX_COLLIDERS colliders per context");
  ColliderDev cd{};
  ypr_rotation(desc->ypr_deg, cd.R);
  for (int a = 0; a < 3; ++a) {
    cd.b[a] = desc->translation[a];
    cd.db[a] = desc->translation_rate[a];
    cd.origin[a] = desc->origin[a];
    cd.dims[a] = desc->dims[a];
    cd.cvel[a] = desc->const_velocity[a];
  }
  cd.s = desc->scale;
  cd.ds = desc->scale_rate;
  cd.inv_h = 1.0f / desc->spacing;
  cd.type = desc->type;
  cd.scene = desc->scene;
  cd.has_vel = desc->velocity != nullptr;
  collider_world_box(cd);
  float *buf = nullptr;
  const size_t floats = (size_t)cells * (cd.has_vel ? 4 : 1);
  cudaError_t e = cudaMalloc(&buf, floats * sizeof(float));
  if (e != cudaSuccess) return fail(MPM_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  c->collider_allocs.push_back(buf);
  ZS_CUDA(cudaMemcpyAsync(buf, desc->sdf, cells * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  cd.sdf = buf;
  cd.vel = nullptr;
  if (cd.has_vel) {
    ZS_CUDA(cudaMemcpyAsync(buf + cells, desc->velocity, 3 * cells * sizeof(float),
                            cudaMemcpyHostToDevice, c->stream));
    cd.vel = buf + cells;
  }
  const int k = (int)c->colliders.size();
  c->colliders.push_back(cd);
  // only the new entry: the device copies of earlier colliders may have moved
  ZS_CUDA(cudaMemcpyAsync(c->d.colliders + k, &c->colliders[k], sizeof(ColliderDev),
                          cudaMemcpyHostToDevice, c->stream));
  ZS_CUDA(cudaStreamSynchronize(c->stream));  // the host sources may go away
  c->prm.n_colliders = k + 1;
  c->prm_dirty = true;
  if (id) *id = k;
  if (k == 0) drop_graphs(c);
  return push_params(c);
}

int32_t mpm_clear_colliders(mpm_ctx *c) {
  int32_t rc = check(c);
  if (rc) return rc;
  c->prm.n_colliders = 0;
  c->prm_dirty = true;
  if ((rc = push_params(c))) return rc;
  ZS_CUDA(cudaStreamSynchronize(c->stream));  // no kernel still reads the sample grids
  for (void *p : c->collider_allocs) cudaFree(p);
  c->collider_allocs.clear();
  if (!c->colliders.empty()) drop_graphs(c);
  c->colliders.clear();
  return MPM_OK;
}

}  // extern "C"

namespace {

// Builds the boundary grid from the context's boundary points (a sync: the
// number of boundary blocks sizes it).
int32_t build_grid_boundary(mpm_ctx *c) {
  DevPtrs &d = c->d;
  const int64_t n = c->bnd_n;
  float *pts = nullptr;
  int32_t *cnt = nullptr;
  double *acc = nullptr;
  int32_t rc = MPM_OK, nb = 0;
  auto done = [&](int32_t r) {
    cudaStreamSynchronize(c->stream);
    dfree(c, pts);
    dfree(c, cnt);
    dfree(c, acc);
    return r;
  };
  ZS_CUDA(cudaStreamSynchronize(c->stream));  // no kernel still reads the old grid
  dfree(c, d.bnd_grid);
  d.bnd_grid = nullptr;
  if (!d.bnd_map && (rc = dalloc(c, &d.bnd_map, (size_t)d.ndir))) return rc;
  ZS_CUDA(cudaMemsetAsync(d.bnd_map, 0xff, (size_t)d.ndir * sizeof(int32_t), c->stream));  // -1
  if ((rc = dalloc(c, &pts, (size_t)n * 10)) || (rc = dalloc(c, &cnt, 1))) return done(rc);
  ZS_CUDA(cudaMemcpyAsync(pts, c->bnd_pts.data(), (size_t)n * 10 * sizeof(float),
                          cudaMemcpyHostToDevice, c->stream));
  ZS_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int32_t), c->stream));
  const SceneParams &S = c->scenes[0];
  float *x = pts, *v = pts + 3 * n, *m = pts + 6 * n, *nrm = pts + 7 * n;
  launch_bnd_mark(d, S, x, n, c->stream);
  launch_bnd_index(d, cnt, c->stream);
  ZS_CUDA(cudaMemcpyAsync(&nb, cnt, sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
  ZS_CUDA(cudaStreamSynchronize(c->stream));
  if ((rc = dalloc(c, &d.bnd_grid, (size_t)std::max(nb, 1) * 128)) ||
      (rc = dalloc(c, &acc, (size_t)std::max(nb, 1) * 64 * 7)))
    return done(rc);
  ZS_CUDA(cudaMemsetAsync(acc, 0, (size_t)std::max(nb, 1) * 64 * 7 * sizeof(double), c->stream));
  launch_bnd_accumulate(d, S, x, v, m, nrm, c->bnd_n_verts, n, acc, c->stream);
  launch_bnd_finalize(d, acc, nb, c->stream);
  if ((rc = launch_check("boundary grid"))) return done(rc);
  return done(MPM_OK);
}

}  // namespace

extern "C" {

int32_t mpm_set_grid_boundary(mpm_ctx *c, int32_t type, int64_t n_verts, int64_t n_eles,
                              const float *x, const float *v, const float *m, const float *nrm) {
  ZS_RANGE("mpm_set_grid_boundary");
  int32_t rc = check(c);
  if (rc) return rc;
  if (c->scenes.size() != 1) return fail(MPM_ERR_INVALID, "a boundary grid needs a one-scene context");
  if (type != MPM_BC_STICKY && type != MPM_BC_SLIP && type != MPM_BC_SEPARATE)
    return fail(MPM_ERR_INVALID, "boundary grid type must be sticky, slip or separate");
  const int64_t n = n_verts + n_eles;
  if (n_verts < 0 || n_eles < 0 || n == 0 || !x || !m || (n_eles > 0 && !nrm))
    return fail(MPM_ERR_INVALID, "invalid boundary points");
  if ((rc = settle(c))) return rc;
  std::vector<float> pts((size_t)n * 10, 0.0f);
  for (int64_t p = 0; p < n; ++p) {
    for (int a = 0; a < 3; ++a) {
      pts[3 * p + a] = x[3 * p + a];
      pts[3 * n + 3 * p + a] = v ? v[3 * p + a] : 0.0f;
      pts[7 * n + 3 * p + a] = (p >= n_verts) ? nrm[3 * p + a] : 0.0f;
    }
    pts[6 * n + p] = m[p];
  }
  c->bnd_pts.swap(pts);
  c->bnd_n = n;
  c->bnd_n_verts = n_verts;
  if (!c->d.bnd_map) drop_graphs(c);  // the graphs gain the boundary pass
  c->d.bnd_type = type;
  if ((rc = build_grid_boundary(c))) return rc;
  drop_graphs(c);  // the new grid's address
  return MPM_OK;
}

int32_t mpm_clear_grid_boundary(mpm_ctx *c) {
  int32_t rc = check(c);
  if (rc) return rc;
  if ((rc = settle(c))) return rc;
  ZS_CUDA(cudaStreamSynchronize(c->stream));
  dfree(c, c->d.bnd_map);
  dfree(c, c->d.bnd_grid);
  if (c->d.bnd_map) drop_graphs(c);
  c->d.bnd_map = nullptr;
  c->d.bnd_grid = nullptr;
  c->bnd_pts.clear();
  c->bnd_n = c->bnd_n_verts = 0;
  return MPM_OK;
}

int32_t mpm_apply_grid_boundary(mpm_ctx *c) {
  int32_t rc = check(c);
  if (rc) return rc;
  if (!c->d.bnd_map) return fail(MPM_ERR_STATE, "no boundary grid (mpm_set_grid_boundary)");
  if (!c->partition_valid) return fail(MPM_ERR_STATE, "call mpm_partition first");
  launch_apply_grid_boundary(c->d, c->stream);
  return launch_check("apply grid boundary");
}

int32_t mpm_boundary_points_from_mesh(int64_t n_verts, const float *pos, const float *vel,
                                      int64_t n_tris, const int32_t *tris, float dx, float *x,
                                      float *v, float *m, float *nrm) {
  if (n_verts < 0 || n_tris < 0 || !pos || (n_tris > 0 && !tris) || !(dx > 0.0f) || !x || !v ||
      !m || !nrm)
    return fail(MPM_ERR_INVALID, "invalid mesh");
  for (int64_t t = 0; t < 3 * n_tris; ++t)
    if (tris[t] < 0 || tris[t] >= n_verts) return fail(MPM_ERR_INVALID, "triangle index out of range");
  auto unit = [](float *a) {
    const float l = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    if (l > 0.0f)
      for (int k = 0; k < 3; ++k) a[k] /= l;
  };
  for (int64_t i = 0; i < n_verts; ++i) {
    for (int k = 0; k < 3; ++k) {
      x[3 * i + k] = pos[3 * i + k];
      v[3 * i + k] = vel ? vel[3 * i + k] : 0.0f;
      nrm[3 * i + k] = 0.0f;
    }
    m[i] = 0.0f;
  }
  for (int64_t t = 0; t < n_tris; ++t) {
    const int32_t *tr = tris + 3 * t;
    const float *p0 = pos + 3 * tr[0], *p1 = pos + 3 * tr[1], *p2 = pos + 3 * tr[2];
    float a[3], b[3], e1[3], e2[3];
    for (int k = 0; k < 3; ++k) {
      e1[k] = p1[k] - p0[k];
      e2[k] = p2[k] - p0[k];
      a[k] = e1[k] / dx;
      b[k] = e2[k] / dx;
    }
    const float cr[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
    const float area = 0.5f * std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
    unit(e1);
    unit(e2);
    float n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                  e1[0] * e2[1] - e1[1] * e2[0]};
    unit(n);
    const int64_t r = n_verts + t;
    m[r] = area;
    for (int k = 0; k < 3; ++k) {
      x[3 * r + k] = (p0[k] + p1[k] + p2[k]) / 3.0f;
      v[3 * r + k] = vel ? (vel[3 * tr[0] + k] + vel[3 * tr[1] + k] + vel[3 * tr[2] + k]) / 3.0f : 0.0f;
      nrm[3 * r + k] = n[k];
    }
    for (int j = 0; j < 3; ++j) {
      m[tr[j]] += area / 3.0f;
      for (int k = 0; k < 3; ++k) nrm[3 * tr[j] + k] += n[k];
    }
  }
  for (int64_t i = 0; i < n_verts; ++i) unit(nrm + 3 * i);
  return MPM_OK;
}

int32_t mpm_step_colliders(mpm_ctx *c, int32_t id, float dt) {
  int32_t rc = check(c);
  if (rc) return rc;
  if (!std::isfinite(dt)) return fail(MPM_ERR_INVALID, "dt must be finite");
  if (id < -1 || id >= (int32_t)c->colliders.size())
    return fail(MPM_ERR_INVALID, "collider id out of range");
  if ((rc = push_params(c))) return rc;
  if (c->prm.n_colliders > 0) launch_step_colliders(c->d, id, dt, c->stream);
  return launch_check("step colliders");
}

int32_t mpm_set_gravity(mpm_ctx *c, float gx, float gy, float gz) {
  int32_t rc = check(c);
  if (rc) return rc;
  for (SceneParams &S : c->scenes) {
    S.gravity[0] = gx;
    S.gravity[1] = gy;
    S.gravity[2] = gz;
  }
  c->prm_dirty = true;
  return push_params(c);
}

}  // extern "C"

namespace {

int32_t upload_impl(mpm_ctx *c, const int64_t *scene_offsets, int64_t n, const float *x,
                    const float *v, const float *C, const float *F, const float *J,
                    const float *m, const float *vol, const int32_t *mat, const float *mu,
                    const float *lam, bool async = false) {
  int32_t rc = check(c);
  if (rc) return rc;
  const int ns = (int)c->scenes.size();
  if (scene_offsets) {
    if (scene_offsets[0] != 0 || scene_offsets[ns] != n)
      return fail(MPM_ERR_INVALID, "scene offsets must run from 0 to n");
    for (int s = 0; s < ns; ++s)
      if (scene_offsets[s + 1] < scene_offsets[s])
        return fail(MPM_ERR_INVALID, "scene offsets must not decrease");
  } else if (ns != 1) {
    return fail(MPM_ERR_INVALID, "a batched context takes mpm_batch_upload");
  }
  if (n < 0 || n > c->d.cap) return fail(MPM_ERR_CAPACITY, "particle count exceeds capacity");
  if (n > 0 && (!x || !m || !vol)) return fail(MPM_ERR_INVALID, "x, m and vol are required");
  if ((mu == nullptr) != (lam == nullptr)) return fail(MPM_ERR_INVALID, "mu and lam go together");
  if (c->n_materials <= 0) return fail(MPM_ERR_STATE, "set materials before uploading");
  const int alt = 1 - c->cur;
  float *st = c->d.pbuf[alt];  // staging: the other buffer is free between substeps
  int32_t *ist = c->d.ibuf[alt];
  const size_t N = (size_t)n;
  IngestSrc src{};
  const float *const hs[9] = {x, v, C, F, J, m, vol, mu, lam};
  const size_t off[9] = {0, 3 * N, 6 * N, 15 * N, 24 * N, 25 * N, 26 * N, 27 * N, 28 * N};
  const int width[9] = {3, 3, 9, 9, 1, 1, 1, 1, 1};
  const float **dsts[9] = {&src.x, &src.v, &src.C, &src.F, &src.J, &src.m, &src.vol, &src.mu, &src.lam};
  for (int a = 0; a < 9; ++a) *dsts[a] = hs[a] ? st + off[a] : nullptr;
  src.mat = mat ? ist : nullptr;
  // chunks of the particle range: the copies of chunk k + 1 (on the copy
  // stream) overlap the material check and ingest of chunk k (on the
  // context's stream); one synchronisation at the end.  An asynchronous
  // upload copies in one piece: its conversion overlaps the next upload of
  // another context instead, and fewer, larger copies keep the link busier
  const int K = n >= (1 << 20) && !async ? kUploadChunks : 1;
  if (!c->copy_stream) {
    ZS_CUDA(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
    for (int k = 0; k <= kUploadChunks; ++k)
      ZS_CUDA(cudaEventCreateWithFlags(&c->copy_ev[k], cudaEventDisableTiming));
  }
  c->prm.n = n;
  c->prm.has_lame = mu ? 1 : 0;
  for (int s = 0; s < ns; ++s) c->scenes[s].p_off = scene_offsets ? scene_offsets[s] : 0;
  c->prm_dirty = true;
  if ((rc = push_params(c))) return rc;
  if (n > 0) {
    ZS_CUDA(cudaEventRecord(c->copy_ev[kUploadChunks], c->stream));  // staging free from here
    ZS_CUDA(cudaStreamWaitEvent(c->copy_stream, c->copy_ev[kUploadChunks], 0));
    ZS_CUDA(cudaMemsetAsync(&c->d.cnt->bad_material, 0, sizeof(int), c->stream));
  }
  for (int k = 0; k < K && n > 0; ++k) {
    const long long b0 = n * k / K, b1 = n * (k + 1) / K;
    for (int a = 0; a < 9; ++a)
      if (hs[a])
        ZS_CUDA(cudaMemcpyAsync(st + off[a] + b0 * width[a], hs[a] + b0 * width[a],
                                (b1 - b0) * width[a] * sizeof(float), cudaMemcpyHostToDevice,
                                c->copy_stream));
    if (mat)
      ZS_CUDA(cudaMemcpyAsync(ist + b0, mat + b0, (b1 - b0) * sizeof(int32_t), cudaMemcpyHostToDevice,
                              c->copy_stream));
    ZS_CUDA(cudaEventRecord(c->copy_ev[k], c->copy_stream));
    ZS_CUDA(cudaStreamWaitEvent(c->stream, c->copy_ev[k], 0));
    if (mat) launch_check_materials(c->d, ist + b0, b1 - b0, c->n_materials, c->stream);
    launch_ingest(c->d, c->cur, src, b0, b1, c->stream);
    launch_stress(c->d, c->cur, c->stream, b0, b1);  // S = vol * tau read by P2G
    if ((rc = launch_check("ingest"))) return rc;
  }
  if (n > 0) {  // ToZSParticles: beta = 0, vms = 0 (Generation.cpp:944-966)
    ZS_CUDA(cudaMemsetAsync(c->d.beta, 0, (size_t)n * sizeof(float), c->stream));
    ZS_CUDA(cudaMemsetAsync(c->d.vms, 0, (size_t)n * sizeof(float), c->stream));
  }
  // a fresh store: clear the status word, the substep gate and the whole
  // directory; substeps queued before the upload no longer matter
  ZS_CUDA(cudaMemsetAsync(&c->d.cnt->status, 0, sizeof(int), c->stream));
  ZS_CUDA(cudaMemsetAsync(&c->d.cnt->halt, 0, 2 * sizeof(int), c->stream));
  c->pending.clear();
  c->pending_total = 0;
  c->started_base = 0;
  c->needs_full_clear = true;
  c->partition_valid = false;
  c->binned = false;
  c->substeps = 0;
  if (async) {  // the verdict of the material check goes to the status word
    if (mat && n > 0) launch_flag_materials(c->d, c->stream);
    return launch_check("upload");
  }
  if (mat && n > 0)
    ZS_CUDA(cudaMemcpyAsync(&c->h_cnt->bad_material, &c->d.cnt->bad_material, sizeof(int),
                            cudaMemcpyDeviceToHost, c->stream));
  ZS_CUDA(cudaStreamSynchronize(c->stream));
  if (mat && n > 0 && c->h_cnt->bad_material) {  // the store is not usable: no particles
    c->prm.n = 0;
    c->prm_dirty = true;
    push_params(c);
    return fail(MPM_ERR_INVALID, "material id out of range (the context holds no particles)");
  }
  return MPM_OK;
}

}  // namespace

extern "C" {

int32_t mpm_particles_upload(mpm_ctx *c, int64_t n, const float *x, const float *v,
                             const float *C, const float *F, const float *J, const float *m,
                             const float *vol, const int32_t *mat, const float *mu,
                             const float *lam) {
  ZS_RANGE("mpm_particles_upload");
  return upload_impl(c, nullptr, n, x, v, C, F, J, m, vol, mat, mu, lam);
}

int32_t mpm_particles_upload_async(mpm_ctx *c, int64_t n, const float *x, const float *v,
                                   const float *C, const float *F, const float *J,
                                   const float *m, const float *vol, const int32_t *mat,
                                   const float *mu, const float *lam) {
  ZS_RANGE("mpm_particles_upload_async");
  return upload_impl(c, nullptr, n, x, v, C, F, J, m, vol, mat, mu, lam, true);
}

int32_t mpm_batch_upload(mpm_ctx *c, const int64_t *scene_offsets, int64_t n, const float *x,
                         const float *v, const float *C, const float *F, const float *J,
                         const float *m, const float *vol, const int32_t *mat, const float *mu,
                         const float *lam) {
  ZS_RANGE("mpm_batch_upload");
  if (!scene_offsets) return fail(MPM_ERR_INVALID, "scene offsets are required");
  return upload_impl(c, scene_offsets, n, x, v, C, F, J, m, vol, mat, mu, lam);
}

int32_t mpm_particles_set_lame(mpm_ctx *c, const float *mu, const float *lam) {
  int32_t rc = check(c);
  if (rc) return rc;
  if ((rc = settle(c))) return rc;
  if (!mu || !lam) return fail(MPM_ERR_INVALID, "mu and lam are required");
  const long long n = c->prm.n;
  if (n == 0) return MPM_OK;
  float *st = c->d.pbuf[1 - c->cur];  // staging: the other buffer is free between substeps
  ZS_CUDA(cudaMemcpyAsync(st, mu, n * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  ZS_CUDA(cudaMemcpyAsync(st + n, lam, n * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  launch_set_lame(c->d, c->cur, st, st + n, n, c->stream);
  if ((rc = launch_check("set lame"))) return rc;
  c->prm.has_lame = 1;
  c->prm_dirty = true;
  if ((rc = push_params(c))) return rc;
  launch_stress(c->d, c->cur, c->stream);  // stored stresses follow the new parameters
  if ((rc = launch_check("stress"))) return rc;
  ZS_CUDA(cudaStreamSynchronize(c->stream));
  return MPM_OK;
}

int32_t mpm_particles_download(mpm_ctx *c, float *x, float *v, float *C, float *F, float *J) {
  ZS_RANGE("mpm_particles_download");
  int32_t rc = check(c);
  if (rc) return rc;
  if ((rc = settle(c))) return rc;
  const long long n = c->prm.n;
  float *st = c->d.pbuf[1 - c->cur];
  // only the requested channels are gathered into upload order
  launch_egest(c->d, c->cur,
               EgestDst{x ? st : nullptr, v ? st + 3 * n : nullptr, C ? st + 6 * n : nullptr,
                        F ? st + 15 * n : nullptr, J ? st + 24 * n : nullptr},
               n, c->stream);
  if ((rc = launch_check("egest"))) return rc;
  const size_t N = (size_t)n;
  auto get = [&](float *h, size_t off, size_t count) -> int32_t {
    if (!h || count == 0) return MPM_OK;
    ZS_CUDA(cudaMemcpyAsync(h, st + off, count * sizeof(float), cudaMemcpyDeviceToHost,
                            c->stream));
    return MPM_OK;
  };
  if ((rc = get(x, 0, 3 * N)) || (rc = get(v, 3 * N, 3 * N)) || (rc = get(C, 6 * N, 9 * N)) ||
      (rc = get(F, 15 * N, 9 * N)) || (rc = get(J, 24 * N, N)))
    return rc;
  ZS_CUDA(cudaStreamSynchronize(c->stream));
  return MPM_OK;
}

int32_t mpm_particles_get_attr(mpm_ctx *c, const char *name, float *values) {
  int32_t rc = check(c);
  if (rc) return rc;
  if ((rc = settle(c))) return rc;
  if (!name || !values) return fail(MPM_ERR_INVALID, "null argument");
  const std::string a(name);
  const long long n = c->prm.n;
  if (a == "cloth_beta") {  // the cloth's vertices (n_verts values)
    if (c->d.cloth.n_verts == 0) return fail(MPM_ERR_STATE, "no cloth in this context");
    ZS_CUDA(cudaMemcpyAsync(values, c->d.cloth.vbeta, c->d.cloth.n_verts * sizeof(float),
                            cudaMemcpyDeviceToHost, c->stream));
    ZS_CUDA(cudaStreamSynchronize(c->stream));
    return MPM_OK;
  }
  if (a == "beta" || a == "vms") {  // planes by upload index
    if (n > 0)
      ZS_CUDA(cudaMemcpyAsync(values, a == "beta" ? c->d.beta : c->d.vms, n * sizeof(float),
                              cudaMemcpyDeviceToHost, c->stream));
    ZS_CUDA(cudaStreamSynchronize(c->stream));
    return MPM_OK;
  }
  int ch = -1;
  if (a == "m") ch = CH_M;
  if (a == "vol") ch = CH_VOL;
  if (a == "J") ch = CH_J;
  if (a == "mu" || a == "lam") {
    if (!c->prm.has_lame) return fail(MPM_ERR_STATE, "no per-particle Lame parameters set");
    ch = a == "mu" ? CH_MU : CH_LAM;
  }
  if (ch < 0) return fail(MPM_ERR_INVALID, "unknown particle attribute '" + a + "'");
  float *st = c->d.pbuf[1 - c->cur];
  launch_egest_channel(c->d, c->cur, ch, st, n, c->stream);
  if ((rc = launch_check("attribute"))) return rc;
  if (n > 0)
    ZS_CUDA(cudaMemcpyAsync(values, st, n * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  ZS_CUDA(cudaStreamSynchronize(c->stream));
  return MPM_OK;
}

int32_t mpm_particles_set_attr(mpm_ctx *c, const char *name, const float *values) {
  int32_t rc = check(c);
  if (rc) return rc;
  if ((rc = settle(c))) return rc;
  if (!name || !values) return fail(MPM_ERR_INVALID, "null argument");
  if (std::string(name) == "cloth_beta") {  // the cloth's vertices (n_verts values)
    if (c->d.cloth.n_verts == 0) return fail(MPM_ERR_STATE, "no cloth in this context");
    ZS_CUDA(cudaMemcpyAsync(c->d.cloth.vbeta, values, c->d.cloth.n_verts * sizeof(float),
                            cudaMemcpyHostToDevice, c->stream));
    ZS_CUDA(cudaStreamSynchronize(c->stream));
    return MPM_OK;
  }
  if (std::string(name) != "beta")
    return fail(MPM_ERR_INVALID, std::string("attribute '") + name + "' cannot be set");
  const long long n = c->prm.n;
  if (n > 0)
    ZS_CUDA(cudaMemcpyAsync(c->d.beta, values, n * sizeof(float), cudaMemcpyHostToDevice,
                            c->stream));
  ZS_CUDA(cudaStreamSynchronize(c->stream));
  return MPM_OK;
}

}  // extern "C"

namespace {

// The per-vertex contribution slots of a cloth's impulses: element corners
// (3 e + corner, the first `per` corners) in element order, then spring ends
// (3 n_eles + 2 s + end) in spring order.
int32_t upload_cloth_slots(mpm_ctx *c, ClothDev &cl, const std::vector<int32_t> &inds, int per,
                           const std::vector<int32_t> &springs) {
  const long long nv = cl.n_verts, ne = cl.n_eles, ns = (long long)springs.size() / 2;
  std::vector<int32_t> ptr(nv + 1, 0), list;
  for (long long e = 0; e < ne; ++e)
    for (int k = 0; k < per; ++k) ++ptr[inds[3 * e + k] + 1];
  for (long long s = 0; s < 2 * ns; ++s) ++ptr[springs[s] + 1];
  for (long long v = 0; v < nv; ++v) ptr[v + 1] += ptr[v];
  list.resize(ptr[nv]);
  std::vector<int32_t> fill(ptr.begin(), ptr.end() - 1);
  for (long long e = 0; e < ne; ++e)
    for (int k = 0; k < per; ++k) list[fill[inds[3 * e + k]]++] = (int32_t)(3 * e + k);
  for (long long s = 0; s < 2 * ns; ++s) list[fill[springs[s]]++] = (int32_t)(3 * ne + s);
  dfree(c, cl.vptr);
  dfree(c, cl.vlist);
  dfree(c, cl.cimp);
  cl.vptr = cl.vlist = nullptr;
  cl.cimp = nullptr;
  int32_t rc;
  if ((rc = dalloc(c, &cl.vptr, (size_t)nv + 1)) || (rc = dalloc(c, &cl.vlist, list.size())) ||
      (rc = dalloc(c, &cl.cimp, (size_t)(3 * ne + 2 * ns))))
    return rc;
  ZS_CUDA(cudaMemcpyAsync(cl.vptr, ptr.data(), ptr.size() * sizeof(int32_t), cudaMemcpyHostToDevice,
                          c->stream));
  if (!list.empty())
    ZS_CUDA(cudaMemcpyAsync(cl.vlist, list.data(), list.size() * sizeof(int32_t),
                            cudaMemcpyHostToDevice, c->stream));
  ZS_CUDA(cudaStreamSynchronize(c->stream));  // the host vectors go away
  return MPM_OK;
}

// The arrays of the cloth's deterministic P2G: records, slots, and the
// partition of its points into blocks of their own, with room for eight
// times the blocks the mesh occupies at creation (more is a capacity
// error of the context).
int32_t alloc_cloth_p2g(mpm_ctx *c, ClothDev &cl, const std::vector<int32_t> &inds, int per,
                        const std::vector<float> &vx, const std::vector<float> &ex) {
  const DevPtrs &d = c->d;
  const SceneParams &S = c->scenes[0];
  const long long np = cl.n_verts + cl.n_eles;
  std::unordered_map<long long, int> blocks;
  auto add = [&](const float *x) {
    long long k = 0;
    for (int a = 0; a < 3; ++a) {
      const int b = (int)std::floor(x[a] * S.inv_dx - 0.5f) >> 2;
      k = k * (1ll << 21) + (b + (1 << 20));
    }
    blocks.emplace(k, 0);
  };
  for (long long i = 0; i < cl.n_verts; ++i) add(&vx[3 * i]);
  for (long long e = 0; e < cl.n_eles; ++e) add(&ex[3 * e]);
  // room for the cloth to spread over 8x its blocks; a grown directory
  // raises the directory's share of the bound (regrow)
  c->cloth_capb_want = std::max<long long>(8 * (long long)blocks.size(), 1024);
  const long long capb = std::min<long long>({d.ndir, np, c->cloth_capb_want});
  cl.cap_cblocks = (int)capb;
  int32_t rc;
  if ((rc = dalloc(c, &cl.crec, (size_t)np * kClothRec)) || (rc = dalloc(c, &cl.ckey, (size_t)np)) ||
      (rc = dalloc(c, &cl.cperm, (size_t)np)) || (rc = dalloc(c, &cl.cperm_tmp, (size_t)np)) ||
      (rc = dalloc(c, &cl.cdir_count, (size_t)d.ndir)) ||
      (rc = dalloc(c, &cl.cdir_fill, (size_t)d.ndir)) || (rc = dalloc(c, &cl.cdir_gb, (size_t)d.ndir)) ||
      (rc = dalloc(c, &cl.cdir_bk, (size_t)d.ndir)) || (rc = dalloc(c, &cl.cdir_flag, (size_t)d.ndir)) ||
      (rc = dalloc(c, &cl.cgb_dir, (size_t)capb)) || (rc = dalloc(c, &cl.cbk_dir, (size_t)capb)) ||
      (rc = dalloc(c, &cl.cbk_start, (size_t)capb)) || (rc = dalloc(c, &cl.cbk_count, (size_t)capb)) ||
      (rc = dalloc(c, &cl.ctile_sums, (size_t)3 * d.ntiles)) ||
      (rc = dalloc(c, &cl.ctile, (size_t)capb * kTileNodes)) ||
      (rc = dalloc(c, &cl.ctile2, (size_t)capb * kTileNodes)) || (rc = dalloc(c, &cl.ccnt, 1)) ||
      (rc = dalloc(c, &cl.cprm, 1)))
    return rc;
  ZS_CUDA(cudaMemsetAsync(cl.cdir_count, 0, (size_t)d.ndir * sizeof(int32_t), c->stream));
  ZS_CUDA(cudaMemsetAsync(cl.cdir_flag, 0, (size_t)d.ndir, c->stream));
  ZS_CUDA(cudaMemsetAsync(cl.ccnt, 0, sizeof(Counters), c->stream));
  SimParams cp{};
  cp.n = np;  // and no collider stepping: auto_step = 0
  ZS_CUDA(cudaMemcpyAsync(cl.cprm, &cp, sizeof(SimParams), cudaMemcpyHostToDevice, c->stream));
  return upload_cloth_slots(c, cl, inds, per, {});
}

}  // namespace

extern "C" {

int32_t mpm_cloth_create(mpm_ctx *c, const mpm_cloth_desc *desc) {
  ZS_RANGE("mpm_cloth_create");
  int32_t rc = check(c);
  if (rc) return rc;
  if (!desc || desc->n_verts <= 0 || desc->n_tris <= 0 || !desc->x || !desc->tris)
    return fail(MPM_ERR_INVALID, "a cloth needs vertices and triangles");
  if (c->scenes.size() != 1) return fail(MPM_ERR_INVALID, "a cloth needs a single-scene context");
  if (c->d.cloth.n_verts > 0) return fail(MPM_ERR_STATE, "one cloth per context");
  if (c->d.differentiable) return fail(MPM_ERR_INVALID, "the differentiable form takes no cloth");
  if (desc->model != MPM_FCR && desc->model != MPM_NHK && desc->model != MPM_STVK)
    return fail(MPM_ERR_INVALID, "cloth model must be fixed-corotated, Neo-Hookean or StVK-Hencky");
  if (desc->kind != MPM_MESH_SURFACE && desc->kind != MPM_MESH_CURVE)
    return fail(MPM_ERR_INVALID, "mesh kind must be MPM_MESH_SURFACE or MPM_MESH_CURVE");
  const bool curve = desc->kind == MPM_MESH_CURVE;
  const int per = curve ? 2 : 3;
  if (!(desc->stiffness_normal > 0.0f) && desc->stiffness_shear != 0.0f)
    return fail(MPM_ERR_INVALID, "stiffness_normal must be positive with a shear stiffness");
  const int64_t nv = desc->n_verts, ne = desc->n_tris;
  if (nv >= (int64_t(1) << 31) || ne >= (int64_t(1) << 31))
    return fail(MPM_ERR_CAPACITY, "cloth larger than 2^31 vertices or triangles");
  for (int64_t i = 0; i < per * ne; ++i)
    if (desc->tris[i] < 0 || desc->tris[i] >= nv) return fail(MPM_ERR_INVALID, "mesh index out of range");
  // ToZSCloth (Generation.cpp:497-688): areas and frames in double, stored as float
  const float E = desc->E, nu = desc->nu;
  const float mu = E / (2.0f * (1.0f + nu)), lam = E * nu / ((1.0f + nu) * (1.0f - 2.0f * nu));
  const float dx = c->scenes[0].dx, rho = desc->density;
  const double feps = 1.1920928955078125e-07;
  std::vector<float> vx(3 * nv), vv(3 * nv, 0.0f), vC(9 * nv, 0.0f), vm(nv), dof(nv, 0.0f);
  std::vector<float> ex(3 * ne), ev(3 * ne, 0.0f), eC(9 * ne, 0.0f), eF(9 * ne), ed(9 * ne),
      eDi(9 * ne), em(ne), evol(ne), emu(ne), elam(ne);
  const float *X = desc->x, *V = desc->v;
  std::vector<int32_t> inds(3 * ne);
  for (int64_t e = 0; e < ne && curve; ++e) {
    // ToZSParticles' curve set-up (Generation.cpp:837-858, 1096-1112)
    const int32_t *t = desc->tris + 2 * e;
    double len2 = 0;
    float d1[3];
    for (int a = 0; a < 3; ++a) {
      const double dd = double(X[3 * t[1] + a]) - double(X[3 * t[0] + a]);
      len2 += dd * dd;
      d1[a] = X[3 * t[1] + a] - X[3 * t[0] + a];
    }
    const float vol = float(std::max(std::sqrt(len2) * double(dx) * double(dx), 10.0 * feps));
    evol[e] = vol;
    em[e] = vol * rho;
    for (int a = 0; a < 3; ++a) {
      ex[3 * e + a] = (X[3 * t[0] + a] + X[3 * t[1] + a]) / 2.0f;
      if (V) ev[3 * e + a] = (V[3 * t[0] + a] + V[3 * t[1] + a]) / 2.0f;
    }
    // n1: a unit vector orthogonal to the segment (Hughes & Moller 1999);
    // n2 = normalize(d1 x n1)
    const double ln[3] = {d1[0], d1[1], d1[2]};
    double o[3];
    if (std::fabs(ln[0]) > std::fabs(ln[2])) {
      o[0] = -ln[1];
      o[1] = ln[0];
      o[2] = 0;
    } else {
      o[0] = 0;
      o[1] = -ln[2];
      o[2] = ln[1];
    }
    const double on = std::sqrt(o[0] * o[0] + o[1] * o[1] + o[2] * o[2]);
    const double n1[3] = {o[0] / on, o[1] / on, o[2] / on};
    const double n2[3] = {ln[1] * n1[2] - ln[2] * n1[1], ln[2] * n1[0] - ln[0] * n1[2],
                          ln[0] * n1[1] - ln[1] * n1[0]};
    const double n2n = std::sqrt(n2[0] * n2[0] + n2[1] * n2[1] + n2[2] * n2[2]);
    float dcol[9];
    for (int a = 0; a < 3; ++a) {
      dcol[a * 3 + 0] = d1[a];
      dcol[a * 3 + 1] = float(n1[a]);
      dcol[a * 3 + 2] = float(n2[a] / n2n);
    }
    const double tl = std::sqrt(double(dcol[0]) * dcol[0] + double(dcol[3]) * dcol[3] + double(dcol[6]) * dcol[6]);
    const double Di[9] = {1 / tl, 0, 0, 0, 1, 0, 0, 0, 1};
    emu[e] = tl <= feps ? 0.0f : mu;
    elam[e] = tl <= feps ? 0.0f : lam;
    for (int i = 0; i < 9; ++i) {
      ed[9 * e + i] = dcol[i];
      eDi[9 * e + i] = float(Di[i]);
    }
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double sum = 0;
        for (int l = 0; l < 3; ++l) sum += double(dcol[i * 3 + l]) * Di[l * 3 + j];
        eF[9 * e + i * 3 + j] = float(sum);
      }
    inds[3 * e] = t[0];
    inds[3 * e + 1] = inds[3 * e + 2] = t[1];
    for (int i = 0; i < 2; ++i) dof[t[i]] += vol / 2.0f;
  }
  for (int64_t e = 0; e < ne && !curve; ++e) {
    const int32_t *t = desc->tris + 3 * e;
    for (int i = 0; i < 3; ++i) inds[3 * e + i] = t[i];
    float d1[3], d2[3];
    for (int a = 0; a < 3; ++a) {
      d1[a] = X[3 * t[1] + a] - X[3 * t[0] + a];
      d2[a] = X[3 * t[2] + a] - X[3 * t[0] + a];
    }
    double e1[3], e2[3];
    for (int a = 0; a < 3; ++a) {
      e1[a] = double(X[3 * t[1] + a]) - double(X[3 * t[0] + a]);
      e2[a] = double(X[3 * t[2] + a]) - double(X[3 * t[0] + a]);
    }
    const double cr[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                          e1[0] * e2[1] - e1[1] * e2[0]};
    const double area = 0.5 * std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
    const float vol = float(std::max(area * double(dx), 10.0 * feps));
    evol[e] = vol;
    em[e] = vol * rho;
    for (int a = 0; a < 3; ++a) {
      ex[3 * e + a] = (X[3 * t[0] + a] + X[3 * t[1] + a] + X[3 * t[2] + a]) / 3.0f;
      if (V) ev[3 * e + a] = (V[3 * t[0] + a] + V[3 * t[1] + a] + V[3 * t[2] + a]) / 3.0f;
    }
    // normal from the normalised edges; rest shape in the triangle's frame:
    // D* = [|d1|, d1.d2/|d1|, 0; 0, |d1 x d2|/|d1|, 0; 0, 0, 1]
    double n1 = 0, n2 = 0, dot = 0;
    for (int a = 0; a < 3; ++a) {
      n1 += double(d1[a]) * d1[a];
      n2 += double(d2[a]) * d2[a];
      dot += double(d1[a]) * d2[a];
    }
    n1 = std::sqrt(n1);
    n2 = std::sqrt(n2);
    const double u1[3] = {d1[0] / n1, d1[1] / n1, d1[2] / n1}, u2[3] = {d2[0] / n2, d2[1] / n2, d2[2] / n2};
    const double nn[3] = {u1[1] * u2[2] - u1[2] * u2[1], u1[2] * u2[0] - u1[0] * u2[2],
                          u1[0] * u2[1] - u1[1] * u2[0]};
    const double nl = std::sqrt(nn[0] * nn[0] + nn[1] * nn[1] + nn[2] * nn[2]);
    const double cx = double(d1[1]) * d2[2] - double(d1[2]) * d2[1], cy = double(d1[2]) * d2[0] - double(d1[0]) * d2[2],
                 cz = double(d1[0]) * d2[1] - double(d1[1]) * d2[0];
    const double a00 = n1, a01 = dot / n1, a11 = std::sqrt(cx * cx + cy * cy + cz * cz) / n1;
    const double Di[9] = {1 / a00, -a01 / (a00 * a11), 0, 0, 1 / a11, 0, 0, 0, 1};
    const bool degenerate = std::fabs(a11) <= 10 * feps || std::fabs(a00) <= 10 * feps;
    emu[e] = degenerate ? 0.0f : mu;
    elam[e] = degenerate ? 0.0f : lam;
    float dcol[9];
    for (int a = 0; a < 3; ++a) {
      dcol[a * 3 + 0] = d1[a];
      dcol[a * 3 + 1] = d2[a];
      dcol[a * 3 + 2] = float(nn[a] / nl);
    }
    for (int i = 0; i < 9; ++i) {
      ed[9 * e + i] = dcol[i];
      eDi[9 * e + i] = float(Di[i]);
    }
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double sum = 0;
        for (int l = 0; l < 3; ++l) sum += double(dcol[i * 3 + l]) * Di[l * 3 + j];
        eF[9 * e + i * 3 + j] = float(sum);
      }
    for (int i = 0; i < 3; ++i) dof[t[i]] += vol / 3.0f;
  }
  for (int64_t p = 0; p < nv; ++p) {
    vm[p] = dof[p] * rho;
    for (int a = 0; a < 3; ++a) {
      vx[3 * p + a] = X[3 * p + a];
      if (V) vv[3 * p + a] = V[3 * p + a];
    }
  }
  ClothDev &cl = c->d.cloth;
  ClothDev nc{};
  auto up = [&](float **dst, const std::vector<float> &h) -> int32_t {
    int32_t r = dalloc(c, dst, h.size());
    if (r) return r;
    ZS_CUDA(cudaMemcpyAsync(*dst, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    return MPM_OK;
  };
  if ((rc = up(&nc.vx, vx)) || (rc = up(&nc.vv, vv)) || (rc = up(&nc.vC, vC)) || (rc = up(&nc.vm, vm)) ||
      (rc = up(&nc.ex, ex)) ||
      (rc = up(&nc.ev, ev)) || (rc = up(&nc.eC, eC)) || (rc = up(&nc.eF, eF)) || (rc = up(&nc.ed, ed)) ||
      (rc = up(&nc.eDmInv, eDi)) || (rc = up(&nc.em, em)) || (rc = up(&nc.evol, evol)) ||
      (rc = up(&nc.emu, emu)) || (rc = up(&nc.elam, elam)) ||
      (rc = up(&nc.vbeta, std::vector<float>(nv, 0.0f))))  // ToZSCloth: beta = 0
    return rc;
  if ((rc = dalloc(c, &nc.inds, (size_t)3 * ne)) || (rc = dalloc(c, &nc.vowner, (size_t)nv)))
    return rc;
  ZS_CUDA(cudaMemcpyAsync(nc.inds, inds.data(), 3 * ne * sizeof(int32_t), cudaMemcpyHostToDevice, c->stream));
  ZS_CUDA(cudaStreamSynchronize(c->stream));
  nc.n_verts = nv;
  nc.n_eles = ne;
  if ((rc = alloc_cloth_p2g(c, nc, inds, curve ? 2 : 3, vx, ex))) return rc;
  nc.kind = desc->kind;
  nc.model = curve ? MPM_STVK : desc->model;  // curves: StVK-Hencky (Generation.cpp:761-769)
  nc.gamma = desc->stiffness_shear;
  nc.k = desc->stiffness_normal;
  nc.fc = std::tan(desc->friction_angle / 3.14159265358979323846f);
  nc.dc = desc->damping_coeff;
  cl = nc;
  drop_graphs(c);  // the substep gains the cloth's kernels
  c->partition_valid = false;
  return MPM_OK;
}

int32_t mpm_cloth_add_bending(mpm_ctx *c, int32_t type, float stiffness, float thickness,
                              int64_t *n_out) {
  int32_t rc = check(c);
  if (rc) return rc;
  ClothDev &cl = c->d.cloth;
  if (cl.n_verts == 0) return fail(MPM_ERR_STATE, "no cloth in this context");
  if (cl.kind != MPM_MESH_SURFACE) return fail(MPM_ERR_INVALID, "bending springs need a triangle mesh");
  if (type == MPM_BENDING_ELEMENT)
    return fail(MPM_ERR_INVALID,
                "element bending springs are undefined in the reference (the pairs are tagged "
                "as vertex springs without vertex indices)");
  if (type != MPM_BENDING_VERTEX && type != MPM_BENDING_ANGLE)
    return fail(MPM_ERR_INVALID, "unknown bending spring type");
  if (cl.n_springs > 0) return fail(MPM_ERR_STATE, "the cloth already has bending springs");
  if (!std::isfinite(stiffness) || !std::isfinite(thickness))
    return fail(MPM_ERR_INVALID, "non-finite bending stiffness or thickness");
  // ConstructBendingSprings (Generation.cu:563-1001) on the host from the
  // cloth's current state: triangles register their directed edges (vi, vj)
  // with vi < vj in cyclic order (tri[2] -> tri[0] -> tri[1] -> tri[2]); an
  // edge vi -> vj with vi > vj whose reverse was registered joins the two
  // triangles, and the vertices opposite the edge form one pair
  const long long nv = cl.n_verts, ne = cl.n_eles;
  std::vector<int32_t> inds(3 * ne);
  std::vector<float> vx(3 * nv), emu(ne), elam(ne);
  ZS_CUDA(cudaMemcpyAsync(inds.data(), cl.inds, inds.size() * 4, cudaMemcpyDeviceToHost, c->stream));
  ZS_CUDA(cudaMemcpyAsync(vx.data(), cl.vx, vx.size() * 4, cudaMemcpyDeviceToHost, c->stream));
  ZS_CUDA(cudaMemcpyAsync(emu.data(), cl.emu, ne * 4, cudaMemcpyDeviceToHost, c->stream));
  ZS_CUDA(cudaMemcpyAsync(elam.data(), cl.elam, ne * 4, cudaMemcpyDeviceToHost, c->stream));
  ZS_CUDA(cudaStreamSynchronize(c->stream));
  std::unordered_map<uint64_t, int32_t> edge_ele;
  edge_ele.reserve(3 * ne);
  auto key = [](int32_t a, int32_t b) { return (uint64_t(uint32_t(a)) << 32) | uint32_t(b); };
  for (long long e = 0; e < ne; ++e) {
    const int32_t *t = &inds[3 * e];
    int32_t vi = t[2];
    for (int v = 0; v < 3; ++v) {
      const int32_t vj = t[v];
      if (vi < vj) edge_ele[key(vi, vj)] = (int32_t)e;
      vi = vj;
    }
  }
  // E, nu from mu, lam: E = mu (3 lam + 2 mu) / (lam + mu), nu = lam / (2 (lam + mu))
  auto E_of = [&](long long e) {
    const double mu = emu[e], lam = elam[e];
    return mu * (3 * lam + 2 * mu) / (lam + mu);
  };
  auto nu_of = [&](long long e) {
    const double mu = emu[e], lam = elam[e];
    return lam / (2 * (lam + mu));
  };
  std::vector<int32_t> sv;
  std::vector<float> sk, srl;
  long long hinges = 0;
  for (long long e = 0; e < ne; ++e) {
    const int32_t *t = &inds[3 * e];
    int32_t vi = t[1], vj = t[2];
    for (int v = 0; v < 3; ++v) {
      const int32_t vk = t[v];
      if (vi > vj) {
        auto it = edge_ele.find(key(vj, vi));
        if (it != edge_ele.end()) {
          const int32_t nb = it->second;
          int32_t other = -1;
          for (int q = 0; q < 3; ++q)
            if (inds[3 * nb + q] != vi && inds[3 * nb + q] != vj) {
              other = inds[3 * nb + q];
              break;
            }
          ++hinges;
          if (type == MPM_BENDING_VERTEX && other >= 0) {
            const double Em = std::min(E_of(e), E_of(nb)), num = std::min(nu_of(e), nu_of(nb));
            sv.push_back(other);
            sv.push_back(vk);
            sk.push_back(float(Em / (24.0 * (1.0 - num * num)) * stiffness));
            double l2 = 0;
            for (int a = 0; a < 3; ++a) {
              const double dd = double(vx[3 * vk + a]) - double(vx[3 * other + a]);
              l2 += dd * dd;
            }
            srl.push_back(float(std::sqrt(l2)));
          }
        }
      }
      vi = vj;
      vj = vk;
    }
  }
  // "angle": the reference's hinge force is identically zero (its angle is
  // declared again inside a block, Transfer.cu:466-480, and the outer one,
  // 0, enters the force), so the hinges are counted and nothing is added
  if (n_out) *n_out = hinges;
  const long long ns = (long long)sk.size();
  if (ns == 0) return MPM_OK;
  if ((rc = dalloc(c, &cl.sv, (size_t)2 * ns)) || (rc = dalloc(c, &cl.sk, (size_t)ns)) ||
      (rc = dalloc(c, &cl.srl, (size_t)ns)))
    return rc;
  ZS_CUDA(cudaMemcpy(cl.sv, sv.data(), sv.size() * 4, cudaMemcpyHostToDevice));
  ZS_CUDA(cudaMemcpy(cl.sk, sk.data(), sk.size() * 4, cudaMemcpyHostToDevice));
  ZS_CUDA(cudaMemcpy(cl.srl, srl.data(), srl.size() * 4, cudaMemcpyHostToDevice));
  cl.thickness = thickness;
  cl.n_springs = ns;
  // the springs' impulse slots join their vertices' lists
  if ((rc = upload_cloth_slots(c, cl, inds, 3, sv))) return rc;
  drop_graphs(c);  // the substep gains the springs' kernel
  return MPM_OK;
}

int32_t mpm_cloth_download(mpm_ctx *c, float *vx, float *vv, float *vC, float *ex, float *ev,
                           float *eC, float *eF, float *ed) {
  ZS_RANGE("mpm_cloth_download");
  int32_t rc = check(c);
  if (rc) return rc;
  if ((rc = settle(c))) return rc;
  const ClothDev &cl = c->d.cloth;
  if (cl.n_verts == 0) return fail(MPM_ERR_STATE, "no cloth in this context");
  auto get = [&](float *h, const float *dsrc, long long count) -> int32_t {
    if (!h) return MPM_OK;
    ZS_CUDA(cudaMemcpyAsync(h, dsrc, count * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    return MPM_OK;
  };
  const long long nv = cl.n_verts, ne = cl.n_eles;
  if ((rc = get(vx, cl.vx, 3 * nv)) || (rc = get(vv, cl.vv, 3 * nv)) || (rc = get(vC, cl.vC, 9 * nv)) ||
      (rc = get(ex, cl.ex, 3 * ne)) || (rc = get(ev, cl.ev, 3 * ne)) || (rc = get(eC, cl.eC, 9 * ne)) ||
      (rc = get(eF, cl.eF, 9 * ne)) || (rc = get(ed, cl.ed, 9 * ne)))
    return rc;
  ZS_CUDA(cudaStreamSynchronize(c->stream));
  return MPM_OK;
}

int32_t mpm_cloth_upload(mpm_ctx *c, const float *vx, const float *vv, const float *vC,
                         const float *ex, const float *ev, const float *eC, const float *eF,
                         const float *ed) {
  ZS_RANGE("mpm_cloth_upload");
  int32_t rc = check(c);
  if (rc) return rc;
  if ((rc = settle(c))) return rc;
  const ClothDev &cl = c->d.cloth;
  if (cl.n_verts == 0) return fail(MPM_ERR_STATE, "no cloth in this context");
  auto put = [&](float *dst, const float *h, long long count) -> int32_t {
    if (!h) return MPM_OK;
    ZS_CUDA(cudaMemcpyAsync(dst, h, count * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    return MPM_OK;
  };
  const long long nv = cl.n_verts, ne = cl.n_eles;
  if ((rc = put(cl.vx, vx, 3 * nv)) || (rc = put(cl.vv, vv, 3 * nv)) ||
      (rc = put(cl.vC, vC, 9 * nv)) || (rc = put(cl.ex, ex, 3 * ne)) ||
      (rc = put(cl.ev, ev, 3 * ne)) || (rc = put(cl.eC, eC, 9 * ne)) ||
      (rc = put(cl.eF, eF, 9 * ne)) || (rc = put(cl.ed, ed, 9 * ne)))
    return rc;
  ZS_CUDA(cudaStreamSynchronize(c->stream));
  c->partition_valid = false;  // the cloth's points moved
  return MPM_OK;
}

int32_t mpm_trackers_create(mpm_ctx *c, int64_t n, const float *x, const float *v) {
  int32_t rc = check(c);
  if (rc) return rc;
  if (n <= 0 || !x) return fail(MPM_ERR_INVALID, "trackers need positions");
  if (c->scenes.size() != 1) return fail(MPM_ERR_INVALID, "trackers need a single-scene context");
  if (c->d.n_trackers > 0) return fail(MPM_ERR_STATE, "one tracker set per context");
  float *tx = nullptr, *tv = nullptr;
  if ((rc = dalloc(c, &tx, (size_t)3 * n)) || (rc = dalloc(c, &tv, (size_t)3 * n))) return rc;
  ZS_CUDA(cudaMemcpyAsync(tx, x, 3 * n * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  if (v)
    ZS_CUDA(cudaMemcpyAsync(tv, v, 3 * n * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  else
    ZS_CUDA(cudaMemsetAsync(tv, 0, 3 * n * sizeof(float), c->stream));
  ZS_CUDA(cudaStreamSynchronize(c->stream));
  c->d.tx = tx;
  c->d.tv = tv;
  c->d.n_trackers = n;
  drop_graphs(c);  // the substep gains the trackers' kernels
  c->partition_valid = false;
  return MPM_OK;
}

int32_t mpm_trackers_download(mpm_ctx *c, float *x, float *v) {
  int32_t rc = check(c);
  if (rc) return rc;
  if ((rc = settle(c))) return rc;
  const long long n = c->d.n_trackers;
  if (n == 0) return fail(MPM_ERR_STATE, "no trackers in this context");
  if (x) ZS_CUDA(cudaMemcpyAsync(x, c->d.tx, 3 * n * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  if (v) ZS_CUDA(cudaMemcpyAsync(v, c->d.tv, 3 * n * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  ZS_CUDA(cudaStreamSynchronize(c->stream));
  return MPM_OK;
}

int32_t mpm_compute_von_mises(mpm_ctx *c, int32_t by_log1p) {
  int32_t rc = check(c);
  if (rc) return rc;
  if ((rc = settle(c))) return rc;
  if (c->prm.n == 0) return MPM_OK;
  if ((rc = push_params(c))) return rc;
  launch_von_mises(c->d, c->cur, by_log1p ? 1 : 0, c->stream);
  return launch_check("von Mises");
}

int32_t mpm_frame_wait(mpm_ctx *c) {
  int32_t rc = check(c);
  if (rc) return rc;
  if (!c->frame_pending) return MPM_OK;
  ZS_CUDA(cudaEventSynchronize(c->frame_done));
  c->frame_pending = false;
  return MPM_OK;
}

int32_t mpm_frame_begin(mpm_ctx *c, float *x, float *v) {
  ZS_RANGE("mpm_frame_begin");
  int32_t rc = check(c);
  if (rc) return rc;
  if ((rc = settle(c))) return rc;
  if ((rc = mpm_frame_wait(c))) return rc;  // the snapshot buffer is free again
  const long long n = c->prm.n;
  if (n == 0) return MPM_OK;
  if (!c->frame_buf) {
    if ((rc = dalloc(c, &c->frame_buf, (size_t)6 * c->d.cap))) return rc;
    ZS_CUDA(cudaStreamCreateWithFlags(&c->frame_stream, cudaStreamNonBlocking));
    ZS_CUDA(cudaEventCreateWithFlags(&c->frame_ready, cudaEventDisableTiming));
    ZS_CUDA(cudaEventCreateWithFlags(&c->frame_done, cudaEventDisableTiming));
  }
  launch_snapshot_xv(c->d, c->cur, c->frame_buf, n, c->stream);
  if ((rc = launch_check("frame snapshot"))) return rc;
  ZS_CUDA(cudaEventRecord(c->frame_ready, c->stream));
  ZS_CUDA(cudaStreamWaitEvent(c->frame_stream, c->frame_ready, 0));
  if (x)
    ZS_CUDA(cudaMemcpyAsync(x, c->frame_buf, 3 * n * sizeof(float), cudaMemcpyDeviceToHost,
                            c->frame_stream));
  if (v)
    ZS_CUDA(cudaMemcpyAsync(v, c->frame_buf + 3 * n, 3 * n * sizeof(float),
                            cudaMemcpyDeviceToHost, c->frame_stream));
  ZS_CUDA(cudaEventRecord(c->frame_done, c->frame_stream));
  c->frame_pending = true;
  return MPM_OK;
}

int32_t mpm_set_transfer(mpm_ctx *c, int32_t scheme) {
  int32_t rc = check(c);
  if (rc) return rc;
  if ((rc = settle(c))) return rc;
  if (scheme < MPM_TRANSFER_APIC || scheme > MPM_TRANSFER_AFLIP)
    return fail(MPM_ERR_INVALID, "unknown transfer scheme");
  if (scheme != MPM_TRANSFER_APIC && c->d.differentiable)
    return fail(MPM_ERR_INVALID, "the differentiable form takes the APIC transfer only");
  if (scheme == c->d.transfer) return MPM_OK;
  DevPtrs &d = c->d;
  if (scheme != MPM_TRANSFER_APIC && !d.grid2) {
    if ((rc = dalloc(c, &d.grid2, (size_t)d.cap_gblocks * 64)) ||
        (rc = dalloc(c, &d.ptile2, (size_t)d.cap_gblocks * kTileNodes)))
      return rc;
    configure_flip_launches(d);
  }
  ZS_CUDA(cudaStreamSynchronize(c->stream));
  d.transfer = scheme;
  c->prm.transfer = scheme;
  c->prm_dirty = true;
  drop_graphs(c);  // the graphs hold the other transfer's kernels
  if ((rc = push_params(c))) return rc;
  if (c->prm.n > 0) {  // the stored stress follows the scheme's Lame parameters
    launch_stress(d, c->cur, c->stream);
    if ((rc = launch_check("stress"))) return rc;
  }
  c->partition_valid = false;  // a stage-path grid of the old scheme is stale
  return MPM_OK;
}

int32_t mpm_compute_particle_beta(mpm_ctx *c, float dt, int32_t collider) {
  ZS_RANGE("mpm_compute_particle_beta");
  int32_t rc = check(c);
  if (rc) return rc;
  if ((rc = settle(c))) return rc;
  if (collider < -2 || collider >= (int32_t)c->colliders.size())
    return fail(MPM_ERR_INVALID, "collider id out of range");
  if (collider == -2 && !c->d.bnd_map)
    return fail(MPM_ERR_STATE, "no boundary grid (mpm_set_grid_boundary)");
  if (collider == -2 && c->d.cloth.n_verts > 0)
    return fail(MPM_ERR_INVALID, "the boundary-grid beta of a cloth is not implemented");
  if ((rc = push_params(c))) return rc;
  if (c->prm.n > 0) launch_particle_beta(c->d, c->cur, dt, collider, c->stream);
  // a triangle cloth's vertices (curves keep beta 0, as in the reference)
  if (c->d.cloth.n_verts > 0 && c->d.cloth.kind == MPM_MESH_SURFACE)
    launch_cloth_beta(c->d, dt, collider, c->stream);
  return launch_check("particle beta");
}

int32_t mpm_partition(mpm_ctx *c) {
  ZS_RANGE("mpm_partition");
  int32_t rc = check(c);
  if (rc) return rc;
  set_auto_step(c, 0);  // the stage path moves colliders only on request
  if ((rc = settle(c))) return rc;
  if ((rc = push_params(c)) || (rc = prepare_partition(c))) return rc;
  enqueue_bin_if_needed(c);
  if (c->d.cloth.n_verts > 0) launch_cloth_mark(c->d, c->stream);
  if (c->d.n_trackers > 0) launch_tracker_mark(c->d, c->stream);
  if (c->auto_regrow) {  // a growing directory: grow it before sorting
    ZS_CUDA(cudaMemcpyAsync(c->h_cnt, c->d.cnt, sizeof(Counters), cudaMemcpyDeviceToHost,
                            c->stream));
    ZS_CUDA(cudaStreamSynchronize(c->stream));
    const int b = c->h_cnt->status;
    if ((b & ST_OUT_OF_DOMAIN) && !(b & (ST_NAN | ST_CAPACITY | ST_MATERIAL))) {
      if ((rc = regrow(c)) || (rc = push_params(c))) return rc;
      enqueue_bin_if_needed(c);
      if (c->d.cloth.n_verts > 0) launch_cloth_mark(c->d, c->stream);
      if (c->d.n_trackers > 0) launch_tracker_mark(c->d, c->stream);
    }
  }
  enqueue_sort(c);
  if ((rc = launch_check("partition"))) return rc;
  c->partition_valid = true;
  return MPM_OK;
}

int32_t mpm_grid_clear(mpm_ctx *c) {
  ZS_RANGE("mpm_grid_clear");
  int32_t rc = check(c);
  if (rc) return rc;
  if (!c->partition_valid) return fail(MPM_ERR_STATE, "grid clear needs a partition");
  launch_grid_clear(c->d, c->stream);
  return launch_check("grid clear");
}

int32_t mpm_p2g(mpm_ctx *c, float dt) {
  ZS_RANGE("mpm_p2g");
  int32_t rc = check(c);
  if (rc) return rc;
  if (!c->partition_valid) return fail(MPM_ERR_STATE, "p2g needs a partition of the current positions");
  if ((rc = set_dt(c, dt))) return rc;
  launch_p2g(c->d, c->cur, c->stream);
  launch_grid_gather(c->d, 0, c->stream);  // grid = m, mv as after the reference P2G
  if (c->d.cloth.n_verts > 0) launch_cloth_p2g(c->d, true, c->stream);
  return launch_check("p2g");
}

int32_t mpm_grid_update(mpm_ctx *c, float dt, float *max_vel_sqr) {
  ZS_RANGE("mpm_grid_update");
  int32_t rc = check(c);
  if (rc) return rc;
  if (!c->partition_valid) return fail(MPM_ERR_STATE, "grid update needs a partition");
  if ((rc = set_dt(c, dt))) return rc;
  ZS_CUDA(cudaMemsetAsync(&c->d.cnt->max_vel_sqr_bits, 0, sizeof(unsigned), c->stream));
  launch_grid_update(c->d, 1, c->stream);
  if ((rc = launch_check("grid update"))) return rc;
  if (max_vel_sqr) {
    ZS_CUDA(cudaMemcpyAsync(c->h_cnt, c->d.cnt, sizeof(Counters), cudaMemcpyDeviceToHost,
                            c->stream));
    ZS_CUDA(cudaStreamSynchronize(c->stream));
    float f;
    std::memcpy(&f, &c->h_cnt->max_vel_sqr_bits, sizeof(float));
    *max_vel_sqr = f;
  }
  return MPM_OK;
}

int32_t mpm_apply_boundary(mpm_ctx *c) {
  ZS_RANGE("mpm_apply_boundary");
  int32_t rc = check(c);
  if (rc) return rc;
  if (!c->partition_valid) return fail(MPM_ERR_STATE, "boundary needs a partition");
  if ((rc = push_params(c))) return rc;
  launch_grid_update(c->d, 2, c->stream);
  if (!c->colliders.empty()) launch_apply_colliders(c->d, -1, c->stream);
  return launch_check("boundary");
}

int32_t mpm_apply_walls(mpm_ctx *c) {
  ZS_RANGE("mpm_apply_walls");
  int32_t rc = check(c);
  if (rc) return rc;
  if (!c->partition_valid) return fail(MPM_ERR_STATE, "boundary needs a partition");
  if ((rc = push_params(c))) return rc;
  launch_grid_update(c->d, 2, c->stream);
  return launch_check("walls");
}

int32_t mpm_apply_collider(mpm_ctx *c, int32_t id) {
  ZS_RANGE("mpm_apply_collider");
  int32_t rc = check(c);
  if (rc) return rc;
  if (!c->partition_valid) return fail(MPM_ERR_STATE, "collider needs a partition");
  if (id < -1 || id >= (int32_t)c->colliders.size())
    return fail(MPM_ERR_INVALID, "collider id out of range");
  if (c->colliders.empty()) return MPM_OK;
  if ((rc = push_params(c))) return rc;
  launch_apply_colliders(c->d, id, c->stream);
  return launch_check("collider");
}

int32_t mpm_g2p(mpm_ctx *c, float dt) {
  ZS_RANGE("mpm_g2p");
  int32_t rc = check(c);
  if (rc) return rc;
  if (!c->partition_valid) return fail(MPM_ERR_STATE, "g2p needs the partition used by p2g");
  if ((rc = set_dt(c, dt))) return rc;
  launch_g2p(c->d, c->cur, 0, 0, c->stream);
  if (c->d.cloth.n_verts > 0) launch_cloth_g2p(c->d, c->stream);
  if (c->d.n_trackers > 0) launch_tracker_g2p(c->d, c->stream);
  if ((rc = launch_check("g2p"))) return rc;
  c->cur = 1 - c->cur;
  c->partition_valid = false;
  c->binned = false;
  c->substeps += 1;
  return MPM_OK;
}

int32_t mpm_return_mapping(mpm_ctx *c) {
  ZS_RANGE("mpm_return_mapping");
  int32_t rc = check(c);
  if (rc) return rc;
  if ((rc = push_params(c))) return rc;
  launch_return_mapping(c->d, c->cur, c->stream);
  return launch_check("return mapping");
}

int32_t mpm_substep(mpm_ctx *c, float dt, int32_t n_substeps) {
  ZS_RANGE("mpm_substep");
  int32_t rc = check(c);
  if (rc) return rc;
  if (n_substeps < 0) return fail(MPM_ERR_INVALID, "negative substep count");
  set_auto_step(c, 1);
  if ((rc = set_dt(c, dt)) || (rc = prepare_partition(c))) return rc;
  if (n_substeps > 0) enqueue_bin_if_needed(c);
  const bool graphs = graphs_enabled();
  for (int32_t k = 0; k < n_substeps; ++k) {
    if (graphs) {
      if ((rc = ensure_graph(c, c->cur))) return rc;
      ZS_CUDA(cudaGraphLaunch(c->graph[c->cur], c->stream));
    } else {
      enqueue_substep(c, c->cur);
      if ((rc = launch_check("substep"))) return rc;
    }
    c->cur = 1 - c->cur;
  }
  c->partition_valid = false;
  c->substeps += n_substeps;
  if (c->auto_regrow && n_substeps > 0) {
    c->pending.emplace_back(dt, n_substeps);
    c->pending_total += n_substeps;
  }
  return MPM_OK;
}

int32_t mpm_substep_timed(mpm_ctx *c, float dt, float *stage_ms, int32_t n_stages) {
  ZS_RANGE("mpm_substep_timed");
  int32_t rc = check(c);
  if (rc) return rc;
  if (!stage_ms || n_stages < MPM_NUM_STAGES)
    return fail(MPM_ERR_INVALID, "stage_ms needs MPM_NUM_STAGES entries");
  set_auto_step(c, 1);
  if ((rc = set_dt(c, dt)) || (rc = prepare_partition(c))) return rc;
  if (!c->events[0]) {
    for (int i = 0; i <= MPM_NUM_STAGES; ++i) ZS_CUDA(cudaEventCreate(&c->events[i]));
  }
  ZS_CUDA(cudaEventRecord(c->events[MPM_STAGE_BIN], c->stream));
  enqueue_bin_if_needed(c);
  enqueue_substep(c, c->cur, c->events);
  if ((rc = launch_check("timed substep"))) return rc;
  ZS_CUDA(cudaEventSynchronize(c->events[MPM_NUM_STAGES]));
  if (uses_persistent(c)) {
    // one kernel: its stages from the times it noted at each barrier (the
    // launch itself counted to the scan)
    float bin = 0.0f, all = 0.0f;
    ZS_CUDA(cudaEventElapsedTime(&bin, c->events[MPM_STAGE_BIN], c->events[MPM_STAGE_SCAN]));
    ZS_CUDA(cudaEventElapsedTime(&all, c->events[MPM_STAGE_SCAN], c->events[MPM_NUM_STAGES]));
    ZS_CUDA(cudaMemcpyAsync(c->h_cnt, c->d.cnt, sizeof(Counters), cudaMemcpyDeviceToHost,
                            c->stream));
    ZS_CUDA(cudaStreamSynchronize(c->stream));
    const unsigned long long *t = c->h_cnt->stage_t;
    auto ms = [&](int a, int b) { return (float)((double)(t[b] - t[a]) * 1e-6); };
    stage_ms[MPM_STAGE_BIN] = bin;
    stage_ms[MPM_STAGE_SCATTER] = ms(2, 3);
    stage_ms[MPM_STAGE_SORT] = ms(3, 4);
    stage_ms[MPM_STAGE_P2G] = ms(4, 5);
    stage_ms[MPM_STAGE_GRID_UPDATE] = ms(5, 6);
    stage_ms[MPM_STAGE_G2P] = ms(6, 7);
    stage_ms[MPM_STAGE_SCAN] = all - ms(2, 7);
  } else {
    for (int i = 0; i < MPM_NUM_STAGES; ++i) {
      float ms = 0.0f;
      ZS_CUDA(cudaEventElapsedTime(&ms, c->events[i], c->events[i + 1]));
      stage_ms[i] = ms;
    }
  }
  c->cur = 1 - c->cur;
  c->partition_valid = false;
  c->substeps += 1;
  return MPM_OK;
}

int32_t mpm_set_launch_config(mpm_ctx *c, const mpm_launch_config *cfg) {
  int32_t rc = check(c);
  if (rc) return rc;
  if (!cfg || cfg->p2g_ctas_per_sm < 0 || cfg->g2p_ctas_per_sm < 0 || cfg->sort_ctas_per_sm < 0 ||
      cfg->stream_ctas_per_sm < 0 || cfg->p2g_ctas_per_sm > 64 || cfg->g2p_ctas_per_sm > 64 ||
      cfg->sort_ctas_per_sm > 64 || cfg->stream_ctas_per_sm > 64 ||
      (cfg->g2p_threads != 0 && cfg->g2p_threads != 128) ||
      cfg->p2g_shape < MPM_P2G_192x128 || cfg->p2g_shape > MPM_P2G_256x256 ||
      (cfg->gather_blocks != 0 && cfg->gather_blocks != 2 && cfg->gather_blocks != 4 &&
       cfg->gather_blocks != 8))
    return fail(MPM_ERR_INVALID, "bad launch configuration");
  ZS_CUDA(cudaStreamSynchronize(c->stream));
  c->d.launch = LaunchConfig{cfg->p2g_ctas_per_sm,    cfg->g2p_ctas_per_sm, cfg->sort_ctas_per_sm,
                             cfg->stream_ctas_per_sm, cfg->g2p_threads,     cfg->p2g_shape,
                             cfg->gather_blocks};
  configure_launches(c->d);
  for (int k = 0; k < 2; ++k)  // the captured graphs hold the old shapes
    if (c->graph[k]) {
      cudaGraphExecDestroy(c->graph[k]);
      c->graph[k] = nullptr;
    }
  return MPM_OK;
}

int32_t mpm_get_launch_config(mpm_ctx *c, mpm_launch_config *cfg) {
  int32_t rc = check(c);
  if (rc) return rc;
  if (!cfg) return fail(MPM_ERR_INVALID, "null config");
  const DevPtrs &d = c->d;
  cfg->p2g_ctas_per_sm = d.grid_p2g / d.num_sms;
  cfg->g2p_ctas_per_sm = d.grid_g2p / d.num_sms;
  cfg->sort_ctas_per_sm = d.grid_sort / d.num_sms;
  cfg->stream_ctas_per_sm = d.grid_stream / d.num_sms;
  cfg->g2p_threads = d.g2p_threads;
  cfg->p2g_shape = d.launch.p2g_shape;
  cfg->gather_blocks = d.launch.gather_blocks == 0 ? 4 : d.launch.gather_blocks;
  return MPM_OK;
}

int32_t mpm_set_differentiable(mpm_ctx *c, int32_t on) {
  int32_t rc = check(c);
  if (rc) return rc;
  if ((rc = settle(c))) return rc;
  if (on && c->d.transfer != MPM_TRANSFER_APIC)
    return fail(MPM_ERR_INVALID, "the differentiable form takes the APIC transfer only");
  if (on && c->d.cloth.n_verts > 0)
    return fail(MPM_ERR_INVALID, "the differentiable form takes no cloth");
  if (on && !c->d.ptile_adj &&
      (rc = dalloc(c, &c->d.ptile_adj, (size_t)c->d.cap_gblocks * kTileNodes)))
    return rc;
  if (on && !c->d.adj_rec && (rc = dalloc(c, &c->d.adj_rec, (size_t)16 * c->d.cap))) return rc;
  if (on && !c->prm.has_lame) {  // the states carry per-particle mu / lam
    launch_lame_from_materials(c->d, c->cur, c->stream);
    if ((rc = launch_check("per-particle Lame parameters"))) return rc;
    c->prm.has_lame = 1;
    c->prm_dirty = true;
    if ((rc = push_params(c))) return rc;
  }
  c->d.differentiable = on ? 1 : 0;
  drop_graphs(c);
  return MPM_OK;
}

int32_t mpm_state_save(mpm_ctx *c, float *dst) {
  ZS_RANGE("mpm_state_save");
  int32_t rc = check(c);
  if (rc) return rc;
  if ((rc = settle(c))) return rc;
  if (!c->d.differentiable) return fail(MPM_ERR_STATE, "state copies need mpm_set_differentiable(ctx, 1)");
  if (!dst) return fail(MPM_ERR_INVALID, "null destination");
  const size_t n = (size_t)c->prm.n;
  if (n == 0) return MPM_OK;
  launch_state_copy(c->d, c->cur, dst, nullptr, (long long)n, c->stream);
  return launch_check("state save");
}

int32_t mpm_state_load(mpm_ctx *c, const float *src) {
  ZS_RANGE("mpm_state_load");
  int32_t rc = check(c);
  if (rc) return rc;
  if ((rc = settle(c))) return rc;
  if (!c->d.differentiable) return fail(MPM_ERR_STATE, "state copies need mpm_set_differentiable(ctx, 1)");
  if (!src) return fail(MPM_ERR_INVALID, "null source");
  const size_t n = (size_t)c->prm.n;
  if (n == 0) return MPM_OK;
  launch_state_copy(c->d, c->cur, nullptr, src, (long long)n, c->stream);
  if ((rc = push_params(c))) return rc;
  launch_stress(c->d, c->cur, c->stream);
  if ((rc = launch_check("state load"))) return rc;
  c->needs_full_clear = true;  // the directory counts described the old positions
  c->binned = false;
  c->partition_valid = false;
  return MPM_OK;
}

int32_t mpm_adjoint_substep(mpm_ctx *c, float dt, const float *adj_next, float *adj_prev,
                            float *grad_mu, float *grad_lam) {
  ZS_RANGE("mpm_adjoint_substep");
  int32_t rc = check(c);
  if (rc) return rc;
  if ((rc = settle(c))) return rc;
  if (!c->d.differentiable) return fail(MPM_ERR_STATE, "the adjoint needs mpm_set_differentiable(ctx, 1)");
  if (c->auto_regrow)
    return fail(MPM_ERR_INVALID, "a rollout needs a fixed block directory (mpm_set_auto_regrow(ctx, 0))");
  if (c->d.bnd_map) return fail(MPM_ERR_INVALID, "the adjoint takes no boundary grid");
  if (!adj_next || !adj_prev || !grad_mu || !grad_lam)
    return fail(MPM_ERR_INVALID, "null adjoint buffer");
  if (!c->differentiable)
    return fail(MPM_ERR_INVALID,
                "the adjoint covers fixed-corotated, Neo-Hookean and StVK-Hencky (with or without "
                "the Drucker-Prager projection) materials, not the equation-of-state fluid, the "
                "stable Neo-Hookean model or von Mises / Cam-Clay plasticity");
  for (const ColliderDev &cd : c->colliders)
    if (cd.db[0] != 0.0f || cd.db[1] != 0.0f || cd.db[2] != 0.0f || cd.ds != 0.0f)
      return fail(MPM_ERR_INVALID, "the adjoint takes static colliders only");
  set_auto_step(c, 0);
  if ((rc = set_dt(c, dt)) || (rc = prepare_partition(c))) return rc;
  enqueue_bin_if_needed(c);
  enqueue_sort(c);
  launch_p2g(c->d, c->cur, c->stream);
  launch_grid_gather(c->d, 3, c->stream);  // grid velocities of this substep
  if (!c->colliders.empty()) launch_apply_colliders(c->d, -1, c->stream);
  const long long n = c->prm.n;
  launch_g2p_adjoint(c->d, c->cur, adj_next, adj_prev, grad_mu, grad_lam, n, c->stream);
  launch_grid_adjoint(c->d, c->stream);
  launch_p2g_adjoint(c->d, c->cur, adj_prev, grad_mu, grad_lam, n, c->stream);
  if ((rc = launch_check("adjoint substep"))) return rc;
  c->partition_valid = true;
  return MPM_OK;
}

int32_t mpm_snapshot_floats(mpm_ctx *c, int64_t *floats) {
  int32_t rc = check(c);
  if (rc) return rc;
  if (!floats) return fail(MPM_ERR_INVALID, "null argument");
  *floats = tiled_elems(c->prm.n, NCH) + tiled_elems(c->prm.n, NICH);
  return MPM_OK;
}

namespace {

// A snapshot buffer as a particle store: the tiled float channels, then the
// tiled int channels of n particles (128-byte aligned: whole tiles).
struct SnapStore {
  float *f;
  int32_t *i;
};
SnapStore snap_store(const mpm_ctx *c, float *base) {
  return SnapStore{base, reinterpret_cast<int32_t *>(base + tiled_elems(c->prm.n, NCH))};
}

int32_t snapshot_copy(mpm_ctx *c, SnapStore dst, const float *src_f, const int32_t *src_i) {
  const long long n = c->prm.n;
  ZS_CUDA(cudaMemcpyAsync(dst.f, src_f, (size_t)tiled_elems(n, NCH) * sizeof(float),
                          cudaMemcpyDeviceToDevice, c->stream));
  ZS_CUDA(cudaMemcpyAsync(dst.i, src_i, (size_t)tiled_elems(n, NICH) * sizeof(int32_t),
                          cudaMemcpyDeviceToDevice, c->stream));
  return MPM_OK;
}

// Runs the kernels with the particle store pair (a -> b) in place of the
// context's own buffers: store 0 = a, store 1 = b, current 0.
struct StoreSwap {
  mpm_ctx *c;
  float *pb[2];
  int32_t *ib[2];
  int cur;
  explicit StoreSwap(mpm_ctx *ctx) : c(ctx), cur(ctx->cur) {
    for (int k = 0; k < 2; ++k) {
      pb[k] = c->d.pbuf[k];
      ib[k] = c->d.ibuf[k];
    }
  }
  void use(SnapStore a, SnapStore b) {
    c->d.pbuf[0] = a.f;
    c->d.ibuf[0] = a.i;
    c->d.pbuf[1] = b.f;
    c->d.ibuf[1] = b.i;
    c->cur = 0;
  }
  ~StoreSwap() {
    for (int k = 0; k < 2; ++k) {
      c->d.pbuf[k] = pb[k];
      c->d.ibuf[k] = ib[k];
    }
    c->cur = cur;
    // the context's own store no longer matches the directory's counts
    c->needs_full_clear = true;
    c->binned = false;
    c->partition_valid = false;
  }
};

void free_psets(mpm_ctx *c) { drop_psets(c); }

// `count` partition sets of `capb` blocks each; false (none kept) when the
// device has not room for them with a margin, so that the rollout takes the
// path that partitions each adjoint substep again.
bool ensure_psets(mpm_ctx *c, int count, int capb) {
  if ((int)c->psets.size() >= count && c->pset_cap >= capb) return true;
  free_psets(c);
  const DevPtrs &d = c->d;
  const size_t per = (size_t)d.cap * 4 + (size_t)d.ndir * 8 + (size_t)capb * 16 +
                     (size_t)capb * (64 + kTileNodes) * sizeof(float4);
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return false;
  const size_t margin = std::max<size_t>(total_b / 16, (size_t)2 << 30);
  if (per * count + margin > free_b) return false;
  bool ok = dalloc(c, &c->pset_cnt, 2 * (size_t)count) == MPM_OK;
  for (int k = 0; ok && k < count; ++k) {
    PartSet p{};
    ok = dalloc(c, &p.perm, (size_t)d.cap) == MPM_OK && dalloc(c, &p.dir_gb, (size_t)d.ndir) == MPM_OK &&
         dalloc(c, &p.dir_bk, (size_t)d.ndir) == MPM_OK && dalloc(c, &p.gb_dir, (size_t)capb) == MPM_OK &&
         dalloc(c, &p.bk_dir, (size_t)capb) == MPM_OK && dalloc(c, &p.bk_start, (size_t)capb) == MPM_OK &&
         dalloc(c, &p.bk_count, (size_t)capb) == MPM_OK &&
         dalloc(c, &p.grid, (size_t)capb * 64) == MPM_OK &&
         dalloc(c, &p.ptile, (size_t)capb * kTileNodes) == MPM_OK;
    c->psets.push_back(p);  // freed with the others if incomplete
  }
  if (!ok) {
    free_psets(c);
    cudaGetLastError();  // the failed allocation is not this call's error
    return false;
  }
  c->pset_cap = capb;
  return true;
}

// Runs the kernels with partition set k in place of the context's own
// partition and grid buffers (and its capacity in blocks).
struct PartSwap {
  mpm_ctx *c;
  PartSet own;
  int cap;
  explicit PartSwap(mpm_ctx *ctx) : c(ctx), cap(ctx->d.cap_gblocks) {
    const DevPtrs &d = c->d;
    own = PartSet{d.perm, d.dir_gb, d.dir_bk, d.gb_dir, d.bk_dir, d.bk_start, d.bk_count,
                  d.grid, d.ptile};
  }
  void set(const PartSet &p, int capb) {
    DevPtrs &d = c->d;
    d.perm = p.perm;
    d.dir_gb = p.dir_gb;
    d.dir_bk = p.dir_bk;
    d.gb_dir = p.gb_dir;
    d.bk_dir = p.bk_dir;
    d.bk_start = p.bk_start;
    d.bk_count = p.bk_count;
    d.grid = p.grid;
    d.ptile = p.ptile;
    d.cap_gblocks = capb;
  }
  ~PartSwap() { set(own, cap); }
};

}  // namespace

int32_t mpm_rollout_forward(mpm_ctx *c, float dt, int32_t n_substeps, int32_t every,
                            const float *state0, float *ckpts, float *seg_states,
                            float *final_state) {
  ZS_RANGE("mpm_rollout_forward");
  int32_t rc = check(c);
  if (rc) return rc;
  if (n_substeps < 0 || every <= 0 || !state0 || !final_state || (n_substeps > 0 && !ckpts))
    return fail(MPM_ERR_INVALID, "invalid rollout arguments");
  if (c->auto_regrow)
    return fail(MPM_ERR_INVALID, "a rollout needs a fixed block directory: the backward recomputes "
                                 "from checkpoints that a moved directory may not cover "
                                 "(mpm_set_auto_regrow(ctx, 0))");
  c->tail.valid = false;
  const long long n = c->prm.n;
  const size_t snap = (size_t)(tiled_elems(n, NCH) + tiled_elems(n, NICH));
  if ((rc = mpm_state_load(c, state0))) return rc;
  // the block counts of these partitions size the backward's kept ones
  ZS_CUDA(cudaMemsetAsync(&c->d.cnt->max_gblocks, 0, 2 * sizeof(int), c->stream));
  const int32_t n_seg = (n_substeps + every - 1) / every;
  const int32_t s_tail = n_substeps > 0 ? (n_seg - 1) * every : 0;
  const bool want_tail = seg_states && n_substeps > 0 && c->differentiable;
  for (int32_t s = 0; s < (want_tail ? s_tail : n_substeps); ++s) {
    if (s % every == 0 &&
        (rc = snapshot_copy(c, snap_store(c, ckpts + (size_t)(s / every) * snap), c->d.pbuf[c->cur],
                            c->d.ibuf[c->cur])))
      return rc;
    if ((rc = mpm_substep(c, dt, 1))) return rc;
  }
  // The last segment through kept snapshots and partitions, sized by the
  // block counts so far with room to double (a segment that outgrows them
  // is run again the plain way).
  bool tail = false;
  Counters before{};
  if (want_tail) {
    if ((rc = mpm_sync(c))) return rc;
    before = *c->h_cnt;
    const int seen = std::max(c->h_cnt->max_gblocks, c->h_cnt->max_buckets);
    const int capb = seen > 0 ? std::min(c->d.cap_gblocks, std::max(2 * seen, seen + 4096))
                              : c->d.cap_gblocks;
    tail = ensure_psets(c, std::min(every, n_substeps), capb);
  }
  if (tail) {
    SnapStore ck = snap_store(c, ckpts + (size_t)(n_seg - 1) * snap);
    if ((rc = snapshot_copy(c, ck, c->d.pbuf[c->cur], c->d.ibuf[c->cur]))) return rc;
    // state s of the segment: its checkpoint, then seg_states slots 1 ..;
    // the final state into slot 0 (the backward's recompute never uses it)
    auto state = [&](int32_t s) {
      return s == s_tail ? ck
                         : snap_store(c, seg_states + (s == n_substeps ? 0 : (size_t)(s - s_tail) * snap));
    };
    {
      StoreSwap swap(c);
      PartSwap pswap(c);
      set_auto_step(c, 1);
      if ((rc = set_dt(c, dt)) || (rc = push_params(c))) return rc;
      for (int32_t s = s_tail; s < n_substeps; ++s) {
        swap.use(state(s), state(s + 1));
        pswap.set(c->psets[s - s_tail], c->pset_cap);
        if ((rc = prepare_partition(c))) return rc;
        enqueue_bin_if_needed(c);
        enqueue_substep(c, 0);
        ZS_CUDA(cudaMemcpyAsync(c->pset_cnt + 2 * (s - s_tail), &c->d.cnt->n_gblocks,
                                2 * sizeof(int), cudaMemcpyDeviceToDevice, c->stream));
        if ((rc = launch_check("rollout forward"))) return rc;
      }
    }
    ZS_CUDA(cudaMemcpyAsync(c->h_cnt, c->d.cnt, sizeof(Counters), cudaMemcpyDeviceToHost, c->stream));
    ZS_CUDA(cudaStreamSynchronize(c->stream));
    if (c->h_cnt->status & ST_CAPACITY) {
      // more blocks than the kept sets hold: the segment again, the plain
      // way, from the counters as they were before it
      ZS_CUDA(cudaMemcpyAsync(c->d.cnt, &before, sizeof(Counters), cudaMemcpyHostToDevice,
                              c->stream));
      ZS_CUDA(cudaMemcpyAsync(c->d.pbuf[c->cur], ck.f, (size_t)tiled_elems(n, NCH) * sizeof(float),
                              cudaMemcpyDeviceToDevice, c->stream));
      ZS_CUDA(cudaMemcpyAsync(c->d.ibuf[c->cur], ck.i,
                              (size_t)tiled_elems(n, NICH) * sizeof(int32_t),
                              cudaMemcpyDeviceToDevice, c->stream));
      ZS_CUDA(cudaStreamSynchronize(c->stream));
      free_psets(c);
      for (int32_t s = s_tail; s < n_substeps; ++s)
        if ((rc = mpm_substep(c, dt, 1))) return rc;
      return mpm_state_save(c, final_state);
    }
    // the final state back into the context's own store
    SnapStore fin = state(n_substeps);
    ZS_CUDA(cudaMemcpyAsync(c->d.pbuf[c->cur], fin.f, (size_t)tiled_elems(n, NCH) * sizeof(float),
                            cudaMemcpyDeviceToDevice, c->stream));
    ZS_CUDA(cudaMemcpyAsync(c->d.ibuf[c->cur], fin.i, (size_t)tiled_elems(n, NICH) * sizeof(int32_t),
                            cudaMemcpyDeviceToDevice, c->stream));
    c->substeps += n_substeps - s_tail;
    c->tail.valid = true;
    c->tail.dt = dt;
    c->tail.n = n_substeps;
    c->tail.every = every;
    c->tail.ckpts = ckpts;
    c->tail.seg = seg_states;
  }
  return mpm_state_save(c, final_state);
}

int32_t mpm_rollout_backward(mpm_ctx *c, float dt, int32_t n_substeps, int32_t every,
                             const float *ckpts, float *seg_states, float *adj, float *adj_tmp,
                             float *grad_mu, float *grad_lam) {
  ZS_RANGE("mpm_rollout_backward");
  int32_t rc = check(c);
  if (rc) return rc;
  if ((rc = settle(c))) return rc;
  if (n_substeps < 0 || every <= 0 || (n_substeps > 0 && (!ckpts || !seg_states)) || !adj ||
      !adj_tmp || !grad_mu || !grad_lam)
    return fail(MPM_ERR_INVALID, "invalid rollout arguments");
  if (!c->d.differentiable) return fail(MPM_ERR_STATE, "the adjoint needs mpm_set_differentiable(ctx, 1)");
  if (!c->differentiable)
    return fail(MPM_ERR_INVALID,
                "the adjoint covers fixed-corotated, Neo-Hookean and StVK-Hencky (with or without "
                "the Drucker-Prager projection) materials, not the equation-of-state fluid, the "
                "stable Neo-Hookean model or von Mises / Cam-Clay plasticity");
  for (const ColliderDev &cd : c->colliders)
    if (cd.db[0] != 0.0f || cd.db[1] != 0.0f || cd.db[2] != 0.0f || cd.ds != 0.0f)
      return fail(MPM_ERR_INVALID, "the adjoint takes static colliders only");
  if (c->d.bnd_map) return fail(MPM_ERR_INVALID, "the adjoint takes no boundary grid");
  const long long n = c->prm.n;
  const size_t snap = (size_t)(tiled_elems(n, NCH) + tiled_elems(n, NICH));
  float *a = adj, *b = adj_tmp;  // adjoint of the next state, of this one
  const int32_t n_seg = (n_substeps + every - 1) / every;
  // Each recomputed substep partitions its state and gathers its grid into
  // a set of its own, which its adjoint then reads instead of partitioning
  // and scattering again (sized by the forward rollout's block counts; the
  // same substeps recomputed bit for bit ask for the same counts).
  ZS_CUDA(cudaMemcpyAsync(c->h_cnt, c->d.cnt, sizeof(Counters), cudaMemcpyDeviceToHost, c->stream));
  ZS_CUDA(cudaStreamSynchronize(c->stream));
  const int seen = std::max(c->h_cnt->max_gblocks, c->h_cnt->max_buckets);
  const int capb =
      seen > 0 ? std::min(c->d.cap_gblocks, seen + std::max(64, seen / 64)) : c->d.cap_gblocks;
  // the forward with these arguments kept its last segment (states in
  // seg_states, partitions in the sets): no recompute for that one
  const bool tail_kept = c->tail.valid && c->tail.dt == dt && c->tail.n == n_substeps &&
                         c->tail.every == every && c->tail.ckpts == ckpts &&
                         c->tail.seg == seg_states && (int)c->psets.size() >= std::min(every, n_substeps);
  c->tail.valid = false;  // the recompute of the other segments overwrites it
  const bool keep =
      n_substeps > 0 && (tail_kept || ensure_psets(c, std::min(every, n_substeps), capb));
  static_assert(offsetof(Counters, n_buckets) == offsetof(Counters, n_gblocks) + sizeof(int),
                "n_gblocks, n_buckets adjacent");
  StoreSwap swap(c);
  PartSwap pswap(c);
  if ((rc = set_dt(c, dt))) return rc;
  // the colliders are static here, so stepping them is the identity: one
  // parameter set for the whole walk (no upload inside a segment)
  set_auto_step(c, 1);
  if ((rc = push_params(c))) return rc;
  const long long nn = c->prm.n;
  // One segment: recompute its states from `ck` (its checkpoint), then take
  // them back through the adjoint substeps, last to first.
  auto segment = [&](int32_t s0, int32_t s1, SnapStore ck, bool kept) -> int32_t {
    // the segment's states: its checkpoint, then the recomputed ones, each
    // substep reading one snapshot and writing the next (no copies)
    auto state = [&](int32_t s) {
      return s == s0 ? ck : snap_store(c, seg_states + (size_t)(s - s0) * snap);
    };
    int32_t r;
    c->needs_full_clear = true;
    c->binned = false;
    for (int32_t s = s0; !kept && s + 1 < s1; ++s) {
      swap.use(state(s), state(s + 1));
      if (keep) pswap.set(c->psets[s - s0], c->pset_cap);
      if ((r = prepare_partition(c))) return r;
      enqueue_bin_if_needed(c);
      enqueue_substep(c, 0);  // bins the new positions: the next one needs no binning
      if (keep)
        ZS_CUDA(cudaMemcpyAsync(c->pset_cnt + 2 * (s - s0), &c->d.cnt->n_gblocks, 2 * sizeof(int),
                                cudaMemcpyDeviceToDevice, c->stream));
      if ((r = launch_check("rollout recompute"))) return r;
    }
    for (int32_t s = s1 - 1; s >= s0; --s) {
      swap.use(state(s), state(s));
      if (keep) pswap.set(c->psets[s - s0], c->pset_cap);
      if (keep && (s + 1 < s1 || kept)) {  // kept by the recompute (or the forward)
        ZS_CUDA(cudaMemcpyAsync(&c->d.cnt->n_gblocks, c->pset_cnt + 2 * (s - s0), 2 * sizeof(int),
                                cudaMemcpyDeviceToDevice, c->stream));
      } else {  // the segment's last substep (not recomputed), or no sets
        c->needs_full_clear = true;  // the counts described another state
        c->binned = false;
        if ((r = prepare_partition(c))) return r;
        enqueue_bin_if_needed(c);
        enqueue_sort(c);
        launch_p2g(c->d, 0, c->stream);
        launch_grid_gather(c->d, 3, c->stream);  // grid velocities of this substep
        if (!c->colliders.empty()) launch_apply_colliders(c->d, -1, c->stream);
      }
      launch_g2p_adjoint(c->d, 0, a, b, grad_mu, grad_lam, nn, c->stream);
      launch_grid_adjoint(c->d, c->stream);
      launch_p2g_adjoint(c->d, 0, b, grad_mu, grad_lam, nn, c->stream);
      if ((r = launch_check("rollout adjoint"))) return r;
      std::swap(a, b);
    }
    return MPM_OK;
  };
  // Full segments of an even length all launch the same operations on the
  // same buffers (the kept partition sets, the segment states; the adjoint
  // pair swapped an even number of times) once each one's checkpoint is
  // copied into slot 0 of seg_states, which no recompute writes: for scenes
  // of up to 4M particles the first is captured as a CUDA graph and the rest
  // replay it, without the per-launch gaps.
  cudaGraphExec_t seg_graph = nullptr;
  struct GraphGuard {
    cudaGraphExec_t *g;
    ~GraphGuard() {
      if (*g) cudaGraphExecDestroy(*g);
    }
  } graph_guard{&seg_graph};
  bool graph_failed = false;
  for (int32_t seg = n_seg - 1; seg >= 0; --seg) {
    const int32_t s0 = seg * every, s1 = std::min(s0 + every, n_substeps);
    const bool kept = tail_kept && seg == n_seg - 1;  // states and sets from the forward
    const SnapStore ck = snap_store(c, const_cast<float *>(ckpts) + (size_t)seg * snap);
    // (large scenes gain nothing from it: their kernels dwarf the launches,
    // and the checkpoint copy would cost more)
    const bool replay = keep && !kept && s1 - s0 == every && every % 2 == 0 && every > 1 &&
                        nn <= (1ll << 22) && graphs_enabled() && !graph_failed;
    if (!replay) {
      if ((rc = segment(s0, s1, ck, kept))) return rc;
      continue;
    }
    const SnapStore slot0 = snap_store(c, seg_states);
    ZS_CUDA(cudaMemcpyAsync(slot0.f, ck.f, snap * sizeof(float), cudaMemcpyDeviceToDevice,
                            c->stream));
    if (!seg_graph) {
      cudaGraph_t g = nullptr;
      float *a0 = a, *b0 = b;
      ZS_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
      const int32_t r = segment(s0, s1, slot0, false);
      cudaError_t e = cudaStreamEndCapture(c->stream, &g);
      if (r == MPM_OK && e == cudaSuccess) e = cudaGraphInstantiate(&seg_graph, g, 0);
      if (g) cudaGraphDestroy(g);
      a = a0;  // the captured segment has not run yet
      b = b0;
      if (r != MPM_OK || e != cudaSuccess) {  // run it (and the rest) without a graph
        seg_graph = nullptr;
        graph_failed = true;
        cudaGetLastError();
        if ((rc = segment(s0, s1, slot0, false))) return rc;
        continue;
      }
    }
    ZS_CUDA(cudaGraphLaunch(seg_graph, c->stream));
  }
  if (a != adj)
    ZS_CUDA(cudaMemcpyAsync(adj, a, (size_t)MPM_ADJ_PLANES * n * sizeof(float),
                            cudaMemcpyDeviceToDevice, c->stream));
  return MPM_OK;
}

int32_t mpm_sync(mpm_ctx *c) {
  ZS_RANGE("mpm_sync");
  int32_t rc = check(c);
  if (rc) return rc;
  ZS_CUDA(cudaMemcpyAsync(c->h_cnt, c->d.cnt, sizeof(Counters), cudaMemcpyDeviceToHost,
                          c->stream));
  ZS_CUDA(cudaStreamSynchronize(c->stream));
  // a growing directory: a particle left it, and no worse error came with it
  for (int round = 0; c->auto_regrow && round < kMaxRegrowRounds; ++round) {
    const int b = c->h_cnt->status;
    if (!(b & ST_OUT_OF_DOMAIN) || (b & (ST_NAN | ST_CAPACITY | ST_MATERIAL | ST_TIMEOUT))) break;
    // the gate let `started` of the queued substeps run; the state after the
    // last of them is complete (the halted ones changed nothing)
    const int64_t started = (int64_t)c->h_cnt->n_started - c->started_base;
    const int64_t halted = std::max<int64_t>(0, c->pending_total - started);
    if (halted & 1) c->cur = 1 - c->cur;
    c->substeps -= halted;
    std::vector<std::pair<float, int32_t>> replay;
    int64_t need = halted;
    for (auto it = c->pending.rbegin(); it != c->pending.rend() && need > 0; ++it) {
      const int32_t k = (int32_t)std::min<int64_t>(need, it->second);
      replay.emplace_back(it->first, k);
      need -= k;
    }
    std::reverse(replay.begin(), replay.end());
    c->pending.clear();
    c->pending_total = 0;
    if ((rc = regrow(c))) return rc;
    for (const auto &r : replay)
      if ((rc = mpm_substep(c, r.first, r.second))) return rc;
    ZS_CUDA(cudaMemcpyAsync(c->h_cnt, c->d.cnt, sizeof(Counters), cudaMemcpyDeviceToHost,
                            c->stream));
    ZS_CUDA(cudaStreamSynchronize(c->stream));
  }
  c->pending.clear();
  c->pending_total = 0;
  c->started_base = c->h_cnt->n_started;
  const int bits = c->h_cnt->status;
  if (bits & (ST_CAPACITY | ST_OUT_OF_DOMAIN)) c->needs_full_clear = true;
  const int32_t st = map_status(bits);
  if (st != MPM_OK) return fail(st, status_text(st));
  return MPM_OK;
}

int32_t mpm_set_auto_regrow(mpm_ctx *c, int32_t on) {
  int32_t rc = check(c);
  if (rc) return rc;
  if (on && c->scenes.size() != 1)
    return fail(MPM_ERR_INVALID, "a growing directory needs a one-scene context");
  if ((rc = settle(c))) return rc;
  if ((on != 0) != c->auto_regrow) {
    ZS_CUDA(cudaStreamSynchronize(c->stream));
    ZS_CUDA(cudaMemsetAsync(&c->d.cnt->halt, 0, 2 * sizeof(int), c->stream));
    c->auto_regrow = on != 0;
    c->pending.clear();
    c->pending_total = 0;
    c->started_base = 0;
    drop_graphs(c);  // the graphs gain or lose the substep gate
  }
  return MPM_OK;
}

int32_t mpm_set_persistent(mpm_ctx *c, int32_t on, uint64_t barrier_limit) {
  int32_t rc = check(c);
  if (rc) return rc;
  if ((rc = settle(c))) return rc;
  if (on) {
    int coop = 0;
    ZS_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, c->device));
    if (!coop || c->d.grid_persist <= 0)
      return fail(MPM_ERR_INVALID, "the device cannot run the persistent substep kernel");
  }
  ZS_CUDA(cudaStreamSynchronize(c->stream));
  c->persistent = on != 0;
  c->prm.barrier_limit = barrier_limit;
  c->prm_dirty = true;
  drop_graphs(c);
  return MPM_OK;
}

int32_t mpm_barrier_selftest(mpm_ctx *c, uint64_t barrier_limit, int32_t *timed_out) {
  if (!timed_out) return fail(MPM_ERR_INVALID, "null output");
  int32_t rc = check(c);
  if (rc) return rc;
  if ((rc = settle(c))) return rc;
  ZS_CUDA(cudaMemcpyAsync(c->h_cnt, c->d.cnt, sizeof(Counters), cudaMemcpyDeviceToHost, c->stream));
  ZS_CUDA(cudaStreamSynchronize(c->stream));
  const Counters keep = *c->h_cnt;
  cudaError_t e = launch_barrier_selftest(c->d, barrier_limit, c->stream);
  if (e != cudaSuccess)
    return fail(MPM_ERR_CUDA, std::string("barrier self-test: ") + cudaGetErrorString(e));
  ZS_CUDA(cudaMemcpyAsync(c->h_cnt, c->d.cnt, sizeof(Counters), cudaMemcpyDeviceToHost, c->stream));
  ZS_CUDA(cudaStreamSynchronize(c->stream));
  *timed_out = (c->h_cnt->status & ST_TIMEOUT) != 0 && c->h_cnt->halt != 0;
  // the context's counters (status word, halt flag) as they were
  ZS_CUDA(cudaMemcpyAsync(c->d.cnt, &keep, sizeof(Counters), cudaMemcpyHostToDevice, c->stream));
  ZS_CUDA(cudaStreamSynchronize(c->stream));
  *c->h_cnt = keep;
  return MPM_OK;
}

// Checkpoint files: a fixed header, then the blocks in the order written
// below, each a plain little-endian array.  The particle store goes in its
// slot order with the upload ids, so a resumed run steps exactly as the
// uninterrupted one.
struct CkptHeader {
  char magic[8];  // "ZSMPMCK1"
  uint32_t version, nch, nich;
  int32_t transfer, has_lame, n_colliders;
  int64_t n, substeps, store_floats, store_ints;
  float dx;
  int32_t reserved;
  int64_t cloth_verts, cloth_eles, trackers;
};
constexpr uint32_t kCkptVersion = 1;
constexpr int kCkptColliderFloats = 10;  // b[3], s, lo[3], hi[3]: the current pose

int32_t mpm_checkpoint_write(mpm_ctx *c, const char *path) {
  ZS_RANGE("mpm_checkpoint_write");
  int32_t rc = check(c);
  if (rc) return rc;
  if (!path) return fail(MPM_ERR_INVALID, "null path");
  if (c->scenes.size() != 1) return fail(MPM_ERR_INVALID, "checkpoints take a one-scene context");
  if ((rc = settle(c))) return rc;
  const DevPtrs &d = c->d;
  const ClothDev &cl = d.cloth;
  CkptHeader h{};
  std::memcpy(h.magic, "ZSMPMCK1", 8);
  h.version = kCkptVersion;
  h.nch = NCH;
  h.nich = NICH;
  h.transfer = d.transfer;
  h.has_lame = c->prm.has_lame;
  h.n_colliders = c->prm.n_colliders;
  h.n = c->prm.n;
  h.substeps = c->substeps;
  h.store_floats = tiled_elems(h.n, NCH);
  h.store_ints = tiled_elems(h.n, NICH);
  h.dx = c->scenes[0].dx;
  h.cloth_verts = cl.n_verts;
  h.cloth_eles = cl.n_eles;
  h.trackers = d.n_trackers;
  std::vector<float> store((size_t)h.store_floats), beta((size_t)h.n);
  std::vector<int32_t> istore((size_t)h.store_ints);
  std::vector<ColliderDev> col((size_t)h.n_colliders);
  ZS_CUDA(cudaMemcpyAsync(store.data(), d.pbuf[c->cur], store.size() * sizeof(float),
                          cudaMemcpyDeviceToHost, c->stream));
  ZS_CUDA(cudaMemcpyAsync(istore.data(), d.ibuf[c->cur], istore.size() * sizeof(int32_t),
                          cudaMemcpyDeviceToHost, c->stream));
  ZS_CUDA(cudaMemcpyAsync(beta.data(), d.beta, beta.size() * sizeof(float), cudaMemcpyDeviceToHost,
                          c->stream));
  if (h.n_colliders > 0)
    ZS_CUDA(cudaMemcpyAsync(col.data(), d.colliders, col.size() * sizeof(ColliderDev),
                            cudaMemcpyDeviceToHost, c->stream));
  // the cloth (vx vv vC ex ev eC eF ed, vertex beta) and the trackers (x, v)
  const long long nv = cl.n_verts, ne = cl.n_eles, nt = d.n_trackers;
  std::vector<std::pair<const float *, long long>> extra;
  if (nv > 0)
    extra = {{cl.vx, 3 * nv}, {cl.vv, 3 * nv}, {cl.vC, 9 * nv}, {cl.ex, 3 * ne}, {cl.ev, 3 * ne},
             {cl.eC, 9 * ne}, {cl.eF, 9 * ne}, {cl.ed, 9 * ne}, {cl.vbeta, nv}};
  if (nt > 0) {
    extra.push_back({d.tx, 3 * nt});
    extra.push_back({d.tv, 3 * nt});
  }
  std::vector<std::vector<float>> ex(extra.size());
  for (size_t k = 0; k < extra.size(); ++k) {
    ex[k].resize((size_t)extra[k].second);
    ZS_CUDA(cudaMemcpyAsync(ex[k].data(), extra[k].first, ex[k].size() * sizeof(float),
                            cudaMemcpyDeviceToHost, c->stream));
  }
  ZS_CUDA(cudaStreamSynchronize(c->stream));
  std::vector<float> poses((size_t)h.n_colliders * kCkptColliderFloats);
  for (int k = 0; k < h.n_colliders; ++k) {
    float *q = &poses[(size_t)k * kCkptColliderFloats];
    for (int a = 0; a < 3; ++a) {
      q[a] = col[k].b[a];
      q[4 + a] = col[k].lo[a];
      q[7 + a] = col[k].hi[a];
    }
    q[3] = col[k].s;
  }
  FILE *f = std::fopen(path, "wb");
  if (!f) return fail(MPM_ERR_INVALID, std::string("cannot open ") + path + " for writing");
  bool ok = std::fwrite(&h, sizeof(h), 1, f) == 1 &&
            std::fwrite(store.data(), sizeof(float), store.size(), f) == store.size() &&
            std::fwrite(istore.data(), sizeof(int32_t), istore.size(), f) == istore.size() &&
            std::fwrite(beta.data(), sizeof(float), beta.size(), f) == beta.size() &&
            std::fwrite(poses.data(), sizeof(float), poses.size(), f) == poses.size();
  for (size_t k = 0; ok && k < ex.size(); ++k)
    ok = std::fwrite(ex[k].data(), sizeof(float), ex[k].size(), f) == ex[k].size();
  ok = std::fclose(f) == 0 && ok;
  if (!ok) return fail(MPM_ERR_INVALID, std::string("writing ") + path + " failed");
  return MPM_OK;
}

int32_t mpm_checkpoint_read(mpm_ctx *c, const char *path) {
  ZS_RANGE("mpm_checkpoint_read");
  int32_t rc = check(c);
  if (rc) return rc;
  if (!path) return fail(MPM_ERR_INVALID, "null path");
  if (c->scenes.size() != 1) return fail(MPM_ERR_INVALID, "checkpoints take a one-scene context");
  if ((rc = settle(c))) return rc;
  DevPtrs &d = c->d;
  ClothDev &cl = d.cloth;
  FILE *f = std::fopen(path, "rb");
  if (!f) return fail(MPM_ERR_INVALID, std::string("cannot open ") + path);
  struct Closer {
    FILE *f;
    ~Closer() { std::fclose(f); }
  } closer{f};
  CkptHeader h{};
  if (std::fread(&h, sizeof(h), 1, f) != 1 || std::memcmp(h.magic, "ZSMPMCK1", 8) != 0)
    return fail(MPM_ERR_INVALID, std::string(path) + " is not a checkpoint of this library");
  if (h.version != kCkptVersion || h.nch != (uint32_t)NCH || h.nich != (uint32_t)NICH)
    return fail(MPM_ERR_INVALID, "the checkpoint's format version or store layout differs");
  if (h.n < 0 || h.n > d.cap || h.store_floats != tiled_elems(h.n, NCH) ||
      h.store_ints != tiled_elems(h.n, NICH))
    return fail(MPM_ERR_INVALID, "the checkpoint's particles do not fit this context");
  if (h.dx != c->scenes[0].dx || h.transfer != d.transfer || h.n_colliders != c->prm.n_colliders ||
      h.cloth_verts != cl.n_verts || h.cloth_eles != cl.n_eles || h.trackers != d.n_trackers)
    return fail(MPM_ERR_INVALID, "the checkpoint was written by a context with another scene "
                                 "(dx, transfer, colliders, cloth or trackers)");
  std::vector<float> store((size_t)h.store_floats), beta((size_t)h.n),
      poses((size_t)h.n_colliders * kCkptColliderFloats);
  std::vector<int32_t> istore((size_t)h.store_ints);
  bool ok = std::fread(store.data(), sizeof(float), store.size(), f) == store.size() &&
            std::fread(istore.data(), sizeof(int32_t), istore.size(), f) == istore.size() &&
            std::fread(beta.data(), sizeof(float), beta.size(), f) == beta.size() &&
            std::fread(poses.data(), sizeof(float), poses.size(), f) == poses.size();
  const long long nv = cl.n_verts, ne = cl.n_eles, nt = d.n_trackers;
  std::vector<std::pair<float *, long long>> extra;
  if (nv > 0)
    extra = {{cl.vx, 3 * nv}, {cl.vv, 3 * nv}, {cl.vC, 9 * nv}, {cl.ex, 3 * ne}, {cl.ev, 3 * ne},
             {cl.eC, 9 * ne}, {cl.eF, 9 * ne}, {cl.ed, 9 * ne}, {cl.vbeta, nv}};
  if (nt > 0) {
    extra.push_back({d.tx, 3 * nt});
    extra.push_back({d.tv, 3 * nt});
  }
  std::vector<std::vector<float>> ex(extra.size());
  for (size_t k = 0; ok && k < extra.size(); ++k) {
    ex[k].resize((size_t)extra[k].second);
    ok = std::fread(ex[k].data(), sizeof(float), ex[k].size(), f) == ex[k].size();
  }
  if (!ok) return fail(MPM_ERR_INVALID, std::string(path) + " is truncated");
  // the ids index per-particle arrays and the materials the parameter table:
  // a file that breaks either is refused before anything reaches the device
  std::vector<char> seen((size_t)h.n, 0);
  for (long long p = 0; p < h.n; ++p) {
    const int32_t id = istore[(size_t)iidx(IC_ID, p)], mat = istore[(size_t)iidx(IC_MAT, p)];
    if (id < 0 || id >= h.n || seen[(size_t)id] || mat < 0 || mat >= c->n_materials)
      return fail(MPM_ERR_INVALID, std::string(path) + " holds invalid particle ids or materials");
    seen[(size_t)id] = 1;
  }
  // the colliders' current poses into their device entries (the samples and
  // the rates stay the context's own)
  std::vector<ColliderDev> col((size_t)h.n_colliders);
  if (h.n_colliders > 0) {
    ZS_CUDA(cudaMemcpy(col.data(), d.colliders, col.size() * sizeof(ColliderDev),
                       cudaMemcpyDeviceToHost));
    for (int k = 0; k < h.n_colliders; ++k) {
      const float *q = &poses[(size_t)k * kCkptColliderFloats];
      for (int a = 0; a < 3; ++a) {
        col[k].b[a] = q[a];
        col[k].lo[a] = q[4 + a];
        col[k].hi[a] = q[7 + a];
      }
      col[k].s = q[3];
    }
  }
  ZS_CUDA(cudaMemcpyAsync(d.pbuf[c->cur], store.data(), store.size() * sizeof(float),
                          cudaMemcpyHostToDevice, c->stream));
  ZS_CUDA(cudaMemcpyAsync(d.ibuf[c->cur], istore.data(), istore.size() * sizeof(int32_t),
                          cudaMemcpyHostToDevice, c->stream));
  ZS_CUDA(cudaMemcpyAsync(d.beta, beta.data(), beta.size() * sizeof(float), cudaMemcpyHostToDevice,
                          c->stream));
  if (h.n_colliders > 0)
    ZS_CUDA(cudaMemcpyAsync(d.colliders, col.data(), col.size() * sizeof(ColliderDev),
                            cudaMemcpyHostToDevice, c->stream));
  for (size_t k = 0; k < ex.size(); ++k)
    ZS_CUDA(cudaMemcpyAsync(extra[k].first, ex[k].data(), ex[k].size() * sizeof(float),
                            cudaMemcpyHostToDevice, c->stream));
  ZS_CUDA(cudaMemsetAsync(d.vms, 0, (size_t)std::max<long long>(h.n, 1) * sizeof(float),
                          c->stream));
  // a fresh store, as after an upload: status word, substep gate, directory
  ZS_CUDA(cudaMemsetAsync(&d.cnt->status, 0, sizeof(int), c->stream));
  ZS_CUDA(cudaMemsetAsync(&d.cnt->halt, 0, 2 * sizeof(int), c->stream));
  ZS_CUDA(cudaStreamSynchronize(c->stream));
  c->prm.n = h.n;
  c->prm.has_lame = h.has_lame;
  c->scenes[0].p_off = 0;
  c->prm_dirty = true;
  if ((rc = push_params(c))) return rc;
  c->pending.clear();
  c->pending_total = 0;
  c->started_base = 0;
  c->substeps = h.substeps;
  c->needs_full_clear = true;  // the directory counts described the old positions
  c->binned = false;
  c->partition_valid = false;
  drop_graphs(c);
  return MPM_OK;
}

int32_t mpm_get_domain(mpm_ctx *c, int32_t block_lo[3], int32_t block_dims[3],
                       int32_t *n_regrows) {
  int32_t rc = check(c);
  if (rc) return rc;
  if ((rc = settle(c))) return rc;
  for (int a = 0; a < 3; ++a) {
    if (block_lo) block_lo[a] = c->scenes[0].block_lo[a];
    if (block_dims) block_dims[a] = c->scenes[0].block_dims[a];
  }
  if (n_regrows) *n_regrows = c->regrows;
  return MPM_OK;
}

int32_t mpm_get_stats(mpm_ctx *c, mpm_stats *out) {
  if (!out) return fail(MPM_ERR_INVALID, "null stats");
  int32_t rc = check(c);
  if (rc) return rc;
  const int32_t st = mpm_sync(c);
  if (st == MPM_ERR_CUDA) return st;
  out->n_particles = c->prm.n;
  out->n_particle_blocks = c->h_cnt->n_buckets;
  out->n_grid_blocks = c->h_cnt->n_gblocks;
  float f;
  std::memcpy(&f, &c->h_cnt->max_vel_sqr_bits, sizeof(float));
  out->max_vel_sqr = f;
  out->status = st;
  out->substeps = c->substeps;
  return MPM_OK;
}

int32_t mpm_partition_download(mpm_ctx *c, int32_t *n_pb, int32_t *pb_dir, int32_t *pb_count,
                               int64_t cap_pb, int32_t *perm, int32_t *n_gb, int32_t *gb_dir,
                               int64_t cap_gb) {
  int32_t rc = check(c);
  if (rc) return rc;
  if (!c->partition_valid) return fail(MPM_ERR_STATE, "no partition of the current positions");
  if ((rc = mpm_sync(c))) return rc;
  const int nb = c->h_cnt->n_buckets, ng = c->h_cnt->n_gblocks;
  if (n_pb) *n_pb = nb;
  if (n_gb) *n_gb = ng;
  if ((pb_dir || pb_count) && cap_pb < nb) return fail(MPM_ERR_CAPACITY, "cap_pb too small");
  if (gb_dir && cap_gb < ng) return fail(MPM_ERR_CAPACITY, "cap_gb too small");
  if (pb_dir) ZS_CUDA(cudaMemcpy(pb_dir, c->d.bk_dir, nb * sizeof(int32_t), cudaMemcpyDeviceToHost));
  if (pb_count)
    ZS_CUDA(cudaMemcpy(pb_count, c->d.bk_count, nb * sizeof(int32_t), cudaMemcpyDeviceToHost));
  if (gb_dir) ZS_CUDA(cudaMemcpy(gb_dir, c->d.gb_dir, ng * sizeof(int32_t), cudaMemcpyDeviceToHost));
  if (perm) {
    const long long n = c->prm.n;
    std::vector<int32_t> p(n), ib((size_t)tiled_elems(n, NICH));
    ZS_CUDA(cudaMemcpy(p.data(), c->d.perm, n * sizeof(int32_t), cudaMemcpyDeviceToHost));
    // the id channel of the first n slots (tiles of the int store)
    ZS_CUDA(cudaMemcpy(ib.data(), c->d.ibuf[c->cur], ib.size() * sizeof(int32_t),
                       cudaMemcpyDeviceToHost));
    const int binned = std::min<long long>(c->h_cnt->n_binned, n);
    for (long long s = 0; s < n; ++s)
      perm[s] = (s < binned && p[s] >= 0 && p[s] < n) ? ib[iidx(IC_ID, p[s])] : -1;
  }
  return MPM_OK;
}

int32_t mpm_grid_download(mpm_ctx *c, float *nodes, int64_t cap_floats) {
  int32_t rc = check(c);
  if (rc) return rc;
  if ((rc = mpm_sync(c))) return rc;
  const long long ng = c->h_cnt->n_gblocks;
  if (!nodes || cap_floats < ng * 256) return fail(MPM_ERR_CAPACITY, "node buffer too small");
  ZS_CUDA(cudaMemcpy(nodes, c->d.grid, ng * 64 * sizeof(float4), cudaMemcpyDeviceToHost));
  return MPM_OK;
}

}  // extern "C"
