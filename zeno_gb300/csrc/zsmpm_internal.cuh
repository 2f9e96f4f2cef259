// Internal declarations shared by the zsmpm translation units.
//
// HBM layout (one context):
//  * particles: two buffers (current / next substep), each `NCH` float
//    channels plus `NICH` int32 channels, tiled by 32 particle slots: element
//    (channel ch, slot p) of a store of nch channels sits at
//    ((p / 32) * nch + ch) * 32 + p % 32.  A warp reads one channel of 32
//    consecutive slots as one 128-byte line, and the channels of a slot are
//    a fixed 128 bytes apart, so every channel access of a particle is one
//    base address plus a constant offset, and the channels of a block of
//    particles share a few pages.  The substep re-orders particles by
//    (block, cell) as G2P writes the next buffer, so the next substep's
//    reads through the sort permutation are near-sequential.
//  * block directory: dense int32 arrays over every 4^3 block of the domain
//    box (a perfect hash of block coordinates), holding particle counts,
//    scatter cursors and the grid block index.
//  * grid: `cap_gblocks` blocks x 64 nodes x float4 (m, mv / v), node cell id
//    (i << 4) | (j << 2) | k inside the block; with the FLIP transfers a
//    second grid of float4 (vstar, 0) in the same node order.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/zsmpm.h"

namespace zsmpm {

// float particle channels (planes)
enum : int {
  CH_X = 0,     // 3
  CH_V = 3,     // 3
  CH_C = 6,     // 9, row-major
  CH_F = 15,    // 9, row-major
  CH_J = 24,    // 1
  CH_M = 25,    // 1
  CH_VOL = 26,  // 1
  CH_MU = 27,   // 1, per-particle override (optional)
  CH_LAM = 28,  // 1, per-particle override (optional)
  CH_S = 29,    // 6, vol * Kirchhoff stress (xx, yy, zz, xy, xz, yz) of the current F
  NCH = 35
};
// int particle channels
enum : int { IC_MAT = 0, IC_ID = 1, NICH = 2 };

// tiled particle store (see the layout note above)
constexpr int kPTile = 32;
__host__ __device__ __forceinline__ long long tix(long long p, int ch, int nch) {
  return ((p >> 5) * nch + ch) * kPTile + (p & (kPTile - 1));
}
__host__ __device__ __forceinline__ long long pidx(int ch, long long p) { return tix(p, ch, NCH); }
__host__ __device__ __forceinline__ long long iidx(int ch, long long p) {
  return tix(p, ch, NICH);
}
// elements of a store of nch channels for `cap` slots
inline long long tiled_elems(long long cap, int nch) {
  return (cap + kPTile - 1) / kPTile * kPTile * nch;
}

// device status bits (OR-ed into Counters::status)
enum : int {
  ST_OUT_OF_DOMAIN = 1,
  ST_CAPACITY = 2,
  ST_NAN = 4,
  ST_BUCKET_OVERSIZE = 8,
  ST_TIMEOUT = 16,
  ST_STENCIL = 32,
  ST_MATERIAL = 64  // a material id of an asynchronous upload out of range
};

// block coordinates (and so node indices, 4 per block) stay inside +-2^27
// blocks, which keeps every node index of a domain an int32
constexpr int kMaxBlockCoord = 1 << 27;
// directory entries of one context (all scenes); key = (entry << 6) | cell
// must stay an int32
constexpr long long kMaxDirBlocks = 1ll << 25;

constexpr int kMaxMaterials = 256;
constexpr int kMaxScenes = 4096;
constexpr int kScanTile = 512;        // directory entries per scan tile
constexpr int kScanThreads = 256;     // 2 entries per thread
constexpr int kScanPerThread = kScanTile / kScanThreads;
constexpr int kTileNodes = 216;       // 6^3 nodes of one particle block's stencils

struct MatParams {
  int type, plastic;
  float mu, lam, alpha, bulk, gamma;
  float yield;                    // von Mises yield stress
  float cc_M, cc_beta, cc_xi, pad;  // Cam-Clay slope, cohesion, hardening
};

struct Counters {
  int n_gblocks;  // grid blocks of the current partition (clamped to capacity)
  int n_buckets;  // non-empty particle blocks
  int status;
  unsigned max_vel_sqr_bits;
  int n_binned;
  int bad_material;  // set by the upload check of material ids
  int n_near;        // grid blocks the fused substep's gather found near a collider
  // growing directory: the substep gate sets `halt` when a particle left the
  // directory, and every kernel of the queued substeps then does nothing;
  // `n_started` counts the substeps the gate let through
  int halt;
  int n_started;
  unsigned bbox[6];  // ordered-bits min x, y, z, max x, y, z of the positions
  // the most grid / particle blocks a partition asked for since the last
  // reset (the differentiable rollout sizes its per-substep partitions by it)
  int max_gblocks, max_buckets;
  // grid-wide barrier of the persistent substep kernel: arrivals and the
  // generation the last arrival publishes; CTAs done with the last stage
  unsigned bar_count, bar_done, bar_gen, pad;
  // global timer (ns) when the last persistent substep started and when it
  // passed each of its stage barriers (the last entry: every CTA done)
  unsigned long long stage_t[8];
};

// Every kernel of the fused substep starts with this test: the substeps
// queued behind one whose particles left the directory leave the state as
// it is, so that the context can grow its directory and replay them.
#define ZSMPM_HALTED(d) ((d).cnt->halt != 0)

// Device-resident parameters; the host updates them with one small copy
// when they change, so captured graphs read the current values.
struct SimParams {
  float dt;
  int has_lame;
  int n_colliders;  // level-set colliders in DevPtrs::colliders
  int auto_step;    // the fused substep advances the colliders by dt
  int transfer;     // MPM_TRANSFER_* (MakeZSGrid "transfer")
  long long n;      // particles of all scenes
  // spins a CTA of the persistent substep waits at a grid barrier before it
  // gives up (ST_TIMEOUT); about 100 ns each
  unsigned long long barrier_limit;
};

// Level-set collider (MakeZSLevelSet + ToZSBoundary): dense signed distance
// grid in collider space, transform X = R^T (p - b) / s.
constexpr int kMaxColliders = MPM_MAX_COLLIDERS;
struct ColliderDev {
  float R[9];       // rotation, row-major
  float b[3], db[3];
  float s, ds;
  float origin[3];
  float inv_h;      // 1 / sample spacing
  int dims[3];
  int type;         // MPM_BC_*
  int scene;        // -1: every scene
  int has_vel;
  float cvel[3];    // material velocity when has_vel == 0
  const float *sdf;
  const float *vel;  // 3 planes, or null
  float lo[3], hi[3];  // world box holding the sample grid (with a margin)
};

// world bounding box of the collider's sample grid under p = s R X + b,
// padded so that rounding in the node test never puts a node the test
// accepts outside it; kept current wherever b or s change
#ifdef __CUDACC__
__host__ __device__
#endif
inline void collider_world_box(ColliderDev &c) {
  float lo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, hi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
  float big = 0.0f;
  for (int k = 0; k < 8; ++k) {
    float X[3];
    for (int a = 0; a < 3; ++a)
      X[a] = c.origin[a] + (((k >> a) & 1) ? (float)(c.dims[a] - 1) / c.inv_h : 0.0f);
    for (int a = 0; a < 3; ++a) {
      const float w = c.s * (c.R[a * 3 + 0] * X[0] + c.R[a * 3 + 1] * X[1] + c.R[a * 3 + 2] * X[2]) + c.b[a];
      lo[a] = w < lo[a] ? w : lo[a];
      hi[a] = w > hi[a] ? w : hi[a];
      const float m = w < 0.0f ? -w : w;
      big = m > big ? m : big;
    }
  }
  const float pad = 1e-4f * (1.0f + big);
  for (int a = 0; a < 3; ++a) {
    c.lo[a] = lo[a] - pad;
    c.hi[a] = hi[a] + pad;
  }
}

// Codimensional cloth (ToZSCloth): vertex and element arrays (AoS, row-major
// 3x3 matrices), the in-plane model and the cloth parameters; n_verts = 0
// when the context holds no cloth.
struct ClothDev {
  long long n_verts, n_eles;
  int kind;                  // MPM_MESH_SURFACE / MPM_MESH_CURVE (inds: 3 per element,
                             // curves use the first 2)
  int model;                 // MPM_FCR / MPM_NHK / MPM_STVK (curves: MPM_STVK)
  float gamma, k, fc, dc;    // shear stiffness, normal stiffness, tan(fa / pi), damping
  float *vx, *vv, *vC, *vm;
  float *vbeta;     // ComputeParticleBeta per vertex (FLIP-style position update)
  int32_t *vowner;  // scratch of the beta pass: the last element of each vertex
  float *ex, *ev, *eC, *eF, *ed, *eDmInv, *em, *evol, *emu, *elam;
  int32_t *inds;
  // vertex bending springs (ConstructBendingSprings "vertex"): vertex pairs,
  // stiffness, rest length; thickness = the model's dx
  long long n_springs;
  int32_t *sv;
  float *sk, *srl;
  float thickness;
  // Deterministic P2G.  The cloth's points (the vertices, then the
  // elements) are partitioned into 4^3 blocks of their own each substep
  // (keys, permutation and block lists below, through the partition's own
  // scan, placement and sort); each point writes one scatter record, and
  // the nodes of a block's 6^3 tile take the records of the cells around
  // them in a fixed order (cells, then points in sorted order).  The element and spring
  // impulses on the vertices are written per contribution slot (3 per
  // element, 2 per spring) and summed per vertex in the fixed order of the
  // vertex's slot list.
  float *crec;                    // kClothRec floats per point, in sorted order
  float4 *cimp;                   // impulse contributions
  int32_t *vptr, *vlist;          // per vertex: its contribution slots
  // key per point, sorted order; cperm_tmp is the sort's scratch, then the
  // inverse permutation (each point's sorted position, where its record goes)
  int32_t *ckey, *cperm, *cperm_tmp;
  int32_t *cdir_count, *cdir_fill, *cdir_gb, *cdir_bk, *cgb_dir, *ctile_sums;
  uint8_t *cdir_flag;             // stays zero: the points make no grid blocks here
  int32_t *cbk_dir, *cbk_start, *cbk_count;
  int cap_cblocks;
  float4 *ctile, *ctile2;         // per cloth block: its 216 node sums (ctile2: FLIP-style vstar)
  Counters *ccnt;
  SimParams *cprm;                // n = the number of points, no collider stepping
};
// floats of a cloth point's scatter record: x, m, b, A, Q, b2 -- the node
// receives W m, W (b + A (x_i - x_p)) and Q grad W (momentum, or vstar on
// FLIP-style grids), and W b2 in vstar
constexpr int kClothRec = 28;

// One scene of a context: its grid spacing, its slice of the concatenated
// block directory, its boundary and gravity.  A context holds one scene
// (the plain substep) or many independent scenes (the batched substep).
struct SceneParams {
  float dx, inv_dx, Dinv;
  float gravity[3];
  int block_lo[3];
  int block_dims[3];
  int dir_off;     // first directory entry of the scene
  int bc_type, bc_thickness;
  int bc_lo[3], bc_hi[3];
  long long p_off;  // first particle of the scene in upload order
};

// Launch shape of the persistent kernels (0 = default); picked by the
// autotuner through mpm_set_launch_config.
struct LaunchConfig {
  int p2g_ctas_per_sm, g2p_ctas_per_sm, sort_ctas_per_sm, stream_ctas_per_sm, g2p_threads;
  int p2g_shape;      // MPM_P2G_* tile shape (threads, chunk)
  int gather_blocks;  // grid blocks per CTA of the grid gather: 2, 4 or 8 (0: 4)
};

struct DevPtrs {
  float *pbuf[2];
  int32_t *ibuf[2];
  long long cap;  // particle plane stride
  int32_t *pkey;  // (directory index << 6) | cell, per storage slot
  int32_t *perm;  // sorted position -> storage slot
  int32_t *perm_tmp;  // scratch of the oversize-block sort
  int32_t *dir_count, *dir_fill, *dir_gb, *dir_bk;
  uint8_t *dir_flag;
  long long ndir;
  int32_t *gb_dir;
  int32_t *bk_dir, *bk_start, *bk_count;
  int cap_gblocks;
  float4 *grid;
  float4 *grid2;      // FLIP transfers: (vstar, 0) per node, else null
  float4 *ptile;      // per particle block: its 6^3 P2G node sums (216 float4)
  float4 *ptile2;     // FLIP transfers: the vstar sums of the same tiles
  float *beta;        // AFLIP positional adjustment per particle, by upload index
                      // (ComputeParticleBeta; 0 at upload), outside the
                      // double-buffered store so that APIC substeps keep it
  float4 *ptile_adj;  // the same for the G2P adjoint (differentiable mode)
  float *adj_rec;     // G2P adjoint scatter records, 16 planes of `cap` (differentiable mode)
  ColliderDev *colliders;  // kMaxColliders entries (device)
  int32_t *near_gb;        // cap_gblocks entries: the grid blocks near a collider
  float *vms;              // ComputeVonMises per particle, by upload index (0 at upload)
  ClothDev cloth;          // n_verts = 0: no cloth
  // ToTrackerParticles: points advected by the grid velocity, no P2G
  long long n_trackers;
  float *tx, *tv;
  int differentiable;  // mpm_set_differentiable: adjoint buffers allocated
  int planar_x;       // pbuf[0] holds positions as 3 planes of `cap` floats (binning only)
  int32_t *tile_sums;
  int ntiles;
  Counters *cnt;
  SimParams *prm;
  SceneParams *scn;  // n_scenes entries
  int n_scenes;
  MatParams *mats;
  int num_sms;
  int grid_p2g, grid_g2p;  // persistent grids: SMs x resident CTAs per SM
  int grid_sort, grid_stream, g2p_threads;
  int transfer;                      // MPM_TRANSFER_* (host copy of SimParams::transfer)
  int hencky;  // some material uses the von Mises / Cam-Clay return mapping
  // persistent grids of the FLIP and AFLIP transfer kernels
  int grid_p2g_flip, grid_p2g_aflip, grid_g2p_flip, grid_g2p_aflip;
  int grid_persist;  // CTAs of the persistent substep kernel (0: it cannot run)
  // boundary grid (mpm_set_grid_boundary; null: none): per directory entry
  // its boundary block or -1, per boundary node (m, v) then (nrm, 0)
  int32_t *bnd_map;
  float4 *bnd_grid;
  int bnd_type;  // MPM_BC_STICKY / SLIP / SEPARATE
  LaunchConfig launch;
};

// The partition and grid of one substep (the buffers a partition, P2G and
// the grid gather write and the adjoint kernels read), for a differentiable
// rollout that keeps them per substep instead of partitioning again.
struct PartSet {
  int32_t *perm, *dir_gb, *dir_bk, *gb_dir, *bk_dir, *bk_start, *bk_count;
  float4 *grid, *ptile;
};

// flip.cu: the FLIP / AFLIP transfers (the launch_* functions of transfer.cu
// dispatch to them when d.transfer is not APIC)
void configure_flip_launches(DevPtrs &d);
void launch_p2g_flip(const DevPtrs &d, int cur, cudaStream_t s);
void launch_grid_gather_flip(const DevPtrs &d, int mode, cudaStream_t s);
void launch_grid_update_flip(const DevPtrs &d, int mode, cudaStream_t s);
void launch_g2p_flip(const DevPtrs &d, int cur, int fuse_rm, int fuse_bin, cudaStream_t s);
// ComputeParticleBeta: collider -1 (volume criterion only) or a collider id
void launch_particle_beta(const DevPtrs &d, int cur, float dt, int collider, cudaStream_t s);

// cloth.cu
void launch_cloth_mark(const DevPtrs &d, cudaStream_t s);
// add_to_grid false: the tiles are left for the grid update (mode bit 4)
void launch_cloth_p2g(const DevPtrs &d, bool add_to_grid, cudaStream_t s);
void launch_cloth_g2p(const DevPtrs &d, cudaStream_t s);
// ComputeParticleBeta on the cloth's vertices (triangle meshes)
void launch_cloth_beta(const DevPtrs &d, float dt, int collider, cudaStream_t s);
void launch_tracker_mark(const DevPtrs &d, cudaStream_t s);
void launch_tracker_g2p(const DevPtrs &d, cudaStream_t s);

// output.cu
void launch_von_mises(const DevPtrs &d, int cur, int by_log1p, cudaStream_t s);
void launch_snapshot_xv(const DevPtrs &d, int cur, float *dst, long long n, cudaStream_t s);

// partition.cu
void launch_bin(const DevPtrs &d, int cur, cudaStream_t s);
void launch_scan(const DevPtrs &d, cudaStream_t s);
void launch_scatter(const DevPtrs &d, cudaStream_t s);
void launch_bucket_sort(const DevPtrs &d, cudaStream_t s);
void launch_grid_clear(const DevPtrs &d, cudaStream_t s);
void launch_full_dir_clear(const DevPtrs &d, cudaStream_t s);
// first kernel of every fused substep of a context that grows its directory
void launch_substep_gate(const DevPtrs &d, cudaStream_t s);
// bounding box of the particle positions (and cloth vertices, trackers) of
// buffer `cur` into Counters::bbox
void launch_bbox(const DevPtrs &d, int cur, cudaStream_t s);

// persistent.cu: the whole fused substep (APIC; `colliders`: level-set
// colliders on the listed blocks) as one cooperative kernel, its barrier
// counter reset on the stream first, with d.grid_persist CTAs: the CTAs
// the context's capacity needs, between one and all the CTAs the SMs hold at
// once (0 if the device cannot run it)
int persistent_grid(const DevPtrs &d);
cudaError_t launch_substep_persistent(const DevPtrs &d, int cur, bool colliders, cudaStream_t s);
// a grid barrier that nothing completes, with `limit` spins: every CTA gives
// up and sets ST_TIMEOUT (the self-test of the bounded wait)
cudaError_t launch_barrier_selftest(const DevPtrs &d, unsigned long long limit, cudaStream_t s);

// transfer.cu
// fills the persistent grid sizes of DevPtrs from the occupancy of each kernel
void configure_launches(DevPtrs &d);
void launch_p2g(const DevPtrs &d, int cur, cudaStream_t s);
// sum of the P2G tiles into the grid; mode bit 1: momentum -> velocity +
// gravity, bit 2: boundary (mode 0 leaves m, mv as the reference P2G does)
void launch_grid_gather(const DevPtrs &d, int mode, cudaStream_t s);
// mode bit 1: momentum -> velocity + gravity, bit 2: boundary, on the grid
void launch_step_colliders(const DevPtrs &d, int id, float dt, cudaStream_t s);
void launch_apply_colliders(const DevPtrs &d, int id, cudaStream_t s);
// every collider on the grid blocks the preceding gather listed as near one
// (the fused substep: colliders stepped before the gather)
void launch_apply_colliders_listed(const DevPtrs &d, cudaStream_t s);
void launch_grid_update(const DevPtrs &d, int mode, cudaStream_t s);
// fuse_rm: return mapping in G2P; fuse_bin: bin the new positions for the
// next partition
void launch_g2p(const DevPtrs &d, int cur, int fuse_rm, int fuse_bin, cudaStream_t s);
void launch_return_mapping(const DevPtrs &d, int cur, cudaStream_t s);
// vol * Kirchhoff stress of every particle from its current F (or J)
// slots [b0, b1) (b1 < 0: every particle)
void launch_stress(const DevPtrs &d, int cur, cudaStream_t s, long long b0 = 0, long long b1 = -1);

// boundary_grid.cu: the boundary grid of one-scene context from boundary
// points (x, v, m, nrm device arrays, the vertex rows first): mark the
// directory entries whose blocks the points' linear stencils touch (bnd_map
// -1 everywhere before), number them (count in *n_blocks), then, with
// accumulators of 7 doubles per node zeroed, add the points and normalise
// into d.bnd_grid.
void launch_bnd_mark(const DevPtrs &d, const SceneParams &S, const float *x, long long n,
                     cudaStream_t s);
void launch_bnd_index(const DevPtrs &d, int32_t *n_blocks, cudaStream_t s);
void launch_bnd_accumulate(const DevPtrs &d, const SceneParams &S, const float *x, const float *v,
                           const float *m, const float *nrm, long long n_verts, long long n,
                           double *acc, cudaStream_t s);
void launch_bnd_finalize(const DevPtrs &d, const double *acc, int n_blocks, cudaStream_t s);
// ApplyGridBoundaryOnZSGrid on the active grid nodes
void launch_apply_grid_boundary(const DevPtrs &d, cudaStream_t s);

// api.cu: the text mpm_last_error() returns on this thread
void set_last_error(const std::string &msg);

// adjoint.cu: the three adjoint kernels of one substep (an / ap: adjoint
// planes of the next / this state, n particles each)
void launch_g2p_adjoint(const DevPtrs &d, int cur, const float *an, float *ap, float *gmu,
                        float *glam, long long n, cudaStream_t s);
void launch_grid_adjoint(const DevPtrs &d, cudaStream_t s);
// the adjoint kernels' launch attributes on the current device (once per
// context, outside any stream capture)
void configure_adjoint();
// cloth.cu: the same for the cloth's tile kernel
void configure_cloth();
void launch_p2g_adjoint(const DevPtrs &d, int cur, float *ap, float *gmu, float *glam, long long n,
                        cudaStream_t s);

// io.cu
struct IngestSrc {
  const float *x, *v, *C, *F, *J, *m, *vol, *mu, *lam;
  const int32_t *mat;
};
void launch_ingest(const DevPtrs &d, int cur, IngestSrc src, long long b0, long long b1,
                   cudaStream_t s);
void launch_check_materials(const DevPtrs &d, const int32_t *mat, long long n, int n_materials,
                            cudaStream_t s);
// the material check's verdict into the status word (asynchronous upload)
void launch_flag_materials(const DevPtrs &d, cudaStream_t s);
void launch_state_copy(const DevPtrs &d, int cur, float *dst, const float *src, long long n,
                       cudaStream_t s);
void launch_set_lame(const DevPtrs &d, int cur, const float *mu, const float *lam, long long n,
                     cudaStream_t s);
// every particle's mu / lam channels from its material
void launch_lame_from_materials(const DevPtrs &d, int cur, cudaStream_t s);
// writes AoS x(3) v(3) C(9) F(9) J(1) planes-of-arrays in upload order into dst
struct EgestDst {
  float *x, *v, *C, *F, *J;
};
void launch_egest(const DevPtrs &d, int cur, EgestDst dst, long long n, cudaStream_t s);
void launch_egest_channel(const DevPtrs &d, int cur, int ch, float *dst, long long n,
                          cudaStream_t s);

#ifdef __CUDACC__
// scene of a (global) directory index: the last scene whose slice starts at
// or before it
__device__ __forceinline__ int scene_of_dir(const DevPtrs &d, int dir) {
  int lo = 0, hi = d.n_scenes - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (d.scn[mid].dir_off <= dir)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// scene of a particle in upload order
__device__ __forceinline__ int scene_of_particle(const DevPtrs &d, long long i) {
  int lo = 0, hi = d.n_scenes - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (d.scn[mid].p_off <= i)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}
#endif

}  // namespace zsmpm
