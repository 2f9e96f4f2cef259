/*
 * zsmpm -- GB300 (sm_103a) MLS-MPM substep behind a plain C ABI.
 *
 * Drop-in boundary for the CuLagrange MPM nodes of zenustech/zeno.  Every
 * entry point takes plain pointers and sizes and returns an int32 status
 * (mpm_status); mpm_last_error() gives the text of the last failure on the
 * calling thread.  Host pointers are AoS as in zeno's PrimitiveObject / the
 * reference TileVector channels: x, v are n x 3 floats, C and F are n x 3 x 3
 * row-major floats (F[9*i + 3*r + c]).
 *
 * Stage entry points mirror the reference node sequence of one substep
 * (paths relative to the zenustech/zeno tree):
 *   mpm_partition       ZSPartitionForZSParticles  projects/CuLagrange/mpm/MPMPipeline.cu:21-112
 *                       + ExpandZSPartition        projects/CuLagrange/mpm/MPMPipeline.cu:121-231
 *   mpm_grid_clear      ZSGridFromZSPartition      projects/CuLagrange/mpm/MPMPipeline.cu:241-267
 *   mpm_p2g             ZSParticleToZSGrid         projects/CuLagrange/mpm/Transfer.cu:985-1060
 *   mpm_grid_update     UpdateZSGrid               projects/CuLagrange/mpm/MPMPipeline.cu:828-940
 *   mpm_apply_boundary  ApplyBoundaryOnZSGrid      projects/CuLagrange/mpm/Boundary.cu:83-163
 *   mpm_g2p             ZSGridToZSParticle         projects/CuLagrange/mpm/Transfer.cu:1069-1173
 *   mpm_return_mapping  ZSReturnMapping            projects/CuLagrange/mpm/MPMPipeline.cu:953-1138
 * and mpm_substep runs the whole sequence on the device (CUDA graph, no host
 * synchronisation), the additive fused node ZSMPMSubstep.
 *
 * Threading: a context is used by one host thread at a time (the reference
 * graph runs nodes serially, zeno/src/core/Graph.cpp:81-95).  All work is
 * ordered on the context's stream.
 */
#ifndef ZSMPM_H
#define ZSMPM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ZSMPM_ABI_VERSION 2

typedef enum mpm_status {
  MPM_OK = 0,
  MPM_ERR_INVALID = 1,       /* bad argument or unsupported option */
  MPM_ERR_CUDA = 2,          /* CUDA runtime error (text in mpm_last_error) */
  MPM_ERR_CAPACITY = 3,      /* more particles / grid blocks than allocated */
  MPM_ERR_OUT_OF_DOMAIN = 4, /* a particle left the block directory */
  MPM_ERR_CFL = 5,           /* a particle moved too far in one substep */
  MPM_ERR_NAN = 6,           /* non-finite state or inverted element */
  MPM_ERR_TIMEOUT = 7,       /* a bounded device-side wait gave up */
  MPM_ERR_NO_DEVICE = 8,     /* no CUDA device / wrong architecture */
  MPM_ERR_STATE = 9          /* call out of order (e.g. p2g before partition) */
} mpm_status;

/* elastic models: ConfigConstitutiveModel "type" (Generation.cu:40-51:
 * fcr, nhk, stvk, snhk), plus the equation-of-state fluid, which the
 * reference nodes do not expose. */
enum { MPM_FCR = 0, MPM_NHK = 1, MPM_STVK = 2, MPM_EOS = 3, MPM_SNHK = 4 };
/* plasticity: ConfigConstitutiveModel "plasticity" (Generation.cu:66-84):
 * non-associative Drucker-Prager (sand), von Mises, Cam-Clay; each runs on
 * the StVK-Hencky model.  A Cam-Clay particle keeps its hardening state
 * log(Jp) in the J channel (upload it there; the reference starts it at
 * -0.04, Generation.cpp:987). */
enum {
  MPM_PLASTIC_NONE = 0,
  MPM_PLASTIC_NADP = 1,
  MPM_PLASTIC_NAVM = 2,
  MPM_PLASTIC_NACC = 3
};
/* collider types: ToZSBoundary "type" (Generation.cu:1601-1611) */
enum { MPM_BC_NONE = 0, MPM_BC_STICKY = 1, MPM_BC_SLIP = 2, MPM_BC_SEPARATE = 3 };
/* grid transfer schemes: MakeZSGrid "transfer" (Generation.cu:1493-1504) */
enum { MPM_TRANSFER_APIC = 0, MPM_TRANSFER_FLIP = 1, MPM_TRANSFER_AFLIP = 2 };

/* Material of ConfigConstitutiveModel (Generation.cu:18-103): E, nu ->
 * Lame parameters; friction angle in degrees (Drucker-Prager, Cam-Clay);
 * bulk modulus and exponent of the equation-of-state fluid; von Mises yield
 * stress; Cam-Clay cohesion beta and hardening xi (the "params" keys
 * friction_angle, yield_stress, beta, xi of Generation.cu:69-82). */
typedef struct mpm_material {
  int32_t type;
  int32_t plasticity;
  float E, nu, density;
  float friction_angle_deg;
  float bulk, gamma;
  float yield_stress;
  float cc_beta, cc_xi;
} mpm_material;

/* Analytic box collider standing in for ToZSBoundary's level set
 * (Generation.cu:1597-1647): walls of `thickness` cells inside the node-index
 * box [lo, hi] on every axis, static (collider velocity 0). */
typedef struct mpm_boundary {
  int32_t type;
  int32_t thickness;
  int32_t lo[3];
  int32_t hi[3];
} mpm_boundary;

/* Level-set collider: MakeZSLevelSet + ToZSBoundary (Generation.cu:1521-1647),
 * resolved per grid node by ApplyBoundaryOnZSGrid (Boundary.cu:83-163).  The
 * signed distance is a dense grid of dims[0] x dims[1] x dims[2] samples (x
 * fastest) at origin + (i, j, k) * spacing in collider space, interpolated
 * trilinearly; its material velocity is 3 planes of the same layout or one
 * constant.  A node at world position p maps to collider space as
 * X = R^T (p - b) / s; it is inside when s * phi(X) < 0, with normal R grad phi
 * and collider velocity R v(X) + db/dt (Boundary.cu:299-301).  R is the
 * rotation of the yaw (about y), pitch (about x) and roll (about z) angles,
 * applied as R = Ry(yaw) Rx(pitch) Rz(roll).  sticky: v = v_obj; slip: the
 * normal part of v - v_obj is removed; separate: only when it points into
 * the collider (ApplyGridBoundaryOnZSGrid, Boundary.cu:56-67). */
typedef struct mpm_collider_desc {
  int32_t type;             /* MPM_BC_STICKY, MPM_BC_SLIP or MPM_BC_SEPARATE */
  int32_t scene;            /* scene of a batched context, -1: every scene */
  int32_t dims[3];          /* samples per axis, >= 2 */
  float origin[3];          /* collider-space position of sample (0, 0, 0) */
  float spacing;            /* sample spacing, > 0 */
  const float *sdf;         /* dims[0]*dims[1]*dims[2] signed distances (host) */
  const float *velocity;    /* 3 planes of material velocity (host), or NULL */
  float const_velocity[3];  /* the material velocity when velocity == NULL */
  float translation[3];     /* b */
  float translation_rate[3];/* db/dt */
  float scale;              /* s, > 0 */
  float scale_rate;         /* ds/dt */
  float ypr_deg[3];         /* yaw, pitch, roll in degrees */
} mpm_collider_desc;

/* Context = MakeZSGrid + MakeZSPartition + the particle store
 * (Generation.cu:1470-1512, Generation.cpp:690-1145).  The sparse grid of
 * 4^3-cell blocks lives inside a block directory: block coordinates
 * [block_lo, block_lo + block_dims) on each axis; particles must stay at
 * least one block inside it. */
typedef struct mpm_ctx_desc {
  int32_t device;          /* CUDA device ordinal (-1: the calling thread's current device) */
  float dx;                /* MakeZSGrid "dx" */
  int32_t block_lo[3];
  int32_t block_dims[3];
  int64_t max_particles;
  int32_t max_grid_blocks; /* 0: derived from max_particles and the directory */
  int32_t flags;           /* reserved, 0 */
} mpm_ctx_desc;

/* One scene of a batched context: many independent scenes (each its own
 * grid spacing, block directory, boundary and gravity) advanced together,
 * every stage one persistent launch over the blocks of all scenes.  The
 * reference has no batching; a scene is what one ZSGrid + ZSPartition +
 * ZSParticles triple holds there. */
typedef struct mpm_scene_desc {
  float dx;
  int32_t block_lo[3];
  int32_t block_dims[3];
  float gravity[3];
  mpm_boundary boundary;
} mpm_scene_desc;

typedef struct mpm_stats {
  int64_t n_particles;
  int32_t n_particle_blocks; /* non-empty 4^3 particle blocks of the last partition */
  int32_t n_grid_blocks;     /* grid blocks after the 1-ring halo */
  float max_vel_sqr;         /* UpdateZSGrid "MaxVelSqr" of the last grid update */
  int32_t status;            /* first device-side error (mpm_status) since the last clear */
  int64_t substeps;          /* substeps run since the particles were uploaded */
} mpm_stats;

typedef struct mpm_ctx mpm_ctx;

/* version of this ABI (ZSMPM_ABI_VERSION) */
int32_t mpm_abi_version(void);

/* text of the last error on this thread ("" if none) */
const char *mpm_last_error(void);

int32_t mpm_ctx_create(const mpm_ctx_desc *desc, mpm_ctx **out);
int32_t mpm_ctx_destroy(mpm_ctx *ctx);
/* A context of n_scenes independent scenes (mpm_set_boundary and
 * mpm_set_gravity then apply to every scene). */
int32_t mpm_batch_create(int32_t device, const mpm_scene_desc *scenes, int32_t n_scenes,
                         int64_t max_particles, int32_t max_grid_blocks, mpm_ctx **out);

/* Order the context's work after / before other work on `stream`
 * (a cudaStream_t; NULL restores the context's own stream). */
int32_t mpm_set_stream(mpm_ctx *ctx, void *stream);

/* ConfigConstitutiveModel: material table indexed by the per-particle id. */
int32_t mpm_set_materials(mpm_ctx *ctx, const mpm_material *mats, int32_t n);
/* ToZSBoundary + ApplyBoundaryOnZSGrid collider */
int32_t mpm_set_boundary(mpm_ctx *ctx, const mpm_boundary *bc);
/* UpdateZSGrid "gravity" / "Accel" inputs (MPMPipeline.cu:838-846) */
int32_t mpm_set_gravity(mpm_ctx *ctx, float gx, float gy, float gz);
/* Level-set colliders (at most MPM_MAX_COLLIDERS per context), applied in
 * order after the box walls by every boundary application.  mpm_substep
 * advances them by dt at the start of each substep; the stage path advances
 * them only through mpm_step_colliders (StepZSBoundary, Generation.cu:1662-1685:
 * b += db/dt dt, s += ds/dt dt). */
#define MPM_MAX_COLLIDERS 16
int32_t mpm_add_collider(mpm_ctx *ctx, const mpm_collider_desc *desc, int32_t *id);
/* Boundary grid (MakeZSGrid transfer="boundary", Generation.cu:1490-1506)
 * of a one-scene context: ZSBoundaryPrimitiveToZSGrid (Transfer.cu:1532-1623)
 * scatters the points with the linear kernel -- m += W m_p, m v += W m_p v_p
 * and, for the n_eles triangle rows after the n_verts vertex rows,
 * m nrm += W m_p nrm_p -- and UpdateZSGrid's boundary branch
 * (MPMPipeline.cu:899-911) sets v = m v / m, nrm = unit(m nrm) (a node no
 * triangle reached keeps a zero normal where the reference divides by zero).
 * Every substep then applies it as ApplyGridBoundaryOnZSGrid
 * (Boundary.cu:18-69) with `type` (MPM_BC_STICKY / SLIP / SEPARATE) to each
 * grid node of non-zero mass whose boundary node has non-zero mass, after
 * the walls and the level-set colliders.  Host arrays: x, v (NULL: zero),
 * nrm (n_verts + n_eles) x 3, m n_verts + n_eles.  The points do not move;
 * set them again to move the boundary.  The adjoint and the persistent
 * substep kernel take no boundary grid (the substep keeps its kernels). */
int32_t mpm_set_grid_boundary(mpm_ctx *ctx, int32_t type, int64_t n_verts, int64_t n_eles,
                              const float *x, const float *v, const float *m, const float *nrm);
int32_t mpm_clear_grid_boundary(mpm_ctx *ctx);
/* ApplyGridBoundaryOnZSGrid alone, for node graphs (after mpm_grid_update) */
int32_t mpm_apply_grid_boundary(mpm_ctx *ctx);
/* ToBoundaryParticles (Generation.cpp:1154-1460, without sprayed points):
 * host-side conversion of a triangle mesh (n_verts positions, velocities or
 * NULL, n_tris index triples) into boundary points, the vertices first, then
 * one point per triangle.  Vertex: m = the sum over its triangles of a third
 * of the triangle's area in units of dx^2, v its velocity, nrm the unit sum
 * of its triangles' normals.  Triangle: m its area in dx^2, x and v the
 * means of its vertices', nrm = unit(unit(p1 - p0) x unit(p2 - p0)).
 * Outputs hold n_verts + n_tris rows (x, v, nrm 3 floats each). */
int32_t mpm_boundary_points_from_mesh(int64_t n_verts, const float *pos, const float *vel,
                                      int64_t n_tris, const int32_t *tris, float dx, float *x,
                                      float *v, float *m, float *nrm);
int32_t mpm_clear_colliders(mpm_ctx *ctx);
/* id: the collider from mpm_add_collider, or -1 for every collider */
int32_t mpm_step_colliders(mpm_ctx *ctx, int32_t id, float dt);

/* Codimensional cloth: ToZSCloth (Generation.cpp:432-689).  A triangle mesh
 * whose vertices and per-triangle quadrature points both carry mass:
 * element volume = area x dx (the thickness), vertex volume = a third of its
 * triangles'; in-plane model MPM_FCR / MPM_NHK / MPM_STVK with E, nu; the
 * ToZSCloth inputs stiffness_shear (gamma), stiffness_normal (k),
 * friction_angle (fa, used as tan(fa / pi) like ZSReturnMapping,
 * MPMPipeline.cu:1120) and damping_coeff (dc).  One cloth per single-scene
 * context, stepped by every substep entry point with the particles
 * (Transfer.cu:656-842 P2G, 1287-1445 G2P, MPMPipeline.cu:973-1011 return
 * mapping, the latter applied in G2P).  Not differentiable. */
typedef struct mpm_cloth_desc {
  int64_t n_verts;
  const float *x; /* n_verts x 3 */
  const float *v; /* n_verts x 3, or NULL (at rest) */
  int64_t n_tris;
  const int32_t *tris; /* n_tris x 3 vertex indices */
  int32_t model;
  float E, nu, density;
  float stiffness_shear, stiffness_normal, friction_angle, damping_coeff;
  /* MPM_MESH_SURFACE: tris holds n_tris triangles (3 indices each);
   * MPM_MESH_CURVE: n_tris segments (2 indices each), ToZSParticles' curve
   * category (Generation.cpp:837-858): element volume = length dx^2, frame
   * d = [p1 - p0, n1, n2], StVK-Hencky cross-section, p2g_curve
   * (Transfer.cu:174-356), curve G2P (:1445-1513), return_mapping_curve
   * (MPMPipeline.cu:1012-1093) */
  int32_t kind;
} mpm_cloth_desc;
enum { MPM_MESH_SURFACE = 0, MPM_MESH_CURVE = 1 };
int32_t mpm_cloth_create(mpm_ctx *ctx, const mpm_cloth_desc *desc);
/* the cloth's state (NULL skips an array): vertices x, v (n_verts x 3), C
 * (n_verts x 9); elements x, v (n_tris x 3), C, F, d (n_tris x 9, row-major) */
int32_t mpm_cloth_download(mpm_ctx *ctx, float *vx, float *vv, float *vC, float *ex, float *ev,
                           float *eC, float *eF, float *ed);
/* the inverse of mpm_cloth_download (NULL keeps an array): the cloth's state
 * from a checkpoint, in the same layout.  The mesh, masses, rest shapes and
 * springs stay as created. */
int32_t mpm_cloth_upload(mpm_ctx *ctx, const float *vx, const float *vv, const float *vC,
                         const float *ex, const float *ev, const float *eC, const float *eF,
                         const float *ed);
/* ConstructBendingSprings (Generation.cu:563-1001) on the context's triangle
 * cloth, from its current state.  MPM_BENDING_VERTEX: one spring between the
 * two vertices opposite each interior (consistently oriented) edge, k = E /
 * (24 (1 - nu^2)) stiffness (the smaller E, nu of the two triangles), rest
 * length their current distance; every substep's P2G then adds, while a
 * spring is shorter than its rest length, impulses -+ thickness^2 len k
 * (1 - len / rl) dt along it to its two vertices (p2g_vert_bending_force,
 * Transfer.cu:357-400; thickness = the model's dx in the reference).
 * MPM_BENDING_ANGLE: the reference's hinge force is identically zero
 * (Transfer.cu:466-480), so the hinges are only counted.
 * MPM_BENDING_ELEMENT fails: the reference tags those pairs as vertex
 * springs without vertex indices (Generation.cu:779, Transfer.cu:374).
 * *n_out (optional) receives the number of pairs / hinges. */
enum { MPM_BENDING_VERTEX = 0, MPM_BENDING_ELEMENT = 1, MPM_BENDING_ANGLE = 2 };
int32_t mpm_cloth_add_bending(mpm_ctx *ctx, int32_t type, float stiffness, float thickness,
                              int64_t *n_out);

/* Checkpoint / resume (a binary, versioned file): the solver state of a
 * one-scene context -- the particle store in its slot order with the upload
 * ids, the per-particle beta, the level-set colliders' current poses, the
 * cloth's and the trackers' state, the substep count -- written to `path`,
 * and read back into a context made with the same scene, materials,
 * colliders, boundary grid, cloth mesh and trackers, which then steps exactly as the
 * uninterrupted run; it then holds the checkpoint's particle count (read
 * it with mpm_get_stats before a download) (frame caches of the reference: GlobalComm::toDisk,
 * zeno/src/extra/GlobalComm.cpp:37,277; the reference keeps no solver state).
 * Read fails with MPM_ERR_INVALID for another format version, a file of
 * another scene (dx, transfer, collider count, cloth or tracker sizes) or
 * more particles than the context holds.  The block directory is not part of
 * the state (the physics does not depend on it): the reading context's must
 * cover the particles, or grow (mpm_set_auto_regrow). */
int32_t mpm_checkpoint_write(mpm_ctx *ctx, const char *path);
int32_t mpm_checkpoint_read(mpm_ctx *ctx, const char *path);

/* ToTrackerParticles (Generation.cu:105-170): n points (x, optional v,
 * n x 3) that join the partition and are advected in every substep's G2P by
 * the grid velocity (Transfer.cu:1259-1285; the grid's transferred "v" also
 * on FLIP grids), with no P2G.  One tracker set per single-scene context. */
int32_t mpm_trackers_create(mpm_ctx *ctx, int64_t n, const float *x, const float *v);
int32_t mpm_trackers_download(mpm_ctx *ctx, float *x, float *v);

/* ToZSParticles (Generation.cpp:690-1145): host arrays -> device store.
 * NULL optional arrays take the reference defaults: v = 0, C = 0, F = I,
 * J = 1.  mu / lam are the per-particle overrides added by
 * AdjustParticleMaterial (Temp.cu:16-56); both NULL or both set.  Large
 * uploads are copied in pieces that overlap the device-side conversion;
 * page-locked host arrays give the full host-link rate.  A material id out
 * of range fails with MPM_ERR_INVALID and leaves the context without
 * particles. */
int32_t mpm_particles_upload(mpm_ctx *ctx, int64_t n, const float *x, const float *v,
                             const float *C, const float *F, const float *J,
                             const float *m, const float *vol, const int32_t *mat,
                             const float *mu, const float *lam);
/* mpm_particles_upload without the final wait: the copies and the
 * conversion are enqueued on the context's streams and the call returns, so
 * that the upload of one context overlaps the substeps and frame copies of
 * another.  The host arrays must stay unchanged until the next
 * synchronising call on the context (mpm_sync, mpm_get_stats, a download);
 * page-locked arrays keep the copies asynchronous.  A material id out of
 * range is reported by the next mpm_sync as MPM_ERR_INVALID (the substeps
 * clamp it meanwhile). */
int32_t mpm_particles_upload_async(mpm_ctx *ctx, int64_t n, const float *x, const float *v,
                                   const float *C, const float *F, const float *J,
                                   const float *m, const float *vol, const int32_t *mat,
                                   const float *mu, const float *lam);
/* Upload of all scenes of a batched context: scene s owns particles
 * [scene_offsets[s], scene_offsets[s+1]) of the arrays (n_scenes + 1 offsets,
 * from 0 to n); arrays as in mpm_particles_upload. */
int32_t mpm_batch_upload(mpm_ctx *ctx, const int64_t *scene_offsets, int64_t n, const float *x,
                         const float *v, const float *C, const float *F, const float *J,
                         const float *m, const float *vol, const int32_t *mat, const float *mu,
                         const float *lam);
/* AdjustParticleMaterial (Temp.cu:16-56): per-particle Lame parameters
 * (host arrays, upload order) that override the material's mu / lam. */
int32_t mpm_particles_set_lame(mpm_ctx *ctx, const float *mu, const float *lam);
/* UpdatePrimitiveFromZSParticles (Generation.cu:1088-1158): device store ->
 * host arrays in the upload order; NULL skips a channel. */
int32_t mpm_particles_download(mpm_ctx *ctx, float *x, float *v, float *C, float *F, float *J);
/* One per-particle attribute in the upload order, by its channel name in the
 * reference's particle store (Generation.cpp:868-903): get "beta", "vms",
 * "m", "vol", "J", "mu", "lam"; set "beta" (host arrays of n floats).  Get
 * "cloth_beta": the beta of the cloth's vertices (n_verts floats), set by
 * mpm_compute_particle_beta on a triangle cloth (and settable). */
int32_t mpm_particles_get_attr(mpm_ctx *ctx, const char *name, float *values);
int32_t mpm_particles_set_attr(mpm_ctx *ctx, const char *name, const float *values);
/* ComputeVonMises (Generation.cu:1873-1920): the von Mises stress of the
 * StVK-Hencky particles (other models keep their value, 0 at upload) from
 * the principal Cauchy stresses c_i = (2 mu e_i + lam sum e) / J, e_i = ln s_i:
 * vms = sqrt(((c0-c1)^2 + (c1-c2)^2 + (c2-c0)^2) / 2), or log10(vms + 1)
 * with by_log1p (the node's default); read back as the attribute "vms". */
int32_t mpm_compute_von_mises(mpm_ctx *ctx, int32_t by_log1p);
/* UpdatePrimitiveFromZSParticles (Generation.cu:1088-1158) off the critical
 * path: mpm_frame_begin snapshots x and v in upload order on the device (on
 * the context's stream, after the work enqueued so far) and copies the
 * snapshot to x, v (n x 3 floats each; page-locked memory makes the copy
 * asynchronous) on a second stream, so substeps enqueued afterwards overlap
 * the copy; mpm_frame_wait blocks until it has landed.  One frame in flight:
 * a second mpm_frame_begin first waits for the previous one. */
int32_t mpm_frame_begin(mpm_ctx *ctx, float *x, float *v);
int32_t mpm_frame_wait(mpm_ctx *ctx);

/* MakeZSGrid "transfer" of the context's grid: MPM_TRANSFER_APIC (default),
 * MPM_TRANSFER_FLIP or MPM_TRANSFER_AFLIP (the grid gains the vstar channel,
 * Generation.cu:1495-1500; P2G Transfer.cu:891-984, grid update
 * MPMPipeline.cu:878-897, boundary on vstar Boundary.cu:90-101, G2P
 * Transfer.cu:1174-1257).  Allocates the vstar grid on first use. */
int32_t mpm_set_transfer(mpm_ctx *ctx, int32_t scheme);
/* ComputeParticleBeta (Boundary.cu:172-516) on the current particles: with
 * collider = -1 beta = 0.5 where det F > 1 (J for the equation-of-state
 * fluid), else 0; with a collider id, first beta = 0 for particles that at
 * x + dt v are inside that collider and move into it; with -2, first beta = 0
 * for particles whose linear stencil at x + dt v has a boundary-grid node
 * (mpm_set_grid_boundary) of non-zero mass with (v - v_b) . nrm_b < 0
 * (Boundary.cu:172-222; particles only, not a cloth). */
int32_t mpm_compute_particle_beta(mpm_ctx *ctx, float dt, int32_t collider);

/* Stage entry points (one reference node each). */
int32_t mpm_partition(mpm_ctx *ctx);
int32_t mpm_grid_clear(mpm_ctx *ctx);
int32_t mpm_p2g(mpm_ctx *ctx, float dt);
/* max_vel_sqr: host pointer that receives MaxVelSqr (synchronises), or NULL */
int32_t mpm_grid_update(mpm_ctx *ctx, float dt, float *max_vel_sqr);
/* the box walls, then every collider in id order */
int32_t mpm_apply_boundary(mpm_ctx *ctx);
/* one ApplyBoundaryOnZSGrid of a wall boundary (Boundary.cu:83-163 with the
 * domain walls only) or of the level-set collider `id` (-1: every collider);
 * node graphs that apply several boundaries call these in graph order */
int32_t mpm_apply_walls(mpm_ctx *ctx);
int32_t mpm_apply_collider(mpm_ctx *ctx, int32_t id);
int32_t mpm_g2p(mpm_ctx *ctx, float dt);
int32_t mpm_return_mapping(mpm_ctx *ctx);

/* n_substeps full substeps (partition, clear, P2G, grid update + boundary,
 * G2P + return mapping) without host synchronisation. */
int32_t mpm_substep(mpm_ctx *ctx, float dt, int32_t n_substeps);

/* One substep like mpm_substep, launched without the graph and with a CUDA
 * event between kernels; stage_ms[i] receives the device time of stage i
 * (MPM_STAGE_*).  The device-timed counterpart of the host timer zeno wraps
 * around every node's apply() when ZENO_BENCHMARKING is on
 * (zeno/src/core/INode.cpp:141-143). */
enum {
  MPM_STAGE_BIN = 0,         /* binning of uploaded positions (0 when G2P binned them) */
  MPM_STAGE_SCAN = 1,        /* directory scan: grid blocks, particle blocks */
  MPM_STAGE_SCATTER = 2,     /* particles into their blocks */
  MPM_STAGE_SORT = 3,        /* canonical (block, cell, index) order */
  MPM_STAGE_P2G = 4,
  MPM_STAGE_GRID_UPDATE = 5, /* tile gather + grid update + boundary */
  MPM_STAGE_G2P = 6,         /* G2P + return mapping + stress + binning */
  MPM_NUM_STAGES = 7
};
int32_t mpm_substep_timed(mpm_ctx *ctx, float dt, float *stage_ms, int32_t n_stages);

/* ---- differentiable form (no counterpart in the reference) ----
 * A state is MPM_STATE_PLANES device planes of n floats each, one entry per
 * storage slot: x (3), v (3), C (9), F (9), J (1), m, vol, mu, lam, then the
 * material id and the upload index as int32 bit patterns.  The substep keeps
 * the particle store sorted by block (each substep writes the particles at
 * their sorted positions), so the slots of consecutive states are in
 * different orders; the upload-index plane says which particle a slot holds.
 * A state whose upload-index plane is 0..n-1 is in upload order.  An adjoint
 * is MPM_ADJ_PLANES planes (x, v, C, F, J) in the slot order of its state. */
#define MPM_STATE_PLANES 31
#define MPM_ADJ_PLANES 25
/* on = 1: per-particle mu / lam (from the state planes), the grid buffers of
 * the adjoint; required by the calls below.  APIC transfer, no cloth. */
int32_t mpm_set_differentiable(mpm_ctx *ctx, int32_t on);
/* copy the current state to / from caller device memory (checkpoints); a
 * load replaces the particles (n stays the uploaded count) */
int32_t mpm_state_save(mpm_ctx *ctx, float *dst_planes);
int32_t mpm_state_load(mpm_ctx *ctx, const float *src_planes);
/* Adjoint of the substep that advances the current state n with dt: given
 * adj_next, the adjoint of state n+1 (slot order of state n+1), writes
 * adj_prev, the adjoint of state n (slot order of state n), and adds the
 * gradients with respect to every particle's mu and lam to grad_mu /
 * grad_lam (n floats each, device, by upload index).  The state is not
 * advanced.  Fixed-corotated, Neo-Hookean and StVK-Hencky materials, the last
 * with or without the Drucker-Prager projection (sand); not the
 * equation-of-state fluid (MPM_ERR_INVALID). */
int32_t mpm_adjoint_substep(mpm_ctx *ctx, float dt, const float *adj_next, float *adj_prev,
                            float *grad_mu, float *grad_lam);
/* Size of one rollout snapshot: the whole particle store of a state as the
 * substep keeps it (tiled channels, the stored stress included), opaque to
 * the caller: 37 x (n rounded up to a multiple of 32) floats. */
int32_t mpm_snapshot_floats(mpm_ctx *ctx, int64_t *floats);
/* Forward of a rollout with checkpoints, in one call: loads state0 (state
 * planes), runs n_substeps substeps of dt, saving a snapshot of the state
 * before substep k * every into ckpts + k * mpm_snapshot_floats (k = 0 ..
 * ceil(n_substeps / every) - 1), and the final state into final_state
 * (state planes); all device memory.  seg_states (optional, `every`
 * snapshots, the backward's scratch): the substeps of the last segment then
 * keep their states there and their partitions and grids in the context, so
 * that the backward that follows with the same arguments takes that segment
 * back without recomputing it (when the device has room for the partitions;
 * otherwise it recomputes it).  A context with a growing directory
 * (mpm_set_auto_regrow) is refused with MPM_ERR_INVALID, here and in the
 * backward: the backward recomputes from checkpoints that a moved directory
 * may not cover. */
int32_t mpm_rollout_forward(mpm_ctx *ctx, float dt, int32_t n_substeps, int32_t every,
                            const float *state0, float *ckpts, float *seg_states,
                            float *final_state);
/* Backward of that rollout, in one call: adj holds the adjoint of the final
 * state; the segments run last to first, each recomputed from its checkpoint
 * (each substep writing the next state straight into its snapshot in
 * seg_states, `every` snapshots, and its partition and grid into a set the
 * context keeps per substep of a segment, when the device has room) and then
 * taken back through the adjoint substep on each snapshot in place, so that
 * adj ends as the adjoint of state0 (adj_tmp: MPM_ADJ_PLANES x n floats of
 * scratch) and grad_mu / grad_lam (by upload index) gain the gradients of
 * every substep.  The context's own particle store is left unspecified: load
 * a state before stepping it again. */
int32_t mpm_rollout_backward(mpm_ctx *ctx, float dt, int32_t n_substeps, int32_t every,
                             const float *ckpts, float *seg_states, float *adj, float *adj_tmp,
                             float *grad_mu, float *grad_lam);

/* Launch shape of the persistent kernels, chosen by the autotuner
 * (zeno_gb300/autotune.py); 0 fields take the defaults (occupancy maximum for
 * P2G / G2P, 8 CTAs per SM for the sort and the streaming kernels).  The
 * reference launches one thread per particle or node (zpc's cuda policy). */
typedef struct mpm_launch_config {
  int32_t p2g_ctas_per_sm;
  int32_t g2p_ctas_per_sm;
  int32_t sort_ctas_per_sm;
  int32_t stream_ctas_per_sm; /* binning, scatter, grid gather */
  int32_t g2p_threads;        /* 128 (0: 128) */
  int32_t p2g_shape;          /* MPM_P2G_* tile shape of the P2G column scatter */
  int32_t gather_blocks;      /* grid blocks per CTA of the grid gather: 2, 4 or 8 (0: 4) */
} mpm_launch_config;
/* P2G tile shapes: threads per CTA and particles per chunk (the 16 cell
 * columns of a block are scattered by 9-lane slots, three per warp) */
enum {
  MPM_P2G_192x128 = 0, /* default: one cell layer per chunk at 8 particles per cell */
  MPM_P2G_192x192 = 1,
  MPM_P2G_192x96 = 2,
  MPM_P2G_256x128 = 3,
  MPM_P2G_256x256 = 4
};
int32_t mpm_set_launch_config(mpm_ctx *ctx, const mpm_launch_config *cfg);
int32_t mpm_get_launch_config(mpm_ctx *ctx, mpm_launch_config *cfg);

/* Wait for the context's stream; returns the device status word.  With a
 * growing directory (mpm_set_auto_regrow) a particle that left the directory
 * is not an error: the directory grows and the halted substeps run again
 * before this returns. */
int32_t mpm_sync(mpm_ctx *ctx);
int32_t mpm_get_stats(mpm_ctx *ctx, mpm_stats *out);

/* Growing block directory, the counterpart of zpc's hashed block table that
 * grows as particles occupy new blocks (projects/CUDA/Structures.hpp:535,
 * zs::bht<int,3,int,16>; inserts at MPMPipeline.cu:75-84).  The dense
 * directory covers a box of blocks fixed at creation; with this switched on
 * (one-scene contexts only), a particle, cloth vertex or tracker that leaves
 * it halts the substeps queued behind it on the device (the state stays the
 * one after the last complete substep), and the next synchronising call
 * (mpm_sync, mpm_get_stats, a download, any call that reads or changes the
 * particles) recentres and enlarges the directory around the particles -- the
 * box of their blocks plus a quarter of its extent, at least 2 blocks, on
 * every side, up to 2^25 blocks -- reallocates it (and the grid-sized buffers
 * if the new box needs more grid blocks), and runs the halted substeps again.
 * Each enqueued substep then also launches one single-thread gate kernel.
 * Off: such a particle is MPM_ERR_OUT_OF_DOMAIN. */
int32_t mpm_set_auto_regrow(mpm_ctx *ctx, int32_t on);
/* The fused substep as ONE persistent kernel: a cooperative launch of as
 * many CTAs as the SMs hold runs the partition (directory scan, placement,
 * in-block sort), P2G, the grid gather and update with walls and level-set
 * colliders, and G2P with the return mapping, stress and binning, with a
 * grid-wide barrier between the stages -- one launch (plus a 4-byte reset of
 * the barrier counter) per substep instead of seven, captured in the
 * context's graph like them.  Results equal those of the stage kernels to
 * rounding (the G2P and P2G use one fixed tile shape).  Applies to APIC
 * contexts without cloth or trackers; others keep the stage kernels.
 * barrier_limit: spins (of about 100 ns) a CTA waits at a barrier before it
 * gives up: the substep then ends early and the status is MPM_ERR_TIMEOUT
 * (the state is that of an incomplete substep).  Returns MPM_ERR_INVALID if
 * the device cannot launch the kernel cooperatively. */
#define MPM_BARRIER_LIMIT_DEFAULT (1ull << 24)
int32_t mpm_set_persistent(mpm_ctx *ctx, int32_t on, uint64_t barrier_limit);
/* Self-test of the bounded barrier: one CTA per SM waits at a barrier that
 * nothing completes, for barrier_limit spins each; *timed_out is 1 when every
 * wait gave up and reported it (the context's status word is left as it
 * was). */
int32_t mpm_barrier_selftest(mpm_ctx *ctx, uint64_t barrier_limit, int32_t *timed_out);
/* The directory box (in 4^3 blocks) and how many times it has grown. */
int32_t mpm_get_domain(mpm_ctx *ctx, int32_t block_lo[3], int32_t block_dims[3],
                       int32_t *n_regrows);

/* Inspection of the last partition (bit-exact tests): sorted directory
 * index and particle count of every non-empty particle block, the particle
 * permutation (sorted position -> index in upload order) and the sorted
 * directory index of every grid block. */
int32_t mpm_partition_download(mpm_ctx *ctx, int32_t *n_pb, int32_t *pb_dir, int32_t *pb_count,
                               int64_t cap_pb, int32_t *perm, int32_t *n_gb, int32_t *gb_dir,
                               int64_t cap_gb);
/* Grid nodes of the last partition: n_grid_blocks x 64 x (m, v0, v1, v2). */
int32_t mpm_grid_download(mpm_ctx *ctx, float *nodes, int64_t cap_floats);

/* Partition without device allocation.  No counterpart in the reference:
 * it serves callers that cannot call cudaMalloc -- hosts that own all device
 * memory through their own allocator or a fixed budget (an engine or
 * renderer plugin, a framework whose caching allocator a stray cudaMalloc
 * would fragment), or code in a real-time loop where cudaMalloc / cudaFree
 * would synchronise the device.  It bins n particles into 4^3 blocks of the
 * block directory (dx, block_lo, block_dims) and sorts them by
 * (block, cell, index), exactly like mpm_partition.
 *   x_planes  device, 3 * n floats: all x, then all y, then all z
 *   perm      device, n ints: sorted position -> particle index
 *   pb_dir, pb_count  device, cap_pb ints: directory index and particle
 *             count of each non-empty block, in sorted order
 *   n_pb      host: number of non-empty blocks
 *   stream    cudaStream_t (NULL: the default stream); the call waits for it.
 * Its scratch is one file-scope device array of 32 MiB that every GPU loading
 * the library holds until the process exits; sizes above
 * ZSMPM_NOALLOC_MAX_PARTICLES particles or ZSMPM_NOALLOC_MAX_BLOCKS directory
 * blocks are rejected with MPM_ERR_CAPACITY (each block_dims entry is checked
 * on its own, so a product that would overflow is rejected too).  The first
 * call on a device sets up that device's scratch address (make it before any
 * stream capture); the address is not valid after cudaDeviceReset.  If cap_pb
 * is below the number of non-empty blocks the call returns MPM_ERR_CAPACITY
 * with *n_pb set to that number.  Calls share the scratch: calls that overlap
 * on the GPU race. */
#define ZSMPM_NOALLOC_MAX_PARTICLES (1 << 20)
#define ZSMPM_NOALLOC_MAX_BLOCKS (1 << 19)
int32_t mpm_partition_noalloc(const float *x_planes, int64_t n, float dx,
                              const int32_t block_lo[3], const int32_t block_dims[3],
                              int32_t *perm, int32_t *pb_dir, int32_t *pb_count,
                              int64_t cap_pb, int32_t *n_pb, void *stream);

#ifdef __cplusplus
}
#endif
#endif
