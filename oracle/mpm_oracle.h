/*
 * CPU oracle for the CuLagrange MLS-MPM substep -- TEST INFRASTRUCTURE ONLY.
 *
 * This library is the checker, never the product: only tests/, the smoke
 * check in __graft_entry__.py and the cpu_baseline / reference legs of
 * bench.py may load it.  The GPU product path never links or calls it.
 *
 * It restates, on the CPU, the node bodies of the reference substep:
 *   ZSPartitionForZSParticles   projects/CuLagrange/mpm/MPMPipeline.cu:73-84
 *   ExpandZSPartition           projects/CuLagrange/mpm/MPMPipeline.cu:131-199
 *   ZSGridFromZSPartition       projects/CuLagrange/mpm/MPMPipeline.cu:256-262
 *   ZSParticleToZSGrid (APIC)   projects/CuLagrange/mpm/Transfer.cu:843-890
 *   UpdateZSGrid (APIC)         projects/CuLagrange/mpm/MPMPipeline.cu:852-877
 *   ApplyBoundaryOnZSGrid       projects/CuLagrange/mpm/Boundary.cu:56-67,105-116
 *   ZSGridToZSParticle (APIC)   projects/CuLagrange/mpm/Transfer.cu:1137-1173
 *   ZSReturnMapping             projects/CuLagrange/mpm/MPMPipeline.cu:953-972
 *   FLIP / AFLIP transfers      projects/CuLagrange/mpm/Transfer.cu:891-984 (P2G),
 *                               MPMPipeline.cu:878-897 (grid update),
 *                               Transfer.cu:1174-1257 (G2P)
 *   ComputeParticleBeta         projects/CuLagrange/mpm/Boundary.cu:172-516
 *                               (no-boundary and level-set forms)
 * The arithmetic the reference delegates to zpc (absent from the reference
 * tree; submodule projects/CUDA/zpc, pinned commit unknown) is restated from
 * the published methods named at each function in mpm_oracle.cpp.
 *
 * Parity status: the reference ships no MPM tests, golden vectors or
 * fixtures and its substep cannot be compiled or run without zpc, so this
 * oracle is pinned only by known-answer tests of its own (rigid motion,
 * free fall, affine reproduction, zero stress at rest, lattice partitions):
 * parity unpinned against reference outputs.
 */
#ifndef ZSMPM_ORACLE_H
#define ZSMPM_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_FCR = 0, ORC_NHK = 1, ORC_STVK = 2, ORC_EOS = 3, ORC_SNHK = 4 };
enum { ORC_PLASTIC_NONE = 0, ORC_PLASTIC_NADP = 1, ORC_PLASTIC_NAVM = 2, ORC_PLASTIC_NACC = 3 };
enum { ORC_BC_NONE = 0, ORC_BC_STICKY = 1, ORC_BC_SLIP = 2, ORC_BC_SEPARATE = 3 };
/* MakeZSGrid "transfer" (Generation.cu:1493-1504) */
enum { ORC_TRANSFER_APIC = 0, ORC_TRANSFER_FLIP = 1, ORC_TRANSFER_AFLIP = 2 };

enum {
  ORC_OK = 0,
  ORC_ERR_INVALID = 1,
  ORC_ERR_OUT_OF_DOMAIN = 4,
  ORC_ERR_NAN = 6,
  ORC_ERR_CAPACITY = 3
};

typedef struct orc_material {
  int32_t type;        /* ORC_FCR / ORC_NHK / ORC_STVK / ORC_EOS / ORC_SNHK */
  int32_t plasticity;  /* ORC_PLASTIC_NONE / _NADP / _NAVM / _NACC */
  float E, nu, density;
  float friction_angle_deg; /* Drucker-Prager / Cam-Clay friction angle */
  float bulk, gamma;        /* equation-of-state fluid */
  float yield_stress;       /* von Mises */
  float cc_beta, cc_xi;     /* Cam-Clay cohesion and hardening; log(Jp) in J */
} orc_material;

/* Level-set collider (MakeZSLevelSet + ToZSBoundary, Generation.cu:1521-1647;
 * resolved per node as in ApplyBoundaryOnZSGrid, Boundary.cu:83-163): dense
 * signed distances sdf[i + dims0 (j + dims1 k)] at origin + (i, j, k) spacing
 * in collider space; X = R^T (p - b) / s with R = Ry(yaw) Rx(pitch) Rz(roll). */
typedef struct orc_collider {
  int32_t type;   /* ORC_BC_STICKY / SLIP / SEPARATE */
  int32_t dims[3];
  float origin[3];
  float spacing;
  const float *sdf;
  const float *velocity; /* 3 planes or NULL */
  float const_velocity[3];
  float translation[3];
  float translation_rate[3];
  float scale;
  float scale_rate;
  float ypr_deg[3];
} orc_collider;

/* Codimensional cloth (ToZSCloth, Generation.cpp:432-689): a triangle mesh
 * whose vertices and per-triangle quadrature points ("elements") both carry
 * mass; element state d = [d1 d2 d3] (two edges and the normal direction),
 * DmInv, F = d DmInv; stepped by the surface branches of the transfer nodes
 * (Transfer.cu:656-842 P2G, 1287-1445 G2P) and ZSReturnMapping
 * (MPMPipeline.cu:973-1011).  Arrays are in/out, row-major 3x3. */
enum { ORC_MESH_SURFACE = 0, ORC_MESH_CURVE = 1 };
typedef struct orc_cloth {
  int32_t kind;           /* ORC_MESH_SURFACE (triangles) or ORC_MESH_CURVE (segments) */
  int32_t model;          /* ORC_FCR / ORC_NHK / ORC_STVK: the in-plane model
                             (curves: StVK-Hencky with the model's mu, lam) */
  float gamma, k, fa, dc; /* ToZSCloth stiffness_shear, stiffness_normal,
                             friction_angle, damping_coeff */
  int64_t n_verts, n_eles;
  double *vx, *vv, *vC;   /* vertices: x (3), v (3), C (9) */
  double *vm;             /* vertex mass */
  double *ex, *ev, *eC, *eF, *ed, *eDmInv; /* elements */
  double *em, *evol, *emu, *elam;
  int32_t *inds;          /* 3 vertex indices per element (curves: the first 2) */
  /* vertex bending springs (ConstructBendingSprings "vertex"): n_springs
   * vertex pairs, stiffness and rest length each; thickness = the model's dx */
  int64_t n_springs;
  const int32_t *spring_v;
  const double *spring_k, *spring_rl;
  double thickness;
  /* ComputeParticleBeta on the surface (NULL: 0): per-vertex beta of the
   * FLIP-style vertex position update x += dt (vstar + beta 0.99 (v0 - v)) */
  double *vbeta;
} orc_cloth;

/* Tracker particles (ToTrackerParticles, Generation.cu:105-170): points
 * that join the partition and are advected by the grid velocity in G2P
 * (Transfer.cu:1259-1285: v = sum W v_i of the grid's "v", x += v dt), with
 * no P2G. */
typedef struct orc_trackers {
  int64_t n;
  double *x, *v; /* n x 3, in/out */
} orc_trackers;

/* Boundary grid (MakeZSGrid transfer="boundary", Generation.cu:1490-1506)
 * filled from boundary points by ZSBoundaryPrimitiveToZSGrid
 * (Transfer.cu:1532-1623: linear kernel, m += W m_p, mv += W m_p v_p, and for
 * the element rows m nrm += W m_p nrm_p), normalised by UpdateZSGrid's
 * boundary branch (MPMPipeline.cu:899-911: v = mv / m, nrm = unit(nrm / m)),
 * and applied to the velocity of every grid node whose mass is non-zero in
 * both grids by ApplyGridBoundaryOnZSGrid (Boundary.cu:18-69), after the
 * walls and the level-set colliders.  Rows 0 .. n_verts-1 are the mesh's
 * vertices (no normal), the n_eles rows after them its triangles. */
typedef struct orc_grid_boundary {
  int32_t type; /* ORC_BC_STICKY / SLIP / SEPARATE */
  int64_t n_verts, n_eles;
  const float *x, *v; /* (n_verts + n_eles) x 3 */
  const float *m;     /* n_verts + n_eles */
  const float *nrm;   /* (n_verts + n_eles) x 3; read for the element rows */
} orc_grid_boundary;

typedef struct orc_scene {
  float dx;
  float gravity[3];
  int32_t block_lo[3];   /* block coordinates (units of 4 cells) of directory origin */
  int32_t block_dims[3]; /* directory extent in blocks */
  int32_t bc_type;       /* ORC_BC_* */
  int32_t bc_thickness;  /* wall thickness in cells */
  int32_t bc_lo[3];      /* node index of the lower domain face */
  int32_t bc_hi[3];      /* node index of the upper domain face */
  int32_t n_materials;
  const orc_material *materials;
  int32_t n_colliders;
  const orc_collider *colliders;
  int32_t collider_autostep; /* 1: advance colliders by dt at the start of each substep */
  int32_t transfer;          /* ORC_TRANSFER_* */
  orc_cloth *cloth;          /* NULL, or one cloth stepped with the particles (FP64 only) */
  orc_trackers *trackers;    /* NULL, or tracker points (FP64 only) */
  const orc_grid_boundary *grid_boundary; /* NULL, or the boundary grid's points */
} orc_scene;

typedef struct orc_stats {
  double max_vel_sqr;
  int64_t n_pblocks;
  int64_t n_gblocks;
  int32_t status;
} orc_stats;

/* Partition of positions x (n x 3, float) into 4^3 blocks.
 * Outputs (caller allocated, capacities given):
 *   pb_dir[cap_pb]   sorted directory index of each non-empty particle block
 *   pb_count[cap_pb] particles per block
 *   perm[n]          stable sort of particle indices by (block, cell, index)
 *   gb_dir[cap_gb]   sorted directory index of each grid block (1-ring halo)
 */
int32_t orc_partition(const orc_scene *scene, int64_t n, const float *x,
                      int64_t cap_pb, int32_t *n_pb, int32_t *pb_dir,
                      int32_t *pb_count, int64_t *perm, int64_t cap_gb,
                      int32_t *n_gb, int32_t *gb_dir);

/* nsteps substeps in double precision, order-stable scatter (the oracle).
 * beta: the particles' AFLIP positional-adjustment factor (NULL: 0). */
int32_t orc_run_f64(const orc_scene *scene, int64_t n, double *x, double *v,
                    double *C, double *F, double *J, const double *m,
                    const double *vol, const int32_t *mat, const double *mu,
                    const double *lam, const double *beta, double dt,
                    int32_t nsteps, int32_t nthreads, orc_stats *stats);

/* ComputeParticleBeta on a triangle cloth (Boundary.cu:316-360, 460-490):
 * per element in index order (a vertex keeps the value of the last element
 * that has it), beta 0 for its vertices when, with collider >= 0, its
 * centroid at x + dt v is inside the collider and moving into it; else 0.2
 * when the normal stretch det F / (|r00 r11 - r10 r01| |det DmInv|) of d =
 * QR exceeds 1, else 0.  Writes cl->vbeta (n_verts). */
int32_t orc_cloth_beta_f64(const orc_scene *scene, orc_cloth *cl, double dt, int32_t collider);

/* Same substeps in single precision with OpenMP (the CPU baseline). */
int32_t orc_run_f32(const orc_scene *scene, int64_t n, float *x, float *v,
                    float *C, float *F, float *J, const float *m,
                    const float *vol, const int32_t *mat, const float *mu,
                    const float *lam, const float *beta, float dt,
                    int32_t nsteps, int32_t nthreads, orc_stats *stats);

/* ComputeParticleBeta (Boundary.cu:172-516) in double precision: with
 * collider < 0 the criterion of the node without a boundary (beta = 0.5 where
 * det F > 1, else 0; J for the equation-of-state fluid); with the index of
 * one of the scene's colliders, first the level-set test at x + dt v
 * (beta = 0 where the particle moves into the collider); with -2, first the
 * test against the scene's boundary grid: beta = 0 where a node of the
 * linear stencil at x + dt v has boundary mass and (v - v_b) . nrm_b < 0. */
/* ComputeVonMises (Generation.cu:1873-1920) in double: for the StVK-Hencky
 * particles vms = sqrt(sum_d (c_d - c_{d+1})^2 / 2) of the principal Cauchy
 * stresses c_i = (2 mu e_i + lam sum e) / J, e_i = ln s_i (s the singular
 * values of F), log10(vms + 1) with by_log1p; other particles keep vms. */
int32_t orc_von_mises_f64(const orc_scene *scene, int64_t n, const double *F,
                          const int32_t *mat, int32_t by_log1p, double *vms);

int32_t orc_particle_beta_f64(const orc_scene *scene, int64_t n, const double *x,
                              const double *v, const double *F, const double *J,
                              const int32_t *mat, double dt, int32_t collider,
                              double *beta);

/* Symmetric 3x3 eigen-decomposition used by the constitutive models
 * (exported for known-answer tests): A = Q diag(w) Q^T, Q column-major
 * eigenvectors stored row-major as Q[i*3+j] = Q_ij. */
void orc_sym_eig3(const double *A, double *w, double *Q);

/* Kirchhoff stress tau = P F^T of one material at deformation F (or J for
 * the equation-of-state fluid) -- exported for known-answer tests. */
int32_t orc_kirchhoff(const orc_material *mat, const double *F, double J,
                      double *tau);

/* Drucker-Prager return mapping of F in place; returns 1 if projected. */
int32_t orc_project_dp(const orc_material *mat, double *F);
/* Von Mises / Cam-Clay return mapping of F (and Cam-Clay's log(Jp)) in
 * place; returns 1 if projected, 0 if inside, -1 degenerate, -2 if the
 * material has neither. */
int32_t orc_project_hencky(const orc_material *mat, double *F, double *logJp);

/* ToZSCloth's set-up of the vertex and element arrays of `out` (allocated
 * by the caller for n_verts / n_tris) from a mesh: positions x, optional
 * velocities v (n_verts x 3 floats), triangles tris (n_tris x 3), the
 * model's dx (thickness), density and E, nu. */
int32_t orc_cloth_init_f64(int64_t n_verts, const float *x, const float *v, int64_t n_tris,
                           const int32_t *tris, float dx, float density, float E, float nu,
                           orc_cloth *out);
/* ToZSParticles' set-up of a curve mesh (Generation.cpp:837-858, 1096-1112):
 * segments (n_segs x 2); element volume = length dx^2, d = [p1 - p0, n1, n2]
 * with n1 a unit vector orthogonal to the segment (Hughes-Moller choice) and
 * n2 = normalize(d1 x n1); D* = diag(|d1|, 1, 1). */
int32_t orc_curve_init_f64(int64_t n_verts, const float *x, const float *v, int64_t n_segs,
                           const int32_t *segs, float dx, float density, float E, float nu,
                           orc_cloth *out);

int32_t orc_max_threads(void);

/* ToBoundaryParticles (Generation.cpp:1154-1460) without sprayed points: a
 * triangle mesh (n_verts positions, velocities or NULL, n_tris index
 * triples) to boundary points, the vertices first, then one point per
 * triangle.  Vertex: m = the sum over its triangles of a third of the
 * triangle's area in units of dx^2, v its velocity, nrm the unit sum of its
 * triangles' normals.  Triangle: m its area in dx^2, x and v the means of its
 * vertices', nrm = unit(unit(p1 - p0) x unit(p2 - p0)).  Outputs hold
 * n_verts + n_tris rows. */
int32_t orc_boundary_points_from_mesh(int64_t n_verts, const float *pos, const float *vel,
                                      int64_t n_tris, const int32_t *tris, float dx,
                                      double *x, double *v, double *m, double *nrm);

#ifdef __cplusplus
}
#endif
#endif
