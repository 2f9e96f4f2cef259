// Codimensional cloth (ToZSCloth, Generation.cpp:432-689; Jiang et al. 2017,
// "Anisotropic elastoplasticity for cloth, knit and hair frictional
// contact"): a triangle mesh whose vertices and per-triangle quadrature
// points ("elements") both carry mass on the MPM grid.
//  * mark: the blocks of every vertex and element and their 26 neighbours
//    join the grid blocks of the next partition (no particle blocks);
//  * P2G (p2g_surface, Transfer.cu:656-842): per element, P from the
//    Gram-Schmidt QR of F (in-plane 2x2 model stress, normal compression -k
//    (1 - r33)^2 and shear gamma terms, P += Q A R^-T), the normal-direction
//    force P_c3 (grad W . d_c3)(-vol dt) and the element's mass and momentum
//    on its 27 nodes (type i), the in-plane force as impulses on its three
//    vertices (type ii); then per vertex its mass, momentum and impulse.
//    FLIP grids take the forces in vstar.  No float atomics: the cloth's
//    points are partitioned into blocks of their own, each point writes a
//    scatter record, each cloth block's node tile sums its records in a
//    fixed order, and the tiles join the grid the particle tiles were
//    gathered into (in the grid update of the whole substep);
//  * G2P (Transfer.cu:1287-1445): vertices as damped APIC (C = skew + (1 -
//    dc) sym; or the FLIP-style blend), then elements: damped C, centroid
//    and mean velocity of their vertices, d1 = p1 - p0, d2 = p2 - p0, d3 +=
//    (dt C + dt^2 / 2 C^2) d3, F = d DmInv, and the surface return mapping
//    (MPMPipeline.cu:973-1011) on d = Q R.
// Curves (ToZSParticles' segment meshes, hair) take the same passes with
// p2g_curve (Transfer.cu:174-356: StVK-Hencky cross-section, stretch
// k (r00 - 1), type ii through DmInv00 on the two vertices), the curve G2P
// (:1445-1513: d2, d3 advected with C) and return_mapping_curve
// (MPMPipeline.cu:1012-1093).
#include <cuda_runtime.h>

#include <algorithm>

#include "binning.cuh"
#include "cloth_grid.cuh"
#include "cp_async.cuh"
#include "colliders.cuh"
#include "mpm_math.cuh"
#include "zsmpm_internal.cuh"

namespace zsmpm {
namespace {

// grid node index of node I of scene 0, or -1 outside the grid blocks
__device__ __forceinline__ long long node_of(const DevPtrs &d, const SceneParams &S, int i0, int i1,
                                             int i2) {
  const int b0 = (i0 >> 2) - S.block_lo[0], b1 = (i1 >> 2) - S.block_lo[1],
            b2 = (i2 >> 2) - S.block_lo[2];
  if ((unsigned)b0 >= (unsigned)S.block_dims[0] || (unsigned)b1 >= (unsigned)S.block_dims[1] ||
      (unsigned)b2 >= (unsigned)S.block_dims[2])
    return -1;
  const int gb = d.dir_gb[S.dir_off + (b0 * S.block_dims[1] + b1) * S.block_dims[2] + b2];
  if (gb < 0 || gb >= d.cap_gblocks) return -1;
  return (long long)gb * 64 + (((i0 & 3) << 4) | ((i1 & 3) << 2) | (i2 & 3));
}

// w' of the quadratic B-spline with respect to the particle position (cells)
__device__ __forceinline__ float wgrad(const Stencil1 &s, int o) {
  return o == 0 ? s.f - 1.5f : (o == 1 ? -2.0f * (s.f - 1.0f) : s.f - 0.5f);
}

// Gram-Schmidt QR of the columns of F (row-major): q2 = q0 x q1, R = Q^T F
// upper triangular with a signed r22
__device__ __forceinline__ void gram_schmidt(const float (&F)[9], float (&Q)[9], float (&R)[9]) {
  const float f0[3] = {F[0], F[3], F[6]}, f1[3] = {F[1], F[4], F[7]}, f2[3] = {F[2], F[5], F[8]};
  const float r00 = sqrtf(f0[0] * f0[0] + f0[1] * f0[1] + f0[2] * f0[2]);
  const float q0[3] = {f0[0] / r00, f0[1] / r00, f0[2] / r00};
  const float r01 = q0[0] * f1[0] + q0[1] * f1[1] + q0[2] * f1[2];
  const float u[3] = {f1[0] - r01 * q0[0], f1[1] - r01 * q0[1], f1[2] - r01 * q0[2]};
  const float r11 = sqrtf(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
  const float q1[3] = {u[0] / r11, u[1] / r11, u[2] / r11};
  const float q2[3] = {q0[1] * q1[2] - q0[2] * q1[1], q0[2] * q1[0] - q0[0] * q1[2],
                       q0[0] * q1[1] - q0[1] * q1[0]};
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    Q[i * 3 + 0] = q0[i];
    Q[i * 3 + 1] = q1[i];
    Q[i * 3 + 2] = q2[i];
  }
#pragma unroll
  for (int i = 0; i < 9; ++i) R[i] = 0.0f;
  R[0] = r00;
  R[1] = r01;
  R[2] = q0[0] * f2[0] + q0[1] * f2[1] + q0[2] * f2[2];
  R[4] = r11;
  R[5] = q1[0] * f2[0] + q1[1] * f2[1] + q1[2] * f2[2];
  R[8] = q2[0] * f2[0] + q2[1] * f2[1] + q2[2] * f2[2];
}

// first Piola-Kirchhoff stress of a 2x2 deformation [a b; c d]: fixed
// corotated 2 mu (F - R) + lam (J - 1) cof F (Stomakhin et al. 2012, R the
// closest rotation), Neo-Hookean mu (F - F^-T) + lam ln J F^-T, StVK-Hencky
// F V diag((2 mu e_i + lam sum e) / s_i^2) V^T (Klar et al. 2016)
__device__ __forceinline__ void first_piola_2d(int model, float mu, float lam, const float (&F)[4],
                                               float (&P)[4]) {
  const float a = F[0], b = F[1], c = F[2], d = F[3];
  const float J = a * d - b * c;
  const float cof[4] = {d, -c, -b, a};
  if (model == MPM_FCR) {
    const float p = a + d, q = c - b, rn = rsqrtf(p * p + q * q);
    const float Rr[4] = {p * rn, -q * rn, q * rn, p * rn};
#pragma unroll
    for (int i = 0; i < 4; ++i) P[i] = 2.0f * mu * (F[i] - Rr[i]) + lam * (J - 1.0f) * cof[i];
    return;
  }
  if (model == MPM_NHK) {
    const float rJ = 1.0f / J, l = lam * logf(J);
#pragma unroll
    for (int i = 0; i < 4; ++i) P[i] = mu * (F[i] - cof[i] * rJ) + l * cof[i] * rJ;
    return;
  }
  const float c00 = a * a + c * c, c01 = a * b + c * d, c11 = b * b + d * d;
  const float tr = c00 + c11, det = c00 * c11 - c01 * c01;
  const float disc = sqrtf(fmaxf(0.0f, 0.25f * (c00 - c11) * (c00 - c11) + c01 * c01));
  const float l0 = 0.5f * tr + disc, l1 = det / l0;  // l1 from the product: no cancellation
  float v0[2];
  if (fabsf(c01) > 0.0f) {
    v0[0] = l0 - c11;
    v0[1] = c01;
  } else if (c00 >= c11) {
    v0[0] = 1.0f;
    v0[1] = 0.0f;
  } else {
    v0[0] = 0.0f;
    v0[1] = 1.0f;
  }
  const float nv = rsqrtf(v0[0] * v0[0] + v0[1] * v0[1]);
  v0[0] *= nv;
  v0[1] *= nv;
  const float v1[2] = {-v0[1], v0[0]};
  const float e0 = 0.5f * logf(l0), e1 = 0.5f * logf(l1);
  const float g0 = (2.0f * mu * e0 + lam * (e0 + e1)) / l0, g1 = (2.0f * mu * e1 + lam * (e0 + e1)) / l1;
  const float S[4] = {g0 * v0[0] * v0[0] + g1 * v1[0] * v1[0], g0 * v0[0] * v0[1] + g1 * v1[0] * v1[1],
                      g0 * v0[1] * v0[0] + g1 * v1[1] * v1[0], g0 * v0[1] * v0[1] + g1 * v1[1] * v1[1]};
  P[0] = a * S[0] + b * S[2];
  P[1] = a * S[1] + b * S[3];
  P[2] = c * S[0] + d * S[2];
  P[3] = c * S[1] + d * S[3];
}

__device__ __forceinline__ void matmul3(const float (&A)[9], const float (&B)[9], float (&C)[9]) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      C[i * 3 + j] = A[i * 3 + 0] * B[0 * 3 + j] + A[i * 3 + 1] * B[1 * 3 + j] + A[i * 3 + 2] * B[2 * 3 + j];
}

// the blocks of the cloth's vertices and elements (and their neighbours)
// join the next partition's grid blocks
__global__ void k_cloth_mark(DevPtrs d) {
  if (ZSMPM_HALTED(d)) return;
  const ClothDev &cl = d.cloth;
  const SceneParams &S = d.scn[0];
  const long long n = cl.n_verts + cl.n_eles;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const float *x = i < cl.n_verts ? cl.vx + 3 * i : cl.ex + 3 * (i - cl.n_verts);
    const int key = bin_key(S, x[0], x[1], x[2], &d.cnt->status);
    if (key < 0) continue;
    const int dd = key >> 6, dy = S.block_dims[1], dz = S.block_dims[2];
    for (int a = -1; a <= 1; ++a)
      for (int b = -1; b <= 1; ++b)
        for (int c = -1; c <= 1; ++c) d.dir_flag[dd + (a * dy + b) * dz + c] = 1;
  }
}

// a point's scatter record at its sorted position, as seven 16-byte stores
__device__ __forceinline__ void store_record(const ClothDev &cl, int pos, const float (&r)[kClothRec]) {
  float4 *dst = reinterpret_cast<float4 *>(cl.crec) + (long long)pos * (kClothRec / 4);
#pragma unroll
  for (int k = 0; k < kClothRec / 4; ++k)
    dst[k] = make_float4(r[4 * k], r[4 * k + 1], r[4 * k + 2], r[4 * k + 3]);
}

// each binned point's sorted position (the inverse of the permutation); and
// (one thread) more cloth blocks than the cloth's block capacity -- the
// points of the blocks left out would be lost -- as a capacity error of the
// context, the cloth partition's counters cleared for the next substep
__global__ void k_cloth_inverse(DevPtrs d) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    Counters *cc = d.cloth.ccnt;
    if ((cc->status & ST_CAPACITY) || cc->max_buckets > d.cloth.cap_cblocks)
      atomicOr(&d.cnt->status, ST_CAPACITY);
    cc->status = 0;
    cc->max_buckets = 0;
  }
  if (ZSMPM_HALTED(d)) return;
  const ClothDev &cl = d.cloth;
  const long long nb = min((long long)cl.ccnt->n_binned, cl.n_verts + cl.n_eles);
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < nb;
       s += (long long)gridDim.x * blockDim.x)
    cl.cperm_tmp[cl.cperm[s]] = (int)s;
}

// Element P2G, first part: the element's stress, its scatter record (type i:
// mass, momentum and the normal-direction force on its 27 nodes), and its
// type (ii) impulses on its vertices, one contribution slot each (no
// atomics).
__global__ void k_cloth_elements(DevPtrs d) {
  if (ZSMPM_HALTED(d)) return;
  const ClothDev &cl = d.cloth;
  const float dt = d.prm->dt;
  const bool affine = d.transfer != MPM_TRANSFER_FLIP;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < cl.n_eles;
       e += (long long)gridDim.x * blockDim.x) {
    // every load first, ahead of the stores (which the compiler may not
    // move them past), so that they are in flight together
    float F[9], dm[9], Q[9], R[9], xe[3], ve[3], Ce[9], Di[4];
#pragma unroll
    for (int i = 0; i < 9; ++i) {
      F[i] = cl.eF[9 * e + i];
      dm[i] = cl.ed[9 * e + i];
      Ce[i] = affine ? cl.eC[9 * e + i] : 0.0f;
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      xe[a] = cl.ex[3 * e + a];
      ve[a] = cl.ev[3 * e + a];
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) Di[i] = cl.eDmInv[9 * e + (i < 2 ? i : i + 1)];  // 0 1 3 4
    const float mass = cl.em[e], vol = cl.evol[e];
    const int key = cl.ckey[cl.n_verts + e];
    const int pos = key >= 0 ? cl.cperm_tmp[cl.n_verts + e] : 0;
    gram_schmidt(F, Q, R);
    const bool curve = cl.kind == MPM_MESH_CURVE;
    const float g = cl.gamma;
    float P[9], A[9], Rt[9];
    if (!curve) {
      // surface: the in-plane block, normal compression and shear
      const float R2[4] = {R[0], R[1], R[3], R[4]};
      float P2[4];
      first_piola_2d(cl.model, cl.emu[e], cl.elam[e], R2, P2);
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        P[i * 3 + 0] = Q[i * 3 + 0] * P2[0] + Q[i * 3 + 1] * P2[2];
        P[i * 3 + 1] = Q[i * 3 + 0] * P2[1] + Q[i * 3 + 1] * P2[3];
        P[i * 3 + 2] = 0.0f;
      }
      float gf = 0.0f;
      if (R[8] < 1.0f) {
        const float vv = 1.0f - R[8];
        gf = -cl.k * vv * vv;
      }
      const float Av[9] = {g * R[2] * R[2], g * R[2] * R[5], g * R[2] * R[8],
                           g * R[2] * R[5], g * R[5] * R[5], g * R[5] * R[8],
                           g * R[2] * R[8], g * R[5] * R[8], gf * R[8]};
      const float i00 = 1.0f / R[0], i11 = 1.0f / R[4], i22 = 1.0f / R[8];
      const float i01 = -R[1] * i00 * i11, i12 = -R[5] * i11 * i22;
      const float i02 = (R[1] * R[5] - R[2] * R[4]) * i00 * i11 * i22;
      const float RiT[9] = {i00, 0.0f, 0.0f, i01, i11, 0.0f, i02, i12, i22};  // R^-T
#pragma unroll
      for (int i = 0; i < 9; ++i) {
        A[i] = Av[i];
        Rt[i] = RiT[i];
      }
    } else {
      // curve: StVK-Hencky cross-section block, stretch k (r00 - 1), shear A
      // times the diagonal of R's cofactors over det R (Transfer.cu:204-237)
      const float R2[4] = {R[4], R[5], 0.0f, R[8]};
      float P2[4];
      first_piola_2d(MPM_STVK, cl.emu[e], cl.elam[e], R2, P2);
      const float Pl[9] = {cl.k * (R[0] - 1.0f), 0.0f, 0.0f, 0.0f, P2[0], P2[1], 0.0f, P2[2], P2[3]};
      float QP[9];
      matmul3(Q, Pl, QP);
#pragma unroll
      for (int i = 0; i < 9; ++i) P[i] = QP[i];
      const float rr = R[1] * R[1] + R[2] * R[2];
      const float a01 = (R[4] * R[1] + R[5] * R[2]) * g, a02 = R[8] * R[2] * g;
      const float Av[9] = {rr * g, a01, a02, a01, 0.0f, 0.0f, a02, 0.0f, 0.0f};
      float invJ = R[0] * R[4] * R[8];
      if (invJ != 0.0f) invJ = 1.0f / invJ;
      const float Rit[9] = {R[4] * R[8] * invJ, 0.0f, 0.0f, 0.0f, R[0] * R[8] * invJ, 0.0f,
                            0.0f, 0.0f, R[0] * R[4] * invJ};
#pragma unroll
      for (int i = 0; i < 9; ++i) {
        A[i] = Av[i];
        Rt[i] = Rit[i];
      }
    }
    float QA[9], T[9];
    matmul3(Q, A, QA);
    matmul3(QA, Rt, T);
#pragma unroll
    for (int i = 0; i < 9; ++i) P[i] += T[i];
    if (key >= 0) {  // a binned point: its record at its sorted position
      const float kf = -vol * dt;
      const float dc1[3] = {dm[1], dm[4], dm[7]}, dc2[3] = {dm[2], dm[5], dm[8]};
      float r[kClothRec];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        r[a] = xe[a];
        r[4 + a] = mass * ve[a];
        r[25 + a] = 0.0f;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          r[7 + a * 3 + c] = mass * Ce[a * 3 + c];
          // surface: P_c3 (grad W . d_c3); curve: P_c2 (grad W . d_c2) too
          r[16 + a * 3 + c] =
              kf * ((curve ? P[a * 3 + 1] * dc1[c] : 0.0f) + P[a * 3 + 2] * dc2[c]);
        }
      }
      r[3] = mass;
      store_record(cl, pos, r);
    }
    float4 *ci = cl.cimp + 3 * e;
    if (curve) {  // type (ii): +-vol dt P_c0 DmInv00 on the two vertices
      const float di = Di[0];
      const float4 f = make_float4(vol * dt * P[0] * di, vol * dt * P[3] * di,
                                   vol * dt * P[6] * di, 0.0f);
      ci[0] = f;
      ci[1] = make_float4(-f.x, -f.y, -f.z, 0.0f);
      continue;
    }
    // type (ii): impulses from the in-plane columns of P through DmInv rows
    const float r0[2] = {Di[0], Di[1]};
    const float r1[2] = {Di[2], Di[3]};
#pragma unroll
    for (int vi = 0; vi < 3; ++vi) {
      float Dr0, Dr1, coeff;
      if (vi == 0) {
        Dr0 = r0[0] + r1[0];
        Dr1 = r0[1] + r1[1];
        coeff = vol * dt;
      } else {
        Dr0 = vi == 1 ? r0[0] : r1[0];
        Dr1 = vi == 1 ? r0[1] : r1[1];
        coeff = -vol * dt;
      }
      ci[vi] = make_float4(coeff * (P[0] * Dr0 + P[1] * Dr1), coeff * (P[3] * Dr0 + P[4] * Dr1),
                           coeff * (P[6] * Dr0 + P[7] * Dr1), 0.0f);
    }
  }
}

// Vertex P2G records: the vertex's impulse (its contribution slots -- its
// elements in index order, then its springs -- summed in that order), mass,
// momentum m (v + C (x_i - x_p)) and the impulse (in the momentum, or in
// vstar on FLIP-style grids).
__global__ void k_cloth_vertex_records(DevPtrs d) {
  if (ZSMPM_HALTED(d)) return;
  const ClothDev &cl = d.cloth;
  const bool flip_style = d.transfer != MPM_TRANSFER_APIC, affine = d.transfer != MPM_TRANSFER_FLIP;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < cl.n_verts;
       p += (long long)gridDim.x * blockDim.x) {
    if (cl.ckey[p] < 0) continue;  // not binned: no record
    float imv[3] = {0.f, 0.f, 0.f};
    const int je = cl.vptr[p + 1];
    for (int j = cl.vptr[p]; j < je; j += 4) {  // four slots' loads in flight, summed in order
      int sl[4];
      float4 c[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) sl[u] = j + u < je ? cl.vlist[j + u] : -1;
#pragma unroll
      for (int u = 0; u < 4; ++u) c[u] = sl[u] >= 0 ? cl.cimp[sl[u]] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (sl[u] >= 0) {
          imv[0] += c[u].x;
          imv[1] += c[u].y;
          imv[2] += c[u].z;
        }
    }
    const float mass = cl.vm[p];
    float r[kClothRec];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      r[a] = cl.vx[3 * p + a];
      r[4 + a] = mass * cl.vv[3 * p + a] + (flip_style ? 0.0f : imv[a]);
      r[25 + a] = flip_style ? imv[a] : 0.0f;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        r[7 + a * 3 + c] = affine ? mass * cl.vC[9 * p + a * 3 + c] : 0.0f;
        r[16 + a * 3 + c] = 0.0f;
      }
    }
    r[3] = mass;
    store_record(cl, cl.cperm_tmp[p], r);
  }
}

// vertex bending springs (p2g_vert_bending_force, Transfer.cu:357-400): a
// spring shorter than its rest length pushes its two vertices apart with
// impulses -+ t^2 len k (1 - len / rl) dt along x1 - x0, into the spring's
// two contribution slots.  The reference scatters each with its vertex's
// weights into the grid's "v" (vstar on FLIP grids); adding it to the
// vertex's impulse, which the vertex P2G scatters the same way, gives the
// same sums.
__global__ void k_cloth_bending(DevPtrs d) {
  if (ZSMPM_HALTED(d)) return;
  const ClothDev &cl = d.cloth;
  const float dt = d.prm->dt, t2 = cl.thickness * cl.thickness;
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < cl.n_springs;
       s += (long long)gridDim.x * blockDim.x) {
    const int a0 = cl.sv[2 * s], a1 = cl.sv[2 * s + 1];
    const float dv[3] = {cl.vx[3 * a1] - cl.vx[3 * a0], cl.vx[3 * a1 + 1] - cl.vx[3 * a0 + 1],
                         cl.vx[3 * a1 + 2] - cl.vx[3 * a0 + 2]};
    const float len = sqrtf(dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2]);
    const float rl = cl.srl[s];
    float4 *ci = cl.cimp + 3 * cl.n_eles + 2 * s;
    if (!(len < rl) || len == 0.0f) {
      ci[0] = ci[1] = make_float4(0.f, 0.f, 0.f, 0.f);
      continue;
    }
    const float c = t2 * len * cl.sk[s] * (1.0f - len / rl) * dt / len;
    ci[0] = make_float4(-c * dv[0], -c * dv[1], -c * dv[2], 0.0f);
    ci[1] = make_float4(c * dv[0], c * dv[1], c * dv[2], 0.0f);
  }
}

// The cloth's points into the blocks of their own partition: key (block,
// cell) per point, warp-aggregated counts per block (no grid blocks).
__global__ void k_cloth_bin(DevPtrs d, DevPtrs dc) {
  // the cloth's partition stages (their own counters) stop with the context:
  // run on stale keys, they would place points at stale block offsets
  if (blockIdx.x == 0 && threadIdx.x == 0) dc.cnt->halt = d.cnt->halt;
  if (ZSMPM_HALTED(d)) return;
  const ClothDev &cl = d.cloth;
  const SceneParams &S = d.scn[0];
  const long long np = cl.n_verts + cl.n_eles;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long base = (long long)blockIdx.x * blockDim.x; base < np; base += stride) {
    const long long i = base + threadIdx.x;
    int key = -1;
    if (i < np) {
      const float *x = i < cl.n_verts ? cl.vx + 3 * i : cl.ex + 3 * (i - cl.n_verts);
      key = bin_key(S, x[0], x[1], x[2], &d.cnt->status);
      cl.ckey[i] = key;
    }
    const int dd = key >> 6;  // -1 for none
    const unsigned peers = __match_any_sync(0xffffffffu, dd);
    if (key >= 0 && (int)(threadIdx.x & 31) == __ffs(peers) - 1)
      atomicAdd(&dc.dir_count[dd], __popc(peers));
  }
}


// One CTA per cloth block at a time, in two passes over shared memory.
// First, for each non-empty cell of the block and each of the 27 stencil
// offsets, the sum over the cell's points in sorted order of their
// contributions to the node at that offset (a work item is a cell and the
// offsets (o0, o1, *): nine items per cell, each reading the cell's records
// once); then each of the tile's 216 nodes adds the sums of the non-empty
// cells around it in cell order.  The records lie in sorted order, so a
// block's records are one contiguous run: they are staged in shared memory
// in chunks of kClothStage points with cp.async, the next chunk (of this
// block or the CTA's next one) in flight while the current one computes.  A
// cell that spans two chunks carries its sums over in shared memory, which
// adds in the same order as one pass would.  kFlip: the grids take vstar
// (FLIP-style transfers), seven sums per node instead of four.
constexpr int kClothTileThreads = 224;  // the 216 nodes of pass 2 in one round
constexpr int kClothStage = 192;
constexpr int kClothStageF4 = kClothStage * (kClothRec / 4);
__host__ __device__ constexpr int cloth_tile_smem(bool flip) {
  return (2 * kClothStageF4 * 4 + 64 * 27 * (flip ? 7 : 4)) * (int)sizeof(float);
}

// the quadratic B-spline weight of node o (0, 1, 2) at fractional offset f
// (cells from the stencil's base) as a (f - b)^2 + c, and its derivative
// e (f - b); stencil1 and wgrad give the same values
struct SplineRow {
  float a, b, c, e;
};
__device__ __forceinline__ SplineRow spline_row(int o) {
  return o == 1 ? SplineRow{-1.0f, 1.0f, 0.75f, -2.0f}
                : SplineRow{0.5f, o == 0 ? 1.5f : 0.5f, 0.0f, 1.0f};
}

template <bool kFlip>
__global__ void __launch_bounds__(kClothTileThreads, 3) k_cloth_tiles(DevPtrs d) {
  constexpr int ch = kFlip ? 7 : 4;  // m, momentum (3)[, vstar (3)]
  if (ZSMPM_HALTED(d)) return;
  // two staging buffers of [kClothStage][7] float4, then the sums [64][27][ch]
  extern __shared__ float4 csmem[];
  float *csum = reinterpret_cast<float *>(csmem + 2 * kClothStageF4);
  const ClothDev &cl = d.cloth;
  const SceneParams &S = d.scn[0];
  const float dx = S.dx, inv_dx = S.inv_dx;
  __shared__ int ccount[64], cstart[65], cells[64], n_cells, carry_cell, last_cell;
  __shared__ unsigned long long cmask;  // the block's non-empty cells so far
  const int nb = min(cl.ccnt->n_buckets, cl.cap_cblocks);
  const long long np = cl.n_verts + cl.n_eles;
  const int t = threadIdx.x;
  const float4 *crec4 = reinterpret_cast<const float4 *>(cl.crec);
  auto block_range = [&](int bb, int &st, int &n) {
    st = cl.cbk_start[bb];
    n = (int)max(0ll, min((long long)cl.cbk_count[bb], np - st));
  };
  auto issue = [&](float4 *buf, int first, int len) {
    const float4 *src = crec4 + (long long)first * (kClothRec / 4);
    for (int j = t; j < len * (kClothRec / 4); j += kClothTileThreads) cp_async16(buf + j, src + j);
  };
  int b = blockIdx.x, c0 = 0, start = 0, cnt = 0;
  if (b < nb) {
    block_range(b, start, cnt);
    issue(csmem, start, min(kClothStage, cnt));
  }
  cp_async_commit();
  for (int it = 0; b < nb; ++it) {
    // the next chunk: of this block, or of the CTA's next block
    int nbk = b, nc0 = c0 + kClothStage, nstart = start, ncnt = cnt;
    if (nc0 >= cnt) {
      nbk = b + gridDim.x;
      nc0 = 0;
      if (nbk < nb) block_range(nbk, nstart, ncnt);
    }
    if (nbk < nb) issue(csmem + ((it + 1) & 1) * kClothStageF4, nstart + nc0, min(kClothStage, ncnt - nc0));
    cp_async_commit();
    float4 *rec = csmem + (it & 1) * kClothStageF4;
    const int len = min(kClothStage, cnt - c0);
    if (t < 64) ccount[t] = 0;
    cp_async_wait<1>();  // this chunk's copies (the next chunk's may be pending)
    __syncthreads();
    // the chunk's cell counts, from its points' positions (the key's cell);
    // each position becomes its offset from the stencil base (in cells)
    for (int r = t; r < len; r += kClothTileThreads) {
      float4 x = rec[r * (kClothRec / 4)];
      const int b0 = particle_base(x.x, inv_dx), b1 = particle_base(x.y, inv_dx),
                b2 = particle_base(x.z, inv_dx);
      atomicAdd(&ccount[sort_cell(b0 & 3, b1 & 3, b2 & 3)], 1);
      x.x = __fsub_rn(__fmul_rn(x.x, inv_dx), (float)b0);
      x.y = __fsub_rn(__fmul_rn(x.y, inv_dx), (float)b1);
      x.z = __fsub_rn(__fmul_rn(x.z, inv_dx), (float)b2);
      rec[r * (kClothRec / 4)] = x;
    }
    __syncthreads();
    if (t < 32) {  // exclusive scan of the 64 cell counts (two per lane), the
                   // list of the chunk's non-empty cells in cell order, the
                   // cell continued from the block's previous chunk
      const int a = ccount[2 * t], c = ccount[2 * t + 1];
      int sum = a + c;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, sum, o);
        if (t >= o) sum += u;
      }
      cstart[2 * t] = sum - a - c;
      cstart[2 * t + 1] = sum - c;
      if (t == 31) cstart[64] = sum;
      const int ne = (a > 0) + (c > 0);
      int incl = ne;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, incl, o);
        if (t >= o) incl += u;
      }
      int pos = incl - ne;
      if (a > 0) cells[pos++] = 2 * t;
      if (c > 0) cells[pos] = 2 * t + 1;
      const unsigned lo = __ballot_sync(0xffffffffu, a > 0), hi = __ballot_sync(0xffffffffu, c > 0);
      __syncwarp();
      if (t == 31) {
        unsigned long long bits = 0;
        for (int k = 0; k < 32; ++k)
          bits |= (unsigned long long)((lo >> k) & 1u) << (2 * k) |
                  (unsigned long long)((hi >> k) & 1u) << (2 * k + 1);
        n_cells = incl;
        carry_cell = c0 > 0 ? last_cell : -1;
        cmask = c0 > 0 ? (cmask | bits) : bits;
        if (incl > 0) last_cell = cells[incl - 1];
      }
    }
    __syncthreads();
    // pass 1 over the chunk's cells
    for (int w = t; w < n_cells * 9; w += kClothTileThreads) {
      const int cell = cells[w / 9], o0 = (w % 9) / 3, o1 = w % 3;
      float *dst = csum + (cell * 27 + o0 * 9 + o1 * 3) * ch;
      const bool carry = cell == carry_cell;  // begun in the block's previous chunk
      float acc[3][ch];
#pragma unroll
      for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int h = 0; h < ch; ++h) acc[k][h] = carry ? dst[k * ch + h] : 0.0f;
      const SplineRow r0 = spline_row(o0), r1 = spline_row(o1);
      const float e0 = r0.e * inv_dx, e1 = r1.e * inv_dx, od0 = (float)o0 * dx, od1 = (float)o1 * dx;
      for (int q = cstart[cell]; q < cstart[cell + 1]; ++q) {
        const float4 *r4 = rec + q * (kClothRec / 4);
        // record: f0 f1 f2 m | b0 b1 b2 A00 | A01 A02 A10 A11 | A12 A20 A21 A22 |
        //         Q00 Q01 Q02 Q10 | Q11 Q12 Q20 Q21 | Q22 b20 b21 b22
        const float4 f_m = r4[0], b_a0 = r4[1], a1 = r4[2], a2 = r4[3], q0 = r4[4], q1 = r4[5],
                     q2 = r4[6];
        const float bv[3] = {b_a0.x, b_a0.y, b_a0.z};
        const float A[9] = {b_a0.w, a1.x, a1.y, a1.z, a1.w, a2.x, a2.y, a2.z, a2.w};
        const float Q[9] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w, q2.x};
        const float t0 = f_m.x - r0.b, t1 = f_m.y - r1.b;
        const float w0 = r0.a * t0 * t0 + r0.c, w1 = r1.a * t1 * t1 + r1.c;
        const float w01 = w0 * w1;
        const float g0 = e0 * t0 * w1, g1 = w0 * e1 * t1;  // d(w0 w1)/dx0, d(w0 w1)/dx1
        const float xi0 = od0 - f_m.x * dx, xi1 = od1 - f_m.y * dx, f2 = f_m.z, f2dx = f2 * dx;
        // the parts of the node's momentum and force that do not depend on o2:
        // b + A (xi0, xi1, 0), and Q (g0, g1, 0) and Q_c2 w01 per row
        float mb[3], qg[3], qz[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          mb[c] = bv[c] + A[c * 3] * xi0 + A[c * 3 + 1] * xi1;
          qg[c] = Q[c * 3] * g0 + Q[c * 3 + 1] * g1;
          qz[c] = Q[c * 3 + 2] * w01 * inv_dx;
        }
#pragma unroll
        for (int o2 = 0; o2 < 3; ++o2) {
          const SplineRow r2 = spline_row(o2);
          const float t2 = f2 - r2.b;
          const float w2 = r2.a * t2 * t2 + r2.c, d2 = r2.e * t2;
          const float W = w01 * w2, xi2 = (float)o2 * dx - f2dx;
          float *a = acc[o2];
          a[0] += W * f_m.w;
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            // W (b + A xi) and Q grad W, grad W = (g0 w2, g1 w2, w01 d2 / dx)
            const float mom = W * (mb[c] + A[c * 3 + 2] * xi2);
            const float fo = qg[c] * w2 + qz[c] * d2;
            if constexpr (kFlip) {
              const float b2v = c == 0 ? q2.y : (c == 1 ? q2.z : q2.w);
              a[1 + c] += mom;
              a[4 + c] += fo + W * b2v;
            } else {
              a[1 + c] += mom + fo;
            }
          }
        }
      }
#pragma unroll
      for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int h = 0; h < ch; ++h) dst[k * ch + h] = acc[k][h];
    }
    if (c0 + kClothStage >= cnt) {  // the block's last chunk
      __syncthreads();
      // pass 2: each node adds the sums of the non-empty cells around it,
      // in cell order
      const unsigned long long mask = cmask;
      for (int nd = t; nd < kTileNodes; nd += kClothTileThreads) {
        const int I = nd / 36, J = (nd / 6) % 6, Kz = nd % 6;
        // the cells (bit (l2 << 4) | (l0 << 2) | l1) whose stencil covers the
        // node: l0 in [I - 2, I], l1 in [J - 2, J], l2 in [Kz - 2, Kz]
        auto span = [](int hi) {  // bits lo..hi of 0..3, lo = hi - 2
          const int h = min(hi, 3), l = max(hi - 2, 0);
          return ((2u << h) - 1u) & ~((1u << l) - 1u);
        };
        const unsigned s0 = span(I), s1 = span(J), s2 = span(Kz);
        unsigned long long sel0 = 0, sel2 = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          if ((s0 >> k) & 1u) sel0 |= 0xFull << (4 * k);
          if ((s2 >> k) & 1u) sel2 |= 0xFFFFull << (16 * k);
        }
        const unsigned long long cand =
            mask & (sel0 * 0x0001000100010001ull) & ((unsigned long long)s1 * 0x1111111111111111ull) & sel2;
        float g[ch];
#pragma unroll
        for (int h = 0; h < ch; ++h) g[h] = 0.0f;
        for (unsigned long long m = cand; m; m &= m - 1) {
          const int cell = __ffsll((long long)m) - 1;
          const int o0 = I - ((cell >> 2) & 3), o1 = J - (cell & 3), o2 = Kz - (cell >> 4);
          const float *src = csum + (cell * 27 + o0 * 9 + o1 * 3 + o2) * ch;
#pragma unroll
          for (int h = 0; h < ch; ++h) g[h] += src[h];
        }
        cl.ctile[(long long)b * kTileNodes + nd] = make_float4(g[0], g[1], g[2], g[3]);
        if constexpr (kFlip)
          cl.ctile2[(long long)b * kTileNodes + nd] = make_float4(g[4], g[5], g[6], 0.0f);
      }
    }
    __syncthreads();  // the chunk's buffer, counts and sums are read no more
    b = nbk;
    c0 = nc0;
    start = nstart;
    cnt = ncnt;
  }
  cp_async_wait<0>();
}

// The cloth tiles into the grid the particle tiles were gathered into (the
// stage path; the whole substep adds them in its grid update): a warp takes
// a grid block (two nodes per lane) and skips it when no cloth block covers
// it.
__global__ void k_cloth_grid_add(DevPtrs d) {
  if (ZSMPM_HALTED(d)) return;
  const ClothDev &cl = d.cloth;
  const SceneParams &S = d.scn[0];
  const bool flip_style = d.transfer != MPM_TRANSFER_APIC;
  const int dy = S.block_dims[1], dz = S.block_dims[2];
  const int lane = threadIdx.x & 31;
  const int ngb = min(d.cnt->n_gblocks, d.cap_gblocks);
  const int warps = gridDim.x * (blockDim.x >> 5);
  for (int gb = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); gb < ngb; gb += warps) {
    const int gdir = d.gb_dir[gb];
    const int ldir = gdir - S.dir_off;
    const int bk = cloth_source(cl, S, gdir, ldir / (dz * dy), (ldir / dz) % dy, ldir % dz, lane);
    if (!__any_sync(0xffffffffu, bk >= 0)) continue;
    int src[8];
#pragma unroll
    for (int o = 0; o < 8; ++o) src[o] = __shfl_sync(0xffffffffu, bk, o);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const long long idx = (long long)gb * 64 + lane + 32 * h;
      float4 g = d.grid[idx], u = flip_style ? d.grid2[idx] : make_float4(0.f, 0.f, 0.f, 0.f);
      if (!add_cloth_tiles(cl, src, lane + 32 * h, flip_style, g, u)) continue;
      d.grid[idx] = g;
      if (flip_style) d.grid2[idx] = u;
    }
  }
}

// sum W v, sum W vstar and the damped affine velocity (from v, or vstar on
// FLIP grids) at x
__device__ __forceinline__ void cloth_gather(const DevPtrs &d, const SceneParams &S, const float *x,
                                             bool flip_style, float dc, float (&vel)[3],
                                             float (&vs)[3], float (&Cn)[9]) {
  const float dx = S.dx, inv_dx = S.inv_dx, Dinv = S.Dinv;
  const Stencil1 s0 = stencil1(x[0], inv_dx), s1 = stencil1(x[1], inv_dx), s2 = stencil1(x[2], inv_dx);
#pragma unroll
  for (int a = 0; a < 3; ++a) vel[a] = vs[a] = 0.0f;
#pragma unroll
  for (int i = 0; i < 9; ++i) Cn[i] = 0.0f;
  // the grid blocks of the (up to) 2 x 2 x 2 blocks the stencil touches,
  // looked up first, so that the 27 node loads below are all in flight
  const int l0 = s0.base & 3, l1 = s1.base & 3, l2 = s2.base & 3;
  const int bb0 = (s0.base >> 2) - S.block_lo[0], bb1 = (s1.base >> 2) - S.block_lo[1],
            bb2 = (s2.base >> 2) - S.block_lo[2];
  const int dy = S.block_dims[1], dz = S.block_dims[2];
  int gbk[8];
#pragma unroll
  for (int o = 0; o < 8; ++o) {
    const int a0 = o >> 2, a1 = (o >> 1) & 1, a2 = o & 1;
    const int c0 = bb0 + a0, c1 = bb1 + a1, c2 = bb2 + a2;
    int gb = -1;
    if ((!a0 || l0 >= 2) && (!a1 || l1 >= 2) && (!a2 || l2 >= 2) &&
        (unsigned)c0 < (unsigned)S.block_dims[0] && (unsigned)c1 < (unsigned)dy &&
        (unsigned)c2 < (unsigned)dz) {
      gb = d.dir_gb[S.dir_off + (c0 * dy + c1) * dz + c2];
      if (gb >= d.cap_gblocks) gb = -1;
    }
    gbk[o] = gb;
  }
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const int n0 = l0 + i, n1 = l1 + j, n2 = l2 + k;
        const int h0 = n0 >> 2, h1 = n1 >> 2, h2 = n2 >> 2;
        // (selects, not a runtime index: the lookups stay in registers)
        const int gb = h0 ? (h1 ? (h2 ? gbk[7] : gbk[6]) : (h2 ? gbk[5] : gbk[4]))
                          : (h1 ? (h2 ? gbk[3] : gbk[2]) : (h2 ? gbk[1] : gbk[0]));
        if (gb < 0) {
          atomicOr(&d.cnt->status, ST_STENCIL);
          continue;
        }
        const long long idx = (long long)gb * 64 + (((n0 & 3) << 4) | ((n1 & 3) << 2) | (n2 & 3));
        const float W = s0.w[i] * s1.w[j] * s2.w[k];
        const float xi[3] = {((float)i - s0.f) * dx, ((float)j - s1.f) * dx, ((float)k - s2.f) * dx};
        const float4 g = d.grid[idx];
        const float v[3] = {g.y, g.z, g.w};
        float u[3] = {v[0], v[1], v[2]};
        if (flip_style) {
          const float4 h = d.grid2[idx];
          vs[0] += W * h.x;
          vs[1] += W * h.y;
          vs[2] += W * h.z;
          u[0] = h.x;
          u[1] = h.y;
          u[2] = h.z;
        }
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          vel[a] += W * v[a];
#pragma unroll
          for (int b = 0; b < 3; ++b) Cn[a * 3 + b] += W * Dinv * u[a] * xi[b];
        }
      }
  float D[9];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b)
      D[a * 3 + b] = 0.5f * (Cn[a * 3 + b] - Cn[b * 3 + a]) + (1.0f - dc) * 0.5f * (Cn[a * 3 + b] + Cn[b * 3 + a]);
#pragma unroll
  for (int i = 0; i < 9; ++i) Cn[i] = D[i];
}

// curve element G2P (Transfer.cu:1445-1513) and return_mapping_curve
// (MPMPipeline.cu:1012-1093, alpha = alpha_tangent = cohesion = 0): the
// cross-section's Hencky strain of R's lower-right block is projected to its
// mean when compressive (to zero when already isotropic within eps) and to
// zero otherwise, the block becomes exp(e_mean) times its closest rotation,
// and the shear (r01, r02) is cleared
__device__ __forceinline__ void curve_g2p(const DevPtrs &d, const ClothDev &cl, long long e, int t0,
                                          int t1, float dt, const float (&Cn)[9]) {
  float dm[9], CC[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) dm[i] = cl.ed[9 * e + i];
  matmul3(Cn, Cn, CC);
  float dn[9];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float p0 = cl.vx[3 * t0 + a], p1 = cl.vx[3 * t1 + a];
    cl.ex[3 * e + a] = (p0 + p1) / 2.0f;
    cl.ev[3 * e + a] = (cl.vv[3 * t0 + a] + cl.vv[3 * t1 + a]) / 2.0f;
    dn[a * 3 + 0] = p1 - p0;
#pragma unroll
    for (int c = 1; c < 3; ++c) {
      float s = dm[a * 3 + c];
#pragma unroll
      for (int b = 0; b < 3; ++b) s += (dt * Cn[a * 3 + b] + 0.5f * dt * dt * CC[a * 3 + b]) * dm[b * 3 + c];
      dn[a * 3 + c] = s;
    }
  }
  float Q[9], R[9];
  gram_schmidt(dn, Q, R);
  const float feps = 1.1920928955078125e-07f;
  const float a = R[4], b = R[5], c = R[7], dd = R[8];
  const float E = 0.5f * (a + dd), Fv = 0.5f * (a - dd), G = 0.5f * (c + b), H = 0.5f * (c - b);
  const float q = sqrtf(E * E + H * H), r = sqrtf(Fv * Fv + G * G);
  float e0 = logf(fmaxf(fabsf(q + r), 128.0f * feps)), e1 = logf(fmaxf(fabsf(q - r), 128.0f * feps));
  const float tr = e0 + e1;
  float em = 0.0f;
  if (tr < 0.0f) {
    const float h0 = e0 - 0.5f * tr, h1 = e1 - 0.5f * tr;
    em = sqrtf(h0 * h0 + h1 * h1) < feps ? 0.0f : 0.5f * tr;
  }
  const float sc = expf(em), rn = 1.0f / sqrtf((a + dd) * (a + dd) + (c - b) * (c - b));
  R[4] = sc * (a + dd) * rn;
  R[5] = -sc * (c - b) * rn;
  R[7] = sc * (c - b) * rn;
  R[8] = sc * (a + dd) * rn;
  R[1] = R[2] = 0.0f;
  matmul3(Q, R, dn);
  float Di[9], Fn[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) Di[i] = cl.eDmInv[9 * e + i];
  matmul3(dn, Di, Fn);
  bool finite = true;
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    cl.ed[9 * e + i] = dn[i];
    cl.eF[9 * e + i] = Fn[i];
    finite = finite && isfinite(Fn[i]);
  }
  if (!finite) atomicOr(&d.cnt->status, ST_NAN);
}

__global__ void k_cloth_g2p_verts(DevPtrs d) {
  if (ZSMPM_HALTED(d)) return;
  const ClothDev &cl = d.cloth;
  const SceneParams &S = d.scn[0];
  const float dt = d.prm->dt;
  const bool flip_style = d.transfer != MPM_TRANSFER_APIC;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < cl.n_verts;
       p += (long long)gridDim.x * blockDim.x) {
    float vel[3], vs[3], Cn[9];
    cloth_gather(d, S, cl.vx + 3 * p, flip_style, cl.dc, vel, vs, Cn);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      if (flip_style) {  // x += dt (vstar + beta 0.99 (v0 - v)), Transfer.cu:1320-1331
        const float d0 = cl.vv[3 * p + a] - vel[a];
        const float beta = cl.vbeta[p];
        cl.vv[3 * p + a] = vs[a] + 0.99f * d0;
        cl.vx[3 * p + a] += dt * (vs[a] + beta * 0.99f * d0);
      } else {
        cl.vv[3 * p + a] = vel[a];
        cl.vx[3 * p + a] += vel[a] * dt;
      }
    }
#pragma unroll
    for (int i = 0; i < 9; ++i) cl.vC[9 * p + i] = Cn[i];
  }
}

// element G2P and the surface return mapping (after the vertices moved)
__global__ void k_cloth_g2p_elements(DevPtrs d) {
  if (ZSMPM_HALTED(d)) return;
  const ClothDev &cl = d.cloth;
  const SceneParams &S = d.scn[0];
  const float dt = d.prm->dt;
  const bool flip_style = d.transfer != MPM_TRANSFER_APIC;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < cl.n_eles;
       e += (long long)gridDim.x * blockDim.x) {
    float vel[3], vs[3], Cn[9];
    cloth_gather(d, S, cl.ex + 3 * e, flip_style, cl.dc, vel, vs, Cn);
#pragma unroll
    for (int i = 0; i < 9; ++i) cl.eC[9 * e + i] = Cn[i];
    int t[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) t[i] = min(max(cl.inds[3 * e + i], 0), (int)cl.n_verts - 1);
    if (cl.kind == MPM_MESH_CURVE) {
      curve_g2p(d, cl, e, t[0], t[1], dt, Cn);
      continue;
    }
    float p[3][3], v[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        p[i][a] = cl.vx[3 * t[i] + a];
        v[i][a] = cl.vv[3 * t[i] + a];
      }
    float dm[9], CC[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) dm[i] = cl.ed[9 * e + i];
    matmul3(Cn, Cn, CC);
    const float d3[3] = {dm[2], dm[5], dm[8]};
    float n3[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      float s = d3[a];
#pragma unroll
      for (int b = 0; b < 3; ++b) s += (dt * Cn[a * 3 + b] + 0.5f * dt * dt * CC[a * 3 + b]) * d3[b];
      n3[a] = s;
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      cl.ex[3 * e + a] = (p[0][a] + p[1][a] + p[2][a]) / 3.0f;
      cl.ev[3 * e + a] = (v[0][a] + v[1][a] + v[2][a]) / 3.0f;
      dm[a * 3 + 0] = p[1][a] - p[0][a];
      dm[a * 3 + 1] = p[2][a] - p[0][a];
      dm[a * 3 + 2] = n3[a];
    }
    // return_mapping_surface on d = Q R
    float Q[9], R[9];
    gram_schmidt(dm, Q, R);
    const float gamma = cl.gamma, k = cl.k, fc = cl.fc;
    bool apply = false;
    if (gamma == 0.0f) {
      R[2] = R[5] = 0.0f;
      R[8] = fminf(R[8], 1.0f);
      apply = true;
    } else if (R[8] > 1.0f) {
      R[2] = R[5] = 0.0f;
      R[8] = 1.0f;
      apply = true;
    } else if (R[8] <= 0.0f) {
      R[2] = R[5] = 0.0f;
      R[8] = fmaxf(R[8], -1.0f);
      apply = true;
    } else if (R[8] < 1.0f) {
      const float rr = R[2] * R[2] + R[5] * R[5], r = R[8] - 1.0f, gk = gamma / k;
      const float zz = fc * r * r;
      if (gk * gk * rr - zz * zz > 0.0f) {
        const float scale = zz / (gk * sqrtf(rr));
        R[2] *= scale;
        R[5] *= scale;
        apply = true;
      }
    }
    if (apply) matmul3(Q, R, dm);
    float Di[9], Fn[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) Di[i] = cl.eDmInv[9 * e + i];
    matmul3(dm, Di, Fn);
    bool finite = true;
#pragma unroll
    for (int i = 0; i < 9; ++i) {
      cl.ed[9 * e + i] = dm[i];
      cl.eF[9 * e + i] = Fn[i];
      finite = finite && isfinite(Fn[i]);
    }
    if (!finite) atomicOr(&d.cnt->status, ST_NAN);
  }
}

// ComputeParticleBeta on a triangle cloth (Boundary.cu:316-360, 460-490):
// each element decides 0.2 (normal stretch det F / (|r00 r11 - r10 r01|
// |det DmInv|) of d = QR above 1) or 0 (else, or, with a collider, its
// centroid at x + dt v inside the collider and moving in) for its three
// vertices.  The reference's elements race for shared vertices; here a
// vertex takes its highest-numbered element's value (the outcome of running
// the elements in index order): a first pass finds that element, the second
// writes.
__global__ void k_cloth_beta_owner(DevPtrs d) {
  const ClothDev &cl = d.cloth;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < cl.n_eles;
       e += (long long)gridDim.x * blockDim.x)
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int t = cl.inds[3 * e + k];
      if (t >= 0 && t < cl.n_verts) atomicMax(&cl.vowner[t], (int)e);
    }
}

__global__ void k_cloth_beta(DevPtrs d, float dt, int collider) {
  const ClothDev &cl = d.cloth;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < cl.n_eles;
       e += (long long)gridDim.x * blockDim.x) {
    float value = -1.0f;
    const float v[3] = {cl.ev[3 * e], cl.ev[3 * e + 1], cl.ev[3 * e + 2]};
    if (collider >= 0) {
      const float x[3] = {cl.ex[3 * e] + dt * v[0], cl.ex[3 * e + 1] + dt * v[1],
                          cl.ex[3 * e + 2] + dt * v[2]};
      float nrm[3], vo[3];
      if (collider_hit(d.colliders[collider], x, nrm, vo) &&
          (v[0] - vo[0]) * nrm[0] + (v[1] - vo[1]) * nrm[1] + (v[2] - vo[2]) * nrm[2] < 0.0f)
        value = 0.0f;
    }
    if (value < 0.0f) {
      float F[9], dm[9], Di[9], Q[9], R[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) {
        F[k] = cl.eF[9 * e + k];
        dm[k] = cl.ed[9 * e + k];
        Di[k] = cl.eDmInv[9 * e + k];
      }
      gram_schmidt(dm, Q, R);
      const float Jn = fabsf(R[0] * R[4] - R[3] * R[1]);
      const float J = det3(F) / (Jn * fabsf(det3(Di)));
      value = J > 1.0f ? 0.2f : 0.0f;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int t = cl.inds[3 * e + k];
      if (t >= 0 && t < cl.n_verts && cl.vowner[t] == (int)e) cl.vbeta[t] = value;
    }
  }
}

// tracker points (ToTrackerParticles): their blocks join the partition
__global__ void k_tracker_mark(DevPtrs d) {
  if (ZSMPM_HALTED(d)) return;
  const SceneParams &S = d.scn[0];
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < d.n_trackers;
       i += (long long)gridDim.x * blockDim.x) {
    const float *x = d.tx + 3 * i;
    const int key = bin_key(S, x[0], x[1], x[2], &d.cnt->status);
    if (key < 0) continue;
    const int dd = key >> 6, dy = S.block_dims[1], dz = S.block_dims[2];
    for (int a = -1; a <= 1; ++a)
      for (int b = -1; b <= 1; ++b)
        for (int c = -1; c <= 1; ++c) d.dir_flag[dd + (a * dy + b) * dz + c] = 1;
  }
}

// tracker G2P (Transfer.cu:1259-1285): v = sum W v_i of the grid's "v"
// channel (also on FLIP grids), x += v dt
__global__ void k_tracker_g2p(DevPtrs d) {
  if (ZSMPM_HALTED(d)) return;
  const SceneParams &S = d.scn[0];
  const float dt = d.prm->dt, inv_dx = S.inv_dx;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < d.n_trackers;
       p += (long long)gridDim.x * blockDim.x) {
    float *x = d.tx + 3 * p;
    const Stencil1 s0 = stencil1(x[0], inv_dx), s1 = stencil1(x[1], inv_dx), s2 = stencil1(x[2], inv_dx);
    float vel[3] = {0.0f, 0.0f, 0.0f};
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        for (int k = 0; k < 3; ++k) {
          const long long idx = node_of(d, S, s0.base + i, s1.base + j, s2.base + k);
          if (idx < 0) {
            atomicOr(&d.cnt->status, ST_STENCIL);
            continue;
          }
          const float W = s0.w[i] * s1.w[j] * s2.w[k];
          const float4 g = d.grid[idx];
          vel[0] += W * g.y;
          vel[1] += W * g.z;
          vel[2] += W * g.w;
        }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      d.tv[3 * p + a] = vel[a];
      x[a] += vel[a] * dt;
    }
  }
}

}  // namespace

void launch_tracker_mark(const DevPtrs &d, cudaStream_t s) {
  k_tracker_mark<<<d.num_sms * 4, 256, 0, s>>>(d);
}

void launch_tracker_g2p(const DevPtrs &d, cudaStream_t s) {
  k_tracker_g2p<<<d.num_sms * 4, 128, 0, s>>>(d);
}

void launch_cloth_beta(const DevPtrs &d, float dt, int collider, cudaStream_t s) {
  cudaMemsetAsync(d.cloth.vowner, 0xff, (size_t)d.cloth.n_verts * sizeof(int32_t), s);  // -1
  k_cloth_beta_owner<<<d.num_sms * 4, 128, 0, s>>>(d);
  k_cloth_beta<<<d.num_sms * 4, 128, 0, s>>>(d, dt, collider);
}

void configure_cloth() {
  cudaFuncSetAttribute(k_cloth_tiles<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       cloth_tile_smem(false));
  cudaFuncSetAttribute(k_cloth_tiles<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       cloth_tile_smem(true));
}

void launch_cloth_mark(const DevPtrs &d, cudaStream_t s) {
  k_cloth_mark<<<d.num_sms * 4, 256, 0, s>>>(d);
}

// The cloth's P2G into the grid that holds the particles' sums: its points'
// own partition (the partition's scan, placement and sort on the cloth's
// arrays), the element stresses, records and impulse slots, the vertex
// records with their impulse sums, the tiles, and (add_to_grid; otherwise
// the grid update adds them, mode bit kGridAddCloth) the tiles into the
// grid.  No float atomics: the result does not depend on the order threads
// run in.
void launch_cloth_p2g(const DevPtrs &d, bool add_to_grid, cudaStream_t s) {
  const ClothDev &cl = d.cloth;
  const long long np = cl.n_verts + cl.n_eles;
  DevPtrs dc = d;
  dc.pkey = cl.ckey;
  dc.perm = cl.cperm;
  dc.perm_tmp = cl.cperm_tmp;
  dc.dir_count = cl.cdir_count;
  dc.dir_fill = cl.cdir_fill;
  dc.dir_flag = cl.cdir_flag;
  dc.dir_gb = cl.cdir_gb;
  dc.dir_bk = cl.cdir_bk;
  dc.gb_dir = cl.cgb_dir;
  dc.bk_dir = cl.cbk_dir;
  dc.bk_start = cl.cbk_start;
  dc.bk_count = cl.cbk_count;
  dc.cap_gblocks = cl.cap_cblocks;
  dc.tile_sums = cl.ctile_sums;
  dc.cnt = cl.ccnt;
  dc.prm = cl.cprm;
  dc.cap = np;
  const int g = d.num_sms * 4;
  k_cloth_bin<<<g, 256, 0, s>>>(d, dc);
  launch_scan(dc, s);
  launch_scatter(dc, s);
  launch_bucket_sort(dc, s);
  k_cloth_inverse<<<g, 256, 0, s>>>(d);
  if (cl.n_springs > 0) k_cloth_bending<<<g, 128, 0, s>>>(d);
  k_cloth_elements<<<g, 128, 0, s>>>(d);
  k_cloth_vertex_records<<<g, 128, 0, s>>>(d);
  const bool flip_style = d.transfer != MPM_TRANSFER_APIC;
  if (flip_style)
    k_cloth_tiles<true><<<d.num_sms * 2, kClothTileThreads, cloth_tile_smem(true), s>>>(d);
  else
    k_cloth_tiles<false><<<d.num_sms * 3, kClothTileThreads, cloth_tile_smem(false), s>>>(d);
  if (add_to_grid) k_cloth_grid_add<<<d.num_sms * 8, 256, 0, s>>>(d);
}

// one point per thread up to 8 CTAs per SM: the gathers are latency-bound
static int cloth_g2p_grid(const DevPtrs &d, long long n) {
  return (int)std::max(1ll, std::min<long long>((n + 127) / 128, 8ll * d.num_sms));
}

void launch_cloth_g2p(const DevPtrs &d, cudaStream_t s) {
  k_cloth_g2p_verts<<<cloth_g2p_grid(d, d.cloth.n_verts), 128, 0, s>>>(d);
  k_cloth_g2p_elements<<<cloth_g2p_grid(d, d.cloth.n_eles), 128, 0, s>>>(d);
}

}  // namespace zsmpm
