// Level-set colliders on grid nodes: ApplyBoundaryOnZSGrid with a level set
// (Boundary.cu:83-163; collider = MakeZSLevelSet + ToZSBoundary,
// Generation.cu:1521-1647).  A node at world position p maps to collider
// space X = R^T (p - b) / s; the signed distance s * phi(X) comes from the
// trilinear interpolant of the collider's sample grid, the normal from that
// interpolant's gradient rotated back (R grad phi / |grad phi|), the collider
// velocity is R v(X) + db/dt (Boundary.cu:299-301).  Inside (phi < 0):
// sticky v = v_obj; slip removes the normal part of v - v_obj; separate does
// so only when it points into the collider (Boundary.cu:56-67).  Outside the
// sample grid a node does not collide.
#pragma once

#include <cuda_runtime.h>

#include "zsmpm_internal.cuh"

namespace zsmpm {

// ApplyBoundaryOnZSGrid with the analytic box walls at node index I: a node
// is in the lower wall of axis a when I_a < lo_a + thickness and in the
// upper wall when I_a > hi_a - thickness; sticky sets v = 0, slip removes the
// wall-normal component, separate removes it only when it points into the
// wall (collider velocity 0, Boundary.cu:56-67).
__device__ __forceinline__ void apply_walls(const SceneParams &S, const int (&I)[3],
                                            float (&vel)[3]) {
  if (S.bc_type == MPM_BC_NONE) return;
  bool any = false;
  const int t = S.bc_thickness;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const bool lower = I[a] < S.bc_lo[a] + t, upper = I[a] > S.bc_hi[a] - t;
    if (!(lower || upper)) continue;
    any = true;
    if (S.bc_type == MPM_BC_SLIP) vel[a] = 0.0f;
    if (S.bc_type == MPM_BC_SEPARATE) {
      if (lower && vel[a] < 0.0f) vel[a] = 0.0f;
      if (upper && vel[a] > 0.0f) vel[a] = 0.0f;
    }
  }
  if (any && S.bc_type == MPM_BC_STICKY) vel[0] = vel[1] = vel[2] = 0.0f;
}

// signed distance (world units), unit normal and collider velocity at p;
// false when p is outside the collider's grid or not inside the collider
__device__ __forceinline__ bool collider_hit(const ColliderDev &c, const float (&p)[3],
                                            float (&n)[3], float (&vo)[3]) {
  float q[3], X[3], u[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) q[a] = (p[a] - c.b[a]) / c.s;
#pragma unroll
  for (int a = 0; a < 3; ++a)  // X = R^T q
    X[a] = c.R[0 * 3 + a] * q[0] + c.R[1 * 3 + a] * q[1] + c.R[2 * 3 + a] * q[2];
  int i0[3];
  float t[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    u[a] = (X[a] - c.origin[a]) * c.inv_h;
    if (!(u[a] >= 0.0f && u[a] <= (float)(c.dims[a] - 1))) return false;
    i0[a] = min((int)floorf(u[a]), c.dims[a] - 2);
    t[a] = u[a] - (float)i0[a];
  }
  const long long sx = 1, sy = c.dims[0], sz = (long long)c.dims[0] * c.dims[1];
  const long long base = i0[0] * sx + i0[1] * sy + i0[2] * sz;
  float f[8];
#pragma unroll
  for (int k = 0; k < 8; ++k)
    f[k] = c.sdf[base + ((k >> 2) & 1) * sx + ((k >> 1) & 1) * sy + (k & 1) * sz];
  // trilinear value and gradient in u (corner k = (kx, ky, kz) bits 2, 1, 0)
  const float tx = t[0], ty = t[1], tz = t[2];
  const float c00 = f[0] + (f[1] - f[0]) * tz, c01 = f[2] + (f[3] - f[2]) * tz;
  const float c10 = f[4] + (f[5] - f[4]) * tz, c11 = f[6] + (f[7] - f[6]) * tz;
  const float c0 = c00 + (c01 - c00) * ty, c1 = c10 + (c11 - c10) * ty;
  const float phi = c0 + (c1 - c0) * tx;
  if (!(phi < 0.0f)) return false;  // s > 0: the sign is phi's
  const float gx = c1 - c0;
  const float gy = (1.0f - tx) * (c01 - c00) + tx * (c11 - c10);
  const float d00 = f[1] - f[0], d01 = f[3] - f[2], d10 = f[5] - f[4], d11 = f[7] - f[6];
  const float gz = (1.0f - tx) * ((1.0f - ty) * d00 + ty * d01) + tx * ((1.0f - ty) * d10 + ty * d11);
  const float g[3] = {gx, gy, gz};  // grad phi up to the positive factor 1/h
  float nr[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) nr[a] = c.R[a * 3 + 0] * g[0] + c.R[a * 3 + 1] * g[1] + c.R[a * 3 + 2] * g[2];
  const float nn = sqrtf(nr[0] * nr[0] + nr[1] * nr[1] + nr[2] * nr[2]);
  const float rn = nn > 0.0f ? 1.0f / nn : 0.0f;
#pragma unroll
  for (int a = 0; a < 3; ++a) n[a] = nr[a] * rn;
  float vl[3] = {c.cvel[0], c.cvel[1], c.cvel[2]};
  if (c.has_vel) {
    const long long plane = sz * c.dims[2];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const float *v = c.vel + a * plane;
      float w[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) w[k] = v[base + ((k >> 2) & 1) * sx + ((k >> 1) & 1) * sy + (k & 1) * sz];
      const float e00 = w[0] + (w[1] - w[0]) * tz, e01 = w[2] + (w[3] - w[2]) * tz;
      const float e10 = w[4] + (w[5] - w[4]) * tz, e11 = w[6] + (w[7] - w[6]) * tz;
      const float e0 = e00 + (e01 - e00) * ty, e1 = e10 + (e11 - e10) * ty;
      vl[a] = e0 + (e1 - e0) * tx;
    }
  }
#pragma unroll
  for (int a = 0; a < 3; ++a)
    vo[a] = c.R[a * 3 + 0] * vl[0] + c.R[a * 3 + 1] * vl[1] + c.R[a * 3 + 2] * vl[2] + c.db[a];
  return true;
}

// one collider on v; returns the action taken: 0 none, 1 sticky, 2 projected
__device__ __forceinline__ int collider_apply(const ColliderDev &c, const float (&p)[3],
                                             float (&v)[3], float (&n)[3]) {
  float vo[3];
  if (!collider_hit(c, p, n, vo)) return 0;
  if (c.type == MPM_BC_STICKY) {
#pragma unroll
    for (int a = 0; a < 3; ++a) v[a] = vo[a];
    return 1;
  }
  const float proj = n[0] * (v[0] - vo[0]) + n[1] * (v[1] - vo[1]) + n[2] * (v[2] - vo[2]);
  if (c.type == MPM_BC_SLIP || (c.type == MPM_BC_SEPARATE && proj < 0.0f)) {
#pragma unroll
    for (int a = 0; a < 3; ++a) v[a] -= proj * n[a];
    return 2;
  }
  return 0;
}

__device__ __forceinline__ bool collider_in_scene(const ColliderDev &c, int scene) {
  return c.scene < 0 || c.scene == scene;
}

// every collider of the scene, in order, on the velocity of the node at p
__device__ __forceinline__ void apply_colliders(const DevPtrs &d, int k0, int k1, int scene,
                                               const float (&p)[3], float (&v)[3]) {
  for (int k = k0; k < k1; ++k) {
    const ColliderDev &c = d.colliders[k];
    if (!collider_in_scene(c, scene) || c.type == MPM_BC_NONE) continue;
    float n[3];
    collider_apply(c, p, v, n);
  }
}

// transpose of apply_colliders: v0 is the velocity the forward pass started
// from, vb the adjoint of its result (replaced by the adjoint of v0).  Each
// collider's action is linear in v on the branch the forward pass took:
// sticky v = v_obj (adjoint 0), projected v - n n^T (v - v_obj) (adjoint
// (I - n n^T) vb).
__device__ __forceinline__ void apply_colliders_adjoint(const DevPtrs &d, int nc, int scene,
                                                       const float (&p)[3], const float (&v0)[3],
                                                       float (&vb)[3]) {
  for (int k = nc - 1; k >= 0; --k) {
    const ColliderDev &c = d.colliders[k];
    if (!collider_in_scene(c, scene) || c.type == MPM_BC_NONE) continue;
    float v[3] = {v0[0], v0[1], v0[2]}, n[3];
    for (int j = 0; j < k; ++j) {  // the forward velocity that reached collider k
      const ColliderDev &cj = d.colliders[j];
      if (!collider_in_scene(cj, scene) || cj.type == MPM_BC_NONE) continue;
      collider_apply(cj, p, v, n);
    }
    const int act = collider_apply(c, p, v, n);
    if (act == 1) {
      vb[0] = vb[1] = vb[2] = 0.0f;
    } else if (act == 2) {
      const float dn = n[0] * vb[0] + n[1] * vb[1] + n[2] * vb[2];
#pragma unroll
      for (int a = 0; a < 3; ++a) vb[a] -= dn * n[a];
    }
  }
}

// does the node box [I0, I0 + 3] dx of a grid block meet the world box of
// one of the colliders k0..k1-1 of the scene
__device__ __forceinline__ bool block_near_colliders(const DevPtrs &d, int k0, int k1, int scene,
                                                     const int (&I0)[3], float dx) {
  const float lo[3] = {(float)I0[0] * dx, (float)I0[1] * dx, (float)I0[2] * dx};
  const float hi[3] = {(float)(I0[0] + 3) * dx, (float)(I0[1] + 3) * dx, (float)(I0[2] + 3) * dx};
  for (int k = k0; k < k1; ++k) {
    const ColliderDev &c = d.colliders[k];
    if (!collider_in_scene(c, scene) || c.type == MPM_BC_NONE) continue;
    if (hi[0] >= c.lo[0] && lo[0] <= c.hi[0] && hi[1] >= c.lo[1] && lo[1] <= c.hi[1] &&
        hi[2] >= c.lo[2] && lo[2] <= c.hi[2])
      return true;
  }
  return false;
}

// the gather's note of a grid block near a collider (its origin I0)
__device__ __forceinline__ void note_near_block(const DevPtrs &d, int nc, int scene,
                                                const int (&I0)[3], float dx, int gb) {
  if (nc > 0 && block_near_colliders(d, 0, nc, scene, I0, dx)) {
    const int i = atomicAdd(&d.cnt->n_near, 1);
    if (i < d.cap_gblocks) d.near_gb[i] = gb;
  }
}

// b += db/dt dt, s += ds/dt dt for every collider (StepZSBoundary)
__device__ __forceinline__ void step_colliders(const DevPtrs &d, int nc, float dt) {
  for (int k = 0; k < nc; ++k) {
    ColliderDev &c = d.colliders[k];
#pragma unroll
    for (int a = 0; a < 3; ++a) c.b[a] += c.db[a] * dt;
    c.s += c.ds * dt;
    collider_world_box(c);
  }
}


}  // namespace zsmpm
