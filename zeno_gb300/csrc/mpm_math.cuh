// Device math of the substep: quadratic B-spline stencil, symmetric 3x3
// eigen-decomposition, Kirchhoff stresses and the Drucker-Prager return
// mapping.  The reference takes these from zpc (absent from the reference
// tree); each routine here is written from the published method it names.
//
// All strain measures are formed from G = F - I, which is exact in FP32 for
// the diagonal (Sterbenz) and unchanged off the diagonal, so that
// E = B - I = G G^T + G + G^T and J - 1 carry small strains without the
// cancellation of forming B = F F^T and subtracting I.
#pragma once

#include <cuda_runtime.h>

#include "zsmpm_internal.cuh"

namespace zsmpm {

struct Sym3 {
  float xx, yy, zz, xy, xz, yz;
};

// One Jacobi rotation on the (p, q) plane, r the third index (Golub & Van
// Loan, Matrix Computations, sym.schur2: theta = (a_qq - a_pp) / (2 a_pq),
// t = sgn(theta) / (|theta| + sqrt(theta^2 + 1)), c = 1/sqrt(1+t^2), s = t c;
// A <- J^T A J, Q <- Q J with J_pp = J_qq = c, J_pq = s, J_qp = -s).
__device__ __forceinline__ void jacobi_rot(float &app, float &aqq, float &apq, float &arp,
                                           float &arq, float (&Q)[9], int p, int q) {
  if (fabsf(apq) <= 1e-30f) return;
  // The rotation only has to be orthogonal: c and s come from one rsqrt, so
  // c^2 + s^2 = 1 to rounding even though t is computed with approximate
  // division; the residual of a_pq is removed by the next sweep.
  const float theta = __fdividef(0.5f * (aqq - app), apq);
  const float at = fabsf(theta);
  float t;
  if (at < 1e15f) {
    const float h = fmaf(theta, theta, 1.0f);
    t = __fdividef(1.0f, at + h * rsqrtf(h));
  } else {
    t = __fdividef(0.5f, at);
  }
  t = copysignf(t, theta);
  const float c = rsqrtf(fmaf(t, t, 1.0f));
  const float s = t * c;
  app = fmaf(-t, apq, app);
  aqq = fmaf(t, apq, aqq);
  apq = 0.0f;
  const float rp = arp, rq = arq;
  arp = c * rp - s * rq;
  arq = s * rp + c * rq;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float qp = Q[k * 3 + p], qq = Q[k * 3 + q];
    Q[k * 3 + p] = c * qp - s * qq;
    Q[k * 3 + q] = s * qp + c * qq;
  }
}

// Cyclic Jacobi on a symmetric 3x3 matrix: A = Q diag(w) Q^T.
__device__ __forceinline__ void sym_eig3(Sym3 a, float (&w)[3], float (&Q)[9]) {
#pragma unroll
  for (int i = 0; i < 9; ++i) Q[i] = (i % 4 == 0) ? 1.0f : 0.0f;
  float d0 = a.xx, d1 = a.yy, d2 = a.zz, o01 = a.xy, o02 = a.xz, o12 = a.yz;
#pragma unroll 1
  for (int sweep = 0; sweep < 5; ++sweep) {
    const float off = o01 * o01 + o02 * o02 + o12 * o12;
    const float dia = d0 * d0 + d1 * d1 + d2 * d2;
    if (off <= 1e-14f * dia || off == 0.0f) break;
    jacobi_rot(d0, d1, o01, o02, o12, Q, 0, 1);  // r = 2: a_r0 = o02, a_r1 = o12
    jacobi_rot(d0, d2, o02, o01, o12, Q, 0, 2);  // r = 1: a_r0 = o01, a_r2 = o12
    jacobi_rot(d1, d2, o12, o01, o02, Q, 1, 2);  // r = 0: a_r1 = o01, a_r2 = o02
  }
  w[0] = d0;
  w[1] = d1;
  w[2] = d2;
}

// Eigenvalues of a symmetric 3x3 matrix from its characteristic cubic in
// trigonometric form (O. K. Smith, "Eigenvalues of a symmetric 3x3 matrix",
// Comm. ACM 4(4):168, 1961): with q = tr(A)/3, p^2 = tr((A - qI)^2)/6 and
// r = det((A - qI)/p)/2, the roots are q + 2p cos(phi + 2 pi k/3),
// phi = acos(r)/3.  Each eigenvalue is accurate to rounding of p, which is all
// the symmetric functions of the eigenvalues below need.
__device__ __forceinline__ void sym_eigvals3(const Sym3 &a, float (&w)[3]) {
  const float q = (a.xx + a.yy + a.zz) * (1.0f / 3.0f);
  const float b0 = a.xx - q, b1 = a.yy - q, b2 = a.zz - q;
  const float off = a.xy * a.xy + a.xz * a.xz + a.yz * a.yz;
  const float p2 = (b0 * b0 + b1 * b1 + b2 * b2 + 2.0f * off) * (1.0f / 6.0f);
  if (!(p2 > 0.0f)) {
    w[0] = w[1] = w[2] = q;
    return;
  }
  const float p = sqrtf(p2);
  const float det = b0 * (b1 * b2 - a.yz * a.yz) - a.xy * (a.xy * b2 - a.yz * a.xz) +
                    a.xz * (a.xy * a.yz - b1 * a.xz);
  const float r = fminf(fmaxf(det / (2.0f * p2 * p), -1.0f), 1.0f);
  const float phi = acosf(r) * (1.0f / 3.0f);
  float sn, cs;
  __sincosf(phi, &sn, &cs);  // phi in [0, pi/3]
  w[0] = fmaf(2.0f * p, cs, q);
  w[2] = fmaf(2.0f * p, -0.5f * cs - 0.8660254037844386f * sn, q);  // cos(phi + 2pi/3)
  w[1] = 3.0f * q - w[0] - w[2];
}

// Fixed-corotated Kirchhoff stress from the stretch invariants, for J > 0:
// tau = 2mu (B - V) + lam (J-1) J I with V = R F^T = sqrt(B).  Cayley-Hamilton
// for V (invariants I1, I2, I3 of V, V^2 = B) gives
//   V = (-B^2 + (I1^2 - I2) B + I1 I3 I) / (I1 I2 - I3)
// (Hoger & Carlson, "Determination of the stretch and rotation in the polar
// decomposition of the deformation gradient", Q. Appl. Math. 42, 1984).  In
// strain variables, B = I + E and s_i = 1 + t_i with t_i = e_i / (1 +
// sqrt(1 + e_i)) (e_i the eigenvalues of E) and e1, e2, e3 the elementary
// symmetric polynomials of the t_i, this is
//   V - I = (e3 (4 + e1) I + (4 + 4 e1 + e1^2 - e2) E - E^2) / D,
//   D = (s1 + s2)(s1 + s3)(s2 + s3) = 8 + 8 e1 + 2 e2 + 2 e1^2 + e1 e2 - e3,
// which keeps small strains free of cancellation and needs no eigenvectors.
__device__ __forceinline__ void fcr_tau_invariant(float mu, float lam, const Sym3 &E, float Jm1,
                                                  Sym3 &tau) {
  float w[3];
  sym_eigvals3(E, w);
  float t[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float e = fmaxf(w[k], -1.0f);
    t[k] = e / (1.0f + sqrtf(1.0f + e));
  }
  const float e1 = t[0] + t[1] + t[2];
  const float e2 = t[0] * t[1] + t[0] * t[2] + t[1] * t[2];
  const float e3 = t[0] * t[1] * t[2];
  const float D = 8.0f + 8.0f * e1 + 2.0f * e2 + 2.0f * e1 * e1 + e1 * e2 - e3;
  const float rD = 1.0f / D;
  const float c0 = e3 * (4.0f + e1) * rD, c1 = (4.0f + 4.0f * e1 + e1 * e1 - e2) * rD;
  // E^2 (symmetric)
  const float qxx = E.xx * E.xx + E.xy * E.xy + E.xz * E.xz;
  const float qyy = E.xy * E.xy + E.yy * E.yy + E.yz * E.yz;
  const float qzz = E.xz * E.xz + E.yz * E.yz + E.zz * E.zz;
  const float qxy = E.xx * E.xy + E.xy * E.yy + E.xz * E.yz;
  const float qxz = E.xx * E.xz + E.xy * E.yz + E.xz * E.zz;
  const float qyz = E.xy * E.xz + E.yy * E.yz + E.yz * E.zz;
  // B - V = E - (V - I)
  const float m2 = 2.0f * mu, k1 = 1.0f - c1;
  const float J = 1.0f + Jm1;
  const float diag = lam * Jm1 * J - m2 * c0;
  tau.xx = m2 * fmaf(qxx, rD, k1 * E.xx) + diag;
  tau.yy = m2 * fmaf(qyy, rD, k1 * E.yy) + diag;
  tau.zz = m2 * fmaf(qzz, rD, k1 * E.zz) + diag;
  tau.xy = m2 * fmaf(qxy, rD, k1 * E.xy);
  tau.xz = m2 * fmaf(qxz, rD, k1 * E.xz);
  tau.yz = m2 * fmaf(qyz, rD, k1 * E.yz);
}

// Q diag(d) Q^T
__device__ __forceinline__ Sym3 qdqt(const float (&Q)[9], float d0, float d1, float d2) {
  Sym3 r;
  r.xx = Q[0] * Q[0] * d0 + Q[1] * Q[1] * d1 + Q[2] * Q[2] * d2;
  r.yy = Q[3] * Q[3] * d0 + Q[4] * Q[4] * d1 + Q[5] * Q[5] * d2;
  r.zz = Q[6] * Q[6] * d0 + Q[7] * Q[7] * d1 + Q[8] * Q[8] * d2;
  r.xy = Q[0] * Q[3] * d0 + Q[1] * Q[4] * d1 + Q[2] * Q[5] * d2;
  r.xz = Q[0] * Q[6] * d0 + Q[1] * Q[7] * d1 + Q[2] * Q[8] * d2;
  r.yz = Q[3] * Q[6] * d0 + Q[4] * Q[7] * d1 + Q[5] * Q[8] * d2;
  return r;
}

// E = F F^T - I from G = F - I, and J - 1 = det(I + G) - 1 expanded in G.
__device__ __forceinline__ void strain_of(const float (&F)[9], Sym3 &E, float &Jm1) {
  const float g0 = F[0] - 1.0f, g1 = F[1], g2 = F[2];
  const float g3 = F[3], g4 = F[4] - 1.0f, g5 = F[5];
  const float g6 = F[6], g7 = F[7], g8 = F[8] - 1.0f;
  E.xx = g0 * g0 + g1 * g1 + g2 * g2 + 2.0f * g0;
  E.yy = g3 * g3 + g4 * g4 + g5 * g5 + 2.0f * g4;
  E.zz = g6 * g6 + g7 * g7 + g8 * g8 + 2.0f * g8;
  E.xy = g0 * g3 + g1 * g4 + g2 * g5 + g1 + g3;
  E.xz = g0 * g6 + g1 * g7 + g2 * g8 + g2 + g6;
  E.yz = g3 * g6 + g4 * g7 + g5 * g8 + g5 + g7;
  const float m2 = (g0 * g4 - g1 * g3) + (g0 * g8 - g2 * g6) + (g4 * g8 - g5 * g7);
  const float dg = g0 * (g4 * g8 - g5 * g7) - g1 * (g3 * g8 - g5 * g6) + g2 * (g3 * g7 - g4 * g6);
  Jm1 = (g0 + g4 + g8) + m2 + dg;
}

// Kirchhoff stress tau = P F^T (the reference scatters -dt*Dinv*vol*P*F^T,
// Transfer.cu:868):
//  fixed corotated (Stomakhin et al. 2012): tau = 2mu U diag(s^2 - s^) U^T
//      + lam (J-1) J I, with B = U S^2 U^T and s^ the singular values with the
//      smallest negated when J < 0 (R F^T = U S^ U^T);
//  Neo-Hookean: tau = mu (B - I) + lam ln(J) I;
//  StVK-Hencky (Klar et al. 2016): tau = U diag(2mu e_i + lam sum e) U^T,
//      e_i = ln s_i;
//  equation-of-state fluid (Tait form, Becker & Teschner 2007):
//      p = K (J^-gamma - 1), tau = -p J I.
// Returns false for an inverted or degenerate state the model cannot take.
__device__ __forceinline__ bool kirchhoff(int type, float mu, float lam, float bulk, float gam,
                                          const float (&F)[9], float Jeos, Sym3 &tau) {
  if (type == MPM_EOS) {
    const float t = -bulk * Jeos * expm1f(-gam * logf(Jeos));
    tau = Sym3{t, t, t, 0.f, 0.f, 0.f};
    return Jeos > 0.0f;
  }
  Sym3 E;
  float Jm1;
  strain_of(F, E, Jm1);
  const float J = 1.0f + Jm1;
  if (type == MPM_NHK) {
    const float diag = lam * log1pf(Jm1);
    tau = Sym3{mu * E.xx + diag, mu * E.yy + diag, mu * E.zz + diag, mu * E.xy, mu * E.xz,
               mu * E.yz};
    return J > 0.0f;
  }
  if (type == MPM_SNHK) {
    // stable Neo-Hookean (Smith, de Goes & Kim 2018, "Stable Neo-Hookean
    // Flesh Simulation"), invariant form Psi = mu/2 (I_C - 3) - mu (J - 1)
    // + lam/2 (J - 1)^2: tau = mu (B - I) + (lam (J - 1) J - mu (J - 1)) I,
    // defined through inversion
    const float diag = Jm1 * (lam * J - mu);
    tau = Sym3{mu * E.xx + diag, mu * E.yy + diag, mu * E.zz + diag, mu * E.xy, mu * E.xz,
               mu * E.yz};
    return true;
  }
  if (type == MPM_FCR && J > 0.0f) {
    fcr_tau_invariant(mu, lam, E, Jm1, tau);
    return true;
  }
  float w[3], Q[9];
  sym_eig3(E, w, Q);
  if (type == MPM_FCR) {  // inverted (J <= 0): sign-fixed singular values
    float d[3], s[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float lamk = fmaxf(w[k], -1.0f);  // eigenvalue of B - I
      s[k] = sqrtf(1.0f + lamk);
      d[k] = s[k] * lamk / (s[k] + 1.0f);     // s^2 - s
    }
    if (J < 0.0f) {
      const int kmin = (s[0] <= s[1] && s[0] <= s[2]) ? 0 : ((s[1] <= s[2]) ? 1 : 2);
#pragma unroll
      for (int k = 0; k < 3; ++k)
        if (k == kmin) d[k] = s[k] * s[k] + s[k];  // s^2 - (-s)
    }
    tau = qdqt(Q, 2.0f * mu * d[0], 2.0f * mu * d[1], 2.0f * mu * d[2]);
    const float diag = lam * Jm1 * J;
    tau.xx += diag;
    tau.yy += diag;
    tau.zz += diag;
    return true;
  }
  // StVK with Hencky strain
  const float e0 = 0.5f * log1pf(w[0]), e1 = 0.5f * log1pf(w[1]), e2 = 0.5f * log1pf(w[2]);
  const float tr = e0 + e1 + e2;
  tau = qdqt(Q, 2.0f * mu * e0 + lam * tr, 2.0f * mu * e1 + lam * tr, 2.0f * mu * e2 + lam * tr);
  return w[0] > -1.0f && w[1] > -1.0f && w[2] > -1.0f;
}

// Non-associative Drucker-Prager return mapping in Hencky strain space
// (Klar et al. 2016, sec. 7.3), the ZSReturnMapping node
// (MPMPipeline.cu:958-971): with F = U S V^T and B = U S^2 U^T the projected
// F is U S' V^T = F + U diag(S'/S - 1) U^T F.  The same decomposition gives
// the StVK-Hencky Kirchhoff stress of the (projected) state,
// tau = U diag(2mu e'_i + lam sum e') U^T.  Returns -1 on a degenerate F,
// 1 if projected, 0 if inside the yield surface.
__device__ __forceinline__ int project_dp(float mu, float lam, float alpha, float (&F)[9],
                                          Sym3 &tau) {
  Sym3 E;
  float Jm1;
  strain_of(F, E, Jm1);
  float w[3], Q[9];
  sym_eig3(E, w, Q);
  if (!(w[0] > -1.0f && w[1] > -1.0f && w[2] > -1.0f)) {
    tau = Sym3{0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    return -1;
  }
  float e0 = 0.5f * log1pf(w[0]), e1 = 0.5f * log1pf(w[1]), e2 = 0.5f * log1pf(w[2]);
  const float tr = e0 + e1 + e2;
  int projected = 1;
  float r0 = 0.f, r1 = 0.f, r2 = 0.f;  // S'/S - 1
  if (tr >= 0.0f) {
    r0 = expm1f(-e0);
    r1 = expm1f(-e1);
    r2 = expm1f(-e2);
    e0 = e1 = e2 = 0.0f;
  } else {
    const float h0 = e0 - tr / 3.0f, h1 = e1 - tr / 3.0f, h2 = e2 - tr / 3.0f;
    const float nrm = sqrtf(h0 * h0 + h1 * h1 + h2 * h2);
    const float dg = nrm + (3.0f * lam + 2.0f * mu) / (2.0f * mu) * tr * alpha;
    if (dg <= 0.0f) {
      projected = 0;
    } else {
      const float k = dg / nrm;
      r0 = expm1f(-k * h0);
      r1 = expm1f(-k * h1);
      r2 = expm1f(-k * h2);
      e0 -= k * h0;
      e1 -= k * h1;
      e2 -= k * h2;
    }
  }
  const float trp = e0 + e1 + e2;
  tau = qdqt(Q, 2.0f * mu * e0 + lam * trp, 2.0f * mu * e1 + lam * trp,
             2.0f * mu * e2 + lam * trp);
  if (!projected) return 0;
  const Sym3 M = qdqt(Q, r0, r1, r2);
  float Fn[9];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    Fn[0 * 3 + j] = F[0 * 3 + j] + M.xx * F[j] + M.xy * F[3 + j] + M.xz * F[6 + j];
    Fn[1 * 3 + j] = F[1 * 3 + j] + M.xy * F[j] + M.yy * F[3 + j] + M.yz * F[6 + j];
    Fn[2 * 3 + j] = F[2 * 3 + j] + M.xz * F[j] + M.yz * F[3 + j] + M.zz * F[6 + j];
  }
#pragma unroll
  for (int i = 0; i < 9; ++i) F[i] = Fn[i];
  return 1;
}

// Return mapping in Hencky strain space for the von Mises and Cam-Clay
// models (ZSReturnMapping, MPMPipeline.cu:953-972, navm / nacc): with
// B = F F^T = U diag(b) U^T and the log stretches e_i = ln(b_i) / 2, a rule
// moves e to e' on the yield surface; F <- U diag(exp(e' - e)) U^T F, and tau
// is the StVK-Hencky stress of e'.  Rules, on h = e - tr(e)/3 and tr(e):
//  von Mises (the Hencky-strain projection of Jiang et al. 2016, "The
//    Material Point Method for Simulating Continuum Materials", SIGGRAPH
//    course, sec. 8.2): with dg = |h| - yield / (2 mu) > 0, e' = e - dg h / |h|;
//  Cam-Clay (Gaume et al. 2018, "Dynamic anticrack propagation in snow",
//    Nat. Commun. 9:3047, Methods): pressure p = -kappa tr(e), kappa = lam +
//    2mu/3, deviatoric q = sqrt(3/2) 2mu |h|, yield surface
//    q^2 (1 + 2 beta) + M^2 (p + beta p0)(p - p0) <= 0 with
//    p0 = kappa sinh(xi max(-log Jp, 0)); beyond the caps p > p0 or
//    p < -beta p0 the state goes to (p0, 0) or (-beta p0, 0), otherwise outside
//    the ellipse it moves toward the ellipse's centre ((1 - beta) p0 / 2, 0)
//    onto the surface (a non-associative return); log Jp gains the plastic
//    volume change tr(e) - tr(e').
// Returns -1 on a degenerate F, 1 if projected, 0 if inside the yield surface.
static __device__ __noinline__ int project_hencky(const MatParams &mp, float mu, float lam,
                                           float (&F)[9], float &logJp, Sym3 &tau) {
  Sym3 E;
  float Jm1;
  strain_of(F, E, Jm1);
  float w[3], Q[9];
  sym_eig3(E, w, Q);
  if (!(w[0] > -1.0f && w[1] > -1.0f && w[2] > -1.0f)) {
    tau = Sym3{0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    return -1;
  }
  const float e[3] = {0.5f * log1pf(w[0]), 0.5f * log1pf(w[1]), 0.5f * log1pf(w[2])};
  const float tr = e[0] + e[1] + e[2];
  const float h[3] = {e[0] - tr / 3.0f, e[1] - tr / 3.0f, e[2] - tr / 3.0f};
  const float nrm = sqrtf(h[0] * h[0] + h[1] * h[1] + h[2] * h[2]);
  float hs = 1.0f, trn = tr;  // e' = hs h + trn / 3
  bool projected = false;
  if (mp.plastic == MPM_PLASTIC_NAVM) {
    const float dg = nrm - mp.yield / (2.0f * mu);
    if (dg > 0.0f) {
      hs = 1.0f - dg / nrm;
      projected = true;
    }
  } else {  // Cam-Clay
    const float kappa = lam + 2.0f * mu / 3.0f;
    const float p0 = kappa * sinhf(mp.cc_xi * fmaxf(-logJp, 0.0f));
    const float beta = mp.cc_beta, M = mp.cc_M;
    const float p = -kappa * tr, q = 1.2247448713915890f * 2.0f * mu * nrm;  // sqrt(3/2)
    float pn = p, qn = q;
    if (p > p0) {
      pn = p0;
      qn = 0.0f;
      projected = true;
    } else if (p < -beta * p0) {
      pn = -beta * p0;
      qn = 0.0f;
      projected = true;
    } else if (q * q * (1.0f + 2.0f * beta) + M * M * (p + beta * p0) * (p - p0) > 0.0f) {
      const float pc = 0.5f * (1.0f - beta) * p0, a = 0.5f * (1.0f + beta) * p0, dp = p - pc;
      const float t = M * a * rsqrtf(q * q * (1.0f + 2.0f * beta) + M * M * dp * dp);
      pn = pc + t * dp;
      qn = t * q;
      projected = true;
    }
    if (projected) {
      trn = -pn / kappa;
      hs = q > 0.0f ? qn / q : 0.0f;
      logJp += tr - trn;
    }
  }
  float en[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) en[k] = hs * h[k] + trn / 3.0f;
  const float trp = en[0] + en[1] + en[2];
  tau = qdqt(Q, 2.0f * mu * en[0] + lam * trp, 2.0f * mu * en[1] + lam * trp,
             2.0f * mu * en[2] + lam * trp);
  if (!projected) return 0;
  const Sym3 Mr = qdqt(Q, expm1f(en[0] - e[0]), expm1f(en[1] - e[1]), expm1f(en[2] - e[2]));
  float Fn[9];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    Fn[0 * 3 + j] = F[0 * 3 + j] + Mr.xx * F[j] + Mr.xy * F[3 + j] + Mr.xz * F[6 + j];
    Fn[1 * 3 + j] = F[1 * 3 + j] + Mr.xy * F[j] + Mr.yy * F[3 + j] + Mr.yz * F[6 + j];
    Fn[2 * 3 + j] = F[2 * 3 + j] + Mr.xz * F[j] + Mr.yz * F[3 + j] + Mr.zz * F[6 + j];
  }
#pragma unroll
  for (int i = 0; i < 9; ++i) F[i] = Fn[i];
  return 1;
}

// The return mapping of a plastic material (ZSReturnMapping) and the stress
// of the result: Drucker-Prager, von Mises or Cam-Clay; `jch` is the J
// channel, which holds log(Jp) for Cam-Clay.
__device__ __forceinline__ int return_mapping(const MatParams &mp, float mu, float lam,
                                              float (&F)[9], float &jch, Sym3 &tau) {
  if (mp.plastic == MPM_PLASTIC_NADP) return project_dp(mu, lam, mp.alpha, F, tau);
  return project_hencky(mp, mu, lam, F, jch, tau);
}

__device__ __forceinline__ float det3(const float (&F)[9]) {
  return F[0] * (F[4] * F[8] - F[5] * F[7]) - F[1] * (F[3] * F[8] - F[5] * F[6]) +
         F[2] * (F[3] * F[7] - F[4] * F[6]);
}

// Quadratic B-spline weights (Hu et al. 2018 MLS-MPM; Jiang et al. 2016
// course notes): f = x/dx - base in [0.5, 1.5),
// w0 = (1.5-f)^2/2, w1 = 3/4 - (f-1)^2, w2 = (f-0.5)^2/2.
struct Stencil1 {
  int base;
  float f;
  float w[3];
};

__device__ __forceinline__ Stencil1 stencil1(float x, float inv_dx) {
  Stencil1 s;
  s.base = __float2int_rd(__fsub_rn(__fmul_rn(x, inv_dx), 0.5f));
  s.f = __fsub_rn(__fmul_rn(x, inv_dx), (float)s.base);
  const float a = 1.5f - s.f, b = s.f - 1.0f, c = s.f - 0.5f;
  s.w[0] = 0.5f * a * a;
  s.w[1] = 0.75f - b * b;
  s.w[2] = 0.5f * c * c;
  return s;
}

}  // namespace zsmpm

namespace zsmpm {

// ---------------------------------------------------------------------------
// Adjoints (vector-Jacobian products) of the Kirchhoff stresses.

__device__ __forceinline__ void cofactor3(const float (&F)[9], float (&c)[9]) {
  c[0] = F[4] * F[8] - F[5] * F[7];
  c[1] = F[5] * F[6] - F[3] * F[8];
  c[2] = F[3] * F[7] - F[4] * F[6];
  c[3] = F[2] * F[7] - F[1] * F[8];
  c[4] = F[0] * F[8] - F[2] * F[6];
  c[5] = F[1] * F[6] - F[0] * F[7];
  c[6] = F[1] * F[5] - F[2] * F[4];
  c[7] = F[2] * F[3] - F[0] * F[5];
  c[8] = F[0] * F[4] - F[1] * F[3];
}

// Fixed corotated, tau = 2mu (F F^T - R F^T) + lam (J^2 - J) I.  Given the
// adjoint tb of tau (3x3), adds to Fb, mub, lamb:
//   Fb += 2mu (tb F + tb^T F - tb^T R - dR^T[tb F]) + lam (2J - 1) tr(tb) cof(F)
//   mub += 2 <tb, F F^T - R F^T>,  lamb += tr(tb) (J^2 - J)
// where dR^T[G] = [K ax(G R^T)]x R is the adjoint of the derivative of the
// polar rotation (F = R S: R^T dR = [w]x with (tr(S) I - S) w = ax(R^T dF),
// ax(M) = (M21 - M12, M02 - M20, M10 - M01)), and K = U diag(1 / (tr s^ - s^_i))
// U^T in the frame of B = F F^T = U S^2 U^T, s^ the sign-fixed singular values.
__device__ __forceinline__ void fcr_vjp(float mu, float lam, const float (&F)[9],
                                        const float (&tb)[9], float (&Fb)[9], float &mub,
                                        float &lamb) {
  Sym3 E;
  float Jm1;
  strain_of(F, E, Jm1);
  const float J = 1.0f + Jm1;
  float w[3], Q[9];
  sym_eig3(E, w, Q);
  float s[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) s[k] = sqrtf(1.0f + fmaxf(w[k], -1.0f));
  if (J < 0.0f) {
    const int kmin = (s[0] <= s[1] && s[0] <= s[2]) ? 0 : ((s[1] <= s[2]) ? 1 : 2);
#pragma unroll
    for (int k = 0; k < 3; ++k)
      if (k == kmin) s[k] = -s[k];
  }
  // R = U diag(1/s^) U^T F,  R F^T = U diag(s^) U^T
  const Sym3 Ui = qdqt(Q, 1.0f / s[0], 1.0f / s[1], 1.0f / s[2]);
  const float Uim[9] = {Ui.xx, Ui.xy, Ui.xz, Ui.xy, Ui.yy, Ui.yz, Ui.xz, Ui.yz, Ui.zz};
  float R[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      R[i * 3 + j] = Uim[i * 3] * F[j] + Uim[i * 3 + 1] * F[3 + j] + Uim[i * 3 + 2] * F[6 + j];
  const Sym3 RFt = qdqt(Q, s[0], s[1], s[2]);
  const float ts = s[0] + s[1] + s[2];
  const Sym3 Kl = qdqt(Q, 1.0f / (ts - s[0]), 1.0f / (ts - s[1]), 1.0f / (ts - s[2]));
  // G = tb F, M = G R^T
  float G[9], M[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      G[i * 3 + j] = tb[i * 3] * F[j] + tb[i * 3 + 1] * F[3 + j] + tb[i * 3 + 2] * F[6 + j];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      M[i * 3 + j] = G[i * 3] * R[j * 3] + G[i * 3 + 1] * R[j * 3 + 1] + G[i * 3 + 2] * R[j * 3 + 2];
  const float a0 = M[7] - M[5], a1 = M[2] - M[6], a2 = M[3] - M[1];
  const float g0 = Kl.xx * a0 + Kl.xy * a1 + Kl.xz * a2;
  const float g1 = Kl.xy * a0 + Kl.yy * a1 + Kl.yz * a2;
  const float g2 = Kl.xz * a0 + Kl.yz * a1 + Kl.zz * a2;
  // [g]x R
  float gR[9];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    gR[0 * 3 + j] = -g2 * R[3 + j] + g1 * R[6 + j];
    gR[1 * 3 + j] = g2 * R[j] - g0 * R[6 + j];
    gR[2 * 3 + j] = -g1 * R[j] + g0 * R[3 + j];
  }
  float cof[9];
  cofactor3(F, cof);
  const float trtb = tb[0] + tb[4] + tb[8];
  const float cj = lam * (2.0f * J - 1.0f) * trtb;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      float tTF = 0.f, tTR = 0.f;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        tTF += tb[k * 3 + i] * F[k * 3 + j];
        tTR += tb[k * 3 + i] * R[k * 3 + j];
      }
      Fb[i * 3 + j] += 2.0f * mu * (G[i * 3 + j] + tTF - tTR - gR[i * 3 + j]) + cj * cof[i * 3 + j];
    }
  // B - R F^T with B = F F^T = I + E
  const float D[9] = {E.xx + 1.0f - RFt.xx, E.xy - RFt.xy, E.xz - RFt.xz,
                      E.xy - RFt.xy, E.yy + 1.0f - RFt.yy, E.yz - RFt.yz,
                      E.xz - RFt.xz, E.yz - RFt.yz, E.zz + 1.0f - RFt.zz};
  float dot = 0.f;
#pragma unroll
  for (int k = 0; k < 9; ++k) dot += tb[k] * D[k];
  mub += 2.0f * dot;
  lamb += trtb * Jm1 * J;
}

// Neo-Hookean, tau = mu (F F^T - I) + lam ln(J) I:
//   Fb += mu (tb + tb^T) F + lam tr(tb) F^-T,  mub += <tb, B - I>,
//   lamb += tr(tb) ln J
__device__ __forceinline__ void nhk_vjp(float mu, float lam, const float (&F)[9],
                                        const float (&tb)[9], float (&Fb)[9], float &mub,
                                        float &lamb) {
  Sym3 E;
  float Jm1;
  strain_of(F, E, Jm1);
  const float J = 1.0f + Jm1;
  float cof[9];
  cofactor3(F, cof);
  const float trtb = tb[0] + tb[4] + tb[8];
  const float cj = lam * trtb / J;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      float v = 0.f;
#pragma unroll
      for (int k = 0; k < 3; ++k) v += (tb[i * 3 + k] + tb[k * 3 + i]) * F[k * 3 + j];
      Fb[i * 3 + j] += mu * v + cj * cof[i * 3 + j];
    }
  const float Em[9] = {E.xx, E.xy, E.xz, E.xy, E.yy, E.yz, E.xz, E.yz, E.zz};
  float dot = 0.f;
#pragma unroll
  for (int k = 0; k < 9; ++k) dot += tb[k] * Em[k];
  mub += dot;
  lamb += trtb * log1pf(Jm1);
}

// ---------------------------------------------------------------------------
// Adjoints of isotropic functions of B = F F^T (StVK-Hencky stress, the
// Drucker-Prager projection).  For T(B) = U diag(t(b)) U^T (b the eigenvalues
// of B, U its eigenvectors) and a symmetric adjoint G of T, the adjoint of B
// is (Daleckii-Krein)
//   B-bar = U [ D o (U^T G U) off the diagonal, diag(Jt^T diag(U^T G U)) ] U^T,
//   D_ij = (t_i - t_j) / (b_i - b_j),  Jt_ik = dt_i / db_k,
// and F-bar += 2 B-bar F.  The divided differences are written as functions
// of u = (b_i - b_j) / b_j; for near-equal eigenvalues (|u| < 1e-3, where the
// FP32 difference of the closed forms cancels) they come from their Taylor
// series in u.  The series are evaluated in FP32: u is an FP32 number, the
// truncation error after the u^3 term is below |u|^4 / 4 < 3e-13, and the
// Horner steps round to a few ulp of the O(1) result, so FP64 arithmetic
// would not change the rounded value (GB300's FP64 rate is a small fraction
// of its FP32 rate, and nearly every particle of a sand column at rest takes
// this branch).

// log1p(u) / u = 1 - u/2 + u^2/3 - u^3/4 + ...
__device__ __forceinline__ float log1p_over(float u) {
  if (fabsf(u) < 1e-3f) return fmaf(-u, fmaf(-u, fmaf(-u, 0.25f, 1.0f / 3.0f), 0.5f), 1.0f);
  return log1pf(u) / u;
}

// ((1 + u)^a - 1) / u = expm1(a log1p(u)) / u
//   = a (1 + u (a-1)/2 + u^2 (a-1)(a-2)/6 + u^3 (a-1)(a-2)(a-3)/24 + ...)
__device__ __forceinline__ float pow1p_m1_over(float a, float u) {
  if (fabsf(u) < 1e-3f) {
    const float c1 = (a - 1.0f) * 0.5f, c2 = c1 * (a - 2.0f) * (1.0f / 3.0f),
                c3 = c2 * (a - 3.0f) * 0.25f;
    return a * fmaf(u, fmaf(u, fmaf(u, c3, c2), c1), 1.0f);
  }
  return expm1f(a * log1pf(u)) / u;
}

// B-bar from the symmetric world-frame adjoint G of T, the eigenvectors Q
// (columns), D (symmetric, off-diagonal used) and Jt; returns B-bar (3x3,
// symmetric) and the eigen-frame diagonal Gh_ii
__device__ __forceinline__ void iso_adjoint(const float (&Q)[9], const float (&G)[9],
                                            const float (&D)[9], const float (&Jt)[9],
                                            float (&Bb)[9], float (&Gd)[3]) {
  float QG[9], Gh[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)  // QG = Q^T G
#pragma unroll
    for (int j = 0; j < 3; ++j)
      QG[i * 3 + j] = Q[0 * 3 + i] * G[0 * 3 + j] + Q[1 * 3 + i] * G[1 * 3 + j] +
                      Q[2 * 3 + i] * G[2 * 3 + j];
#pragma unroll
  for (int i = 0; i < 3; ++i)  // Gh = Q^T G Q
#pragma unroll
    for (int j = 0; j < 3; ++j)
      Gh[i * 3 + j] = QG[i * 3 + 0] * Q[0 * 3 + j] + QG[i * 3 + 1] * Q[1 * 3 + j] +
                      QG[i * 3 + 2] * Q[2 * 3 + j];
  float H[9];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    Gd[i] = Gh[i * 4];
#pragma unroll
    for (int j = 0; j < 3; ++j) H[i * 3 + j] = i == j ? 0.0f : Gh[i * 3 + j] * D[i * 3 + j];
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) H[k * 4] = Gd[0] * Jt[0 * 3 + k] + Gd[1] * Jt[1 * 3 + k] + Gd[2] * Jt[2 * 3 + k];
  float QH[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)  // QH = Q H
#pragma unroll
    for (int j = 0; j < 3; ++j)
      QH[i * 3 + j] = Q[i * 3 + 0] * H[0 * 3 + j] + Q[i * 3 + 1] * H[1 * 3 + j] +
                      Q[i * 3 + 2] * H[2 * 3 + j];
#pragma unroll
  for (int i = 0; i < 3; ++i)  // Bb = Q H Q^T
#pragma unroll
    for (int j = 0; j < 3; ++j)
      Bb[i * 3 + j] = QH[i * 3 + 0] * Q[j * 3 + 0] + QH[i * 3 + 1] * Q[j * 3 + 1] +
                      QH[i * 3 + 2] * Q[j * 3 + 2];
}

// Fb += 2 Bb F
__device__ __forceinline__ void add_2BbF(const float (&Bb)[9], const float (&F)[9],
                                         float (&Fb)[9]) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      Fb[i * 3 + j] += 2.0f * (Bb[i * 3 + 0] * F[0 * 3 + j] + Bb[i * 3 + 1] * F[1 * 3 + j] +
                               Bb[i * 3 + 2] * F[2 * 3 + j]);
}

// StVK-Hencky, tau = U diag(2mu e_i + lam sum e) U^T, e_i = log(b_i) / 2: given
// the adjoint tb of tau (3x3), adds to Fb, mub, lamb.  D_ij = mu (log b_i -
// log b_j) / (b_i - b_j), Jt_ik = (2mu delta_ik + lam) / (2 b_k).
__device__ __forceinline__ void hencky_vjp(float mu, float lam, const float (&F)[9],
                                           const float (&tb)[9], float (&Fb)[9], float &mub,
                                           float &lamb) {
  Sym3 E;
  float Jm1;
  strain_of(F, E, Jm1);
  float w[3], Q[9];
  sym_eig3(E, w, Q);
  float b[3], e[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    b[k] = 1.0f + w[k];
    e[k] = 0.5f * log1pf(w[k]);
  }
  float G[9], D[9], Jt[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      G[i * 3 + j] = 0.5f * (tb[i * 3 + j] + tb[j * 3 + i]);
      D[i * 3 + j] = i == j ? 0.0f : mu * log1p_over((w[i] - w[j]) / b[j]) / b[j];
      Jt[i * 3 + j] = ((i == j ? 2.0f * mu : 0.0f) + lam) / (2.0f * b[j]);
    }
  float Bb[9], Gd[3];
  iso_adjoint(Q, G, D, Jt, Bb, Gd);
  add_2BbF(Bb, F, Fb);
  const float tr = e[0] + e[1] + e[2];
  mub += 2.0f * (Gd[0] * e[0] + Gd[1] * e[1] + Gd[2] * e[2]);
  lamb += (Gd[0] + Gd[1] + Gd[2]) * tr;
}

// Adjoint of the Drucker-Prager projection F_new = N(B) F (project_dp, B the
// trial B = F F^T, N = U diag(m) U^T, m_i = exp(e'_i - e_i)): given Fb =
// F_new-bar, replaces it by the trial F-bar N F_new-bar + 2 B-bar F (B-bar from
// G = sym(F_new-bar F^T)) and adds the yield condition's mu, lam terms.
// Cases (the same tests on the same FP32 eigenvalues as project_dp):
//   elastic: N = I;
//   tension (sum e >= 0): m_i = b_i^-1/2, Jt_ii = -b_i^-3/2 / 2,
//       D_ij = -1 / (s_i s_j (s_i + s_j)), s = sqrt(b);
//   projected: m_i = exp(g_i), g = -k h, h = e - tr/3, k = 1 + c alpha tr / |h|,
//       c = (3 lam + 2 mu) / (2 mu); dg_i/de_j = -P_ij - c alpha (h^_i + tr (P_ij -
//       h^_i h^_j) / |h|), P = I - 1/3, Jt_ij = m_i dg_i/de_j / (2 b_j), and
//       D_ij = m_j ((b_i/b_j)^(-k/2) - 1) / (b_i - b_j).
__device__ __forceinline__ void dp_projection_vjp(float mu, float lam, float alpha,
                                                  const float (&F)[9], float (&Fb)[9],
                                                  float &mub, float &lamb) {
  Sym3 E;
  float Jm1;
  strain_of(F, E, Jm1);
  float w[3], Q[9];
  sym_eig3(E, w, Q);
  if (!(w[0] > -1.0f && w[1] > -1.0f && w[2] > -1.0f)) return;  // degenerate: forward flagged it
  float b[3], e[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    b[k] = 1.0f + w[k];
    e[k] = 0.5f * log1pf(w[k]);
  }
  const float tr = e[0] + e[1] + e[2];
  float m[3], D[9], Jt[9];
  float hh[3] = {0.f, 0.f, 0.f}, c = 0.f;
  bool projected = false;
  if (tr >= 0.0f) {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      m[i] = expf(-e[i]);
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const float si = sqrtf(b[i]), sj = sqrtf(b[j]);
        D[i * 3 + j] = i == j ? 0.0f : -1.0f / (si * sj * (si + sj));
        Jt[i * 3 + j] = i == j ? -0.5f / (b[i] * si) : 0.0f;
      }
    }
  } else {
    const float h0 = e[0] - tr / 3.0f, h1 = e[1] - tr / 3.0f, h2 = e[2] - tr / 3.0f;
    const float nrm = sqrtf(h0 * h0 + h1 * h1 + h2 * h2);
    c = (3.0f * lam + 2.0f * mu) / (2.0f * mu);
    const float dg = nrm + c * tr * alpha;
    if (dg <= 0.0f) return;  // elastic: F_new = F
    projected = true;
    const float k = dg / nrm;
    const float h[3] = {h0, h1, h2};
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      hh[i] = h[i] / nrm;
      m[i] = expf(-k * h[i]);
    }
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const float P = (i == j ? 1.0f : 0.0f) - 1.0f / 3.0f;
        const float dgde = -P - c * alpha * (hh[i] + tr * (P - hh[i] * hh[j]) / nrm);
        Jt[i * 3 + j] = m[i] * dgde / (2.0f * b[j]);
        D[i * 3 + j] =
            i == j ? 0.0f : m[j] * pow1p_m1_over(-0.5f * k, (w[i] - w[j]) / b[j]) / b[j];
      }
  }
  // G = sym(F_new-bar F^T)
  float G[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const float a = Fb[i * 3 + 0] * F[j * 3 + 0] + Fb[i * 3 + 1] * F[j * 3 + 1] +
                      Fb[i * 3 + 2] * F[j * 3 + 2];
      const float t = Fb[j * 3 + 0] * F[i * 3 + 0] + Fb[j * 3 + 1] * F[i * 3 + 1] +
                      Fb[j * 3 + 2] * F[i * 3 + 2];
      G[i * 3 + j] = 0.5f * (a + t);
    }
  float Bb[9], Gd[3];
  iso_adjoint(Q, G, D, Jt, Bb, Gd);
  // N F_new-bar
  const Sym3 N = qdqt(Q, m[0], m[1], m[2]);
  const float Nm[9] = {N.xx, N.xy, N.xz, N.xy, N.yy, N.yz, N.xz, N.yz, N.zz};
  float out[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      out[i * 3 + j] = Nm[i * 3 + 0] * Fb[0 * 3 + j] + Nm[i * 3 + 1] * Fb[1 * 3 + j] +
                       Nm[i * 3 + 2] * Fb[2 * 3 + j];
  add_2BbF(Bb, F, out);
#pragma unroll
  for (int k = 0; k < 9; ++k) Fb[k] = out[k];
  if (projected) {
    // dg_i/dc = -alpha tr h^_i; dc/dmu = -3 lam / (2 mu^2), dc/dlam = 3 / (2 mu)
    const float dLdc = -alpha * tr * (Gd[0] * m[0] * hh[0] + Gd[1] * m[1] * hh[1] +
                                      Gd[2] * m[2] * hh[2]);
    mub += dLdc * (-3.0f * lam / (2.0f * mu * mu));
    lamb += dLdc * (3.0f / (2.0f * mu));
  }
}

// dw/df of the quadratic B-spline weights (per axis): w0' = f - 1.5,
// w1' = -2 (f - 1), w2' = f - 0.5
__device__ __forceinline__ void stencil_dw(float f, float (&dw)[3]) {
  dw[0] = f - 1.5f;
  dw[1] = -2.0f * (f - 1.0f);
  dw[2] = f - 0.5f;
}

}  // namespace zsmpm
