// CPU oracle for the CuLagrange MLS-MPM substep -- TEST INFRASTRUCTURE ONLY.
//
// The GPU product never links or calls this file.  It is the checker used by
// tests/, by the smoke check and by the CPU legs of bench.py.  Templated on
// the real type: the double build is the physics oracle (order-stable
// scatter: particle blocks are processed in 8 parity colours, so every grid
// node receives its contributions in one fixed order whatever the thread
// count); the float build with OpenMP is the timed CPU baseline.
//
// Reference node bodies restated here (file:line within zenustech/zeno):
//   binning            projects/CuLagrange/mpm/MPMPipeline.cu:73-84
//   halo expansion     projects/CuLagrange/mpm/MPMPipeline.cu:131-199
//   grid clear         projects/CuLagrange/mpm/MPMPipeline.cu:256-262
//   APIC P2G           projects/CuLagrange/mpm/Transfer.cu:849-889
//   grid update        projects/CuLagrange/mpm/MPMPipeline.cu:852-877
//   boundary           projects/CuLagrange/mpm/Boundary.cu:56-67,105-116
//   APIC G2P           projects/CuLagrange/mpm/Transfer.cu:1139-1173
//   return mapping     projects/CuLagrange/mpm/MPMPipeline.cu:958-971
//   particle init      projects/CuLagrange/mpm/Generation.cpp:944-966
//   FLIP / AFLIP P2G   projects/CuLagrange/mpm/Transfer.cu:891-984
//   FLIP grid update   projects/CuLagrange/mpm/MPMPipeline.cu:878-897
//   FLIP / AFLIP G2P   projects/CuLagrange/mpm/Transfer.cu:1174-1257
//   particle beta      projects/CuLagrange/mpm/Boundary.cu:172-516
// zpc (which holds the arithmetic) is absent; each restated formula below
// names the published method it follows.
#include "mpm_oracle.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <type_traits>
#include <unordered_map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

template <class R> struct Params {
  R mu, lam, alpha, bulk, gamma;
  R yield, ccM, ccbeta, ccxi;
  int type, plastic;
};

template <class R> Params<R> material_params(const orc_material &m) {
  // Lame parameters from (E, nu): the standard relations the reference
  // obtains from zs::lame_parameters (projects/CuLagrange/mpm/Temp.cu:47).
  Params<R> p;
  const R E = R(m.E), nu = R(m.nu);
  p.mu = E / (R(2) * (R(1) + nu));
  p.lam = E * nu / ((R(1) + nu) * (R(1) - R(2) * nu));
  // Drucker-Prager cone coefficient, Klar et al. 2016 "Drucker-Prager
  // elastoplasticity for sand animation", sec. 7.3.
  const R phi = R(m.friction_angle_deg) * R(3.14159265358979323846) / R(180);
  const R s = std::sin(phi);
  p.alpha = std::sqrt(R(2) / R(3)) * R(2) * s / (R(3) - s);
  p.bulk = R(m.bulk);
  p.gamma = R(m.gamma);
  p.yield = R(m.yield_stress);
  // Cam-Clay critical-state slope: the Mohr-Coulomb compression match
  p.ccM = R(6) * s / (R(3) - s);
  p.ccbeta = R(m.cc_beta);
  p.ccxi = R(m.cc_xi);
  p.type = m.type;
  p.plastic = m.plasticity;
  return p;
}

// Cyclic Jacobi eigen-decomposition of a symmetric 3x3 matrix (Golub & Van
// Loan, Matrix Computations, 4th ed., Alg. 8.5.2 with sym.schur2).
// A = Q diag(w) Q^T.
template <class R> void sym_eig3(const R *A_, R *w, R *Q, int max_sweeps) {
  R A[9];
  for (int i = 0; i < 9; ++i) A[i] = A_[i];
  for (int i = 0; i < 9; ++i) Q[i] = (i % 4 == 0) ? R(1) : R(0);
  const int P[3] = {0, 0, 1}, Qi[3] = {1, 2, 2};
  for (int sweep = 0; sweep < max_sweeps; ++sweep) {
    const R off = A[1] * A[1] + A[2] * A[2] + A[5] * A[5];
    const R dia = A[0] * A[0] + A[4] * A[4] + A[8] * A[8];
    if (off == R(0) || off <= dia * std::numeric_limits<R>::epsilon() *
                                     std::numeric_limits<R>::epsilon() * R(1e-2))
      break;
    for (int r = 0; r < 3; ++r) {
      const int p = P[r], q = Qi[r];
      const R apq = A[p * 3 + q];
      if (apq == R(0)) continue;
      const R theta = (A[q * 3 + q] - A[p * 3 + p]) / (R(2) * apq);
      const R t = (theta >= R(0) ? R(1) : R(-1)) /
                  (std::fabs(theta) + std::sqrt(theta * theta + R(1)));
      const R c = R(1) / std::sqrt(t * t + R(1)), s = t * c;
      for (int k = 0; k < 3; ++k) {  // A <- A J
        const R akp = A[k * 3 + p], akq = A[k * 3 + q];
        A[k * 3 + p] = c * akp - s * akq;
        A[k * 3 + q] = s * akp + c * akq;
      }
      for (int k = 0; k < 3; ++k) {  // A <- J^T A
        const R apk = A[p * 3 + k], aqk = A[q * 3 + k];
        A[p * 3 + k] = c * apk - s * aqk;
        A[q * 3 + k] = s * apk + c * aqk;
      }
      for (int k = 0; k < 3; ++k) {  // Q <- Q J
        const R qkp = Q[k * 3 + p], qkq = Q[k * 3 + q];
        Q[k * 3 + p] = c * qkp - s * qkq;
        Q[k * 3 + q] = s * qkp + c * qkq;
      }
    }
  }
  w[0] = A[0];
  w[1] = A[4];
  w[2] = A[8];
}

template <class R> inline R det3(const R *F) {
  return F[0] * (F[4] * F[8] - F[5] * F[7]) - F[1] * (F[3] * F[8] - F[5] * F[6]) +
         F[2] * (F[3] * F[7] - F[4] * F[6]);
}

template <class R> inline void mul_ABt(const R *A, const R *B, R *out) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      R s = 0;
      for (int k = 0; k < 3; ++k) s += A[i * 3 + k] * B[j * 3 + k];
      out[i * 3 + j] = s;
    }
}

template <class R> inline void mul_AB(const R *A, const R *B, R *out) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      R s = 0;
      for (int k = 0; k < 3; ++k) s += A[i * 3 + k] * B[k * 3 + j];
      out[i * 3 + j] = s;
    }
}

// Q diag(d) Q^T
template <class R> inline void qdqt(const R *Q, const R *d, R *out) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      R s = 0;
      for (int k = 0; k < 3; ++k) s += Q[i * 3 + k] * d[k] * Q[j * 3 + k];
      out[i * 3 + j] = s;
    }
}

constexpr int kSweeps = 30;

// Kirchhoff stress tau = P F^T.  The reference scatters
// contrib = -dt * Dinv * vol * P * F^T (Transfer.cu:868); tau is that P F^T.
//   fixed corotated (Stomakhin et al. 2012): P = 2mu(F-R) + lam(J-1)J F^-T,
//     tau = 2mu(B - R F^T) + lam(J-1)J I with B = F F^T, R F^T = U S^ U^T
//     (S^ = singular values with the smallest negated when J < 0).
//   Neo-Hookean: P = mu(F - F^-T) + lam ln(J) F^-T, tau = mu(B - I) + lam ln(J) I.
//   StVK with Hencky strain (Klar et al. 2016): tau = U(2mu ln S + lam tr(ln S))U^T.
//   equation-of-state fluid (Tait, Becker & Teschner 2007):
//     p = K(J^-gamma - 1), tau = -p J I.
// U and S come from the eigen-decomposition of B = U S^2 U^T.
template <class R>
bool kirchhoff(const Params<R> &p, const R *F, R J, R *tau) {
  for (int i = 0; i < 9; ++i) tau[i] = 0;
  if (p.type == ORC_EOS) {
    if (!(J > R(0))) return false;
    const R t = p.bulk * (J - std::pow(J, R(1) - p.gamma));
    tau[0] = tau[4] = tau[8] = t;
    return true;
  }
  R B[9];
  mul_ABt(F, F, B);
  if (p.type == ORC_SNHK) {
    // stable Neo-Hookean, invariant form (Smith, de Goes & Kim 2018):
    // Psi = mu/2 (I_C - 3) - mu (J - 1) + lam/2 (J - 1)^2,
    // P = mu F + (lam (J - 1) - mu) J F^-T, tau = mu B + (lam (J - 1) - mu) J I
    const R Jf = det3(F);
    for (int i = 0; i < 9; ++i) tau[i] = p.mu * B[i];
    const R diag = (p.lam * (Jf - R(1)) - p.mu) * Jf;
    tau[0] += diag;
    tau[4] += diag;
    tau[8] += diag;
    return std::isfinite(tau[0]);
  }
  if (p.type == ORC_NHK) {
    const R Jf = det3(F);
    if (!(Jf > R(0))) return false;
    for (int i = 0; i < 9; ++i) tau[i] = p.mu * B[i];
    const R diag = -p.mu + p.lam * std::log(Jf);
    tau[0] += diag;
    tau[4] += diag;
    tau[8] += diag;
    return true;
  }
  R w[3], Q[9];
  sym_eig3(B, w, Q, kSweeps);
  if (p.type == ORC_FCR) {
    const R Jf = det3(F);
    R sig[3];
    for (int k = 0; k < 3; ++k) sig[k] = std::sqrt(std::max(w[k], R(0)));
    if (Jf < R(0)) {
      int kmin = 0;
      for (int k = 1; k < 3; ++k)
        if (sig[k] < sig[kmin]) kmin = k;
      sig[kmin] = -sig[kmin];
    }
    R S[9];
    qdqt(Q, sig, S);
    for (int i = 0; i < 9; ++i) tau[i] = R(2) * p.mu * (B[i] - S[i]);
    const R diag = p.lam * (Jf - R(1)) * Jf;
    tau[0] += diag;
    tau[4] += diag;
    tau[8] += diag;
    return std::isfinite(tau[0]);
  }
  // StVK with Hencky strain
  R eps[3];
  for (int k = 0; k < 3; ++k) {
    if (!(w[k] > R(0))) return false;
    eps[k] = R(0.5) * std::log(w[k]);
  }
  const R tr = eps[0] + eps[1] + eps[2];
  R d[3];
  for (int k = 0; k < 3; ++k) d[k] = R(2) * p.mu * eps[k] + p.lam * tr;
  qdqt(Q, d, tau);
  return true;
}

// Non-associative Drucker-Prager return mapping in Hencky strain space
// (Klar et al. 2016, Alg. 2 / sec. 7.3); applied by the reference's
// ZSReturnMapping node after G2P (MPMPipeline.cu:958-971).  With
// F = U S V^T and B = F F^T = U S^2 U^T, the projected F is
// U S' V^T = U (S'/S) U^T F.
template <class R> int project_dp(const Params<R> &p, R *F) {
  R B[9], w[3], Q[9];
  mul_ABt(F, F, B);
  sym_eig3(B, w, Q, kSweeps);
  R sig[3], eps[3];
  for (int k = 0; k < 3; ++k) {
    sig[k] = std::sqrt(std::max(w[k], R(0)));
    if (!(sig[k] > R(0))) return -1;
    eps[k] = std::log(sig[k]);
  }
  const R tr = eps[0] + eps[1] + eps[2];
  R sig_new[3];
  if (tr >= R(0)) {
    sig_new[0] = sig_new[1] = sig_new[2] = R(1);
  } else {
    R ehat[3];
    for (int k = 0; k < 3; ++k) ehat[k] = eps[k] - tr / R(3);
    const R nrm = std::sqrt(ehat[0] * ehat[0] + ehat[1] * ehat[1] + ehat[2] * ehat[2]);
    const R dg = nrm + (R(3) * p.lam + R(2) * p.mu) / (R(2) * p.mu) * tr * p.alpha;
    if (dg <= R(0)) return 0;
    for (int k = 0; k < 3; ++k) sig_new[k] = std::exp(eps[k] - dg / nrm * ehat[k]);
  }
  R ratio[3], Mr[9], Fn[9];
  for (int k = 0; k < 3; ++k) ratio[k] = sig_new[k] / sig[k];
  qdqt(Q, ratio, Mr);
  mul_AB(Mr, F, Fn);
  for (int i = 0; i < 9; ++i) F[i] = Fn[i];
  return 1;
}

// Von Mises and Cam-Clay return mappings in Hencky strain space (the navm /
// nacc options of ConfigConstitutiveModel, Generation.cu:71-82, applied by
// ZSReturnMapping, MPMPipeline.cu:958-971).  With F = U S V^T and the log
// stretches e = ln S, a rule moves e to e' and F <- U exp(e') V^T =
// U (exp(e')/S) U^T F.  On h = e - tr(e)/3:
//   von Mises (Jiang et al. 2016, "The Material Point Method for Simulating
//     Continuum Materials", SIGGRAPH course, sec. 8.2): if
//     dg = |h| - yield / (2 mu) > 0, e' = e - dg h / |h|;
//   Cam-Clay (Gaume et al. 2018, "Dynamic anticrack propagation in snow",
//     Nat. Commun. 9:3047, Methods): p = -kappa tr(e) (kappa = lam + 2mu/3),
//     q = sqrt(3/2) 2mu |h|, p0 = kappa sinh(xi max(-log Jp, 0)); states past
//     the caps go to (p0, 0) / (-beta p0, 0); outside the ellipse
//     q^2 (1 + 2 beta) + M^2 (p + beta p0)(p - p0) = 0 they move along the
//     line to its centre ((1 - beta) p0 / 2, 0) onto it; e' keeps the
//     direction of h with |h'| = q' / (sqrt(3/2) 2mu) and tr(e') = -p'/kappa;
//     log Jp += tr(e) - tr(e').
template <class R> int project_hencky(const Params<R> &p, R *F, R &logJp) {
  R B[9], w[3], Q[9];
  mul_ABt(F, F, B);
  sym_eig3(B, w, Q, kSweeps);
  R sig[3], e[3];
  for (int k = 0; k < 3; ++k) {
    sig[k] = std::sqrt(std::max(w[k], R(0)));
    if (!(sig[k] > R(0))) return -1;
    e[k] = std::log(sig[k]);
  }
  const R tr = e[0] + e[1] + e[2];
  R h[3];
  for (int k = 0; k < 3; ++k) h[k] = e[k] - tr / R(3);
  const R nrm = std::sqrt(h[0] * h[0] + h[1] * h[1] + h[2] * h[2]);
  R hs = R(1), trn = tr;
  bool projected = false;
  if (p.plastic == ORC_PLASTIC_NAVM) {
    const R dg = nrm - p.yield / (R(2) * p.mu);
    if (dg > R(0)) {
      hs = R(1) - dg / nrm;
      projected = true;
    }
  } else {
    const R kappa = p.lam + R(2) * p.mu / R(3);
    const R p0 = kappa * std::sinh(p.ccxi * std::max(-logJp, R(0)));
    const R beta = p.ccbeta, M = p.ccM;
    const R pr = -kappa * tr, q = std::sqrt(R(1.5)) * R(2) * p.mu * nrm;
    R pn = pr, qn = q;
    if (pr > p0) {
      pn = p0;
      qn = R(0);
      projected = true;
    } else if (pr < -beta * p0) {
      pn = -beta * p0;
      qn = R(0);
      projected = true;
    } else if (q * q * (R(1) + R(2) * beta) + M * M * (pr + beta * p0) * (pr - p0) > R(0)) {
      const R pc = R(0.5) * (R(1) - beta) * p0, a = R(0.5) * (R(1) + beta) * p0, dp = pr - pc;
      const R t = M * a / std::sqrt(q * q * (R(1) + R(2) * beta) + M * M * dp * dp);
      pn = pc + t * dp;
      qn = t * q;
      projected = true;
    }
    if (projected) {
      trn = -pn / kappa;
      hs = q > R(0) ? qn / q : R(0);
      logJp += tr - trn;
    }
  }
  if (!projected) return 0;
  R ratio[3], Mr[9], Fn[9];
  for (int k = 0; k < 3; ++k) ratio[k] = std::exp(hs * h[k] + trn / R(3)) / sig[k];
  qdqt(Q, ratio, Mr);
  mul_AB(Mr, F, Fn);
  for (int i = 0; i < 9; ++i) F[i] = Fn[i];
  return 1;
}

struct Partition {
  std::vector<int32_t> pb_dir;   // directory index of each particle block (sorted)
  std::vector<int64_t> pb_start; // offset of the block in perm
  std::vector<int32_t> pb_count;
  std::vector<int64_t> perm;     // sorted position -> particle index
  std::vector<int32_t> gb_dir;   // directory index of each grid block (sorted)
  std::vector<int32_t> dir2gb;   // directory index -> grid block or -1
};

struct Dir {
  int32_t lo[3], dims[3];
  int64_t size() const { return int64_t(dims[0]) * dims[1] * dims[2]; }
  void coords(int64_t d, int32_t *c) const {
    c[2] = int32_t(d % dims[2]);
    c[1] = int32_t((d / dims[2]) % dims[1]);
    c[0] = int32_t(d / (int64_t(dims[1]) * dims[2]));
  }
  int64_t index(const int32_t *c) const {
    return (int64_t(c[0]) * dims[1] + c[1]) * dims[2] + c[2];
  }
};

// Block of a particle: base = floor(x / dx - 0.5), key = base - (base & 3)
// (MPMPipeline.cu:78-83).  Computed in the precision of R: one rounded
// multiply by 1/dx, one rounded subtraction of 0.5, then floor.
template <class R> inline void particle_base(const R *x, R inv_dx, int32_t *base) {
  for (int d = 0; d < 3; ++d) {
    R c = x[d] * inv_dx;
    c = c - R(0.5);
    base[d] = int32_t(std::floor(c));
  }
}

// Partition + 1-ring expansion (ZSPartitionForZSParticles followed by one
// iteration of ExpandZSPartition over all 26 neighbours).  Particle blocks
// are sorted by directory index; inside a block particles are ordered by
// (cell id, particle index), which is the stable order by (block, cell).
// extra: point sets (cloth vertices and elements) whose blocks and their 26
// neighbours join the grid blocks without forming particle blocks
struct PointSet {
  const double *x;
  int64_t n;
};

template <class R>
int build_partition(const orc_scene &sc, int64_t n, const R *x, Partition &P, int nthreads,
                    const std::vector<PointSet> &extra = {}) {
  Dir dir;
  for (int d = 0; d < 3; ++d) {
    dir.lo[d] = sc.block_lo[d];
    dir.dims[d] = sc.block_dims[d];
    if (dir.dims[d] < 3) return ORC_ERR_INVALID;
  }
  const int64_t D = dir.size();
  if (D >= (int64_t(1) << 26)) return ORC_ERR_INVALID;
  const R inv_dx = R(1) / R(sc.dx);
  std::vector<int32_t> key(n);  // directory index * 64 + cell
  int bad = 0;
#pragma omp parallel for num_threads(nthreads) reduction(| : bad) schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    int32_t base[3], bc[3];
    particle_base(x + 3 * i, inv_dx, base);
    bool ok = true;
    for (int d = 0; d < 3; ++d) {
      bc[d] = (base[d] >> 2) - dir.lo[d];
      if (bc[d] < 1 || bc[d] > dir.dims[d] - 2) ok = false;
    }
    if (!ok) {
      bad |= 1;
      key[i] = -1;
      continue;
    }
    // z-major cell id inside the block, (z << 4) | (x << 2) | y
    const int32_t cell = ((base[2] & 3) << 4) | ((base[0] & 3) << 2) | (base[1] & 3);
    key[i] = int32_t(dir.index(bc) * 64 + cell);
  }
  if (bad) return ORC_ERR_OUT_OF_DOMAIN;

  // counting sort by block, stable in particle index
  std::vector<int64_t> count(D + 1, 0);
  for (int64_t i = 0; i < n; ++i) count[key[i] >> 6]++;
  std::vector<int64_t> start(D + 1, 0);
  for (int64_t d = 0; d < D; ++d) start[d + 1] = start[d] + count[d];
  std::vector<int64_t> tmp(n), fill(start.begin(), start.end());
  for (int64_t i = 0; i < n; ++i) tmp[fill[key[i] >> 6]++] = i;

  P.pb_dir.clear();
  P.pb_start.clear();
  P.pb_count.clear();
  for (int64_t d = 0; d < D; ++d)
    if (count[d]) {
      P.pb_dir.push_back(int32_t(d));
      P.pb_start.push_back(start[d]);
      P.pb_count.push_back(int32_t(count[d]));
    }
  // inside each block: stable counting sort by cell id
  P.perm.assign(n, 0);
  const int64_t nb = int64_t(P.pb_dir.size());
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 16)
  for (int64_t b = 0; b < nb; ++b) {
    const int64_t s0 = P.pb_start[b], c = P.pb_count[b];
    int64_t cc[65] = {0};
    for (int64_t s = s0; s < s0 + c; ++s) cc[(key[tmp[s]] & 63) + 1]++;
    for (int k = 0; k < 64; ++k) cc[k + 1] += cc[k];
    for (int64_t s = s0; s < s0 + c; ++s) {
      const int64_t i = tmp[s];
      P.perm[s0 + cc[key[i] & 63]++] = i;
    }
  }

  // halo: every particle block and its 26 neighbours
  std::vector<uint8_t> mark(D, 0);
  for (const PointSet &ps : extra)
    for (int64_t i = 0; i < ps.n; ++i) {
      int32_t base[3], bc[3];
      particle_base(ps.x + 3 * i, 1.0 / double(sc.dx), base);
      for (int d = 0; d < 3; ++d) {
        bc[d] = (base[d] >> 2) - dir.lo[d];
        if (bc[d] < 1 || bc[d] > dir.dims[d] - 2) return ORC_ERR_OUT_OF_DOMAIN;
      }
      for (int a = -1; a <= 1; ++a)
        for (int b = -1; b <= 1; ++b)
          for (int c = -1; c <= 1; ++c) {
            const int32_t cn[3] = {bc[0] + a, bc[1] + b, bc[2] + c};
            mark[dir.index(cn)] = 1;
          }
    }
  for (int64_t b = 0; b < nb; ++b) {
    int32_t c[3];
    dir.coords(P.pb_dir[b], c);
    for (int i = -1; i <= 1; ++i)
      for (int j = -1; j <= 1; ++j)
        for (int k = -1; k <= 1; ++k) {
          const int32_t cn[3] = {c[0] + i, c[1] + j, c[2] + k};
          mark[dir.index(cn)] = 1;
        }
  }
  P.gb_dir.clear();
  P.dir2gb.assign(D, -1);
  for (int64_t d = 0; d < D; ++d)
    if (mark[d]) {
      P.dir2gb[d] = int32_t(P.gb_dir.size());
      P.gb_dir.push_back(int32_t(d));
    }
  return ORC_OK;
}

template <class R> struct Sim {
  // colliders with their moving state (b, s) in R
  struct Col {
    const orc_collider *c;
    R Rm[9], b[3], s;
  };
  std::vector<Col> cols;

  const orc_scene &sc;
  Dir dir;
  std::vector<Params<R>> mats;
  int nthreads;
  Partition P;
  // [gb][64][kNG] = m, mv (then v), and for the FLIP transfers vstar: the
  // momentum change of the grid forces (then the updated velocity)
  static constexpr int kNG = 7;
  std::vector<R> grid;
  R max_vel_sqr = 0;

  // Boundary grid nodes by node index (ZSBoundaryPrimitiveToZSGrid,
  // Transfer.cu:1532-1623, then UpdateZSGrid's boundary branch,
  // MPMPipeline.cu:899-911); the boundary points do not move.
  struct BNode {
    R m, v[3], n[3];
  };
  std::unordered_map<int64_t, BNode> bgrid;
  static int64_t node_key(const int32_t *I) {
    return ((int64_t(I[0]) + (1 << 20)) << 42) | ((int64_t(I[1]) + (1 << 20)) << 21) |
           (int64_t(I[2]) + (1 << 20));
  }
  void build_grid_boundary() {
    const orc_grid_boundary *gb = sc.grid_boundary;
    if (!gb) return;
    const float inv_dx = 1.0f / sc.dx;
    std::unordered_map<int64_t, std::array<R, 7>> acc;
    const int64_t np = gb->n_verts + gb->n_eles;
    for (int64_t p = 0; p < np; ++p) {
      // linear kernel: nodes base, base + 1 per axis, base = floor(x / dx)
      int32_t base[3];
      R w[3][2];
      for (int d = 0; d < 3; ++d) {
        const float c = gb->x[3 * p + d] * inv_dx;
        base[d] = int32_t(std::floor(c));
        const R f = R(c) - R(base[d]);
        w[d][0] = R(1) - f;
        w[d][1] = f;
      }
      const R m = R(gb->m[p]);
      const bool with_n = p >= gb->n_verts;
      for (int o = 0; o < 8; ++o) {
        const int32_t I[3] = {base[0] + (o >> 2), base[1] + ((o >> 1) & 1), base[2] + (o & 1)};
        const R W = w[0][o >> 2] * w[1][(o >> 1) & 1] * w[2][o & 1];
        auto &a = acc.try_emplace(node_key(I), std::array<R, 7>{}).first->second;
        a[0] += W * m;
        for (int d = 0; d < 3; ++d) a[1 + d] += W * m * R(gb->v[3 * p + d]);
        if (with_n)
          for (int d = 0; d < 3; ++d) a[4 + d] += W * m * R(gb->nrm[3 * p + d]);
      }
    }
    for (const auto &kv : acc) {
      const auto &a = kv.second;
      BNode b{};
      b.m = a[0];
      if (a[0] != R(0)) {
        for (int d = 0; d < 3; ++d) b.v[d] = a[1 + d] / a[0];
        // unit(nrm / m); a node no triangle reached keeps a zero normal
        const R nn = std::sqrt(a[4] * a[4] + a[5] * a[5] + a[6] * a[6]);
        if (nn > R(0))
          for (int d = 0; d < 3; ++d) b.n[d] = a[4 + d] / nn;
      }
      bgrid.emplace(kv.first, b);
    }
  }

  // ApplyGridBoundaryOnZSGrid (Boundary.cu:18-69) on the velocity of the
  // node at index I (a node of non-zero mass)
  void apply_grid_boundary(const int32_t *I, R *vel) const {
    if (bgrid.empty()) return;
    const auto it = bgrid.find(node_key(I));
    if (it == bgrid.end() || it->second.m == R(0)) return;
    const BNode &b = it->second;
    if (sc.grid_boundary->type == ORC_BC_STICKY) {
      for (int d = 0; d < 3; ++d) vel[d] = b.v[d];
      return;
    }
    R u[3];
    for (int d = 0; d < 3; ++d) u[d] = vel[d] - b.v[d];
    const R proj = b.n[0] * u[0] + b.n[1] * u[1] + b.n[2] * u[2];
    if (sc.grid_boundary->type == ORC_BC_SLIP || (sc.grid_boundary->type == ORC_BC_SEPARATE && proj < 0))
      for (int d = 0; d < 3; ++d) u[d] -= proj * b.n[d];
    for (int d = 0; d < 3; ++d) vel[d] = u[d] + b.v[d];
  }

  Sim(const orc_scene &s, int nt) : sc(s), nthreads(nt) {
    for (int d = 0; d < 3; ++d) {
      dir.lo[d] = s.block_lo[d];
      dir.dims[d] = s.block_dims[d];
    }
    for (int i = 0; i < s.n_materials; ++i) mats.push_back(material_params<R>(s.materials[i]));
    for (int i = 0; i < s.n_colliders; ++i) {
      Col c;
      c.c = &s.colliders[i];
      rotation_ypr(c.c->ypr_deg, c.Rm);
      for (int a = 0; a < 3; ++a) c.b[a] = R(c.c->translation[a]);
      c.s = R(c.c->scale);
      cols.push_back(c);
    }
    build_grid_boundary();
  }

  // R = Ry(yaw) Rx(pitch) Rz(roll), angles in degrees
  static void rotation_ypr(const float *ypr, R *Rm) {
    const R k = R(3.14159265358979323846) / R(180);
    const R cy = std::cos(R(ypr[0]) * k), sy = std::sin(R(ypr[0]) * k);
    const R cp = std::cos(R(ypr[1]) * k), sp = std::sin(R(ypr[1]) * k);
    const R cr = std::cos(R(ypr[2]) * k), sr = std::sin(R(ypr[2]) * k);
    const R Ry[9] = {cy, 0, sy, 0, 1, 0, -sy, 0, cy};
    const R Rx[9] = {1, 0, 0, 0, cp, -sp, 0, sp, cp};
    const R Rz[9] = {cr, -sr, 0, sr, cr, 0, 0, 0, 1};
    R A[9];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        A[i * 3 + j] = 0;
        for (int l = 0; l < 3; ++l) A[i * 3 + j] += Ry[i * 3 + l] * Rx[l * 3 + j];
      }
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        Rm[i * 3 + j] = 0;
        for (int l = 0; l < 3; ++l) Rm[i * 3 + j] += A[i * 3 + l] * Rz[l * 3 + j];
      }
  }

  // StepZSBoundary (Generation.cu:1662-1685): b += db/dt dt, s += ds/dt dt
  void step_colliders(R dt) {
    for (Col &c : cols) {
      for (int a = 0; a < 3; ++a) c.b[a] += R(c.c->translation_rate[a]) * dt;
      c.s += R(c.c->scale_rate) * dt;
    }
  }

  // Level-set collider `cl` at world position p (ApplyBoundaryOnZSGrid with a
  // level set, Boundary.cu:83-163): trilinear signed distance and its gradient
  // at X = R^T (p - b) / s; inside when negative; unit normal R grad phi /
  // |R grad phi|, collider velocity R v(X) + db/dt (Boundary.cu:299-301).
  // False outside the sample grid or outside the collider.
  bool collider_hit(const Col &cl, const R *p, R *nrm, R *vo) const {
    const orc_collider &c = *cl.c;
    R q[3], X[3], u[3], t[3];
    int64_t i0[3];
    for (int a = 0; a < 3; ++a) q[a] = (p[a] - cl.b[a]) / cl.s;
    for (int a = 0; a < 3; ++a) X[a] = cl.Rm[0 * 3 + a] * q[0] + cl.Rm[1 * 3 + a] * q[1] + cl.Rm[2 * 3 + a] * q[2];
    for (int a = 0; a < 3; ++a) {
      u[a] = (X[a] - R(c.origin[a])) / R(c.spacing);
      if (!(u[a] >= 0 && u[a] <= R(c.dims[a] - 1))) return false;
    }
    for (int a = 0; a < 3; ++a) {
      i0[a] = std::min<int64_t>(int64_t(std::floor(u[a])), c.dims[a] - 2);
      t[a] = u[a] - R(i0[a]);
    }
    const int64_t sx = 1, sy = c.dims[0], sz = int64_t(c.dims[0]) * c.dims[1];
    auto at = [&](const float *g, int dx, int dy, int dz) {
      return R(g[(i0[0] + dx) * sx + (i0[1] + dy) * sy + (i0[2] + dz) * sz]);
    };
    auto tri = [&](const float *g, R *grad) {
      R val = 0;
      if (grad) grad[0] = grad[1] = grad[2] = 0;
      for (int k = 0; k < 8; ++k) {
        const int bx = (k >> 2) & 1, by = (k >> 1) & 1, bz = k & 1;
        const R wx = bx ? t[0] : R(1) - t[0], wy = by ? t[1] : R(1) - t[1],
                wz = bz ? t[2] : R(1) - t[2];
        const R f = at(g, bx, by, bz);
        val += wx * wy * wz * f;
        if (grad) {
          grad[0] += (bx ? R(1) : R(-1)) * wy * wz * f;
          grad[1] += wx * (by ? R(1) : R(-1)) * wz * f;
          grad[2] += wx * wy * (bz ? R(1) : R(-1)) * f;
        }
      }
      return val;
    };
    R g[3];
    const R phi = tri(c.sdf, g);
    if (!(phi < 0)) return false;
    R nr[3];
    for (int a = 0; a < 3; ++a) nr[a] = cl.Rm[a * 3 + 0] * g[0] + cl.Rm[a * 3 + 1] * g[1] + cl.Rm[a * 3 + 2] * g[2];
    const R nn = std::sqrt(nr[0] * nr[0] + nr[1] * nr[1] + nr[2] * nr[2]);
    const R rn = nn > 0 ? R(1) / nn : R(0);
    for (int a = 0; a < 3; ++a) nrm[a] = nr[a] * rn;
    R vl[3] = {R(c.const_velocity[0]), R(c.const_velocity[1]), R(c.const_velocity[2])};
    if (c.velocity) {
      const int64_t plane = sz * c.dims[2];
      for (int a = 0; a < 3; ++a) vl[a] = tri(c.velocity + a * plane, nullptr);
    }
    for (int a = 0; a < 3; ++a)
      vo[a] = cl.Rm[a * 3 + 0] * vl[0] + cl.Rm[a * 3 + 1] * vl[1] + cl.Rm[a * 3 + 2] * vl[2] +
              R(c.translation_rate[a]);
    return true;
  }

  // The level-set colliders on the velocity of the node at index I, in order;
  // sticky / slip / separate as ApplyGridBoundaryOnZSGrid (Boundary.cu:56-67).
  void apply_colliders(const int32_t *I, R *vel) const {
    R p[3];
    for (int a = 0; a < 3; ++a) p[a] = R(I[a]) * R(sc.dx);
    for (const Col &cl : cols) {
      R nrm[3], vo[3];
      if (!collider_hit(cl, p, nrm, vo)) continue;
      if (cl.c->type == ORC_BC_STICKY) {
        for (int a = 0; a < 3; ++a) vel[a] = vo[a];
        continue;
      }
      const R proj = nrm[0] * (vel[0] - vo[0]) + nrm[1] * (vel[1] - vo[1]) + nrm[2] * (vel[2] - vo[2]);
      if (cl.c->type == ORC_BC_SLIP || (cl.c->type == ORC_BC_SEPARATE && proj < 0))
        for (int a = 0; a < 3; ++a) vel[a] -= proj * nrm[a];
    }
  }

  // Quadratic B-spline stencil (Hu et al. 2018 MLS-MPM; Jiang et al. 2016
  // course notes): f = x/dx - base in [0.5, 1.5),
  // w0 = (1.5-f)^2/2, w1 = 3/4 - (f-1)^2, w2 = (f-0.5)^2/2.
  // dw[d][o] = d w_o / d f, the derivative with respect to the particle's
  // position in cells: w0' = f - 3/2, w1' = -2 (f - 1), w2' = f - 1/2.
  struct Stencil {
    int32_t base[3];
    R fx[3];
    R w[3][3];
    R dw[3][3];
  };
  void stencil(const R *x, Stencil &st) const {
    const R inv_dx = R(1) / R(sc.dx);
    particle_base(x, inv_dx, st.base);
    for (int d = 0; d < 3; ++d) {
      const R f = x[d] * inv_dx - R(st.base[d]);
      st.fx[d] = f;
      st.w[d][0] = R(0.5) * (R(1.5) - f) * (R(1.5) - f);
      st.w[d][1] = R(0.75) - (f - R(1)) * (f - R(1));
      st.w[d][2] = R(0.5) * (f - R(0.5)) * (f - R(0.5));
      st.dw[d][0] = f - R(1.5);
      st.dw[d][1] = R(-2) * (f - R(1));
      st.dw[d][2] = f - R(0.5);
    }
  }
  R *node(const int32_t *I) {
    int32_t bc[3];
    for (int d = 0; d < 3; ++d) bc[d] = (I[d] >> 2) - dir.lo[d];
    const int32_t gb = P.dir2gb[dir.index(bc)];
    const int cell = ((I[0] & 3) << 4) | ((I[1] & 3) << 2) | (I[2] & 3);
    return &grid[(int64_t(gb) * 64 + cell) * kNG];
  }

  // ZSGridToZSParticle for tracker points (Transfer.cu:1259-1285): the
  // grid's "v" channel interpolated, x += v dt
  void tracker_g2p(orc_trackers &tk, double dt) {
    for (int64_t p = 0; p < tk.n; ++p) {
      Stencil st;
      stencil(tk.x + 3 * p, st);
      double vel[3] = {0, 0, 0};
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
          for (int k = 0; k < 3; ++k) {
            const int32_t I[3] = {st.base[0] + i, st.base[1] + j, st.base[2] + k};
            const double W = st.w[0][i] * st.w[1][j] * st.w[2][k];
            const R *nd = node(I);
            for (int a = 0; a < 3; ++a) vel[a] += W * nd[1 + a];
          }
      for (int a = 0; a < 3; ++a) {
        tk.v[3 * p + a] = vel[a];
        tk.x[3 * p + a] += vel[a] * dt;
      }
    }
  }

  // ---- codimensional cloth (FP64 only) ----
  //
  // Gram-Schmidt QR of the columns of F (Jiang et al. 2017, sec. 4): q0 =
  // f0 / |f0|, q1 the normalised part of f1 orthogonal to q0, q2 = q0 x q1;
  // R = Q^T F upper triangular with a signed R22 (negative once the element
  // is inverted through its normal).
  static void gram_schmidt(const double *F, double *Q, double *Rm) {
    double f[3][3];
    for (int j = 0; j < 3; ++j)
      for (int i = 0; i < 3; ++i) f[j][i] = F[i * 3 + j];
    auto dot = [](const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; };
    double q0[3], q1[3], q2[3];
    const double r00 = std::sqrt(dot(f[0], f[0]));
    for (int i = 0; i < 3; ++i) q0[i] = f[0][i] / r00;
    const double r01 = dot(q0, f[1]);
    double u[3];
    for (int i = 0; i < 3; ++i) u[i] = f[1][i] - r01 * q0[i];
    const double r11 = std::sqrt(dot(u, u));
    for (int i = 0; i < 3; ++i) q1[i] = u[i] / r11;
    q2[0] = q0[1] * q1[2] - q0[2] * q1[1];
    q2[1] = q0[2] * q1[0] - q0[0] * q1[2];
    q2[2] = q0[0] * q1[1] - q0[1] * q1[0];
    for (int i = 0; i < 3; ++i) {
      Q[i * 3 + 0] = q0[i];
      Q[i * 3 + 1] = q1[i];
      Q[i * 3 + 2] = q2[i];
    }
    for (int i = 0; i < 9; ++i) Rm[i] = 0;
    Rm[0] = r00;
    Rm[1] = r01;
    Rm[2] = dot(q0, f[2]);
    Rm[4] = r11;
    Rm[5] = dot(q1, f[2]);
    Rm[8] = dot(q2, f[2]);
  }

  // first Piola-Kirchhoff stress of a 2x2 deformation [a b; c d] (the
  // in-plane part of R): fixed corotated P = 2 mu (F - R) + lam (J - 1) cof F
  // (R the closest rotation, Stomakhin et al. 2012), Neo-Hookean P = mu (F -
  // F^-T) + lam ln J F^-T, StVK-Hencky P = U diag((2 mu e_i + lam sum e) /
  // s_i) V^T, e_i = ln s_i (Klar et al. 2016).
  static void first_piola_2d(int model, double mu, double lam, const double *F2, double *P2) {
    const double a = F2[0], b = F2[1], c = F2[2], d = F2[3];
    const double J = a * d - b * c;
    const double cof[4] = {d, -c, -b, a};  // J F^-T
    if (model == ORC_FCR) {
      const double p = a + d, q = c - b, nn = std::sqrt(p * p + q * q);
      const double Rr[4] = {p / nn, -q / nn, q / nn, p / nn};
      for (int i = 0; i < 4; ++i) P2[i] = 2 * mu * (F2[i] - Rr[i]) + lam * (J - 1) * cof[i];
      return;
    }
    if (model == ORC_NHK) {
      for (int i = 0; i < 4; ++i) P2[i] = mu * (F2[i] - cof[i] / J) + lam * std::log(J) * cof[i] / J;
      return;
    }
    // StVK-Hencky: P = F V diag((2 mu e_i + lam tr e) / s_i^2) V^T from F^T F = V S^2 V^T
    const double c00 = a * a + c * c, c01 = a * b + c * d, c11 = b * b + d * d;
    const double tr = c00 + c11, det = c00 * c11 - c01 * c01;
    const double disc = std::sqrt(std::max(0.0, 0.25 * tr * tr - det));
    const double l0 = 0.5 * tr + disc, l1 = 0.5 * tr - disc;
    double v0[2];
    if (std::fabs(c01) > 1e-300) {
      v0[0] = l0 - c11;
      v0[1] = c01;
    } else if (c00 >= c11) {
      v0[0] = 1;
      v0[1] = 0;
    } else {
      v0[0] = 0;
      v0[1] = 1;
    }
    const double nv = std::sqrt(v0[0] * v0[0] + v0[1] * v0[1]);
    v0[0] /= nv;
    v0[1] /= nv;
    const double v1[2] = {-v0[1], v0[0]};
    const double e0 = 0.5 * std::log(l0), e1 = 0.5 * std::log(l1);
    const double g0 = (2 * mu * e0 + lam * (e0 + e1)) / l0, g1 = (2 * mu * e1 + lam * (e0 + e1)) / l1;
    const double S[4] = {g0 * v0[0] * v0[0] + g1 * v1[0] * v1[0], g0 * v0[0] * v0[1] + g1 * v1[0] * v1[1],
                         g0 * v0[1] * v0[0] + g1 * v1[1] * v1[0], g0 * v0[1] * v0[1] + g1 * v1[1] * v1[1]};
    P2[0] = a * S[0] + b * S[2];
    P2[1] = a * S[1] + b * S[3];
    P2[2] = c * S[0] + d * S[2];
    P2[3] = c * S[1] + d * S[3];
  }

  // gradient of the node weight with respect to the particle position
  void weight_grad(const Stencil &st, int i, int j, int k, double *g) const {
    const double inv_dx = 1.0 / double(sc.dx);
    g[0] = st.dw[0][i] * st.w[1][j] * st.w[2][k] * inv_dx;
    g[1] = st.w[0][i] * st.dw[1][j] * st.w[2][k] * inv_dx;
    g[2] = st.w[0][i] * st.w[1][j] * st.dw[2][k] * inv_dx;
  }

  // p2g_curve (Transfer.cu:174-356) for one segment: the cross-section
  // block of R through the StVK-Hencky model, P00 = k (r00 - 1), P = Q P,
  // shear A (gamma) times the diagonal of R's cofactors over det R as the
  // reference computes it, the force P_c23 (d_c23^T grad W)(-vol dt) on the
  // element's nodes (type i), +-vol dt P_c0 DmInv00 on its two vertices
  // (type ii)
  void curve_p2g(orc_cloth &cl, int64_t e, const double *Q, const double *Rm, double dt,
                 std::vector<double> &imp) {
    const int tr = sc.transfer;
    const bool flip_style = tr != ORC_TRANSFER_APIC, affine = tr != ORC_TRANSFER_FLIP;
    const double dx = sc.dx;
    const double *dm = cl.ed + 9 * e, *Di = cl.eDmInv + 9 * e;
    const double R2[4] = {Rm[4], Rm[5], 0.0, Rm[8]};
    double P2[4];
    first_piola_2d(ORC_STVK, cl.emu[e], cl.elam[e], R2, P2);
    double Pl[9] = {double(cl.k) * (Rm[0] - 1), 0, 0, 0, P2[0], P2[1], 0, P2[2], P2[3]}, P[9];
    mul_AB(Q, Pl, P);
    const double g = cl.gamma;
    const double rr = Rm[1] * Rm[1] + Rm[2] * Rm[2];
    double A[9] = {rr * g, (Rm[4] * Rm[1] + Rm[5] * Rm[2]) * g, Rm[8] * Rm[2] * g, 0, 0, 0, 0, 0, 0};
    A[3] = A[1];
    A[6] = A[2];
    double invJ = Rm[0] * Rm[4] * Rm[8];
    if (invJ != 0) invJ = 1 / invJ;
    const double Rit[9] = {Rm[4] * Rm[8] * invJ, 0, 0, 0, Rm[0] * Rm[8] * invJ, 0, 0, 0, Rm[0] * Rm[4] * invJ};
    double QA[9], T[9];
    mul_AB(Q, A, QA);
    mul_AB(QA, Rit, T);
    for (int i = 0; i < 9; ++i) P[i] += T[i];
    const double mass = cl.em[e], vol = cl.evol[e];
    const double *ve = cl.ev + 3 * e, *Ce = cl.eC + 9 * e;
    Stencil st;
    stencil(cl.ex + 3 * e, st);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        for (int k = 0; k < 3; ++k) {
          const int32_t I[3] = {st.base[0] + i, st.base[1] + j, st.base[2] + k};
          const double xixp[3] = {(i - st.fx[0]) * dx, (j - st.fx[1]) * dx, (k - st.fx[2]) * dx};
          const double W = st.w[0][i] * st.w[1][j] * st.w[2][k];
          double gw[3];
          weight_grad(st, i, j, k, gw);
          const double s1 = (dm[1] * gw[0] + dm[4] * gw[1] + dm[7] * gw[2]) * (-vol * dt);
          const double s2 = (dm[2] * gw[0] + dm[5] * gw[1] + dm[8] * gw[2]) * (-vol * dt);
          R *nd = node(I);
          nd[0] += W * mass;
          for (int a = 0; a < 3; ++a) {
            const double vft = P[a * 3 + 1] * s1 + P[a * 3 + 2] * s2;
            const double Cx = affine ? Ce[a * 3 + 0] * xixp[0] + Ce[a * 3 + 1] * xixp[1] + Ce[a * 3 + 2] * xixp[2] : 0.0;
            nd[1 + a] += W * mass * (ve[a] + Cx) + (flip_style ? 0.0 : vft);
            if (flip_style) nd[4 + a] += vft;
          }
        }
    const int32_t *t = cl.inds + 3 * e;
    for (int a = 0; a < 3; ++a) {
      const double f = vol * dt * P[a * 3 + 0] * Di[0];
      imp[3 * t[0] + a] += f;
      imp[3 * t[1] + a] -= f;
    }
  }

  // ZSParticleToZSGrid for the cloth (p2g_surface, Transfer.cu:656-842):
  // each element scatters its mass and momentum and the normal-direction
  // force P_c3 (grad W . d_c3) (-vol dt) (type i), and hands the in-plane
  // force to its vertices as impulses (type ii); then each vertex scatters
  // its mass, momentum and impulse.  FLIP grids take the forces in vstar.
  void cloth_p2g(orc_cloth &cl, double dt) {
    const int tr = sc.transfer;
    const bool flip_style = tr != ORC_TRANSFER_APIC, affine = tr != ORC_TRANSFER_FLIP;
    const double dx = sc.dx;
    std::vector<double> imp(3 * cl.n_verts, 0.0);
    const bool curve = cl.kind == ORC_MESH_CURVE;
    for (int64_t e = 0; e < cl.n_eles; ++e) {
      const double *F = cl.eF + 9 * e, *dm = cl.ed + 9 * e, *Di = cl.eDmInv + 9 * e;
      double Q[9], Rm[9];
      gram_schmidt(F, Q, Rm);
      if (curve) {
        curve_p2g(cl, e, Q, Rm, dt, imp);
        continue;
      }
      const double R2[4] = {Rm[0], Rm[1], Rm[3], Rm[4]};
      double P2[4];
      first_piola_2d(cl.model, cl.emu[e], cl.elam[e], R2, P2);
      double P[9];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
          P[i * 3 + j] = j < 2 ? Q[i * 3 + 0] * P2[0 * 2 + j] + Q[i * 3 + 1] * P2[1 * 2 + j] : 0.0;
      const double g = cl.gamma;
      double gf = 0;
      if (Rm[8] < 1) {
        const double vv = 1 - Rm[8];
        gf = -double(cl.k) * vv * vv;
      }
      double A[9] = {g * Rm[2] * Rm[2], g * Rm[2] * Rm[5], g * Rm[2] * Rm[8],
                     0, g * Rm[5] * Rm[5], g * Rm[5] * Rm[8], 0, 0, gf * Rm[8]};
      A[3] = A[1];
      A[6] = A[2];
      A[7] = A[5];
      // R^-1 of the upper-triangular R, then P += Q A R^-T
      const double i00 = 1 / Rm[0], i11 = 1 / Rm[4], i22 = 1 / Rm[8];
      const double i01 = -Rm[1] * i00 * i11, i12 = -Rm[5] * i11 * i22;
      const double i02 = (Rm[1] * Rm[5] - Rm[2] * Rm[4]) * i00 * i11 * i22;
      const double Ri[9] = {i00, i01, i02, 0, i11, i12, 0, 0, i22};
      double QA[9], T[9];
      mul_AB(Q, A, QA);
      mul_ABt(QA, Ri, T);
      for (int i = 0; i < 9; ++i) P[i] += T[i];
      const double Pc3[3] = {P[2], P[5], P[8]}, dc3[3] = {dm[2], dm[5], dm[8]};
      const double mass = cl.em[e], vol = cl.evol[e];
      const double *ve = cl.ev + 3 * e, *Ce = cl.eC + 9 * e;
      Stencil st;
      stencil(cl.ex + 3 * e, st);
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
          for (int k = 0; k < 3; ++k) {
            const int32_t I[3] = {st.base[0] + i, st.base[1] + j, st.base[2] + k};
            const double xixp[3] = {(i - st.fx[0]) * dx, (j - st.fx[1]) * dx, (k - st.fx[2]) * dx};
            const double W = st.w[0][i] * st.w[1][j] * st.w[2][k];
            double gw[3];
            weight_grad(st, i, j, k, gw);
            const double s = (gw[0] * dc3[0] + gw[1] * dc3[1] + gw[2] * dc3[2]) * (-vol * dt);
            R *nd = node(I);
            nd[0] += W * mass;
            for (int a = 0; a < 3; ++a) {
              const double Cx = affine ? Ce[a * 3 + 0] * xixp[0] + Ce[a * 3 + 1] * xixp[1] + Ce[a * 3 + 2] * xixp[2] : 0.0;
              nd[1 + a] += W * mass * (ve[a] + Cx) + (flip_style ? 0.0 : Pc3[a] * s);
              if (flip_style) nd[4 + a] += Pc3[a] * s;
            }
          }
      // type (ii): vertex impulses from the in-plane columns of P
      const double r0[2] = {Di[0], Di[1]}, r1[2] = {Di[3], Di[4]};
      const int32_t *t = cl.inds + 3 * e;
      for (int vi = 0; vi < 3; ++vi) {
        double Dr[2], coeff;
        if (vi == 0) {
          Dr[0] = r0[0] + r1[0];
          Dr[1] = r0[1] + r1[1];
          coeff = vol * dt;
        } else {
          const double *r = vi == 1 ? r0 : r1;
          Dr[0] = r[0];
          Dr[1] = r[1];
          coeff = -vol * dt;
        }
        for (int a = 0; a < 3; ++a) imp[3 * t[vi] + a] += coeff * (P[a * 3 + 0] * Dr[0] + P[a * 3 + 1] * Dr[1]);
      }
    }
    // vertex bending springs (p2g_vert_bending_force, Transfer.cu:357-400):
    // while a spring between the two vertices opposite an interior edge is
    // shorter than its rest length, impulses -+ t^2 len k (1 - len / rl) dt
    // along x1 - x0 on its ends, scattered with each end's weights -- the
    // same sums as adding them to the ends' vertex impulses
    for (int64_t s = 0; s < cl.n_springs; ++s) {
      const int32_t a0 = cl.spring_v[2 * s], a1 = cl.spring_v[2 * s + 1];
      const double *x0 = cl.vx + 3 * a0, *x1 = cl.vx + 3 * a1;
      double dir[3] = {x1[0] - x0[0], x1[1] - x0[1], x1[2] - x0[2]};
      const double len = std::sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
      const double rl = cl.spring_rl[s];
      if (!(len < rl) || len == 0) continue;
      const double c = cl.thickness * cl.thickness * len * cl.spring_k[s] * (1 - len / rl) * dt / len;
      for (int a = 0; a < 3; ++a) {
        imp[3 * a0 + a] -= c * dir[a];
        imp[3 * a1 + a] += c * dir[a];
      }
    }
    for (int64_t p = 0; p < cl.n_verts; ++p) {
      const double mass = cl.vm[p], *vp = cl.vv + 3 * p, *Cp = cl.vC + 9 * p;
      Stencil st;
      stencil(cl.vx + 3 * p, st);
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
          for (int k = 0; k < 3; ++k) {
            const int32_t I[3] = {st.base[0] + i, st.base[1] + j, st.base[2] + k};
            const double xixp[3] = {(i - st.fx[0]) * dx, (j - st.fx[1]) * dx, (k - st.fx[2]) * dx};
            const double W = st.w[0][i] * st.w[1][j] * st.w[2][k];
            R *nd = node(I);
            nd[0] += W * mass;
            for (int a = 0; a < 3; ++a) {
              const double Cx = affine ? Cp[a * 3 + 0] * xixp[0] + Cp[a * 3 + 1] * xixp[1] + Cp[a * 3 + 2] * xixp[2] : 0.0;
              if (flip_style) {
                nd[1 + a] += W * mass * (vp[a] + Cx);
                nd[4 + a] += W * imp[3 * p + a];
              } else {
                nd[1 + a] += W * (mass * (vp[a] + Cx) + imp[3 * p + a]);
              }
            }
          }
    }
  }

  // affine velocity Dinv sum W u_i (x_i - x_p)^T at x with u = v or vstar,
  // and sum W v, sum W vstar; symmetric part damped by (1 - dc)
  void cloth_gather(const double *x, bool use_vstar, double dc, double *vel, double *vs,
                    double *Cn) {
    const double dx = sc.dx, Dinv = 4.0 / (dx * dx);
    Stencil st;
    stencil(x, st);
    for (int a = 0; a < 3; ++a) vel[a] = vs[a] = 0;
    for (int i = 0; i < 9; ++i) Cn[i] = 0;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        for (int k = 0; k < 3; ++k) {
          const int32_t I[3] = {st.base[0] + i, st.base[1] + j, st.base[2] + k};
          const double xixp[3] = {(i - st.fx[0]) * dx, (j - st.fx[1]) * dx, (k - st.fx[2]) * dx};
          const double W = st.w[0][i] * st.w[1][j] * st.w[2][k];
          const R *nd = node(I);
          for (int a = 0; a < 3; ++a) {
            vel[a] += W * nd[1 + a];
            vs[a] += W * nd[4 + a];
            const double u = use_vstar ? nd[4 + a] : nd[1 + a];
            for (int b = 0; b < 3; ++b) Cn[a * 3 + b] += W * Dinv * u * xixp[b];
          }
        }
    double D[9];
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b)
        D[a * 3 + b] = 0.5 * (Cn[a * 3 + b] - Cn[b * 3 + a]) + (1 - dc) * 0.5 * (Cn[a * 3 + b] + Cn[b * 3 + a]);
    for (int i = 0; i < 9; ++i) Cn[i] = D[i];
  }

  // ZSGridToZSParticle for the cloth (Transfer.cu:1287-1445): vertices as
  // damped APIC (or the FLIP-style blend with the vertices' beta), then elements: damped
  // C, centroid position and mean velocity of their vertices, d1 = p1 - p0,
  // d2 = p2 - p0, d3 += (dt C + dt^2 / 2 C^2) d3, F = d DmInv.
  void cloth_g2p(orc_cloth &cl, double dt) {
    const bool flip_style = sc.transfer != ORC_TRANSFER_APIC;
    const double dc = cl.dc;
    for (int64_t p = 0; p < cl.n_verts; ++p) {
      double vel[3], vs[3], Cn[9];
      cloth_gather(cl.vx + 3 * p, flip_style, dc, vel, vs, Cn);
      for (int a = 0; a < 3; ++a) {
        if (flip_style) {
          const double d0 = cl.vv[3 * p + a] - vel[a];
          const double beta = cl.vbeta ? cl.vbeta[p] : 0.0;
          cl.vv[3 * p + a] = vs[a] + 0.99 * d0;
          cl.vx[3 * p + a] += dt * (vs[a] + beta * 0.99 * d0);
        } else {
          cl.vv[3 * p + a] = vel[a];
          cl.vx[3 * p + a] += vel[a] * dt;
        }
      }
      for (int i = 0; i < 9; ++i) cl.vC[9 * p + i] = Cn[i];
    }
    for (int64_t e = 0; e < cl.n_eles; ++e) {
      double vel[3], vs[3], Cn[9];
      cloth_gather(cl.ex + 3 * e, flip_style, dc, vel, vs, Cn);
      for (int i = 0; i < 9; ++i) cl.eC[9 * e + i] = Cn[i];
      const int32_t *t = cl.inds + 3 * e;
      if (cl.kind == ORC_MESH_CURVE) {  // Transfer.cu:1445-1513
        const double *p0 = cl.vx + 3 * t[0], *p1 = cl.vx + 3 * t[1];
        double *d = cl.ed + 9 * e;
        double CC[9], M[9];
        mul_AB(Cn, Cn, CC);
        for (int i = 0; i < 9; ++i) M[i] = dt * Cn[i] + 0.5 * dt * dt * CC[i];
        double dn[9];
        for (int a = 0; a < 3; ++a) {
          cl.ex[3 * e + a] = (p0[a] + p1[a]) / 2;
          cl.ev[3 * e + a] = (cl.vv[3 * t[0] + a] + cl.vv[3 * t[1] + a]) / 2;
          dn[a * 3 + 0] = p1[a] - p0[a];
          for (int c = 1; c < 3; ++c)
            dn[a * 3 + c] = d[a * 3 + c] + M[a * 3 + 0] * d[0 * 3 + c] + M[a * 3 + 1] * d[1 * 3 + c] +
                            M[a * 3 + 2] * d[2 * 3 + c];
        }
        for (int i = 0; i < 9; ++i) d[i] = dn[i];
        mul_AB(d, cl.eDmInv + 9 * e, cl.eF + 9 * e);
        continue;
      }
      const double *p0 = cl.vx + 3 * t[0], *p1 = cl.vx + 3 * t[1], *p2 = cl.vx + 3 * t[2];
      double *d = cl.ed + 9 * e;
      double d3[3] = {d[2], d[5], d[8]}, CC[9], M[9], n3[3];
      mul_AB(Cn, Cn, CC);
      for (int i = 0; i < 9; ++i) M[i] = dt * Cn[i] + 0.5 * dt * dt * CC[i];
      for (int a = 0; a < 3; ++a) n3[a] = d3[a] + M[a * 3 + 0] * d3[0] + M[a * 3 + 1] * d3[1] + M[a * 3 + 2] * d3[2];
      for (int a = 0; a < 3; ++a) {
        cl.ex[3 * e + a] = (p0[a] + p1[a] + p2[a]) / 3;
        cl.ev[3 * e + a] = (cl.vv[3 * t[0] + a] + cl.vv[3 * t[1] + a] + cl.vv[3 * t[2] + a]) / 3;
        d[a * 3 + 0] = p1[a] - p0[a];
        d[a * 3 + 1] = p2[a] - p0[a];
        d[a * 3 + 2] = n3[a];
      }
      mul_AB(d, cl.eDmInv + 9 * e, cl.eF + 9 * e);
    }
  }

  // return_mapping_curve (MPMPipeline.cu:1012-1093) with its hard-coded
  // alpha = alpha_tangent = cohesion = 0: the cross-section's Hencky strain
  // e = ln |s| of R's lower-right block (|s| >= 128 eps) is projected to its
  // mean part when compressive (sum e < 0; to zero if already isotropic within
  // eps) and to zero otherwise, so that block becomes exp(e_mean) times its
  // closest rotation; the frictional shear (r01, r02) is then always removed
  // (zero cohesion cone).
  void curve_return_mapping(orc_cloth &cl, int64_t e, const double *Q, double *Rm) {
    const double feps = 1.1920928955078125e-07;
    const double a = Rm[4], b = Rm[5], c = Rm[7], dd = Rm[8];
    // singular values of [a b; c d]
    const double E = 0.5 * (a + dd), Fv = 0.5 * (a - dd), G = 0.5 * (c + b), H = 0.5 * (c - b);
    const double q = std::sqrt(E * E + H * H), r = std::sqrt(Fv * Fv + G * G);
    const double s0 = q + r, s1 = q - r;
    double eps[2] = {std::log(std::max(std::fabs(s0), feps * 128)), std::log(std::max(std::fabs(s1), feps * 128))};
    const double tr = eps[0] + eps[1];
    if (tr < 0) {
      const double h0 = eps[0] - 0.5 * tr, h1 = eps[1] - 0.5 * tr;
      const double hn = std::sqrt(h0 * h0 + h1 * h1);
      if (hn < feps)
        eps[0] = eps[1] = 0;
      else
        eps[0] = eps[1] = 0.5 * tr;
    } else {
      eps[0] = eps[1] = 0;
    }
    const double scale = std::exp(eps[0]);  // both equal
    const double p = a + dd, qq = c - b, nn = std::sqrt(p * p + qq * qq);
    Rm[4] = scale * p / nn;
    Rm[5] = -scale * qq / nn;
    Rm[7] = scale * qq / nn;
    Rm[8] = scale * p / nn;
    // shear: gamma == 0, or gamma |R2 r| > 0 with zero cohesion, clears it
    Rm[1] = Rm[2] = 0;
    mul_AB(Q, Rm, cl.ed + 9 * e);
    mul_AB(cl.ed + 9 * e, cl.eDmInv + 9 * e, cl.eF + 9 * e);
  }

  // ZSReturnMapping for the cloth (return_mapping_surface,
  // MPMPipeline.cu:973-1011) on R of d = Q R: no shear resistance beyond
  // friction, no tension across the normal; fc = tan(fa / pi) as the node
  // computes it (MPMPipeline.cu:1120).
  void cloth_return_mapping(orc_cloth &cl) {
    const double gamma = cl.gamma, k = cl.k, fc = std::tan(double(cl.fa) / 3.14159265358979323846);
    for (int64_t e = 0; e < cl.n_eles; ++e) {
      double *d = cl.ed + 9 * e;
      double Q[9], Rm[9];
      gram_schmidt(d, Q, Rm);
      if (cl.kind == ORC_MESH_CURVE) {
        curve_return_mapping(cl, e, Q, Rm);
        continue;
      }
      bool apply = false;
      if (gamma == 0) {
        Rm[2] = Rm[5] = 0;
        Rm[8] = std::min(Rm[8], 1.0);
        apply = true;
      } else if (Rm[8] > 1) {
        Rm[2] = Rm[5] = 0;
        Rm[8] = 1;
        apply = true;
      } else if (Rm[8] <= 0) {
        Rm[2] = Rm[5] = 0;
        Rm[8] = std::max(Rm[8], -1.0);
        apply = true;
      } else if (Rm[8] < 1) {
        const double rr = Rm[2] * Rm[2] + Rm[5] * Rm[5], r = Rm[8] - 1, gk = gamma / k;
        const double zz = fc * r * r;
        if (gk * gk * rr - zz * zz > 0) {
          const double scale = zz / (gk * std::sqrt(rr));
          Rm[2] *= scale;
          Rm[5] *= scale;
          apply = true;
        }
      }
      if (apply) {
        mul_AB(Q, Rm, d);
        mul_AB(d, cl.eDmInv + 9 * e, cl.eF + 9 * e);
      }
    }
  }

  int substep(int64_t n, R *x, R *v, R *C, R *F, R *J, const R *m, const R *vol,
              const int32_t *mat, const R *mu, const R *lam, const R *beta, R dt) {
    const int tr = sc.transfer;
    if (sc.collider_autostep) step_colliders(dt);  // the fused substep's collider time
    std::vector<PointSet> extra;
    if (std::is_same<R, double>::value && sc.cloth) {
      extra.push_back({sc.cloth->vx, sc.cloth->n_verts});
      extra.push_back({sc.cloth->ex, sc.cloth->n_eles});
    }
    if (std::is_same<R, double>::value && sc.trackers) extra.push_back({sc.trackers->x, sc.trackers->n});
    int rc = build_partition<R>(sc, n, x, P, nthreads, extra);
    if (rc) return rc;
    // ZSGridFromZSPartition: zero every channel of every block
    grid.assign(P.gb_dir.size() * 64 * kNG, R(0));

    const R dx = R(sc.dx), inv_dx = R(1) / dx;
    const R Dinv = R(4) * inv_dx * inv_dx;
    int bad = 0;

    // P2G in 8 parity colours of the particle-block coordinates: two blocks
    // of one colour are >= 2 blocks apart on some axis, so their stencils
    // (blocks K..K+1 per axis) never overlap.
    const int64_t nb = int64_t(P.pb_dir.size());
    for (int colour = 0; colour < 8; ++colour) {
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 1) reduction(| : bad)
      for (int64_t b = 0; b < nb; ++b) {
        int32_t c[3];
        dir.coords(P.pb_dir[b], c);
        if ((((c[0] & 1) << 2) | ((c[1] & 1) << 1) | (c[2] & 1)) != colour) continue;
        for (int64_t s = P.pb_start[b]; s < P.pb_start[b] + P.pb_count[b]; ++s) {
          const int64_t p = P.perm[s];
          Params<R> mp = mats[mat[p]];
          // per-particle override (Transfer.cu:861-864, 950-953); the FLIP
          // P2G has none (Transfer.cu:897-907)
          if (mu && lam && tr != ORC_TRANSFER_FLIP) {
            mp.mu = mu[p];
            mp.lam = lam[p];
          }
          R tau[9];
          if (!kirchhoff(mp, F + 9 * p, J[p], tau)) bad |= 1;
          // contrib = -dt Dinv vol P F^T (APIC, AFLIP), -dt vol P F^T (FLIP,
          // which contracts it with the weight gradient instead)
          R contrib[9];
          const R kc = tr == ORC_TRANSFER_FLIP ? -dt * vol[p] : -dt * Dinv * vol[p];
          for (int i = 0; i < 9; ++i) contrib[i] = kc * tau[i];
          Stencil st;
          stencil(x + 3 * p, st);
          const R *Cp = C + 9 * p, *vp = v + 3 * p;
          const R mass = m[p];
          for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j)
              for (int k = 0; k < 3; ++k) {
                const int32_t I[3] = {st.base[0] + i, st.base[1] + j, st.base[2] + k};
                const R xixp[3] = {(R(i) - st.fx[0]) * dx, (R(j) - st.fx[1]) * dx,
                                   (R(k) - st.fx[2]) * dx};
                const R W = st.w[0][i] * st.w[1][j] * st.w[2][k];
                R *g = node(I);
                g[0] += mass * W;
                if (tr == ORC_TRANSFER_FLIP) {
                  // Transfer.cu:924-934: v += W m v_p, vstar += W (contrib grad W)
                  // with grad W = d W / d x_p
                  const R gw[3] = {st.dw[0][i] * st.w[1][j] * st.w[2][k] * inv_dx,
                                   st.w[0][i] * st.dw[1][j] * st.w[2][k] * inv_dx,
                                   st.w[0][i] * st.w[1][j] * st.dw[2][k] * inv_dx};
                  for (int d = 0; d < 3; ++d) {
                    const R fdt = contrib[d * 3 + 0] * gw[0] + contrib[d * 3 + 1] * gw[1] +
                                  contrib[d * 3 + 2] * gw[2];
                    g[1 + d] += W * mass * vp[d];
                    g[4 + d] += W * fdt;
                  }
                  continue;
                }
                for (int d = 0; d < 3; ++d) {
                  const R Cx = Cp[d * 3 + 0] * xixp[0] + Cp[d * 3 + 1] * xixp[1] +
                               Cp[d * 3 + 2] * xixp[2];
                  const R fdt = contrib[d * 3 + 0] * xixp[0] + contrib[d * 3 + 1] * xixp[1] +
                                contrib[d * 3 + 2] * xixp[2];
                  if (tr == ORC_TRANSFER_AFLIP) {  // Transfer.cu:976-980
                    g[1 + d] += W * (mass * (vp[d] + Cx));
                    g[4 + d] += W * fdt;
                  } else {
                    g[1 + d] += W * (mass * (vp[d] + Cx) + fdt);
                  }
                }
              }
        }
      }
    }

    if constexpr (std::is_same<R, double>::value)
      if (sc.cloth) cloth_p2g(*sc.cloth, double(dt));

    // UpdateZSGrid (APIC branch) then ApplyBoundaryOnZSGrid, node-wise
    const int64_t ng = int64_t(P.gb_dir.size());
    R vmax = 0;
    const R g[3] = {R(sc.gravity[0]), R(sc.gravity[1]), R(sc.gravity[2])};
#pragma omp parallel for num_threads(nthreads) reduction(max : vmax) schedule(static)
    for (int64_t gb = 0; gb < ng; ++gb) {
      int32_t c[3];
      dir.coords(P.gb_dir[gb], c);
      for (int cell = 0; cell < 64; ++cell) {
        R *nd = &grid[(gb * 64 + cell) * kNG];
        if (nd[0] == R(0)) continue;
        const R rm = R(1) / nd[0];
        const int32_t I[3] = {(c[0] + dir.lo[0]) * 4 + (cell >> 4),
                              (c[1] + dir.lo[1]) * 4 + ((cell >> 2) & 3),
                              (c[2] + dir.lo[2]) * 4 + (cell & 3)};
        R vel[3];
        if (tr == ORC_TRANSFER_APIC) {
          for (int d = 0; d < 3; ++d) vel[d] = nd[1 + d] * rm + g[d] * dt;
          vmax = std::max(vmax, vel[0] * vel[0] + vel[1] * vel[1] + vel[2] * vel[2]);
          apply_bc(I, vel);
          apply_colliders(I, vel);
          apply_grid_boundary(I, vel);
          for (int d = 0; d < 3; ++d) nd[1 + d] = vel[d];
        } else {
          // MPMPipeline.cu:882-893: v = mv / m; vstar = vstar / m + v + g dt;
          // MaxVelSqr of vstar; the boundary acts on vstar (Boundary.cu:90-101)
          R vs[3];
          for (int d = 0; d < 3; ++d) {
            vel[d] = nd[1 + d] * rm;
            vs[d] = nd[4 + d] * rm + vel[d] + g[d] * dt;
          }
          vmax = std::max(vmax, vs[0] * vs[0] + vs[1] * vs[1] + vs[2] * vs[2]);
          apply_bc(I, vs);
          apply_colliders(I, vs);
          apply_grid_boundary(I, vs);
          for (int d = 0; d < 3; ++d) {
            nd[1 + d] = vel[d];
            nd[4 + d] = vs[d];
          }
        }
      }
    }
    max_vel_sqr = vmax;

    // G2P (+ F update) and the Drucker-Prager return mapping
#pragma omp parallel for num_threads(nthreads) schedule(static) reduction(| : bad)
    for (int64_t p = 0; p < n; ++p) {
      Stencil st;
      stencil(x + 3 * p, st);
      // vel = sum W v_i; vs = sum W vstar_i (FLIP transfers); Cn = Dinv sum W
      // u_i (x_i - x_p)^T with u = v (APIC) or vstar (AFLIP), or the velocity
      // gradient sum vstar_i (grad W)^T (FLIP)
      R vel[3] = {0, 0, 0}, vs[3] = {0, 0, 0}, Cn[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
          for (int k = 0; k < 3; ++k) {
            const int32_t I[3] = {st.base[0] + i, st.base[1] + j, st.base[2] + k};
            const R xixp[3] = {(R(i) - st.fx[0]) * dx, (R(j) - st.fx[1]) * dx,
                               (R(k) - st.fx[2]) * dx};
            const R W = st.w[0][i] * st.w[1][j] * st.w[2][k];
            const R *gv = node(I) + 1, *gs = node(I) + 4;
            if (tr == ORC_TRANSFER_FLIP) {
              const R gw[3] = {st.dw[0][i] * st.w[1][j] * st.w[2][k] * inv_dx,
                               st.w[0][i] * st.dw[1][j] * st.w[2][k] * inv_dx,
                               st.w[0][i] * st.w[1][j] * st.dw[2][k] * inv_dx};
              for (int a = 0; a < 3; ++a) {
                vel[a] += gv[a] * W;
                vs[a] += gs[a] * W;
                for (int bb = 0; bb < 3; ++bb) Cn[a * 3 + bb] += gs[a] * gw[bb];
              }
              continue;
            }
            const R *gu = tr == ORC_TRANSFER_AFLIP ? gs : gv;
            for (int a = 0; a < 3; ++a) {
              vel[a] += gv[a] * W;
              vs[a] += gs[a] * W;
              for (int bb = 0; bb < 3; ++bb) Cn[a * 3 + bb] += W * Dinv * gu[a] * xixp[bb];
            }
          }
      if (tr == ORC_TRANSFER_APIC) {
        for (int a = 0; a < 3; ++a) {
          v[3 * p + a] = vel[a];
          x[3 * p + a] += vel[a] * dt;
        }
        for (int i = 0; i < 9; ++i) C[9 * p + i] = Cn[i];
      } else {
        // Transfer.cu:1203-1211 (AFLIP), 1245-1250 (FLIP): flip = 0.99,
        // v = vstar + flip (v_p - vel); AFLIP x += dt (vstar + beta flip
        // (v_p - vel)) and C = Cn; FLIP x += dt vstar, C unchanged
        const R flip = R(0.99);
        const R bp = beta ? beta[p] : R(0);
        for (int a = 0; a < 3; ++a) {
          const R d0 = v[3 * p + a] - vel[a];
          v[3 * p + a] = vs[a] + flip * d0;
          x[3 * p + a] += tr == ORC_TRANSFER_AFLIP ? dt * (vs[a] + bp * flip * d0) : vs[a] * dt;
        }
        if (tr == ORC_TRANSFER_AFLIP)
          for (int i = 0; i < 9; ++i) C[9 * p + i] = Cn[i];
      }
      const Params<R> &mp = mats[mat[p]];
      R *Fp = F + 9 * p;
      if (mp.type == ORC_EOS) {
        J[p] *= R(1) + dt * (Cn[0] + Cn[4] + Cn[8]);
        const R s = std::cbrt(J[p]);
        for (int i = 0; i < 9; ++i) Fp[i] = (i % 4 == 0) ? s : R(0);
      } else {
        R A[9], Fn[9];
        for (int i = 0; i < 9; ++i) A[i] = dt * Cn[i] + ((i % 4 == 0) ? R(1) : R(0));
        mul_AB(A, Fp, Fn);
        for (int i = 0; i < 9; ++i) Fp[i] = Fn[i];
        Params<R> pp = mp;
        if (mu && lam) {
          pp.mu = mu[p];
          pp.lam = lam[p];
        }
        if (mp.plastic == ORC_PLASTIC_NADP) {
          if (project_dp(pp, Fp) < 0) bad |= 1;
        } else if (mp.plastic == ORC_PLASTIC_NAVM || mp.plastic == ORC_PLASTIC_NACC) {
          if (project_hencky(pp, Fp, J[p]) < 0) bad |= 1;  // J holds log(Jp) for Cam-Clay
        }
        if (mp.plastic != ORC_PLASTIC_NACC) J[p] = det3(Fp);
      }
      for (int i = 0; i < 9; ++i)
        if (!std::isfinite(Fp[i])) bad |= 1;
      if (!std::isfinite(x[3 * p]) || !std::isfinite(x[3 * p + 1]) || !std::isfinite(x[3 * p + 2]))
        bad |= 1;
    }
    if constexpr (std::is_same<R, double>::value) {
      if (sc.cloth) {
        cloth_g2p(*sc.cloth, double(dt));
        cloth_return_mapping(*sc.cloth);
      }
      if (sc.trackers) tracker_g2p(*sc.trackers, double(dt));
    }
    return bad ? ORC_ERR_NAN : ORC_OK;
  }

  // Box walls of the analytic collider in node-index space: a node is in the
  // lower wall of axis d when I_d < lo_d + thickness and in the upper wall
  // when I_d > hi_d - thickness.  Collider semantics follow
  // Boundary.cu:56-67 with a static wall (v_object = 0): sticky sets v to 0,
  // slip removes the wall-normal component, separate removes it only when it
  // points into the wall.
  void apply_bc(const int32_t *I, R *vel) const {
    if (sc.bc_type == ORC_BC_NONE) return;
    const int t = sc.bc_thickness;
    bool any = false;
    for (int d = 0; d < 3; ++d) {
      const bool lower = I[d] < sc.bc_lo[d] + t;
      const bool upper = I[d] > sc.bc_hi[d] - t;
      if (!(lower || upper)) continue;
      any = true;
      if (sc.bc_type == ORC_BC_SLIP) vel[d] = 0;
      if (sc.bc_type == ORC_BC_SEPARATE) {
        if (lower && vel[d] < 0) vel[d] = 0;
        if (upper && vel[d] > 0) vel[d] = 0;
      }
    }
    if (any && sc.bc_type == ORC_BC_STICKY) vel[0] = vel[1] = vel[2] = 0;
  }
};

template <class R>
int32_t run(const orc_scene *scene, int64_t n, R *x, R *v, R *C, R *F, R *J, const R *m,
            const R *vol, const int32_t *mat, const R *mu, const R *lam, const R *beta, R dt,
            int32_t nsteps, int32_t nthreads, orc_stats *stats) {
  if (!scene || n < 0 || nsteps < 0) return ORC_ERR_INVALID;
  if (scene->transfer < ORC_TRANSFER_APIC || scene->transfer > ORC_TRANSFER_AFLIP)
    return ORC_ERR_INVALID;
  if ((scene->cloth || scene->trackers) && !std::is_same<R, double>::value) return ORC_ERR_INVALID;
  for (int64_t p = 0; p < n; ++p)
    if (mat[p] < 0 || mat[p] >= scene->n_materials) return ORC_ERR_INVALID;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
  nthreads = 1;
#endif
  Sim<R> sim(*scene, nthreads);
  int32_t rc = ORC_OK;
  for (int32_t s = 0; s < nsteps && rc == ORC_OK; ++s)
    rc = sim.substep(n, x, v, C, F, J, m, vol, mat, mu, lam, beta, dt);
  if (stats) {
    stats->max_vel_sqr = double(sim.max_vel_sqr);
    stats->n_pblocks = int64_t(sim.P.pb_dir.size());
    stats->n_gblocks = int64_t(sim.P.gb_dir.size());
    stats->status = rc;
  }
  return rc;
}

}  // namespace

extern "C" {

int32_t orc_partition(const orc_scene *scene, int64_t n, const float *x, int64_t cap_pb,
                      int32_t *n_pb, int32_t *pb_dir, int32_t *pb_count, int64_t *perm,
                      int64_t cap_gb, int32_t *n_gb, int32_t *gb_dir) {
  if (!scene || n < 0) return ORC_ERR_INVALID;
  Partition P;
  int nt = 1;
#ifdef _OPENMP
  nt = omp_get_max_threads();
#endif
  const int rc = build_partition<float>(*scene, n, x, P, nt);
  if (rc) return rc;
  *n_pb = int32_t(P.pb_dir.size());
  *n_gb = int32_t(P.gb_dir.size());
  if (int64_t(P.pb_dir.size()) > cap_pb || int64_t(P.gb_dir.size()) > cap_gb)
    return ORC_ERR_CAPACITY;
  std::copy(P.pb_dir.begin(), P.pb_dir.end(), pb_dir);
  std::copy(P.pb_count.begin(), P.pb_count.end(), pb_count);
  std::copy(P.perm.begin(), P.perm.end(), perm);
  std::copy(P.gb_dir.begin(), P.gb_dir.end(), gb_dir);
  return ORC_OK;
}

int32_t orc_run_f64(const orc_scene *scene, int64_t n, double *x, double *v, double *C, double *F,
                    double *J, const double *m, const double *vol, const int32_t *mat,
                    const double *mu, const double *lam, const double *beta, double dt,
                    int32_t nsteps, int32_t nthreads, orc_stats *stats) {
  return run<double>(scene, n, x, v, C, F, J, m, vol, mat, mu, lam, beta, dt, nsteps, nthreads,
                     stats);
}

int32_t orc_run_f32(const orc_scene *scene, int64_t n, float *x, float *v, float *C, float *F,
                    float *J, const float *m, const float *vol, const int32_t *mat,
                    const float *mu, const float *lam, const float *beta, float dt,
                    int32_t nsteps, int32_t nthreads, orc_stats *stats) {
  return run<float>(scene, n, x, v, C, F, J, m, vol, mat, mu, lam, beta, dt, nsteps, nthreads,
                    stats);
}

// ComputeVonMises (Generation.cu:1873-1920): singular values of F from the
// eigenvalues of F^T F (Jacobi), Hencky strains e_i = ln s_i, principal
// Cauchy stresses c_i = (2 mu e_i + lam sum e) / (s0 s1 s2) of the
// StVK-Hencky model (Klar et al. 2016), vms = sqrt(((c0 - c1)^2 + (c1 - c2)^2
// + (c2 - c0)^2) / 2), log10(vms + 1) with by_log1p.
int32_t orc_von_mises_f64(const orc_scene *scene, int64_t n, const double *F, const int32_t *mat,
                          int32_t by_log1p, double *vms) {
  if (!scene || n < 0 || !vms) return ORC_ERR_INVALID;
  for (int64_t p = 0; p < n; ++p) {
    if (mat[p] < 0 || mat[p] >= scene->n_materials) return ORC_ERR_INVALID;
    const Params<double> mp = material_params<double>(scene->materials[mat[p]]);
    if (mp.type != ORC_STVK) continue;
    const double *Fp = F + 9 * p;
    double A[9], w[3], Q[9];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        A[i * 3 + j] = 0;
        for (int k = 0; k < 3; ++k) A[i * 3 + j] += Fp[k * 3 + i] * Fp[k * 3 + j];
      }
    sym_eig3<double>(A, w, Q, kSweeps);
    double e[3], tr = 0;
    for (int i = 0; i < 3; ++i) {
      e[i] = 0.5 * std::log(w[i]);
      tr += e[i];
    }
    const double J = std::exp(tr);
    double c[3];
    for (int i = 0; i < 3; ++i) c[i] = (2.0 * mp.mu * e[i] + mp.lam * tr) / J;
    double s2 = 0;
    for (int d = 0; d < 3; ++d) s2 += (c[d] - c[(d + 1) % 3]) * (c[d] - c[(d + 1) % 3]);
    const double v = std::sqrt(0.5 * s2);
    vms[p] = by_log1p ? std::log10(v + 1.0) : v;
  }
  return ORC_OK;
}

// ComputeParticleBeta (Boundary.cu:172-516) without a boundary (:490-499)
// and with a level-set boundary (determine_beta_sdf, :285-315): at
// x + dt v, a particle inside the collider moving into it, (v - v_obj) . n
// < 0, gets beta = 0; otherwise beta = 0.5 where J = det F > Jp_critical = 1
// (the value for every model here; 1.1 is the Cam-Clay one), else 0.  The
// equation-of-state fluid keeps J instead of F.
int32_t orc_particle_beta_f64(const orc_scene *scene, int64_t n, const double *x, const double *v,
                              const double *F, const double *J, const int32_t *mat, double dt,
                              int32_t collider, double *beta) {
  if (!scene || n < 0 || !beta || collider >= scene->n_colliders || collider < -2 ||
      (collider == -2 && !scene->grid_boundary))
    return ORC_ERR_INVALID;
  Sim<double> sim(*scene, 1);
  for (int64_t p = 0; p < n; ++p) {
    if (mat[p] < 0 || mat[p] >= scene->n_materials) return ORC_ERR_INVALID;
    if (collider == -2) {
      // the boundary grid (Boundary.cu:172-222): at x + dt v, a node of the
      // linear stencil with boundary mass where (v - v_b) . nrm_b < 0
      const float inv_dx = 1.0f / scene->dx;
      int32_t base[3];
      for (int a = 0; a < 3; ++a)
        base[a] = int32_t(std::floor(float(x[3 * p + a] + dt * v[3 * p + a]) * inv_dx));
      bool in = false;
      for (int o = 0; o < 8 && !in; ++o) {
        const int32_t I[3] = {base[0] + (o >> 2), base[1] + ((o >> 1) & 1), base[2] + (o & 1)};
        const auto it = sim.bgrid.find(sim.node_key(I));
        if (it == sim.bgrid.end() || it->second.m == 0) continue;
        const auto &b = it->second;
        in = (v[3 * p] - b.v[0]) * b.n[0] + (v[3 * p + 1] - b.v[1]) * b.n[1] +
                 (v[3 * p + 2] - b.v[2]) * b.n[2] < 0;
      }
      if (in) {
        beta[p] = 0;
        continue;
      }
    }
    if (collider >= 0) {
      double pos[3], nrm[3], vo[3];
      for (int a = 0; a < 3; ++a) pos[a] = x[3 * p + a] + dt * v[3 * p + a];
      if (sim.collider_hit(sim.cols[collider], pos, nrm, vo)) {
        const double vn = (v[3 * p] - vo[0]) * nrm[0] + (v[3 * p + 1] - vo[1]) * nrm[1] +
                          (v[3 * p + 2] - vo[2]) * nrm[2];
        if (vn < 0) {
          beta[p] = 0;
          continue;
        }
      }
    }
    const double Jp = sim.mats[mat[p]].type == ORC_EOS ? J[p] : det3(F + 9 * p);
    beta[p] = Jp > 1.0 ? 0.5 : 0.0;
  }
  return ORC_OK;
}

int32_t orc_cloth_beta_f64(const orc_scene *scene, orc_cloth *cl, double dt, int32_t collider) {
  if (!scene || !cl || !cl->vbeta || collider >= scene->n_colliders) return ORC_ERR_INVALID;
  if (cl->kind != ORC_MESH_SURFACE) return ORC_ERR_INVALID;
  Sim<double> sim(*scene, 1);
  for (int64_t e = 0; e < cl->n_eles; ++e) {
    const int32_t *t = cl->inds + 3 * e;
    const double *ve = cl->ev + 3 * e;
    double value = -1;
    if (collider >= 0) {
      double pos[3], nrm[3], vo[3];
      for (int a = 0; a < 3; ++a) pos[a] = cl->ex[3 * e + a] + dt * ve[a];
      if (sim.collider_hit(sim.cols[collider], pos, nrm, vo) &&
          (ve[0] - vo[0]) * nrm[0] + (ve[1] - vo[1]) * nrm[1] + (ve[2] - vo[2]) * nrm[2] < 0)
        value = 0;
    }
    if (value < 0) {
      double Q[9], Rm[9];
      Sim<double>::gram_schmidt(cl->ed + 9 * e, Q, Rm);
      const double Jn = std::fabs(Rm[0] * Rm[4] - Rm[3] * Rm[1]);
      const double J0inv = std::fabs(det3(cl->eDmInv + 9 * e));
      const double J = det3(cl->eF + 9 * e) / (Jn * J0inv);
      value = J > 1.0 ? 0.2 : 0.0;
    }
    for (int k = 0; k < 3; ++k) cl->vbeta[t[k]] = value;
  }
  return ORC_OK;
}

void orc_sym_eig3(const double *A, double *w, double *Q) { sym_eig3<double>(A, w, Q, kSweeps); }

int32_t orc_kirchhoff(const orc_material *mat, const double *F, double J, double *tau) {
  const Params<double> p = material_params<double>(*mat);
  return kirchhoff<double>(p, F, J, tau) ? 1 : 0;
}

int32_t orc_project_dp(const orc_material *mat, double *F) {
  const Params<double> p = material_params<double>(*mat);
  return project_dp<double>(p, F);
}

int32_t orc_project_hencky(const orc_material *mat, double *F, double *logJp) {
  const Params<double> p = material_params<double>(*mat);
  if (p.plastic != ORC_PLASTIC_NAVM && p.plastic != ORC_PLASTIC_NACC) return -2;
  double lj = logJp ? *logJp : 0.0;
  const int r = project_hencky<double>(p, F, lj);
  if (logJp) *logJp = lj;
  return r;
}

// ToZSCloth (Generation.cpp:489-688): per triangle, area A (double), vol =
// max(A dx, 10 eps_float), centroid position and velocity, d = [p1 - p0,
// p2 - p0, n] with n = normalize(normalize(d1) x normalize(d2)); each vertex
// gets a third of the volume of its triangles; m = vol density.  The rest
// shape D* = [|d1|, d1.d2/|d1|, 0; 0, |d1 x d2|/|d1|, 0; 0, 0, 1] (d1, d2 in
// the triangle's own frame: the reference rotates n to z and d1 to x),
// DmInv = D*^-1, F = d DmInv; a triangle with a near-zero side of D* gets
// mu = lam = 0.
int32_t orc_cloth_init_f64(int64_t n_verts, const float *x, const float *v, int64_t n_tris,
                           const int32_t *tris, float dx, float density, float E, float nu,
                           orc_cloth *out) {
  if (!out || n_verts < 0 || n_tris < 0) return ORC_ERR_INVALID;
  const float mu = E / (2.0f * (1.0f + nu)), lam = E * nu / ((1.0f + nu) * (1.0f - 2.0f * nu));
  std::vector<float> dof_vol(n_verts, 0.0f);
  const double feps = std::numeric_limits<float>::epsilon();
  for (int64_t e = 0; e < n_tris; ++e) {
    const int32_t *t = tris + 3 * e;
    for (int i = 0; i < 3; ++i)
      if (t[i] < 0 || t[i] >= n_verts) return ORC_ERR_INVALID;
    double p[3][3];
    for (int i = 0; i < 3; ++i)
      for (int a = 0; a < 3; ++a) p[i][a] = x[3 * t[i] + a];
    double e1[3], e2[3], cr[3];
    for (int a = 0; a < 3; ++a) {
      e1[a] = p[1][a] - p[0][a];
      e2[a] = p[2][a] - p[0][a];
    }
    cr[0] = e1[1] * e2[2] - e1[2] * e2[1];
    cr[1] = e1[2] * e2[0] - e1[0] * e2[2];
    cr[2] = e1[0] * e2[1] - e1[1] * e2[0];
    const double area = 0.5 * std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
    const float vol = float(std::max(area * double(dx), feps * 10.0));
    out->evol[e] = vol;
    out->em[e] = double(vol * density);
    for (int a = 0; a < 3; ++a) {
      const float c = (x[3 * t[0] + a] + x[3 * t[1] + a] + x[3 * t[2] + a]) / 3.0f;
      out->ex[3 * e + a] = c;
      out->ev[3 * e + a] = v ? double((v[3 * t[0] + a] + v[3 * t[1] + a] + v[3 * t[2] + a]) / 3.0f) : 0.0;
    }
    // d columns in float as the reference stores them
    float d1[3], d2[3];
    for (int a = 0; a < 3; ++a) {
      d1[a] = x[3 * t[1] + a] - x[3 * t[0] + a];
      d2[a] = x[3 * t[2] + a] - x[3 * t[0] + a];
    }
    const double n1 = std::sqrt(double(d1[0]) * d1[0] + double(d1[1]) * d1[1] + double(d1[2]) * d1[2]);
    const double n2 = std::sqrt(double(d2[0]) * d2[0] + double(d2[1]) * d2[1] + double(d2[2]) * d2[2]);
    double u1[3], u2[3], nn[3];
    for (int a = 0; a < 3; ++a) {
      u1[a] = d1[a] / n1;
      u2[a] = d2[a] / n2;
    }
    nn[0] = u1[1] * u2[2] - u1[2] * u2[1];
    nn[1] = u1[2] * u2[0] - u1[0] * u2[2];
    nn[2] = u1[0] * u2[1] - u1[1] * u2[0];
    const double nl = std::sqrt(nn[0] * nn[0] + nn[1] * nn[1] + nn[2] * nn[2]);
    float n3[3];
    for (int a = 0; a < 3; ++a) n3[a] = float(nn[a] / nl);
    double *d = out->ed + 9 * e;
    for (int a = 0; a < 3; ++a) {
      d[a * 3 + 0] = d1[a];
      d[a * 3 + 1] = d2[a];
      d[a * 3 + 2] = n3[a];
    }
    // rest shape in the triangle's frame, from the stored (float) columns
    const double t0[3] = {d1[0], d1[1], d1[2]}, t1[3] = {d2[0], d2[1], d2[2]};
    const double l0 = std::sqrt(t0[0] * t0[0] + t0[1] * t0[1] + t0[2] * t0[2]);
    const double dot01 = t0[0] * t1[0] + t0[1] * t1[1] + t0[2] * t1[2];
    const double cx = t0[1] * t1[2] - t0[2] * t1[1], cy = t0[2] * t1[0] - t0[0] * t1[2],
                 cz = t0[0] * t1[1] - t0[1] * t1[0];
    const double a00 = l0, a01 = dot01 / l0, a11 = std::sqrt(cx * cx + cy * cy + cz * cz) / l0;
    double Di[9] = {1 / a00, -a01 / (a00 * a11), 0, 0, 1 / a11, 0, 0, 0, 1};
    const bool degenerate = std::fabs(a11) <= 10 * feps || std::fabs(a00) <= 10 * feps;
    out->emu[e] = degenerate ? 0.0 : mu;
    out->elam[e] = degenerate ? 0.0 : lam;
    for (int i = 0; i < 9; ++i) out->eDmInv[9 * e + i] = float(Di[i]);
    double Fd[9];
    mul_AB(d, Di, Fd);
    for (int i = 0; i < 9; ++i) out->eF[9 * e + i] = float(Fd[i]);
    for (int i = 0; i < 9; ++i) out->eC[9 * e + i] = 0;
    for (int i = 0; i < 3; ++i) {
      out->inds[3 * e + i] = t[i];
      dof_vol[t[i]] += vol / 3.0f;
    }
  }
  for (int64_t p = 0; p < n_verts; ++p) {
    out->vm[p] = double(dof_vol[p] * density);
    for (int a = 0; a < 3; ++a) {
      out->vx[3 * p + a] = x[3 * p + a];
      out->vv[3 * p + a] = v ? v[3 * p + a] : 0.0f;
    }
    for (int i = 0; i < 9; ++i) out->vC[9 * p + i] = 0;
  }
  out->n_verts = n_verts;
  out->n_eles = n_tris;
  return ORC_OK;
}

int32_t orc_curve_init_f64(int64_t n_verts, const float *x, const float *v, int64_t n_segs,
                           const int32_t *segs, float dx, float density, float E, float nu,
                           orc_cloth *out) {
  if (!out || n_verts < 0 || n_segs < 0) return ORC_ERR_INVALID;
  const float mu = E / (2.0f * (1.0f + nu)), lam = E * nu / ((1.0f + nu) * (1.0f - 2.0f * nu));
  std::vector<float> dof_vol(n_verts, 0.0f);
  const double feps = std::numeric_limits<float>::epsilon();
  for (int64_t e = 0; e < n_segs; ++e) {
    const int32_t *t = segs + 2 * e;
    for (int i = 0; i < 2; ++i)
      if (t[i] < 0 || t[i] >= n_verts) return ORC_ERR_INVALID;
    double len2 = 0;
    float d1[3];
    for (int a = 0; a < 3; ++a) {
      const double dd = double(x[3 * t[1] + a]) - double(x[3 * t[0] + a]);
      len2 += dd * dd;
      d1[a] = x[3 * t[1] + a] - x[3 * t[0] + a];
    }
    const float vol = float(std::max(std::sqrt(len2) * double(dx) * double(dx), feps * 10.0));
    out->evol[e] = vol;
    out->em[e] = double(vol * density);
    for (int a = 0; a < 3; ++a) {
      out->ex[3 * e + a] = (x[3 * t[0] + a] + x[3 * t[1] + a]) / 2.0f;
      out->ev[3 * e + a] = v ? double((v[3 * t[0] + a] + v[3 * t[1] + a]) / 2.0f) : 0.0;
    }
    const double ln[3] = {d1[0], d1[1], d1[2]};
    // a vector orthogonal to ln (Hughes & Moller 1999)
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
    double n1[3] = {o[0] / on, o[1] / on, o[2] / on};
    double n2[3] = {ln[1] * n1[2] - ln[2] * n1[1], ln[2] * n1[0] - ln[0] * n1[2], ln[0] * n1[1] - ln[1] * n1[0]};
    const double n2n = std::sqrt(n2[0] * n2[0] + n2[1] * n2[1] + n2[2] * n2[2]);
    double *d = out->ed + 9 * e;
    for (int a = 0; a < 3; ++a) {
      d[a * 3 + 0] = d1[a];
      d[a * 3 + 1] = float(n1[a]);
      d[a * 3 + 2] = float(n2[a] / n2n);
    }
    const double tl = std::sqrt(d[0] * d[0] + d[3] * d[3] + d[6] * d[6]);
    const double Di[9] = {1 / tl, 0, 0, 0, 1, 0, 0, 0, 1};
    out->emu[e] = tl <= feps ? 0.0 : mu;
    out->elam[e] = tl <= feps ? 0.0 : lam;
    for (int i = 0; i < 9; ++i) out->eDmInv[9 * e + i] = float(Di[i]);
    double Fd[9];
    mul_AB(d, Di, Fd);
    for (int i = 0; i < 9; ++i) out->eF[9 * e + i] = float(Fd[i]);
    for (int i = 0; i < 9; ++i) out->eC[9 * e + i] = 0;
    out->inds[3 * e + 0] = t[0];
    out->inds[3 * e + 1] = t[1];
    out->inds[3 * e + 2] = t[1];
    for (int i = 0; i < 2; ++i) dof_vol[t[i]] += vol / 2.0f;
  }
  for (int64_t p = 0; p < n_verts; ++p) {
    out->vm[p] = double(dof_vol[p] * density);
    for (int a = 0; a < 3; ++a) {
      out->vx[3 * p + a] = x[3 * p + a];
      out->vv[3 * p + a] = v ? v[3 * p + a] : 0.0f;
    }
    for (int i = 0; i < 9; ++i) out->vC[9 * p + i] = 0;
  }
  out->n_verts = n_verts;
  out->n_eles = n_segs;
  return ORC_OK;
}

int32_t orc_boundary_points_from_mesh(int64_t n_verts, const float *pos, const float *vel,
                                      int64_t n_tris, const int32_t *tris, float dx,
                                      double *x, double *v, double *m, double *nrm) {
  if (n_verts < 0 || n_tris < 0 || !pos || (n_tris > 0 && !tris) || !(dx > 0) || !x || !v || !m ||
      !nrm)
    return ORC_ERR_INVALID;
  for (int64_t t = 0; t < 3 * n_tris; ++t)
    if (tris[t] < 0 || tris[t] >= n_verts) return ORC_ERR_INVALID;
  auto unit = [](double *a) {
    const double l = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    if (l > 0)
      for (int d = 0; d < 3; ++d) a[d] /= l;
  };
  for (int64_t i = 0; i < n_verts; ++i) {
    for (int d = 0; d < 3; ++d) {
      x[3 * i + d] = pos[3 * i + d];
      v[3 * i + d] = vel ? vel[3 * i + d] : 0.0;
      nrm[3 * i + d] = 0.0;
    }
    m[i] = 0.0;
  }
  for (int64_t t = 0; t < n_tris; ++t) {
    const int32_t *tr = tris + 3 * t;
    double p[3][3];
    for (int k = 0; k < 3; ++k)
      for (int d = 0; d < 3; ++d) p[k][d] = pos[3 * tr[k] + d];
    double a[3], b[3];
    for (int d = 0; d < 3; ++d) {
      a[d] = (p[1][d] - p[0][d]) / dx;
      b[d] = (p[2][d] - p[0][d]) / dx;
    }
    const double cr[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2],
                          a[0] * b[1] - a[1] * b[0]};
    const double area = 0.5 * std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
    double e1[3], e2[3];
    for (int d = 0; d < 3; ++d) {
      e1[d] = p[1][d] - p[0][d];
      e2[d] = p[2][d] - p[0][d];
    }
    unit(e1);
    unit(e2);
    double n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                   e1[0] * e2[1] - e1[1] * e2[0]};
    unit(n);
    const int64_t r = n_verts + t;
    m[r] = area;
    for (int d = 0; d < 3; ++d) {
      x[3 * r + d] = (p[0][d] + p[1][d] + p[2][d]) / 3.0;
      v[3 * r + d] = vel ? (double(vel[3 * tr[0] + d]) + vel[3 * tr[1] + d] + vel[3 * tr[2] + d]) / 3.0
                         : 0.0;
      nrm[3 * r + d] = n[d];
    }
    for (int k = 0; k < 3; ++k) {
      m[tr[k]] += area / 3.0;
      for (int d = 0; d < 3; ++d) nrm[3 * tr[k] + d] += n[d];
    }
  }
  for (int64_t i = 0; i < n_verts; ++i) unit(nrm + 3 * i);
  return ORC_OK;
}

int32_t orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
