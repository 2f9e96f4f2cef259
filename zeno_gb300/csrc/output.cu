// Particle output: ComputeVonMises (Generation.cu:1873-1920) and the frame
// snapshot behind asynchronous write-back (UpdatePrimitiveFromZSParticles,
// Generation.cu:1088-1158, without the host-side reorder loop: the store is
// put back into upload order on the device).
#include <cuda_runtime.h>

#include "mpm_math.cuh"
#include "zsmpm_internal.cuh"

namespace zsmpm {
namespace {

// von Mises stress of the StVK-Hencky particles from the principal Cauchy
// stresses c_i = (2 mu e_i + lam sum e) / J, e_i = ln s_i (s the singular
// values of F, from the eigenvalues of F F^T - I), J = s0 s1 s2:
// vms = sqrt(((c0 - c1)^2 + (c1 - c2)^2 + (c2 - c0)^2) / 2), where lam drops
// out; log10(vms + 1) with by_log1p.  The material's mu (the reference passes
// the model, no per-particle override); other models keep their value.
__global__ void k_von_mises(DevPtrs d, const float *__restrict__ pb,
                            const int32_t *__restrict__ ib, int by_log1p) {
  const long long n = d.prm->n;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    const int id = ib[iidx(IC_ID, p)];
    if (id < 0 || id >= n) continue;
    const MatParams mp = d.mats[min(max(ib[iidx(IC_MAT, p)], 0), kMaxMaterials - 1)];
    if (mp.type != MPM_STVK) continue;
    float F[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) F[k] = pb[pidx((CH_F + k), p)];
    Sym3 E;
    float Jm1, w[3];
    strain_of(F, E, Jm1);
    sym_eigvals3(E, w);
    const float e0 = 0.5f * log1pf(w[0]), e1 = 0.5f * log1pf(w[1]), e2 = 0.5f * log1pf(w[2]);
    const float J = expf(e0 + e1 + e2);
    const float a = e0 - e1, b = e1 - e2, c = e2 - e0;
    const float vms = 2.0f * mp.mu / J * sqrtf(0.5f * (a * a + b * b + c * c));
    d.vms[id] = by_log1p ? log10f(vms + 1.0f) : vms;
  }
}

// x (3n) | v (3n) of the store in upload order
__global__ void k_snapshot_xv(const float *__restrict__ pb, const int32_t *__restrict__ ib,
                              float *__restrict__ dst, long long n) {
  float *x = dst, *v = dst + 3 * n;
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < n;
       s += (long long)gridDim.x * blockDim.x) {
    const long long u = ib[iidx(IC_ID, s)];
    if (u < 0 || u >= n) continue;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      x[3 * u + k] = pb[pidx((CH_X + k), s)];
      v[3 * u + k] = pb[pidx((CH_V + k), s)];
    }
  }
}

}  // namespace

void launch_von_mises(const DevPtrs &d, int cur, int by_log1p, cudaStream_t s) {
  k_von_mises<<<d.num_sms * 8, 256, 0, s>>>(d, d.pbuf[cur], d.ibuf[cur], by_log1p);
}

void launch_snapshot_xv(const DevPtrs &d, int cur, float *dst, long long n, cudaStream_t s) {
  if (n <= 0) return;
  k_snapshot_xv<<<d.num_sms * 8, 256, 0, s>>>(d.pbuf[cur], d.ibuf[cur], dst, n);
}

}  // namespace zsmpm
