// Upload / download of the particle store: the user's AoS arrays (staged in
// device memory) <-> the SoA planes, keeping the upload order in the id plane
// so that downloads return particles in the order they were uploaded, as the
// reference's TileVector never reorders (Generation.cpp:937-1000,
// Generation.cu:1088-1158).
#include <cuda_runtime.h>

#include "zsmpm_internal.cuh"

namespace zsmpm {
namespace {

__global__ void k_ingest(float *__restrict__ pb, int32_t *__restrict__ ib, long long cap,
                         IngestSrc src, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      pb[(CH_X + k) * cap + i] = src.x[3 * i + k];
      pb[(CH_V + k) * cap + i] = src.v ? src.v[3 * i + k] : 0.0f;
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      pb[(CH_C + k) * cap + i] = src.C ? src.C[9 * i + k] : 0.0f;
      pb[(CH_F + k) * cap + i] = src.F ? src.F[9 * i + k] : ((k % 4 == 0) ? 1.0f : 0.0f);
    }
    pb[CH_J * cap + i] = src.J ? src.J[i] : 1.0f;
    pb[CH_M * cap + i] = src.m[i];
    pb[CH_VOL * cap + i] = src.vol[i];
    if (src.mu) {
      pb[CH_MU * cap + i] = src.mu[i];
      pb[CH_LAM * cap + i] = src.lam[i];
    }
    ib[IC_MAT * cap + i] = src.mat ? src.mat[i] : 0;
    ib[IC_ID * cap + i] = (int32_t)i;
  }
}

// dst layout: x (3n) | v (3n) | C (9n) | F (9n) | J (n), each in upload order
__global__ void k_egest(const float *__restrict__ pb, const int32_t *__restrict__ ib,
                        long long cap, float *__restrict__ dst, long long n) {
  float *x = dst, *v = dst + 3 * n, *C = dst + 6 * n, *F = dst + 15 * n, *J = dst + 24 * n;
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < n;
       s += (long long)gridDim.x * blockDim.x) {
    const long long u = ib[IC_ID * cap + s];
    if (u < 0 || u >= n) continue;  // slot not rewritten after a binning error
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      x[3 * u + k] = pb[(CH_X + k) * cap + s];
      v[3 * u + k] = pb[(CH_V + k) * cap + s];
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      C[9 * u + k] = pb[(CH_C + k) * cap + s];
      F[9 * u + k] = pb[(CH_F + k) * cap + s];
    }
    J[u] = pb[CH_J * cap + s];
  }
}

// per-particle Lame overrides given in upload order -> storage order
__global__ void k_set_lame(float *__restrict__ pb, const int32_t *__restrict__ ib, long long cap,
                           const float *__restrict__ mu, const float *__restrict__ lam,
                           long long n) {
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < n;
       s += (long long)gridDim.x * blockDim.x) {
    const long long u = ib[IC_ID * cap + s];
    if (u < 0 || u >= n) continue;
    pb[CH_MU * cap + s] = mu[u];
    pb[CH_LAM * cap + s] = lam[u];
  }
}

}  // namespace

void launch_set_lame(const DevPtrs &d, int cur, const float *mu, const float *lam, long long n,
                     cudaStream_t s) {
  if (n <= 0) return;
  k_set_lame<<<d.num_sms * 8, 256, 0, s>>>(d.pbuf[cur], d.ibuf[cur], d.cap, mu, lam, n);
}

void launch_ingest(const DevPtrs &d, int cur, IngestSrc src, long long n, cudaStream_t s) {
  if (n <= 0) return;
  k_ingest<<<d.num_sms * 8, 256, 0, s>>>(d.pbuf[cur], d.ibuf[cur], d.cap, src, n);
}

void launch_egest(const DevPtrs &d, int cur, float *dst, long long n, cudaStream_t s) {
  if (n <= 0) return;
  k_egest<<<d.num_sms * 8, 256, 0, s>>>(d.pbuf[cur], d.ibuf[cur], d.cap, dst, n);
}

}  // namespace zsmpm
