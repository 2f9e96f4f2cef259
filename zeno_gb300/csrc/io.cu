// Upload / download of the particle store: the user's AoS arrays (staged in
// device memory) <-> the SoA planes, keeping the upload order in the id plane
// so that downloads return particles in the order they were uploaded, as the
// reference's TileVector never reorders (Generation.cpp:937-1000,
// Generation.cu:1088-1158).
#include <cuda_runtime.h>

#include "zsmpm_internal.cuh"

namespace zsmpm {
namespace {

// particles [b0, b1) of the staged arrays into slots b0..b1-1
__global__ void k_ingest(float *__restrict__ pb, int32_t *__restrict__ ib, long long cap,
                         IngestSrc src, long long b0, long long b1) {
  for (long long i = b0 + blockIdx.x * (long long)blockDim.x + threadIdx.x; i < b1;
       i += (long long)gridDim.x * blockDim.x) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      pb[pidx((CH_X + k), i)] = src.x[3 * i + k];
      pb[pidx((CH_V + k), i)] = src.v ? src.v[3 * i + k] : 0.0f;
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      pb[pidx((CH_C + k), i)] = src.C ? src.C[9 * i + k] : 0.0f;
      pb[pidx((CH_F + k), i)] = src.F ? src.F[9 * i + k] : ((k % 4 == 0) ? 1.0f : 0.0f);
    }
    pb[pidx(CH_J, i)] = src.J ? src.J[i] : 1.0f;
    pb[pidx(CH_M, i)] = src.m[i];
    pb[pidx(CH_VOL, i)] = src.vol[i];
    if (src.mu) {
      pb[pidx(CH_MU, i)] = src.mu[i];
      pb[pidx(CH_LAM, i)] = src.lam[i];
    }
    ib[iidx(IC_MAT, i)] = src.mat ? src.mat[i] : 0;
    ib[iidx(IC_ID, i)] = (int32_t)i;
  }
}

// x (n x 3), v, C (n x 9), F, J in upload order; any destination may be
// null, device memory or host memory the device can address
__global__ void k_egest(const float *__restrict__ pb, const int32_t *__restrict__ ib,
                        long long cap, EgestDst o, long long n) {
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < n;
       s += (long long)gridDim.x * blockDim.x) {
    const long long u = ib[iidx(IC_ID, s)];
    if (u < 0 || u >= n) continue;  // slot not rewritten after a binning error
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      if (o.x) o.x[3 * u + k] = pb[pidx((CH_X + k), s)];
      if (o.v) o.v[3 * u + k] = pb[pidx((CH_V + k), s)];
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      if (o.C) o.C[9 * u + k] = pb[pidx((CH_C + k), s)];
      if (o.F) o.F[9 * u + k] = pb[pidx((CH_F + k), s)];
    }
    if (o.J) o.J[u] = pb[pidx(CH_J, s)];
  }
}

// one float channel of the store -> dst in upload order
__global__ void k_egest_channel(const float *__restrict__ pb, const int32_t *__restrict__ ib,
                                int ch, float *__restrict__ dst, long long n) {
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < n;
       s += (long long)gridDim.x * blockDim.x) {
    const long long u = ib[iidx(IC_ID, s)];
    if (u < 0 || u >= n) continue;
    dst[u] = pb[pidx(ch, s)];
  }
}

// per-particle Lame overrides given in upload order -> storage order
__global__ void k_set_lame(float *__restrict__ pb, const int32_t *__restrict__ ib, long long cap,
                           const float *__restrict__ mu, const float *__restrict__ lam,
                           long long n) {
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < n;
       s += (long long)gridDim.x * blockDim.x) {
    const long long u = ib[iidx(IC_ID, s)];
    if (u < 0 || u >= n) continue;
    pb[pidx(CH_MU, s)] = mu[u];
    pb[pidx(CH_LAM, s)] = lam[u];
  }
}

__global__ void k_lame_from_materials(const DevPtrs d, float *__restrict__ pb,
                                      const int32_t *__restrict__ ib) {
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < d.prm->n;
       s += (long long)gridDim.x * blockDim.x) {
    const MatParams mp = d.mats[min(max(ib[iidx(IC_MAT, s)], 0), kMaxMaterials - 1)];
    pb[pidx(CH_MU, s)] = mp.mu;
    pb[pidx(CH_LAM, s)] = mp.lam;
  }
}

// state planes [MPM_STATE_PLANES][n] of every slot <-> the tiled store:
// x v C F J m vol mu lam are the store's float channels 0..28, then the
// material id and the upload index (int32 bits); dst != null saves,
// src != null loads
static_assert(MPM_STATE_PLANES == CH_LAM + 1 + NICH && CH_S == CH_LAM + 1,
              "state planes: float channels up to lam, then the int channels");
__global__ void k_state_copy(float *__restrict__ pb, int32_t *__restrict__ ib,
                             float *__restrict__ dst, const float *__restrict__ src, long long n) {
  constexpr int NF = CH_LAM + 1;
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < n;
       s += (long long)gridDim.x * blockDim.x) {
    if (dst) {
#pragma unroll
      for (int k = 0; k < NF; ++k) dst[k * n + s] = pb[pidx(k, s)];
      dst[(NF + IC_MAT) * n + s] = __int_as_float(ib[iidx(IC_MAT, s)]);
      dst[(NF + IC_ID) * n + s] = __int_as_float(ib[iidx(IC_ID, s)]);
    } else {
#pragma unroll
      for (int k = 0; k < NF; ++k) pb[pidx(k, s)] = src[k * n + s];
      ib[iidx(IC_MAT, s)] = __float_as_int(src[(NF + IC_MAT) * n + s]);
      ib[iidx(IC_ID, s)] = __float_as_int(src[(NF + IC_ID) * n + s]);
    }
  }
}

// every material id in [0, n_materials)? (bad_material was zeroed before)
__global__ void k_check_materials(const int32_t *__restrict__ mat, long long n, int n_materials,
                                  Counters *cnt) {
  bool bad = false;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    bad |= (unsigned)mat[i] >= (unsigned)n_materials;
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) cnt->bad_material = 1;
}

__global__ void k_flag_materials(Counters *cnt) {
  if (cnt->bad_material) atomicOr(&cnt->status, ST_MATERIAL);
}

}  // namespace

void launch_flag_materials(const DevPtrs &d, cudaStream_t s) {
  k_flag_materials<<<1, 1, 0, s>>>(d.cnt);
}

void launch_check_materials(const DevPtrs &d, const int32_t *mat, long long n, int n_materials,
                            cudaStream_t s) {
  if (n <= 0) return;
  k_check_materials<<<d.num_sms * 4, 256, 0, s>>>(mat, n, n_materials, d.cnt);
}

void launch_state_copy(const DevPtrs &d, int cur, float *dst, const float *src, long long n,
                       cudaStream_t s) {
  if (n <= 0) return;
  k_state_copy<<<d.num_sms * 8, 256, 0, s>>>(d.pbuf[cur], d.ibuf[cur], dst, src, n);
}

void launch_egest_channel(const DevPtrs &d, int cur, int ch, float *dst, long long n,
                          cudaStream_t s) {
  if (n <= 0) return;
  k_egest_channel<<<d.num_sms * 8, 256, 0, s>>>(d.pbuf[cur], d.ibuf[cur], ch, dst, n);
}

void launch_set_lame(const DevPtrs &d, int cur, const float *mu, const float *lam, long long n,
                     cudaStream_t s) {
  if (n <= 0) return;
  k_set_lame<<<d.num_sms * 8, 256, 0, s>>>(d.pbuf[cur], d.ibuf[cur], d.cap, mu, lam, n);
}

void launch_lame_from_materials(const DevPtrs &d, int cur, cudaStream_t s) {
  k_lame_from_materials<<<d.num_sms * 8, 256, 0, s>>>(d, d.pbuf[cur], d.ibuf[cur]);
}

void launch_ingest(const DevPtrs &d, int cur, IngestSrc src, long long b0, long long b1,
                   cudaStream_t s) {
  if (b1 <= b0) return;
  k_ingest<<<d.num_sms * 8, 256, 0, s>>>(d.pbuf[cur], d.ibuf[cur], d.cap, src, b0, b1);
}

void launch_egest(const DevPtrs &d, int cur, EgestDst dst, long long n, cudaStream_t s) {
  if (n <= 0) return;
  k_egest<<<d.num_sms * 8, 256, 0, s>>>(d.pbuf[cur], d.ibuf[cur], d.cap, dst, n);
}

}  // namespace zsmpm
