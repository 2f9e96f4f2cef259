// Asynchronous global -> shared copies (cp.async, sm_80 and later) for the
// staged particle and grid loads of the transfer kernels: a thread issues
// many copies without holding the values in registers, commits them as a
// group and waits for the group before a barrier, so that the loads of the
// next chunk of particles are in flight while the current chunk computes.
#pragma once

#include <cuda_runtime.h>

namespace zsmpm {

__device__ __forceinline__ unsigned smem_addr(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

// 4 bytes; both addresses 4-byte aligned
__device__ __forceinline__ void cp_async4(void *smem, const void *gmem) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(smem_addr(smem)), "l"(gmem)
               : "memory");
}

// 16 bytes; both addresses 16-byte aligned
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_addr(smem)), "l"(gmem)
               : "memory");
}

__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}

// wait until at most N of this thread's committed groups are pending
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

}  // namespace zsmpm
