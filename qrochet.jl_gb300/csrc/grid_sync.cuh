// Bounded grid-wide barrier for cooperative launches, shared by the Jacobi sweeps (svd.cu) and
// the persistent Householder QR (qr.cu).
#pragma once
#include "common.cuh"

namespace qr {
namespace {

// Grid-wide barrier for a cooperative launch (all CTAs resident).  bar[0] counts arrivals over the
// whole launch (and over consecutive launches of the same grid size that share the counters): the
// CTA whose arrival is number a waits until the count reaches the next multiple of the grid size,
// polling with an acquire load, so one atomic per CTA and one cache line carry the barrier.  The
// wait is bounded: after 2^22 polls the CTA records a timeout in bar[2] and proceeds; every CTA
// checks bar[2] after the barrier and leaves, so the kernel always returns.  bar[1] is unused.
__device__ __forceinline__ unsigned ld_acquire_gpu_u32(const unsigned* a) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(a) : "memory");
  return v;
}
__device__ __forceinline__ bool grid_barrier(unsigned* bar) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();  // this CTA's writes are visible before its arrival
    const unsigned arrived = atomicAdd(&bar[0], 1u) + 1u;
    const unsigned target = (arrived + gridDim.x - 1u) / gridDim.x * gridDim.x;
    unsigned polls = 0;
    while (ld_acquire_gpu_u32(&bar[0]) < target) {
      if (((volatile unsigned*)bar)[2]) break;
      if (++polls > (1u << 22)) {
        atomicExch(&bar[2], 1u);
        break;
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ((volatile unsigned*)bar)[2] == 0u;
}

}  // namespace
}  // namespace qr
