// Bounded grid-wide barrier for cooperative launches, shared by the Jacobi sweeps (svd.cu) and
// the persistent Householder QR (qr.cu).
#pragma once
#include "common.cuh"

namespace qr {
namespace {

// Grid-wide barrier for a cooperative launch (all CTAs resident).  The wait is bounded: after
// ~2^22 polls (about a second) the CTA records a timeout in bar[2] and proceeds; every CTA checks
// bar[2] after the barrier and leaves the sweep, so the kernel always returns.
__device__ __forceinline__ bool grid_barrier(unsigned* bar) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* vb = bar;
    const unsigned gen = vb[1];
    __threadfence();
    const unsigned arrived = atomicAdd(&bar[0], 1u) + 1u;
    if (arrived == gridDim.x) {
      atomicExch(&bar[0], 0u);
      __threadfence();
      atomicAdd(&bar[1], 1u);
    } else {
      unsigned polls = 0;
      while (vb[1] == gen) {
        if (++polls > (1u << 22)) {
          atomicExch(&bar[2], 1u);
          break;
        }
        __nanosleep(200);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ((volatile unsigned*)bar)[2] == 0u;
}

}  // namespace
}  // namespace qr
