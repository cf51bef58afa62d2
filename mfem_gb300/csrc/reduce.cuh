// Deterministic block reductions and last-tile detection.
//
// A tile reduces its values with a fixed shuffle tree, writes one partial
// per tile, and the last tile of a scene to arrive (atomic ticket; no
// waiting) sums that scene's partials in tile order.
#pragma once
#include "device_math.cuh"
#include "kernels.cuh"

namespace mfem_gpu {

// Reduce v[0..NQ) over the block (sums for q < nsum, maxima otherwise) and
// have thread 0 store them to part[0..NQ).  blockDim.x must be a multiple of 32.
template <int NQ>
__device__ __forceinline__ void block_partial(double (&v)[NQ], int nsum, double* part) {
  __shared__ double red[32][NQ];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      double o = __shfl_down_sync(0xffffffffu, v[q], off);
      v[q] = (q < nsum) ? v[q] + o : fmax(v[q], o);
    }
  }
  if (lane == 0) {
#pragma unroll
    for (int q = 0; q < NQ; ++q) red[warp][q] = v[q];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      double a = red[0][q];
      for (int w = 1; w < nw; ++w) a = (q < nsum) ? a + red[w][q] : fmax(a, red[w][q]);
      part[q] = a;
    }
  }
}

// Compensated (Neumaier) block sum of per-thread KSum values; thread 0 writes
// (s, c) to part[0], part[1].
__device__ __forceinline__ void block_ksum(KSum v, double* part) {
  __shared__ double rs[32], rc[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    KSum o;
    o.s = __shfl_down_sync(0xffffffffu, v.s, off);
    o.c = __shfl_down_sync(0xffffffffu, v.c, off);
    v.merge(o);
  }
  if (lane == 0) {
    rs[warp] = v.s;
    rc[warp] = v.c;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    KSum a{rs[0], rc[0]};
    for (int w = 1; w < nw; ++w) a.merge(KSum{rs[w], rc[w]});
    part[0] = a.s;
    part[1] = a.c;
  }
}

// True in every thread of the block that finished a scene's tile set last.
// No thread waits: the last arrival is decided by an atomic ticket.
__device__ __forceinline__ bool last_tile(unsigned int* ctr, int count) {
  __shared__ int s_last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    unsigned int prev = atomicAdd(ctr, 1u);
    s_last = (prev + 1u == (unsigned int)count) ? 1 : 0;
    if (s_last) *ctr = 0u;
  }
  __syncthreads();
  if (s_last) __threadfence();
  return s_last != 0;
}

__device__ __forceinline__ double ld_partial(const double* p) { return __ldcg(p); }

}  // namespace mfem_gpu
