// Deterministic block reductions and last-tile detection.
//
// A tile reduces its values with a fixed shuffle tree and writes one partial
// per quantity; partials are stored quantity-major (partials[q*pstride+tile]).
// The last tile of a scene to arrive (atomic ticket; no thread ever waits)
// reduces that scene's partials with the whole block in a fixed order.
#pragma once
#include "device_math.cuh"
#include "kernels.cuh"

namespace mfem_gpu {

// Block-wide sum / max of one double per thread; every thread gets the result.
// blockDim.x must be a multiple of 32.
__device__ __forceinline__ double block_sum_all(double v) {
  __shared__ double red[32];
  __shared__ double out;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = red[0];
    for (int w = 1; w < nw; ++w) a += red[w];
    out = a;
  }
  __syncthreads();
  return out;
}

__device__ __forceinline__ double block_max_all(double v) {
  __shared__ double red[32];
  __shared__ double out;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, off));
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = red[0];
    for (int w = 1; w < nw; ++w) a = fmax(a, red[w]);
    out = a;
  }
  __syncthreads();
  return out;
}

// Compensated (Neumaier) block sum; every thread gets (s, c).
__device__ __forceinline__ KSum block_ksum_all(KSum v) {
  __shared__ double rs[32], rc[32];
  __shared__ double os, oc;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    KSum o;
    o.s = __shfl_down_sync(0xffffffffu, v.s, off);
    o.c = __shfl_down_sync(0xffffffffu, v.c, off);
    v.merge(o);
  }
  __syncthreads();
  if (lane == 0) {
    rs[warp] = v.s;
    rc[warp] = v.c;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    KSum a{rs[0], rc[0]};
    for (int w = 1; w < nw; ++w) a.merge(KSum{rs[w], rc[w]});
    os = a.s;
    oc = a.c;
  }
  __syncthreads();
  return KSum{os, oc};
}

// Tile partial writes (thread 0 stores).
__device__ __forceinline__ void put_sum(double v, double* partials, int pstride, int q, int tile) {
  v = block_sum_all(v);
  if (threadIdx.x == 0) partials[(size_t)q * pstride + tile] = v;
}
__device__ __forceinline__ void put_max(double v, double* partials, int pstride, int q, int tile) {
  v = block_max_all(v);
  if (threadIdx.x == 0) partials[(size_t)q * pstride + tile] = v;
}
__device__ __forceinline__ void put_ksum(KSum v, double* partials, int pstride, int q, int tile) {
  v = block_ksum_all(v);
  if (threadIdx.x == 0) {
    partials[(size_t)q * pstride + tile] = v.s;
    partials[(size_t)(q + 1) * pstride + tile] = v.c;
  }
}

// Reductions of a scene's partials [first, first+count) by the whole block.
__device__ __forceinline__ double scene_sum(const double* partials, int pstride, int q, int first,
                                            int count) {
  const double* p = partials + (size_t)q * pstride + first;
  double s = 0;
  for (int i = threadIdx.x; i < count; i += blockDim.x) s += __ldcg(p + i);
  return block_sum_all(s);
}
__device__ __forceinline__ double scene_max(const double* partials, int pstride, int q, int first,
                                            int count) {
  const double* p = partials + (size_t)q * pstride + first;
  double s = 0;
  for (int i = threadIdx.x; i < count; i += blockDim.x) s = fmax(s, __ldcg(p + i));
  return block_max_all(s);
}
__device__ __forceinline__ double scene_ksum(const double* partials, int pstride, int q, int first,
                                             int count) {
  const double* ps = partials + (size_t)q * pstride + first;
  const double* pc = partials + (size_t)(q + 1) * pstride + first;
  KSum s{0.0, 0.0};
  for (int i = threadIdx.x; i < count; i += blockDim.x) s.merge(KSum{__ldcg(ps + i), __ldcg(pc + i)});
  return block_ksum_all(s).value();
}

// True in every thread of the block that finished a scene's tile set last.
// No thread waits: the last arrival is decided by atomic tickets, first per
// group of kTicketGroup tiles (distinct addresses, so the increments do not
// serialise on one L2 line), then per scene by the last tile of each group.
__device__ __forceinline__ bool last_tile(const SceneDev& sd, int table, int tix) {
  __shared__ int s_last;
  __syncthreads();
  if (threadIdx.x == 0) {
    const int local = tix - sd.tile_first[table];
    const int count = sd.tile_count[table];
    const int grp = local / kTicketGroup;
    const int ngrp = (count + kTicketGroup - 1) / kTicketGroup;
    const int in_grp = min(kTicketGroup, count - grp * kTicketGroup);
    unsigned int* gc = sd.gctr + (size_t)table * sd.gmax + grp;
    __threadfence();
    int last = 0;
    if (atomicAdd(gc, 1u) + 1u == (unsigned int)in_grp) {
      *gc = 0u;
      __threadfence();
      unsigned int* sc = &sd.sc->ctr[table];
      if (atomicAdd(sc, 1u) + 1u == (unsigned int)ngrp) {
        *sc = 0u;
        last = 1;
      }
    }
    s_last = last;
  }
  __syncthreads();
  if (s_last) __threadfence();
  return s_last != 0;
}

}  // namespace mfem_gpu
