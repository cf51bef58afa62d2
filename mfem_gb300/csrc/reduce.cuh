// Precision traits of the two paths and deterministic reductions.
//
// Ext is the high-precision type of a path: df64 (float pairs, FP32 pipe) in
// the mixed path, double in the all-FP64 path.  Positions, the stretch
// variable s, the residual chain and per-thread accumulations use Ext; a
// warp reduces in Ext with a fixed shuffle tree and converts once to double;
// a tile writes one double partial per quantity (quantity-major,
// partials[q*pstride+tile]); the last tile of a scene (atomic tickets, no
// thread waits) reduces that scene's partials with the whole block in a
// fixed order.
#pragma once
#include "device_math.cuh"
#include "kernels.cuh"

namespace mfem_gpu {

template <typename Real> struct Ext;
template <> struct Ext<float> {
  using T = df64;
  __device__ static T ld(const void* p, size_t i) { return df_load(static_cast<const float2*>(p)[i]); }
  __device__ static void st(void* p, size_t i, T v) { static_cast<float2*>(p)[i] = df_store(v); }
  __device__ static double to_d(T v) { return v.to_double(); }
  __device__ static float to_real(T v) { return __fadd_rn(v.hi, v.lo); }
};
template <> struct Ext<double> {
  using T = double;
  __device__ static T ld(const void* p, size_t i) { return static_cast<const double*>(p)[i]; }
  __device__ static void st(void* p, size_t i, T v) { static_cast<double*>(p)[i] = v; }
  __device__ static double to_d(T v) { return v; }
  __device__ static double to_real(T v) { return v; }
};

__device__ __forceinline__ df64 shfl_down(df64 v, int off) {
  return df64(__shfl_down_sync(0xffffffffu, v.hi, off), __shfl_down_sync(0xffffffffu, v.lo, off));
}
__device__ __forceinline__ double shfl_down(double v, int off) { return __shfl_down_sync(0xffffffffu, v, off); }
__device__ __forceinline__ float shfl_down(float v, int off) { return __shfl_down_sync(0xffffffffu, v, off); }
__device__ __forceinline__ double to_double_any(df64 v) { return v.to_double(); }
__device__ __forceinline__ double to_double_any(double v) { return v; }

// Writes NS sums (Ext per thread) and NM maxima (double per thread) of the
// block as tile partials at quantities q0, q0+1, ...: the first `npairs`
// sums as compensated (s, c) pairs, the other sums as plain doubles, then
// the maxima.
template <typename E, int NS, int NM>
__device__ __forceinline__ void tile_partials(E* sums, double* maxs, double* partials, int pstride,
                                              int q0, int tile, int npairs) {
  __shared__ double red[32][NS + NM];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int q = 0; q < NS; ++q)
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) sums[q] = sums[q] + shfl_down(sums[q], off);
#pragma unroll
  for (int q = 0; q < NM; ++q)
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) maxs[q] = fmax(maxs[q], shfl_down(maxs[q], off));
  __syncthreads();
  if (lane == 0) {
#pragma unroll
    for (int q = 0; q < NS; ++q) red[warp][q] = to_double_any(sums[q]);
#pragma unroll
    for (int q = 0; q < NM; ++q) red[warp][NS + q] = maxs[q];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int qo = q0;
#pragma unroll
    for (int q = 0; q < NS; ++q) {
      KSum a{red[0][q], 0.0};
      for (int w = 1; w < nw; ++w) a.add(red[w][q]);
      if (q < npairs) {
        partials[(size_t)qo * pstride + tile] = a.s;
        partials[(size_t)(qo + 1) * pstride + tile] = a.c;
        qo += 2;
      } else {
        partials[(size_t)qo * pstride + tile] = a.value();
        qo += 1;
      }
    }
#pragma unroll
    for (int q = 0; q < NM; ++q) {
      double m = red[0][NS + q];
      for (int w = 1; w < nw; ++w) m = fmax(m, red[w][NS + q]);
      partials[(size_t)qo * pstride + tile] = m;
      qo += 1;
    }
  }
}

// Block-wide double reductions returning the result to every thread.
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
