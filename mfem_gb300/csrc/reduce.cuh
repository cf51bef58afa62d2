// Precision traits of the two paths and deterministic reductions.
//
// Ext is the high-precision type of a path: df64 (float pairs, FP32 pipe) in
// the mixed path, double in the all-FP64 path.  Positions, the stretch
// variable s, the residual chain and per-thread accumulations use Ext; a
// warp reduces in Ext with a fixed shuffle tree; a tile writes one Ext
// partial per quantity (quantity-major, partials[q*pstride+tile]); the last
// tile of a scene (atomic tickets, no thread waits) reduces that scene's
// partials in Ext with the whole block in a fixed order, and one thread
// converts the result to double for the scene's scalars.
#pragma once
#include "device_math.cuh"
#include "kernels.cuh"

namespace mfem_gpu {

template <typename Real> struct Ext;
template <> struct Ext<float> {
  using T = df64;
  // a double constant of the scene as the path's Ext / Real value
  __device__ static T c(double, float2 x) { return df64(x.x, x.y); }
  __device__ static float r(double, float2 x) { return x.x; }
  __device__ static T ld(const void* p, size_t i) { return df_load(static_cast<const float2*>(p)[i]); }
  __device__ static void st(void* p, size_t i, T v) { static_cast<float2*>(p)[i] = df_store(v); }
  __device__ static double to_d(T v) { return v.to_double(); }
  __device__ static float to_real(T v) { return __fadd_rn(v.hi, v.lo); }
};
template <> struct Ext<double> {
  using T = double;
  __device__ static T c(double d, float2) { return d; }
  __device__ static double r(double d, float2) { return d; }
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

// A tile partial is an 8-byte slot: a double (FP64 path), a df64 as a
// float pair, or a float maximum (mixed path).  Keeping the whole reduction
// (warp tree, block combine, scene sum) in the path's own types keeps FP64
// instructions out of the mixed path: on GB300 one FP64 warp instruction
// occupies the FP64 pipe for 64 cycles, so a scalar FP64 chain in a block's
// tail stalls the whole block behind its thread 0.
template <typename T> struct Slot;
template <> struct Slot<df64> {
  __device__ static void put(double* p, df64 v) { *reinterpret_cast<float2*>(p) = make_float2(v.hi, v.lo); }
  __device__ static df64 get(const double* p) {
    const float2 f = __ldcg(reinterpret_cast<const float2*>(p));
    return df64(f.x, f.y);
  }
  __device__ static df64 sget(const double* p) {
    const float2 f = *reinterpret_cast<const float2*>(p);
    return df64(f.x, f.y);
  }
};
template <> struct Slot<double> {
  __device__ static void put(double* p, double v) { *p = v; }
  __device__ static double get(const double* p) { return __ldcg(p); }
  __device__ static double sget(const double* p) { return *p; }
};
template <> struct Slot<float> {
  __device__ static void put(double* p, float v) { *reinterpret_cast<float*>(p) = v; }
  __device__ static float get(const double* p) { return __ldcg(reinterpret_cast<const float*>(p)); }
  __device__ static float sget(const double* p) { return *reinterpret_cast<const float*>(p); }
};

// Addition in the reduction trees (df64: the one-TwoSum addition of
// df64.cuh, about 2^-47 of the operands per addition).
__device__ __forceinline__ df64 radd(df64 a, df64 b) { return a + b; }
__device__ __forceinline__ double radd(double a, double b) { return a + b; }

// Reduces the per-warp values red[w][q] (w < nw <= 32) in warp 0 with a
// shuffle tree; the result is valid in lane 0.  Fixed order.
template <typename T, bool kSum>
__device__ __forceinline__ T warp0_combine(const double* red_q, int stride, int nw) {
  const int lane = threadIdx.x & 31;
  T a = lane < nw ? Slot<T>::sget(red_q + (size_t)lane * stride) : T(0);
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const T o = shfl_down(a, off);
    a = kSum ? radd(a, o) : fmax(a, o);
  }
  return a;
}

// Writes NS sums (type E) and NM maxima (type M) of the block as tile
// partials at quantities q0, q0+1, ... (sums first).  Fixed reduction
// order: a shuffle tree per warp, then a shuffle tree over the warps in
// warp 0; thread 0 writes the partials.
template <typename E, typename M, int NS, int NM>
__device__ __forceinline__ void tile_partials(E* sums, M* maxs, double* partials, int pstride,
                                              int q0, int tile) {
  __shared__ double red[32][NS + NM];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int q = 0; q < NS; ++q)
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) sums[q] = radd(sums[q], shfl_down(sums[q], off));
#pragma unroll
  for (int q = 0; q < NM; ++q)
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) maxs[q] = fmax(maxs[q], shfl_down(maxs[q], off));
  __syncthreads();
  if (lane == 0) {
#pragma unroll
    for (int q = 0; q < NS; ++q) Slot<E>::put(&red[warp][q], sums[q]);
#pragma unroll
    for (int q = 0; q < NM; ++q) Slot<M>::put(&red[warp][NS + q], maxs[q]);
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int q = 0; q < NS; ++q) {
      const E a = warp0_combine<E, true>(&red[0][q], NS + NM, nw);
      if (lane == 0) Slot<E>::put(partials + (size_t)(q0 + q) * pstride + tile, a);
    }
#pragma unroll
    for (int q = 0; q < NM; ++q) {
      const M m = warp0_combine<M, false>(&red[0][NS + q], NS + NM, nw);
      if (lane == 0) Slot<M>::put(partials + (size_t)(q0 + NS + q) * pstride + tile, m);
    }
  }
}

// Block-wide reductions returning the result to every thread.
template <typename E>
__device__ __forceinline__ E block_sum_all(E v) {
  __shared__ double red[32];
  __shared__ double out;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v = radd(v, shfl_down(v, off));
  __syncthreads();
  if (lane == 0) Slot<E>::put(&red[warp], v);
  __syncthreads();
  if (warp == 0) {
    const E a = warp0_combine<E, true>(red, 1, nw);
    if (lane == 0) Slot<E>::put(&out, a);
  }
  __syncthreads();
  return Slot<E>::sget(&out);
}

template <typename M>
__device__ __forceinline__ M block_max_all(M v) {
  __shared__ double red[32];
  __shared__ double out;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v = fmax(v, shfl_down(v, off));
  __syncthreads();
  if (lane == 0) Slot<M>::put(&red[warp], v);
  __syncthreads();
  if (warp == 0) {
    const M a = warp0_combine<M, false>(red, 1, nw);
    if (lane == 0) Slot<M>::put(&out, a);
  }
  __syncthreads();
  return Slot<M>::sget(&out);
}

// Reductions of a scene's partials [first, first+count) by the whole block,
// each thread over a fixed strided subset, then the block tree.
template <typename E>
__device__ __forceinline__ E scene_sum(const double* partials, int pstride, int q, int first, int count) {
  const double* p = partials + (size_t)q * pstride + first;
  E s = E(0);
  for (int i = threadIdx.x; i < count; i += blockDim.x) s = radd(s, Slot<E>::get(p + i));
  return block_sum_all<E>(s);
}
template <typename M>
__device__ __forceinline__ M scene_max(const double* partials, int pstride, int q, int first, int count) {
  const double* p = partials + (size_t)q * pstride + first;
  M s = M(0);
  for (int i = threadIdx.x; i < count; i += blockDim.x) s = fmax(s, Slot<M>::get(p + i));
  return block_max_all<M>(s);
}

// NQ sums of a scene's partials at quantities q0.. in one pass: each thread
// over a fixed strided subset of tiles, then one block tree for all NQ.
template <typename E, int NQ>
__device__ __forceinline__ void scene_sums(const double* partials, int pstride, int q0, int first,
                                           int count, E* out) {
  __shared__ double red[32][NQ];
  __shared__ double res[NQ];
  E s[NQ];
#pragma unroll
  for (int q = 0; q < NQ; ++q) s[q] = E(0);
  for (int i = threadIdx.x; i < count; i += blockDim.x)
#pragma unroll
    for (int q = 0; q < NQ; ++q) s[q] = radd(s[q], Slot<E>::get(partials + (size_t)(q0 + q) * pstride + first + i));
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int q = 0; q < NQ; ++q)
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s[q] = radd(s[q], shfl_down(s[q], off));
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < NQ; ++q) Slot<E>::put(&red[warp][q], s[q]);
  __syncthreads();
  if (warp == 0)
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      const E a = warp0_combine<E, true>(&red[0][q], NQ, nw);
      if (lane == 0) Slot<E>::put(&res[q], a);
    }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < NQ; ++q) out[q] = Slot<E>::sget(&res[q]);
}

// Scalar arithmetic of a scene's finalizer (one thread).  The mixed path
// keeps FP64 division and square root out (each a multi-instruction
// sequence on the 1/64-rate FP64 pipe, microseconds on one thread):
// quotients in df64, square roots in FP32 (they only feed tolerance tests
// and reports).
template <typename Real> struct Fin;
template <> struct Fin<float> {
  __device__ static double div(double a, double b) { return (df64(a) / df64(b)).to_double(); }
  __device__ static double sqrt(double a) { return double(sqrtf(float(a))); }
  __device__ static double sqrt_ratio(double a, double b) { return double(sqrtf(float(a) / float(b))); }
};
template <> struct Fin<double> {
  __device__ static double div(double a, double b) { return a / b; }
  __device__ static double sqrt(double a) { return ::sqrt(a); }
  __device__ static double sqrt_ratio(double a, double b) { return ::sqrt(a / b); }
};

// Atomic add with acquire-release semantics at GPU scope: orders this
// thread's earlier writes (the tile's partials) before the ticket, and the
// last arrival sees every other tile's partials, without a separate fence.
__device__ __forceinline__ unsigned int atom_add_acq_rel(unsigned int* p, unsigned int v) {
  unsigned int old;
  asm volatile("atom.add.acq_rel.gpu.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}

// True in every thread of the block that finished a scene's tile set last.
// No thread waits: the last arrival is decided by atomic tickets, first per
// group of kTicketGroup tiles (distinct addresses, so the increments do not
// serialise on one L2 line), then per scene by the last tile of each group.
// Thread 0 wrote the tile's partials, so its acquire-release tickets carry
// them; the block barrier then extends what thread 0 acquired to the block.
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
    int last = 0;
    if (atom_add_acq_rel(gc, 1u) + 1u == (unsigned int)in_grp) {
      *gc = 0u;
      unsigned int* sc = &sd.sc->ctr[table];
      if (atom_add_acq_rel(sc, 1u) + 1u == (unsigned int)ngrp) {
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

// Phases of a Newton iteration in the ticked multi-step form: K1 and the
// assembly, the PCG's init, its iterations, the local solve, the line
// search, the update.  The kernels' finalizers move a scene along them in
// every form; only a ticked scene's kernels check them.
enum : int { kPhNewton = 0, kPhPcgInit = 1, kPhPcg = 2, kPhLocal = 3, kPhLs = 4, kPhApply = 5 };
__device__ __forceinline__ bool not_my_phase(const SceneScalars* sc, int ph) { return sc->ticked && sc->nph != ph; }

// Ends a scene's Newton loop for this timestep (thread 0 of its last tile).
// In the one-step form the batch counts one scene fewer; in the multi-step
// form (steps_target > 0) the scene is flagged for k_step_turn, which
// retires it only after its last step.
__device__ __forceinline__ void end_newton_loop(SceneScalars* sc, BatchCounters* ctrs) {
  sc->newton_active = 0;
  if (sc->steps_target > 0) sc->turn = 1;
  else atomicSub(&ctrs->newton_active, 1);
}

// The per-step Newton, PCG and line-search state of a scene at the start of
// a timestep.
__device__ __forceinline__ void reset_step_scalars(SceneScalars* sc) {
  sc->newton_active = 1;
  sc->newton_iter = 0;
  sc->converged_by_residual = 0;
  sc->status = 0;
  sc->E = 0;
  sc->E_prev = 0;
  sc->eres = 0;
  sc->decrement = 0;
  sc->rhs_norm0 = 0;
  sc->rhs_norm = 0;
  sc->cg_active = 0;
  sc->cg_iter = 0;
  sc->cg_total = 0;
  sc->cg_status = 0;
  sc->cg_err = 0;
  sc->ls_active = 0;
  sc->ls_iter = 0;
  sc->ls_ok = 0;
  sc->ls_total = 0;
  sc->alpha_ls = 1.0;
  sc->alpha_ls_f = 1.0f;
  sc->procrustes_fail = 0;
  sc->nph = kPhNewton;
  sc->cg_scale_exp = 0;
}


}  // namespace mfem_gpu
