// Row-parallel kernels: deterministic assembly of the 3x3-block CSR system
// and the Jacobi / block-Jacobi preconditioned conjugate gradient.
//
//   k_assemble   LHS = PMP + A_mixed and RHS = -PM(x - x~ - h^2 f) - PJW dSdF gl
//                Assembler::update_matrix (sparse_utils.cpp:141-203) gathers
//                each block's element contributions in a fixed sorted order;
//                here one warp owns one block row and sums, in element order,
//                the contributions of the elements incident to its vertex,
//                so no atomics are used and the result is bit-reproducible.
//   k_cg_*       Eigen::ConjugateGradient<.., Lower|Upper, DiagonalPreconditioner>
//                with zero initial guess (eigen_iterative_solver.h:20-29):
//                stop when |r|^2 < tol^2 |b|^2, at most max_iterative_solver_iters.
//                Vectors are Real; every inner product is accumulated in the
//                path's high precision (double, or float-float in the mixed
//                path).
#include <cfloat>

#include "device_math.cuh"
#include "kernels.cuh"
#include "async_copy.cuh"
#include "reduce.cuh"

namespace mfem_gpu {

namespace {

// offset of entry (l, m) of local block (i, j) in the element record
__device__ __forceinline__ int rec_offset(int i, int j, int l, int m) {
  if (i > j) {
    int t = i; i = j; j = t;
    t = l; l = m; m = t;
  }
  const int start = (i == 0) ? 0 : (i == 1 ? 33 : (i == 2 ? 57 : 72));
  if (i == j) {
    if (l > m) { int t = l; l = m; m = t; }
    return start + (l == 0 ? m : (l == 1 ? 2 + m : 5));
  }
  return start + 6 + 9 * (j - i - 1) + 3 * l + m;
}

// Three components of a row of a 4-padded vector: one 16-byte access in
// FP32, two in FP64.  kCo: the load bypasses L1 (data written by other
// blocks earlier in the same launch).
template <bool kCo>
__device__ __forceinline__ void ld3(const float* p, float v[3]) {
  const float4 t = kCo ? __ldcg(reinterpret_cast<const float4*>(p)) : *reinterpret_cast<const float4*>(p);
  v[0] = t.x;
  v[1] = t.y;
  v[2] = t.z;
}
template <bool kCo>
__device__ __forceinline__ void ld3(const double* p, double v[3]) {
  const double2 a = kCo ? __ldcg(reinterpret_cast<const double2*>(p)) : *reinterpret_cast<const double2*>(p);
  const double2 b = kCo ? __ldcg(reinterpret_cast<const double2*>(p) + 1) : reinterpret_cast<const double2*>(p)[1];
  v[0] = a.x;
  v[1] = a.y;
  v[2] = b.x;
}
__device__ __forceinline__ void st3(float* p, const float v[3]) {
  *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], 0.f);
}
__device__ __forceinline__ void st3(double* p, const double v[3]) {
  reinterpret_cast<double2*>(p)[0] = make_double2(v[0], v[1]);
  reinterpret_cast<double2*>(p)[1] = make_double2(v[2], 0.0);
}

// Loads of data that other blocks wrote earlier in the same launch: in the
// persistent PCG (kCo) they bypass L1, which is not coherent across SMs;
// between separate launches a plain load is fine.
template <bool kCo, typename T> __device__ __forceinline__ T ldv(const T* p) {
  if constexpr (kCo) return __ldcg(p);
  else return *p;
}

// Pair w of a packed ELL slot; the column of pair 0 is stored as the
// integer's bits in the first word.
template <bool kCo>
__device__ __forceinline__ float2 ld_pair(const float* ell, size_t pair) {
  const float2* p = reinterpret_cast<const float2*>(ell) + pair;
  return kCo ? __ldcg(p) : *p;
}
template <bool kCo>
__device__ __forceinline__ double2 ld_pair(const double* ell, size_t pair) {
  const double2* p = reinterpret_cast<const double2*>(ell) + pair;
  return kCo ? __ldcg(p) : *p;
}
// L2 policies for the PCG's SpMV: the matrix is streamed once per iteration
// (evict first, no L1 allocation, read-only path), while the vectors the
// SpMV gathers at neighbouring rows are kept (evict last).  Without them the
// 115 MB matrix stream of a 1M-tet scene pushes the 4 MB vectors out of L2.
__device__ __forceinline__ unsigned long long l2_evict_first() {
  unsigned long long p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ unsigned long long l2_evict_last() {
  unsigned long long p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ float2 ld_stream(const float* ell, size_t pair, unsigned long long pol) {
  float2 v;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;"
               : "=f"(v.x), "=f"(v.y) : "l"(reinterpret_cast<const float2*>(ell) + pair), "l"(pol));
  return v;
}
__device__ __forceinline__ double2 ld_stream(const double* ell, size_t pair, unsigned long long pol) {
  double2 v;
  asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.v2.f64 {%0, %1}, [%2], %3;"
               : "=d"(v.x), "=d"(v.y) : "l"(reinterpret_cast<const double2*>(ell) + pair), "l"(pol));
  return v;
}
// Gather of a row's three components with the keep policy (between
// launches only: the persistent form bypasses L1 instead).
__device__ __forceinline__ void ld3_keep(const float* p, float v[3], unsigned long long pol) {
  float4 t;
  asm volatile("ld.global.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
               : "=f"(t.x), "=f"(t.y), "=f"(t.z), "=f"(t.w) : "l"(p), "l"(pol));
  v[0] = t.x;
  v[1] = t.y;
  v[2] = t.z;
}
__device__ __forceinline__ void ld3_keep(const double* p, double v[3], unsigned long long pol) {
  double2 a, b;
  asm volatile("ld.global.L2::cache_hint.v2.f64 {%0, %1}, [%2], %3;" : "=d"(a.x), "=d"(a.y) : "l"(p), "l"(pol));
  asm volatile("ld.global.L2::cache_hint.v2.f64 {%0, %1}, [%2], %3;" : "=d"(b.x), "=d"(b.y) : "l"(p + 2), "l"(pol));
  v[0] = a.x;
  v[1] = a.y;
  v[2] = b.x;
}
template <bool kCo, typename Real>
__device__ __forceinline__ void ld3_gather(const Real* p, Real v[3], unsigned long long pol) {
  if constexpr (kCo) ld3<true>(p, v);
  else ld3_keep(p, v, pol);
}

__device__ __forceinline__ int pair_col(float2 w) { return __float_as_int(w.x); }
__device__ __forceinline__ int pair_col(double2 w) { return (int)__double_as_longlong(w.x); }

// x of the mixed-path PCG in df64: a row is 4 float pairs (32 bytes).
struct X3 {
  df64 v[3];
};
__device__ __forceinline__ X3 zero_x3() { return X3{{df64(0.f), df64(0.f), df64(0.f)}}; }
template <bool kCo>
__device__ __forceinline__ X3 xe_load(const void* base, int row) {
  const float4* p = static_cast<const float4*>(base) + 2 * (size_t)row;
  const float4 a = kCo ? __ldcg(p) : p[0];
  const float4 b = kCo ? __ldcg(p + 1) : p[1];
  return X3{{df64(a.x, a.y), df64(a.z, a.w), df64(b.x, b.y)}};
}
__device__ __forceinline__ void xe_store(void* base, int row, const X3& x) {
  float4* p = static_cast<float4*>(base) + 2 * (size_t)row;
  p[0] = make_float4(x.v[0].hi, x.v[0].lo, x.v[1].hi, x.v[1].lo);
  p[1] = make_float4(x.v[2].hi, x.v[2].lo, 0.f, 0.f);
}

constexpr int kAsmWindow = 64;  // block slots per warp accumulated in shared memory per pass
constexpr int kAsmUnroll = 8;   // incidences whose record entries are in flight together
static_assert(kAsmUnroll == 8, "the 4 entries past 32 of 8 incidences fill one warp");

// Jacobi or block-Jacobi inverse of a free row from its diagonal block D
// (row-major 3x3; zero where the row has no diagonal block).
template <typename Real>
__device__ __forceinline__ void write_row_precond(const SceneDev& sd, int row, const Real* D) {
  Real* dinv = static_cast<Real*>(sd.dinv);
  if (sd.block_jacobi) {
    // inverse of the 3x3 diagonal block (row-major)
    Real c00 = D[4] * D[8] - D[5] * D[7], c01 = D[5] * D[6] - D[3] * D[8],
         c02 = D[3] * D[7] - D[4] * D[6];
    Real det = D[0] * c00 + D[1] * c01 + D[2] * c02;
    if (det != Real(0)) {
      Real id = Real(1) / det;
      dinv[9 * row + 0] = c00 * id;
      dinv[9 * row + 1] = (D[2] * D[7] - D[1] * D[8]) * id;
      dinv[9 * row + 2] = (D[1] * D[5] - D[2] * D[4]) * id;
      dinv[9 * row + 3] = c01 * id;
      dinv[9 * row + 4] = (D[0] * D[8] - D[2] * D[6]) * id;
      dinv[9 * row + 5] = (D[2] * D[3] - D[0] * D[5]) * id;
      dinv[9 * row + 6] = c02 * id;
      dinv[9 * row + 7] = (D[1] * D[6] - D[0] * D[7]) * id;
      dinv[9 * row + 8] = (D[0] * D[4] - D[1] * D[3]) * id;
    } else {
#pragma unroll
      for (int k = 0; k < 9; ++k) dinv[9 * row + k] = (k % 4 == 0) ? Real(1) : Real(0);
    }
  } else {
    // DiagonalPreconditioner: 1/a_ii, or 1 where a_ii == 0
    Real dj[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const Real d = D[4 * c];
      dj[c] = d != Real(0) ? Real(1) / d : Real(1);
    }
    st3(dinv + 4 * (size_t)row, dj);
  }
}

template <typename Real>
__global__ void __launch_bounds__(256) k_assemble(const Tile* tiles, const SceneDev* sds,
                                                            double* partials, int pstride,
                                                            BatchCounters* ctrs) {
  __shared__ unsigned short offtab[4][4][9];
  __shared__ Real acc_s[8][kAsmWindow * 9];
  for (int k = threadIdx.x; k < 144; k += blockDim.x) {
    const int i = k / 36, j = (k / 9) % 4, rc = k % 9;
    offtab[i][j][rc] = (unsigned short)rec_offset(i, j, rc / 3, rc % 3);
  }
  __syncthreads();
  const int tix = blockIdx.x;
  const Tile t = tiles[tix];
  const SceneDev& sd = sds[t.scene];
  SceneScalars* sc = sd.sc;
  if (!sc->newton_active || not_my_phase(sc, kPhNewton)) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  typename Ext<Real>::T rn2 = typename Ext<Real>::T(0);
  for (int rr = warp; rr < kRowTile; rr += 8) {
  const int row = t.begin + rr;
  if (row < t.end) {
    constexpr int RB = sizeof(Real);
    const int rb = sd.b_ptr[row], nb = sd.b_ptr[row + 1] - rb;
    const int ib = sd.inc_ptr[row], ie = sd.inc_ptr[row + 1];
    const int v = sd.free_vert[row];
    // ---- right-hand side in Ext: -sum_b m_vb (x_b - xt_b) + element shares
    using E = typename Ext<Real>::T;
    const Real* mval = static_cast<const Real*>(sd.m_val);
    E acc[3] = {E(0), E(0), E(0)};
    for (int q = sd.m_ptr[v] + lane; q < sd.m_ptr[v + 1]; q += 32) {
      const int b = sd.m_col[q];
      const E m = E(mval[q]);
#pragma unroll
      for (int c = 0; c < 3; ++c)
        acc[c] = acc[c] - m * (Ext<Real>::ld(sd.x, 3 * (size_t)b + c) - Ext<Real>::ld(sd.xt, 3 * (size_t)b + c));
    }
    // the row's first 32 incidences, one a lane: the RHS shares and the
    // block pass below read them from registers
    const int2 inc0 = ib + lane < ie ? sd.inc[ib + lane] : make_int2(0, 0);
    for (int k = ib + lane; k < ie; k += 32) {
      const int2 ic = k < ib + 32 ? inc0 : sd.inc[k];
      const void* rp = sd.rec + (size_t)ic.x * rec_bytes(RB) + rec_rhs_offset(RB);
#pragma unroll
      for (int c = 0; c < 3; ++c) acc[c] = acc[c] + Ext<Real>::ld(rp, 3 * (ic.y & 3) + c);
    }
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) acc[c] = acc[c] + shfl_down(acc[c], off);
    if (lane == 0) {
      Real* rhs = static_cast<Real*>(sd.rhs);
      E r2 = E(0);
      Real rv[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        rv[c] = Real(Ext<Real>::to_real(acc[c]));
        r2 = r2 + acc[c] * acc[c];
      }
      st3(rhs + 4 * (size_t)row, rv);
      rn2 = rn2 + r2;
    }
    // ---- block values: the warp accumulates the row's blocks in shared
    // memory, one incidence (element, local vertex i) at a time; lane l < 36
    // adds entry l % 9 of local block (i, l / 9) to that block's column slot.
    // Slots of one incidence are distinct, so the adds never collide, and
    // every entry sums its contributions in element order.
    const int slice = row >> 5, rs = row & 31;
    const int soff = sd.slice_off[slice], slen = (sd.slice_off[slice + 1] - soff) >> 5;
    Real* val = static_cast<Real*>(sd.ell);
    const Real* bm = static_cast<const Real*>(sd.b_mass) + rb;
    Real* acc_w = acc_s[warp];
    // the diagonal block's slot (the row's own column)
    int qd = -1;
    for (int q0 = 0; q0 < nb; q0 += 32) {
      const bool hit = (q0 + lane < nb) && sd.b_col[rb + q0 + lane] == row;
      const unsigned bal = __ballot_sync(0xffffffffu, hit);
      if (bal && qd < 0) qd = q0 + __ffs(bal) - 1;
    }
    for (int w0 = 0; w0 < nb; w0 += kAsmWindow) {
      const int wn = min(kAsmWindow, nb - w0);
      for (int o = lane; o < 9 * wn; o += 32) acc_w[o] = Real(0);
      __syncwarp();
      // kAsmUnroll incidences per round: their record entries are loaded
      // first (independent gathers in flight together), then added in
      // incidence order with the warp synchronised between incidences, so
      // every entry still sums its contributions in element order.
      for (int c0 = ib; c0 < ie; c0 += 32) {
        const int cn = min(32, ie - c0);
        const int2 my = c0 == ib ? inc0 : (lane < cn ? sd.inc[c0 + lane] : make_int2(0, 0));
        for (int k0 = 0; k0 < cn; k0 += kAsmUnroll) {
          // entry l < 32 of incidence k0 + u in lane l; entries 32..35 of
          // incidence k0 + lane / 4 in lane (lane % 4) + 32
          Real av[kAsmUnroll], aw = Real(0);
          int sv[kAsmUnroll], sw = -1;
          {
            const int uw = lane >> 2, lw = 32 + (lane & 3);
            const int2 icw = make_int2(__shfl_sync(0xffffffffu, my.x, (k0 + uw) & 31),
                                       __shfl_sync(0xffffffffu, my.y, (k0 + uw) & 31));
            if (k0 + uw < cn) {
              const int i = icw.y & 3, j = lw / 9, ent = lw - 9 * j;
              const int slot = (icw.y >> (2 + 7 * j)) & 127, sl = slot - w0;
              if (slot != 127 && sl >= 0 && sl < wn) {
                sw = 9 * sl + ent;
                aw = reinterpret_cast<const Real*>(sd.rec + (size_t)icw.x * rec_bytes(RB))[offtab[i][j][ent]];
              }
            }
          }
#pragma unroll
          for (int u = 0; u < kAsmUnroll; ++u) {
            sv[u] = -1;
            av[u] = Real(0);
            const int2 ic = make_int2(__shfl_sync(0xffffffffu, my.x, (k0 + u) & 31),
                                      __shfl_sync(0xffffffffu, my.y, (k0 + u) & 31));
            if (k0 + u < cn) {
              const int i = ic.y & 3, j = lane / 9, ent = lane - 9 * j;
              const int slot = (ic.y >> (2 + 7 * j)) & 127, sl = slot - w0;
              if (slot != 127 && sl >= 0 && sl < wn) {
                sv[u] = 9 * sl + ent;
                av[u] = reinterpret_cast<const Real*>(sd.rec + (size_t)ic.x * rec_bytes(RB))[offtab[i][j][ent]];
              }
            }
          }
#pragma unroll
          for (int u = 0; u < kAsmUnroll; ++u) {
            if (sv[u] >= 0) acc_w[sv[u]] += av[u];
            if ((lane >> 2) == u && sw >= 0) acc_w[sw] += aw;
            __syncwarp();
          }
        }
      }
      for (int o = lane; o < 9 * wn; o += 32) {
        const int q = o / 9, ent = o - 9 * q;
        val[ell_entry(soff, w0 + q, rs, ent)] =
            acc_w[o] + ((ent == 0 || ent == 4 || ent == 8) ? bm[w0 + q] : Real(0));
      }
      if (lane == 0 && qd >= w0 && qd < w0 + wn) {
        // the diagonal block as written above, from shared memory
        Real D[9];
#pragma unroll
        for (int k = 0; k < 9; ++k)
          D[k] = acc_w[9 * (qd - w0) + k] + ((k == 0 || k == 4 || k == 8) ? bm[qd] : Real(0));
        write_row_precond(sd, row, D);
      }
      __syncwarp();
    }
    // padding blocks of the slice beyond this row's length are zero
    for (int o = lane; o < 9 * (slen - nb); o += 32) {
      const int q = nb + o / 9, ent = o % 9;
      val[ell_entry(soff, q, rs, ent)] = Real(0);
    }
    // ---- preconditioner of a row without a diagonal block
    if (lane == 0 && qd < 0) {
      const Real Z[9] = {Real(0), Real(0), Real(0), Real(0), Real(0), Real(0), Real(0), Real(0), Real(0)};
      write_row_precond(sd, row, Z);
    }
  }
  }
  {
    typename Ext<Real>::T sums[1] = {rn2};
    tile_partials<typename Ext<Real>::T, Real, 1, 0>(sums, nullptr, partials, pstride, 0, tix);
  }
  if (last_tile(sd, TB_ROW, tix)) {
    const auto s_ = scene_sum<typename Ext<Real>::T>(partials, pstride, 0, sd.tile_first[TB_ROW],
                                                     sd.tile_count[TB_ROW]);
    if (threadIdx.x == 0) {
      const double s = to_double_any(s_);
      const double rn = Fin<Real>::sqrt(s);
      if (sc->newton_iter == 0) sc->rhs_norm0 = rn;
      sc->rhs_norm = rn;
      // |rhs_k| <= tol * max(|rhs_0|, |h^2 P M f|)
      if (sd.res_tol > 0 && ((sc->newton_iter > 0 && rn <= sd.res_tol * sc->rhs_norm0) ||
                             rn <= sd.res_tol * sd.load_norm)) {
        sc->converged_by_residual = 1;
        end_newton_loop(sc, ctrs);
      }
      if (!(s == s) || isinf(s)) {
        sc->status = 4;  // MFEM_ERR_NONFINITE
        if (sc->newton_active) end_newton_loop(sc, ctrs);
      }
      if (sc->newton_active) sc->nph = kPhPcgInit;
    }
  }
}

// ---------------------------------------------------------------- PCG ---
// Products of two Reals carried exactly in Ext (TwoProduct in the mixed path).
__device__ __forceinline__ df64 exact_prod(float a, float b) { return two_prod(a, b); }
__device__ __forceinline__ double exact_prod(double a, double b) { return a * b; }

// z = D^{-1} r for one row (Jacobi or 3x3 block Jacobi).
template <typename Real>
__device__ __forceinline__ void apply_prec(const SceneDev& sd, int row, const Real r[3], Real z[3]) {
  const Real* dinv = static_cast<const Real*>(sd.dinv);
  if (sd.block_jacobi) {
    const Real* D = dinv + 9 * (size_t)row;
#pragma unroll
    for (int c = 0; c < 3; ++c) z[c] = D[3 * c] * r[0] + D[3 * c + 1] * r[1] + D[3 * c + 2] * r[2];
  } else {
    Real d[3];
    ld3<false>(dinv + 4 * (size_t)row, d);
#pragma unroll
    for (int c = 0; c < 3; ++c) z[c] = d[c] * r[c];
  }
}

// ------------------------------------------------------------- PCG ------
// Every kernel writes tile partials; the last tile of a scene to finish
// (atomic tickets, no thread waits) reduces them in a fixed order and sets
// the scene's scalars (alpha, beta, the stopping test) for the next kernel.

// r = b, z = D^{-1} b, x = 0, rz; one thread per row.
template <typename Real>
__global__ void __launch_bounds__(kCgThreads) k_cg_init(const Tile* tiles, const SceneDev* sds,
                                                        double* partials, int pstride,
                                                        BatchCounters* ctrs) {
  const int tix = blockIdx.x;
  const Tile t = tiles[tix];
  const SceneDev& sd = sds[t.scene];
  SceneScalars* sc = sd.sc;
  if (!sc->newton_active || not_my_phase(sc, kPhPcgInit)) return;
  using E = typename Ext<Real>::T;
  E dots[2] = {E(0), E(0)};  // r.r, r.z
  const int row = t.begin + threadIdx.x;
  if (row < t.end) {
    const size_t k = 4 * (size_t)row;
    Real r[3], z[3];
    ld3<false>(static_cast<const Real*>(sd.rhs) + k, r);
    apply_prec<Real>(sd, row, r, z);
    const Real zero[3] = {Real(0), Real(0), Real(0)};
    st3(static_cast<Real*>(sd.cg_r) + k, r);
    st3(static_cast<Real*>(sd.cg_z) + k, z);
    st3(static_cast<Real*>(sd.cg_x) + k, zero);
    if (sd.cg_xe) xe_store(sd.cg_xe, row, zero_x3());
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      dots[0] = dots[0] + exact_prod(r[c], r[c]);
      dots[1] = dots[1] + exact_prod(r[c], z[c]);
    }
  }
  tile_partials<E, Real, 2, 0>(dots, nullptr, partials, pstride, 0, tix);
  if (last_tile(sd, TB_CG, tix)) {
    const int t0 = sd.tile_first[TB_CG], tc = sd.tile_count[TB_CG];
    E v[2];
    scene_sums<E, 2>(partials, pstride, 0, t0, tc, v);
    if (threadIdx.x == 0) {
      const double rrs = to_double_any(v[0]), rzs = to_double_any(v[1]);
      sc->cg_rhs_norm2 = rrs;
      sc->cg_iter = 0;
      sc->beta = 0.0;
      sc->beta_f = 0.0f;
      sc->rz = rzs;
      sc->cg_err = 0.0;
      if (rrs == 0.0) {
        sc->cg_active = 0;
        sc->nph = kPhLocal;
      } else {
        const double thr = fmax(sd.cg_tol * sd.cg_tol * rrs, DBL_MIN);
        sc->cg_threshold = thr;
        if (rrs < thr || sd.max_cg <= 0) {
          sc->cg_active = 0;
          sc->nph = kPhLocal;
          sc->cg_err = 1.0;
        } else {
          sc->cg_active = 1;
          atomicAdd(&ctrs->cg_active, 1);
        }
      }
    }
  }
}

// Ap = A p with p = z + beta p_prev formed on the fly (so the p update needs
// no kernel of its own); p is written to the other buffer of the pair.
// One thread per row over the sliced-ELL layout: every matrix load of a
// warp is one coalesced access, the column arriving with the first pair.
template <typename Real, bool kCo>
__device__ __forceinline__ void cg_spmv_tile(int tix, const Tile* tiles, const SceneDev* sds,
                                             double* partials, int pstride) {
  const Tile t = tiles[tix];
  const SceneDev& sd = sds[t.scene];
  SceneScalars* sc = sd.sc;
  if (!ldv<kCo>(&sc->cg_active)) return;
  const int it = ldv<kCo>(&sc->cg_iter);
  const Real beta = sizeof(Real) == 4 ? Real(ldv<kCo>(&sc->beta_f)) : Real(ldv<kCo>(&sc->beta));
  const bool first = (it == 0);
  const Real* z = static_cast<const Real*>(sd.cg_z);
  const Real* pin = static_cast<const Real*>(sd.cg_p[(it + 1) & 1]);
  Real* pout = static_cast<Real*>(sd.cg_p[it & 1]);
  Real* Ap = static_cast<Real*>(sd.cg_Ap);
  const Real* ell = static_cast<const Real*>(sd.ell);
  using E = typename Ext<Real>::T;
  E pAp[1] = {E(0)};
  const int row = t.begin + threadIdx.x;
  if (row < t.end) {
    const int slice = row >> 5, rs = row & 31;
    const int soff = sd.slice_off[slice], slen = (sd.slice_off[slice + 1] - soff) >> 5;
    const unsigned long long pol_s = l2_evict_first(), pol_k = l2_evict_last();
    Real acc0 = 0, acc1 = 0, acc2 = 0;
#pragma unroll 4
    for (int k = 0; k < slen; ++k) {
      const size_t q = ell_pair(soff, k, rs, 0);
      const auto w0 = ld_stream(ell, q, pol_s), w1 = ld_stream(ell, q + 32, pol_s),
                 w2 = ld_stream(ell, q + 64, pol_s), w3 = ld_stream(ell, q + 96, pol_s),
                 w4 = ld_stream(ell, q + 128, pol_s);
      const int col = pair_col(w0);
      Real p[3];
      ld3_gather<kCo>(z + 4 * (size_t)col, p, pol_k);
      if (!first) {
        Real pp[3];
        ld3_gather<kCo>(pin + 4 * (size_t)col, pp, pol_k);
#pragma unroll
        for (int c = 0; c < 3; ++c) p[c] += beta * pp[c];
      }
      acc0 += w0.y * p[0] + w1.x * p[1] + w1.y * p[2];
      acc1 += w2.x * p[0] + w2.y * p[1] + w3.x * p[2];
      acc2 += w3.y * p[0] + w4.x * p[1] + w4.y * p[2];
    }
    const Real acc[3] = {acc0, acc1, acc2};
    Real p[3];
    ld3<kCo>(z + 4 * (size_t)row, p);
    if (!first) {
      Real pp[3];
      ld3<kCo>(pin + 4 * (size_t)row, pp);
#pragma unroll
      for (int c = 0; c < 3; ++c) p[c] += beta * pp[c];
    }
    st3(pout + 4 * (size_t)row, p);
    st3(Ap + 4 * (size_t)row, acc);
#pragma unroll
    for (int c = 0; c < 3; ++c) pAp[0] = pAp[0] + exact_prod(p[c], acc[c]);
  }
  tile_partials<E, Real, 1, 0>(pAp, nullptr, partials, pstride, 0, tix);
  if (last_tile(sd, TB_CG, tix)) {
    E s[1];
    scene_sums<E, 1>(partials, pstride, 0, sd.tile_first[TB_CG], sd.tile_count[TB_CG], s);
    if (threadIdx.x == 0) {
      const double a = Fin<Real>::div(ldv<kCo>(&sc->rz), to_double_any(s[0]));
      sc->alpha = a;
      sc->alpha_f = float(a);
    }
  }
}

// x += alpha p, r -= alpha Ap, z = D^{-1} r, then beta and the stopping test.
template <typename Real, bool kCo>
__device__ __forceinline__ void cg_update_tile(int tix, const Tile* tiles, const SceneDev* sds,
                                               double* partials, int pstride, BatchCounters* ctrs) {
  const Tile t = tiles[tix];
  const SceneDev& sd = sds[t.scene];
  SceneScalars* sc = sd.sc;
  if (!ldv<kCo>(&sc->cg_active)) return;
  const int it = ldv<kCo>(&sc->cg_iter);
  const Real alpha = sizeof(Real) == 4 ? Real(ldv<kCo>(&sc->alpha_f)) : Real(ldv<kCo>(&sc->alpha));
  using E = typename Ext<Real>::T;
  E dots[2] = {E(0), E(0)};  // r.r, r.z
  const int row = t.begin + threadIdx.x;
  if (row < t.end) {
    const size_t k = 4 * (size_t)row;
    Real* x = static_cast<Real*>(sd.cg_x) + k;
    Real* r = static_cast<Real*>(sd.cg_r) + k;
    Real xv[3], pv[3], rv[3], av[3], z[3];
    ld3<kCo>(x, xv);
    ld3<kCo>(static_cast<const Real*>(sd.cg_p[it & 1]) + k, pv);
    ld3<kCo>(r, rv);
    ld3<kCo>(static_cast<const Real*>(sd.cg_Ap) + k, av);
    if (sizeof(Real) == 4 && sd.cg_xe) {
      // x in df64: x += alpha p with the exact product, x rounded for readers
      X3 xe = xe_load<kCo>(sd.cg_xe, row);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        xe.v[c] = xe.v[c] + two_prod(float(alpha), float(pv[c]));
        xv[c] = Real(Ext<float>::to_real(xe.v[c]));
      }
      xe_store(sd.cg_xe, row, xe);
    } else {
#pragma unroll
      for (int c = 0; c < 3; ++c) xv[c] += alpha * pv[c];
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      rv[c] -= alpha * av[c];
      dots[0] = dots[0] + exact_prod(rv[c], rv[c]);
    }
    st3(x, xv);
    st3(r, rv);
    apply_prec<Real>(sd, row, rv, z);
    st3(static_cast<Real*>(sd.cg_z) + k, z);
#pragma unroll
    for (int c = 0; c < 3; ++c) dots[1] = dots[1] + exact_prod(rv[c], z[c]);
  }
  tile_partials<E, Real, 2, 0>(dots, nullptr, partials, pstride, 0, tix);
  if (last_tile(sd, TB_CG, tix)) {
    E v[2];
    scene_sums<E, 2>(partials, pstride, 0, sd.tile_first[TB_CG], sd.tile_count[TB_CG], v);
    if (threadIdx.x == 0) {
      const double rrs = to_double_any(v[0]), rzs = to_double_any(v[1]);
      sc->cg_err = Fin<Real>::sqrt_ratio(rrs, ldv<kCo>(&sc->cg_rhs_norm2));
      bool stop = false;
      if (rrs < ldv<kCo>(&sc->cg_threshold)) {
        stop = true;
      } else {
        const double rz_old = ldv<kCo>(&sc->rz);
        const double b = Fin<Real>::div(rzs, rz_old);
        sc->beta = b;
        sc->beta_f = float(b);
        sc->rz_prev = rz_old;
        sc->rz = rzs;
        sc->cg_iter = it + 1;
        if (it + 1 >= sd.max_cg) {
          stop = true;
          sc->cg_status = 5;  // MFEM_ERR_CG_MAXITER
        }
      }
      if (!(rrs == rrs)) {
        stop = true;
        sc->status = 4;
      }
      if (stop) {
        sc->cg_total = ldv<kCo>(&sc->cg_total) + ldv<kCo>(&sc->cg_iter);
        sc->cg_active = 0;
        sc->nph = kPhLocal;
        atomicSub(&ctrs->cg_active, 1);
      }
    }
  }
}

// Residual replacement of the mixed path (reliable updates): r = b - A x
// with x in df64, each FP32 matrix entry times x as an exact product summed
// in df64, then z = D^{-1} r, (r, r) and (r, z).  The last tile restarts
// beta from the true (r, z) and applies the stopping test to the true
// residual.  The search direction is kept.
template <bool kCo>
__device__ __forceinline__ void cg_replace_tile(int tix, const Tile* tiles, const SceneDev* sds,
                                                double* partials, int pstride, BatchCounters* ctrs) {
  const Tile t = tiles[tix];
  const SceneDev& sd = sds[t.scene];
  SceneScalars* sc = sd.sc;
  if (!ldv<kCo>(&sc->cg_active) || !sd.cg_xe) return;
  if (ldv<kCo>(&sc->cg_iter) % kCgReplace != 0) return;
  const float* ell = static_cast<const float*>(sd.ell);
  df64 dots[2] = {df64(0.f), df64(0.f)};
  const int row = t.begin + threadIdx.x;
  if (row < t.end) {
    const int slice = row >> 5, rs = row & 31;
    const int soff = sd.slice_off[slice], slen = (sd.slice_off[slice + 1] - soff) >> 5;
    df64 acc[3] = {df64(0.f), df64(0.f), df64(0.f)};
    for (int k = 0; k < slen; ++k) {
      const size_t q = ell_pair(soff, k, rs, 0);
      const float2 w0 = ld_pair<false>(ell, q), w1 = ld_pair<false>(ell, q + 32),
                   w2 = ld_pair<false>(ell, q + 64), w3 = ld_pair<false>(ell, q + 96),
                   w4 = ld_pair<false>(ell, q + 128);
      const X3 xc = xe_load<kCo>(sd.cg_xe, pair_col(w0));
      const float a[9] = {w0.y, w1.x, w1.y, w2.x, w2.y, w3.x, w3.y, w4.x, w4.y};
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const float aij = a[3 * i + j];
          acc[i] = acc[i] + two_prod(aij, xc.v[j].hi) + df64(aij * xc.v[j].lo);
        }
    }
    float b[3], r[3], z[3];
    ld3<false>(static_cast<const float*>(sd.rhs) + 4 * (size_t)row, b);
#pragma unroll
    for (int c = 0; c < 3; ++c) r[c] = Ext<float>::to_real(df64(b[c]) - acc[c]);
    apply_prec<float>(sd, row, r, z);
    st3(static_cast<float*>(sd.cg_r) + 4 * (size_t)row, r);
    st3(static_cast<float*>(sd.cg_z) + 4 * (size_t)row, z);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      dots[0] = dots[0] + exact_prod(r[c], r[c]);
      dots[1] = dots[1] + exact_prod(r[c], z[c]);
    }
  }
  tile_partials<df64, float, 2, 0>(dots, nullptr, partials, pstride, 0, tix);
  if (last_tile(sd, TB_CG, tix)) {
    df64 v[2];
    scene_sums<df64, 2>(partials, pstride, 0, sd.tile_first[TB_CG], sd.tile_count[TB_CG], v);
    if (threadIdx.x == 0) {
      const double rrs = to_double_any(v[0]), rzs = to_double_any(v[1]);
      sc->cg_err = Fin<float>::sqrt_ratio(rrs, ldv<kCo>(&sc->cg_rhs_norm2));
      if (rrs < ldv<kCo>(&sc->cg_threshold) || !(rrs == rrs)) {
        if (!(rrs == rrs)) sc->status = 4;
        // x_{cg_iter} meets the threshold: as in Eigen, that iteration is not counted
        const int done = ldv<kCo>(&sc->cg_iter) - 1;
        sc->cg_iter = done;
        sc->cg_total = ldv<kCo>(&sc->cg_total) + done;
        sc->cg_status = 0;
        sc->cg_active = 0;
        sc->nph = kPhLocal;
        atomicSub(&ctrs->cg_active, 1);
      } else {
        const double b2 = Fin<float>::div(rzs, ldv<kCo>(&sc->rz_prev));
        sc->beta = b2;
        sc->beta_f = float(b2);
        sc->rz = rzs;
      }
    }
  }
}

__global__ void __launch_bounds__(kCgThreads) k_cg_replace(const Tile* tiles, const SceneDev* sds,
                                                           double* partials, int pstride,
                                                           BatchCounters* ctrs) {
  cg_replace_tile<false>(blockIdx.x, tiles, sds, partials, pstride, ctrs);
}

// At most 40 registers in FP32, so that six blocks fit on an SM and a
// 1M-tet scene's PCG rows (873 tiles) run in one wave on 152 SMs.
template <typename Real>
__global__ void __launch_bounds__(kCgThreads, sizeof(Real) == 4 ? 6 : 4) k_cg_spmv(
    const Tile* tiles, const SceneDev* sds, double* partials, int pstride, BatchCounters* ctrs) {
  cg_spmv_tile<Real, false>(blockIdx.x, tiles, sds, partials, pstride);
}

template <typename Real>
__global__ void __launch_bounds__(kCgThreads) k_cg_update(const Tile* tiles, const SceneDev* sds,
                                                          double* partials, int pstride,
                                                          BatchCounters* ctrs) {
  cg_update_tile<Real, false>(blockIdx.x, tiles, sds, partials, pstride, ctrs);
}

// ------------------------------------------- single-reduction PCG ---
// Chronopoulos and Gear's PCG ("s-step" with s = 1): with u = M^{-1} r and
// w = A u, one iteration is
//   p_i = u_i + b_i p_{i-1},  s_i = w_i + b_i s_{i-1},
//   x_{i+1} = x_i + a_i p_i,  r_{i+1} = r_i - a_i s_i,  u_{i+1} = M^{-1} r_{i+1},
//   w_{i+1} = A u_{i+1},  g = (r, u), d = (w, u), rr = (r, r) at i+1,
//   b_{i+1} = g_{i+1} / g_i,  a_{i+1} = g_{i+1} / (d_{i+1} - b_{i+1} g_{i+1} / a_i),
// so its three inner products reduce together and an iteration is ONE
// launch: the SpMV needs u_{i+1} at neighbouring rows, which each thread
// forms from the previous iteration's r, w and s of that row (kept by
// iteration parity, so no row is overwritten while another block reads it).
// In exact arithmetic the iterates are those of the two-reduction PCG.

// acc += B u for one packed ELL slot (pairs (col, a00) (a01, a02) (a10, a11)
// (a12, a20) (a21, a22)), as explicit FMA chains: every form of the fused
// iteration (registers or staged through shared memory) rounds alike.
template <typename P, typename Real>
__device__ __forceinline__ void ell_block_fma(const P& w0, const P& w1, const P& w2, const P& w3, const P& w4,
                                              const Real u[3], Real& a0, Real& a1, Real& a2) {
  a0 = fma(w1.y, u[2], fma(w1.x, u[1], fma(w0.y, u[0], a0)));
  a1 = fma(w3.x, u[2], fma(w2.y, u[1], fma(w2.x, u[0], a1)));
  a2 = fma(w4.y, u[2], fma(w4.x, u[1], fma(w3.y, u[0], a2)));
}

// u_{i+1} of a row from r_i, w_i, s_{i-1}: the same operations, in the same
// order, wherever a row's value is formed.
template <typename Real>
__device__ __forceinline__ void cgf_next(const SceneDev& sd, int row, const Real r[3], const Real w[3],
                                         const Real sp[3], Real a, Real b, Real s[3], Real rn[3],
                                         Real u[3]) {
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    s[c] = fma(b, sp[c], w[c]);
    rn[c] = fma(-a, s[c], r[c]);
  }
  apply_prec<Real>(sd, row, rn, u);
}

__device__ __forceinline__ void cgf_verify_step(const SceneDev& sd, BatchCounters* ctrs, double rr, double g,
                                                double d, double su, double ps, int it);

// The three inner products of one tile as tile partials; the scene's last
// tile reduces them and sets a, b of the next iteration and the stopping
// test (Eigen's |r|^2 < tol^2 |b|^2).  A bounded wait that ran out in this
// launch (ctrs->error) ends the solve.
template <typename Real, bool kInit, int NQ = 3>
__device__ __forceinline__ void cgf_finish(const SceneDev& sd, BatchCounters* ctrs,
                                           typename Ext<Real>::T (&dots)[NQ], double* partials,
                                           int pstride, int tix, int it) {
  using E = typename Ext<Real>::T;
  SceneScalars* sc = sd.sc;
  tile_partials<E, Real, NQ, 0>(dots, nullptr, partials, pstride, 0, tix);
  if (last_tile(sd, TB_CG, tix)) {
    E v[NQ];
    scene_sums<E, NQ>(partials, pstride, 0, sd.tile_first[TB_CG], sd.tile_count[TB_CG], v);
    if (threadIdx.x == 0) {
      const double rr = to_double_any(v[0]), g = to_double_any(v[1]), d = to_double_any(v[2]);
      const double su = NQ > 3 ? to_double_any(v[NQ > 3 ? 3 : 0]) : 0.0;
      const double ps = NQ > 4 ? to_double_any(v[NQ > 4 ? 4 : 0]) : 0.0;
      if (kInit) {
        sc->cg_rhs_norm2 = rr;
        sc->cg_iter = 0;
        sc->cg_err = 0.0;
        sc->cgf_phase = 0;
        sc->cgf_rounds = 0;
        const double thr = fmax(sd.cg_tol * sd.cg_tol * rr, DBL_MIN);
        sc->cg_threshold = thr;
        if (rr == 0.0) {
          sc->cg_active = 0;
          sc->nph = kPhLocal;
        } else if (rr < thr || sd.max_cg <= 0) {
          sc->cg_active = 0;
          sc->nph = kPhLocal;
          sc->cg_err = 1.0;
        } else {
          sc->cg_active = 1;
          atomicAdd(&ctrs->cg_active, 1);
        }
        sc->nph = sc->cg_active ? kPhPcg : kPhLocal;
        const double a0 = Fin<Real>::div(g, d);
        sc->cgf_gamma[0] = g;
        sc->alpha = a0;
        sc->alpha_f = float(a0);
        sc->beta = 0.0;
        sc->beta_f = 0.0f;
      } else if (sizeof(Real) == 4 && sd.cg_xe) {
        cgf_verify_step(sd, ctrs, rr, g, d, su, ps, it);
      } else {
        bool stop = false;
        sc->cg_err = Fin<Real>::sqrt_ratio(rr, sc->cg_rhs_norm2);
        if (rr < sc->cg_threshold) {
          stop = true;
        } else {
          const double bn = Fin<Real>::div(g, sc->cgf_gamma[0]);
          const double an = Fin<Real>::div(g, d - Fin<Real>::div(bn * g, sc->alpha));
          sc->beta = bn;
          sc->beta_f = float(bn);
          sc->alpha = an;
          sc->alpha_f = float(an);
          sc->cgf_gamma[0] = g;
          sc->cg_iter = it + 1;
          if (it + 1 >= sd.max_cg) {
            stop = true;
            sc->cg_status = 5;  // MFEM_ERR_CG_MAXITER
          }
        }
        if (!(rr == rr)) {
          stop = true;
          sc->status = 4;
        }
        if (*(volatile int*)&ctrs->error) stop = true;  // the host reports MFEM_ERR_TIMEOUT
        if (stop) {
          sc->cg_total += sc->cg_iter;
          sc->cg_active = 0;
          sc->nph = kPhLocal;
          atomicSub(&ctrs->cg_active, 1);
        }
      }
    }
  }
}

// ---------------------------------------- verified stop (mixed path) ---
// In FP32 the single-reduction recurrences drift: the recursive residual
// meets the tolerance while the true |b - A x| / |b| sits several times
// above it (x itself rounded to FP32 floors it near eps32 |A||x| / |b|).
// So when the recursion says "converged", the mixed path verifies before it
// stops, in three further launches of the same kernel (the scene's
// cgf_phase selects the work; the iteration count does not move):
//   1  r = b - A (x_e + x), with each FP32 matrix entry times the df64
//      x_e + x as an exact product summed in df64 (the reliable residual);
//      u = M^-1 r;
//   2  x_e += x, x = 0 (the FP32 x restarts as a correction, so its
//      rounding shrinks with what is left to solve); w = A u and s = A p
//      (the recursions' drift starts again from zero); the inner products
//      of the true residual.  If it meets the tolerance: phase 3.
//      Otherwise the recursion continues from the replaced r, w and s:
//      the next direction u + b p is made A-conjugate to p directly (b =
//      -(A p, u) / (p, A p)), because the drifted recursion's
//      gamma_prev no longer describes the true residual, and a from the
//      exact (p_new, A p_new).  After kCgfRounds failed verifications the
//      next recursive stop is accepted as it is;
//   3  x_e += x, and x = round(x_e) for the readers of the solution; stop.
// A stop on max_iterative_solver_iters or a non-finite residual also goes
// through phase 3, so the solution is always x_e + x.

// The finalizer's part for the mixed path (thread 0 of the scene's last tile).
constexpr int kCgfRounds = 4;
__device__ __forceinline__ void cgf_verify_step(const SceneDev& sd, BatchCounters* ctrs, double rr, double g,
                                                double d, double su, double ps, int it) {
  SceneScalars* sc = sd.sc;
  const int ph = sc->cgf_phase;
  if (ph == 1) {
    sc->cgf_phase = 2;
    return;
  }
  if (ph == 3 || *(volatile int*)&ctrs->error) {
    sc->cg_total += sc->cg_iter;
    sc->cg_active = 0;
    sc->nph = kPhLocal;
    atomicSub(&ctrs->cg_active, 1);
    return;
  }
  sc->cg_err = Fin<float>::sqrt_ratio(rr, sc->cg_rhs_norm2);
  if (!(rr == rr)) {
    sc->status = 4;
    sc->cgf_phase = 3;
    return;
  }
  if (rr < sc->cg_threshold) {
    // phase 0: the recursion's residual passes, verify it (unless the
    // verifications are used up); phase 2: the true residual passes, write
    // the solution
    sc->cgf_phase = (ph == 0 && sc->cgf_rounds < kCgfRounds) ? 1 : 3;
    return;
  }
  double bn, an;
  if (ph == 2) {
    // A failed verification.  The recursion's gamma had drifted below the
    // true residual's, so b = gamma / gamma_prev would be far too large: the
    // new direction is made A-conjugate to the last one directly,
    // b = -(A p, u) / (p, A p), and (p_new, A p_new) = d + 2 b (A p, u) +
    // b^2 (p, A p) from phase 2's exact A p.
    sc->cgf_rounds += 1;
    bn = -Fin<float>::div(su, ps);
    an = Fin<float>::div(g, d + 2.0 * bn * su + bn * bn * ps);
  } else {
    bn = Fin<float>::div(g, sc->cgf_gamma[0]);
    an = Fin<float>::div(g, d - Fin<float>::div(bn * g, sc->alpha));
  }
  sc->beta = bn;
  sc->beta_f = float(bn);
  sc->alpha = an;
  sc->alpha_f = float(an);
  sc->cgf_gamma[0] = g;
  sc->cg_iter = it + 1;
  sc->cgf_phase = 0;
  if (it + 1 >= sd.max_cg) {
    sc->cg_status = 5;  // MFEM_ERR_CG_MAXITER
    sc->cgf_phase = 3;
  }
}

// One launch of phases 1..3 for one tile (plain loads: these are a few
// launches per solve).
template <bool kScaled>
__device__ __noinline__ void cgf_verify_tile(int ph, int tix, const Tile* tiles, const SceneDev* sds,
                                             double* partials, int pstride, BatchCounters* ctrs) {
  const Tile t = tiles[tix];
  const SceneDev& sd = sds[t.scene];
  SceneScalars* sc = sd.sc;
  const int it = sc->cg_iter;
  float* r_cur = static_cast<float*>(sd.cgf_r[(it + 1) & 1]);  // r_{it+1}, replaced in phase 1
  float* w_cur = static_cast<float*>(sd.cgf_w[(it + 1) & 1]);  // w_{it+1}, replaced in phase 2
  float* x = static_cast<float*>(sd.cg_x);
  float* u = static_cast<float*>(sd.cg_z);
  const float* ell = static_cast<const float*>(sd.ell);
  // (r,r), (r,u), (w,u) and in phase 2 also (A p, u), (p, A p)
  df64 dots[5] = {df64(0.f), df64(0.f), df64(0.f), df64(0.f), df64(0.f)};
  const int row = t.begin + threadIdx.x;
  if (row < t.end) {
    const size_t k4 = 4 * (size_t)row;
    const int slice = row >> 5, rs = row & 31;
    const int soff = sd.slice_off[slice], slen = (sd.slice_off[slice + 1] - soff) >> 5;
    if (ph == 1) {
      df64 acc[3] = {df64(0.f), df64(0.f), df64(0.f)};
      for (int k = 0; k < slen; ++k) {
        const size_t q = ell_pair(soff, k, rs, 0);
        const float2 w0 = ld_pair<false>(ell, q), w1 = ld_pair<false>(ell, q + 32),
                     w2 = ld_pair<false>(ell, q + 64), w3 = ld_pair<false>(ell, q + 96),
                     w4 = ld_pair<false>(ell, q + 128);
        const int col = pair_col(w0);
        X3 xc = xe_load<false>(sd.cg_xe, col);
        float xf[3];
        ld3<false>(x + 4 * (size_t)col, xf);
#pragma unroll
        for (int j = 0; j < 3; ++j) xc.v[j] = xc.v[j] + df64(xf[j]);
        const float a[9] = {w0.y, w1.x, w1.y, w2.x, w2.y, w3.x, w3.y, w4.x, w4.y};
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            const float aij = a[3 * i + j];
            acc[i] = acc[i] + two_prod(aij, xc.v[j].hi) + df64(aij * xc.v[j].lo);
          }
      }
      float bv[3], r[3], z[3];
      ld3<false>(static_cast<const float*>(sd.rhs) + k4, bv);
#pragma unroll
      for (int c = 0; c < 3; ++c) r[c] = Ext<float>::to_real(df64(ldexpf(bv[c], sc->cg_scale_exp)) - acc[c]);
      apply_prec<float>(sd, row, r, z);
      st3(r_cur + k4, kScaled ? z : r);  // the scaled form keeps r~ = M^-1 r (= u)
      if (!kScaled) st3(u + k4, z);
    } else if (ph == 2) {
      // fold x into x_e
      X3 xe = xe_load<false>(sd.cg_xe, row);
      float xf[3];
      ld3<false>(x + k4, xf);
#pragma unroll
      for (int c = 0; c < 3; ++c) xe.v[c] = xe.v[c] + df64(xf[c]);
      xe_store(sd.cg_xe, row, xe);
      const float zero[3] = {0.f, 0.f, 0.f};
      st3(x + k4, zero);
      // w = A u with u of the neighbours as phase 1 stored it, and s = A p
      // (the recursion's s_it, whose drift is what moves r away from b - A x)
      const float* pv = static_cast<const float*>(sd.cg_p[0]);
      float acc0 = 0.f, acc1 = 0.f, acc2 = 0.f, sa0 = 0.f, sa1 = 0.f, sa2 = 0.f;
      for (int k = 0; k < slen; ++k) {
        const size_t q = ell_pair(soff, k, rs, 0);
        const float2 w0 = ld_pair<false>(ell, q), w1 = ld_pair<false>(ell, q + 32),
                     w2 = ld_pair<false>(ell, q + 64), w3 = ld_pair<false>(ell, q + 96),
                     w4 = ld_pair<false>(ell, q + 128);
        const size_t c4 = 4 * (size_t)pair_col(w0);
        float uc[3], pc[3];
        ld3<false>((kScaled ? r_cur : u) + c4, uc);
        ld3<false>(pv + c4, pc);
        ell_block_fma(w0, w1, w2, w3, w4, uc, acc0, acc1, acc2);
        ell_block_fma(w0, w1, w2, w3, w4, pc, sa0, sa1, sa2);
      }
      float* s_cur = static_cast<float*>(sd.cgf_s[it & 1]);  // s_it
      float un[3], rn[3];
      ld3<false>((kScaled ? r_cur : u) + k4, un);
      if (kScaled) {
        float dv[3];
        ld3<false>(static_cast<const float*>(sd.dinv) + k4, dv);
#pragma unroll
        for (int c = 0; c < 3; ++c) rn[c] = un[c] / dv[c];
        const float ws[3] = {dv[0] * acc0, dv[1] * acc1, dv[2] * acc2};
        const float ss[3] = {dv[0] * sa0, dv[1] * sa1, dv[2] * sa2};
        st3(w_cur + k4, ws);
        st3(s_cur + k4, ss);
      } else {
        ld3<false>(r_cur + k4, rn);
        const float wn[3] = {acc0, acc1, acc2};
        const float sn[3] = {sa0, sa1, sa2};
        st3(w_cur + k4, wn);
        st3(s_cur + k4, sn);
      }
      const float wn[3] = {acc0, acc1, acc2};
      const float san[3] = {sa0, sa1, sa2};
      float po[3];
      ld3<false>(pv + k4, po);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        dots[0] = dots[0] + exact_prod(rn[c], rn[c]);
        dots[1] = dots[1] + exact_prod(rn[c], un[c]);
        dots[2] = dots[2] + exact_prod(wn[c], un[c]);
        dots[3] = dots[3] + exact_prod(san[c], un[c]);
        dots[4] = dots[4] + exact_prod(po[c], san[c]);
      }
    } else {
      // the solution: x_e + x in x_e, and rounded to FP32 in x for its
      // readers, scaled back by 2^-cg_scale_exp
      X3 xe = xe_load<false>(sd.cg_xe, row);
      float xf[3];
      ld3<false>(x + k4, xf);
      const int ue = -sc->cg_scale_exp;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        xe.v[c] = xe.v[c] + df64(xf[c]);
        xe.v[c] = df64(ldexpf(xe.v[c].hi, ue), ldexpf(xe.v[c].lo, ue));
        xf[c] = Ext<float>::to_real(xe.v[c]);
      }
      xe_store(sd.cg_xe, row, xe);
      st3(x + k4, xf);
    }
  }
  cgf_finish<float, false, 5>(sd, ctrs, dots, partials, pstride, tix, it);
}

// One launch of the single-reduction PCG (init: r0 = b, x = 0, p = 0,
// s_{-1} = 0, u0 = M^{-1} b, w0 = A u0).  The scene's last tile reduces the
// three inner products and sets a, b of the next iteration.
//
// kScaled (Jacobi preconditioner, M = diag(A)): r, w and s are kept scaled
// by M^{-1} (r~ = M^{-1} r, ...).  The recurrences are linear, so
// s~ = w~ + b s~_prev and u = r~ - a s~: a neighbour's u needs three
// gathers and no preconditioner gather, and u is r~ itself (no u vector).
// The own row unscales r = r~ / M^{-1} for the inner products.
template <typename Real, bool kInit, bool kScaled>
__device__ __forceinline__ void cgf_tile(int tix, const Tile* tiles, const SceneDev* sds,
                                         double* partials, int pstride, BatchCounters* ctrs) {
  const Tile t = tiles[tix];
  const SceneDev& sd = sds[t.scene];
  SceneScalars* sc = sd.sc;
  if (kInit ? (!sc->newton_active || not_my_phase(sc, kPhPcgInit)) : !sc->cg_active) return;
  if constexpr (!kInit && sizeof(Real) == 4) {
    if (const int ph = sc->cgf_phase) {
      cgf_verify_tile<kScaled>(ph, tix, tiles, sds, partials, pstride, ctrs);
      return;
    }
  }
  const int it = kInit ? 0 : sc->cg_iter;
  const Real a = kInit ? Real(0) : (sizeof(Real) == 4 ? Real(sc->alpha_f) : Real(sc->alpha));
  const Real b = kInit ? Real(0) : (sizeof(Real) == 4 ? Real(sc->beta_f) : Real(sc->beta));
  // old (read) and new (written) buffers of the ping-ponged vectors
  const Real* r_old = static_cast<const Real*>(kInit ? sd.rhs : sd.cgf_r[it & 1]);
  const Real* w_old = static_cast<const Real*>(sd.cgf_w[it & 1]);
  const Real* s_old = static_cast<const Real*>(sd.cgf_s[(it + 1) & 1]);
  Real* r_new = static_cast<Real*>(sd.cgf_r[kInit ? 0 : (it + 1) & 1]);
  Real* w_new = static_cast<Real*>(sd.cgf_w[kInit ? 0 : (it + 1) & 1]);
  Real* s_new = static_cast<Real*>(sd.cgf_s[kInit ? 1 : it & 1]);
  Real* x = static_cast<Real*>(sd.cg_x);
  Real* u = static_cast<Real*>(sd.cg_z);
  Real* p = static_cast<Real*>(sd.cg_p[0]);
  const Real* ell = static_cast<const Real*>(sd.ell);
  using E = typename Ext<Real>::T;
  E dots[3] = {E(0), E(0), E(0)};  // (r,r), (r,u), (w,u) at it+1
  const int row = t.begin + threadIdx.x;
  if (row < t.end) {
    const size_t k4 = 4 * (size_t)row;
    Real un[3], rn[3], dv[3];
    if (kScaled) ld3<false>(static_cast<const Real*>(sd.dinv) + k4, dv);
    if (kInit) {
      ld3<false>(r_old + k4, rn);
      if constexpr (sizeof(Real) == 4) {
#pragma unroll
        for (int c = 0; c < 3; ++c) rn[c] = ldexpf(rn[c], sc->cg_scale_exp);
      }
      apply_prec<Real>(sd, row, rn, un);
      const Real zero[3] = {Real(0), Real(0), Real(0)};
      st3(x + k4, zero);
      st3(p + k4, zero);
      st3(s_new + k4, zero);
      if (sizeof(Real) == 4 && sd.cg_xe) xe_store(sd.cg_xe, row, zero_x3());
    } else {
      Real rv[3], wv[3], sp[3], sv[3], uv[3], pv[3], xv[3];
      ld3<false>(r_old + k4, rv);
      ld3<false>(w_old + k4, wv);
      ld3<false>(s_old + k4, sp);
      if (kScaled) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          sv[c] = fma(b, sp[c], wv[c]);
          un[c] = fma(-a, sv[c], rv[c]);
          rn[c] = un[c] / dv[c];
          uv[c] = rv[c];  // u_i = r~_i
        }
      } else {
        cgf_next<Real>(sd, row, rv, wv, sp, a, b, sv, rn, un);
        ld3<false>(u + k4, uv);
      }
      ld3<false>(p + k4, pv);
      ld3<false>(x + k4, xv);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        pv[c] = fma(b, pv[c], uv[c]);
        xv[c] = fma(a, pv[c], xv[c]);
      }
      st3(p + k4, pv);
      st3(x + k4, xv);
      st3(s_new + k4, sv);
    }
    if (kScaled) {
      st3(r_new + k4, un);
    } else {
      st3(r_new + k4, rn);
      st3(u + k4, un);
    }
    // w_{i+1} = A u_{i+1}
    const int slice = row >> 5, rs = row & 31;
    const int soff = sd.slice_off[slice], slen = (sd.slice_off[slice + 1] - soff) >> 5;
    const unsigned long long pol_s = l2_evict_first(), pol_k = l2_evict_last();
    Real acc0 = 0, acc1 = 0, acc2 = 0;
#pragma unroll 1
    for (int k = 0; k < slen; ++k) {
      const size_t q = ell_pair(soff, k, rs, 0);
      const auto w0 = ld_stream(ell, q, pol_s), w1 = ld_stream(ell, q + 32, pol_s),
                 w2 = ld_stream(ell, q + 64, pol_s), w3 = ld_stream(ell, q + 96, pol_s),
                 w4 = ld_stream(ell, q + 128, pol_s);
      const int col = pair_col(w0);
      const size_t c4 = 4 * (size_t)col;
      Real uc[3];
      if (kInit) {
        Real bc[3];
        ld3_keep(r_old + c4, bc, pol_k);
        if constexpr (sizeof(Real) == 4) {
#pragma unroll
          for (int c = 0; c < 3; ++c) bc[c] = ldexpf(bc[c], sc->cg_scale_exp);
        }
        apply_prec<Real>(sd, col, bc, uc);
      } else {
        Real rc[3], wc[3], spc[3], sc_[3], rnc[3];
        ld3_keep(r_old + c4, rc, pol_k);
        ld3_keep(w_old + c4, wc, pol_k);
        ld3_keep(s_old + c4, spc, pol_k);
        if (kScaled) {
#pragma unroll
          for (int c = 0; c < 3; ++c) uc[c] = fma(-a, fma(b, spc[c], wc[c]), rc[c]);
        } else {
          cgf_next<Real>(sd, col, rc, wc, spc, a, b, sc_, rnc, uc);
        }
      }
      ell_block_fma(w0, w1, w2, w3, w4, uc, acc0, acc1, acc2);
    }
    const Real wn[3] = {acc0, acc1, acc2};
    if (kScaled) {
      // the row's M^{-1} again (an L1/L2 hit) rather than held across the loop
      ld3<false>(static_cast<const Real*>(sd.dinv) + k4, dv);
      const Real ws[3] = {dv[0] * acc0, dv[1] * acc1, dv[2] * acc2};
      st3(w_new + k4, ws);
    } else {
      st3(w_new + k4, wn);
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      dots[0] = dots[0] + exact_prod(rn[c], rn[c]);
      dots[1] = dots[1] + exact_prod(rn[c], un[c]);
      dots[2] = dots[2] + exact_prod(wn[c], un[c]);
    }
  }
  cgf_finish<Real, kInit>(sd, ctrs, dots, partials, pstride, tix, it);
}

// Mixed path: the power of two 2^k with max |2^k b_i| in [0.5, 1), taken
// from the entries' largest magnitude (no squares, so nothing underflows on
// the way); the PCG then runs on 2^k b.  Scaling by a power of two is exact,
// so for right-hand sides well inside FP32's range the iterates are those of
// the unscaled solve, scaled.
__global__ void __launch_bounds__(kCgThreads) k_cgf_scale(const Tile* tiles, const SceneDev* sds,
                                                         double* partials, int pstride, BatchCounters* ctrs) {
  const Tile t = tiles[blockIdx.x];
  const SceneDev& sd = sds[t.scene];
  SceneScalars* sc = sd.sc;
  if (!sc->newton_active || not_my_phase(sc, kPhPcgInit)) return;
  float m[1] = {0.f};
  const int row = t.begin + threadIdx.x;
  if (row < t.end) {
    float bv[3];
    ld3<false>(static_cast<const float*>(sd.rhs) + 4 * (size_t)row, bv);
    m[0] = fmaxf(fabsf(bv[0]), fmaxf(fabsf(bv[1]), fabsf(bv[2])));
  }
  tile_partials<df64, float, 0, 1>(nullptr, m, partials, pstride, 0, blockIdx.x);
  if (last_tile(sd, TB_CG, blockIdx.x)) {
    const float mx = scene_max<float>(partials, pstride, 0, sd.tile_first[TB_CG], sd.tile_count[TB_CG]);
    if (threadIdx.x == 0) {
      int e = 0;
      if (mx > 0.f && isfinite(mx)) frexpf(mx, &e);
      sc->cg_scale_exp = -e;
    }
  }
}

// kScaled: every scene of the batch uses the Jacobi preconditioner.
template <typename Real, bool kScaled>
__global__ void __launch_bounds__(kCgThreads) k_cgf_init(const Tile* tiles, const SceneDev* sds,
                                                         double* partials, int pstride,
                                                         BatchCounters* ctrs) {
  cgf_tile<Real, true, kScaled>(blockIdx.x, tiles, sds, partials, pstride, ctrs);
}

template <typename Real, bool kScaled>
__global__ void __launch_bounds__(kCgThreads, sizeof(Real) == 4 ? 6 : 4) k_cgf_iter(
    const Tile* tiles, const SceneDev* sds, double* partials, int pstride, BatchCounters* ctrs) {
  cgf_tile<Real, false, kScaled>(blockIdx.x, tiles, sds, partials, pstride, ctrs);
}


// ------------------------------------------- staged fused iteration ---
// The same iteration as cgf_tile (not the init), with the matrix streamed
// through shared memory: each warp owns one 32-row slice of the packed
// sliced ELL, whose ELL slot k (the 32 rows' block k: 160 pairs, contiguous
// in global memory) is one bulk copy (cp.async.bulk, the TMA engine) into a
// ring of S stages, completed on one mbarrier per stage.  Lane 0 keeps S
// slots in flight: a stage is refilled with slot k + S as soon as the warp
// has read slot k out of it.  The column -> gather -> FMA chain of a slot
// then starts from shared memory, and the DRAM latency of the matrix stream
// is hidden behind the S - 1 slots ahead instead of sitting in every
// slot's chain.  Arithmetic and its order are those of cgf_tile (bitwise
// the same results).
//
// Shared memory: (blockDim / 32) warps x S stages x 160 pairs, then S
// mbarriers per warp.  Every wait is bounded; one that runs out raises
// ctrs->error, waits (bounded) for the warp's copies still in flight and
// leaves the rest of the slice undone.
template <typename Real> struct PairOf;
template <> struct PairOf<float> { using T = float2; };
template <> struct PairOf<double> { using T = double2; };

constexpr int kSlotPairs = 160;  // pairs of one ELL slot of a 32-row slice

template <typename Real, int S>
constexpr size_t cgf_staged_smem_bytes(int warps) {
  return (size_t)warps * S * kSlotPairs * sizeof(typename PairOf<Real>::T) + (size_t)warps * S * 8;
}

// L2 policy of the matrix stream: all lines evict-first (keep = 0), or half
// of them evict-last (keep = 1), so that about half the matrix can stay in
// L2 from one iteration to the next.
template <int kKeep>
__device__ __forceinline__ unsigned long long l2_matrix_policy() {
  unsigned long long p;
  if constexpr (kKeep == 0)
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  else
    asm volatile("createpolicy.fractional.L2::evict_last.L2::evict_first.b64 %0, 0.5;" : "=l"(p));
  return p;
}

// Programmatic dependent launch: this grid lets the next one launch, and
// waits for the previous one's completion (and its writes) before it reads
// anything the previous iteration wrote.
__device__ __forceinline__ void griddep_launch_dependents() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename Real, bool kScaled, int S, int kKeep, int U, bool kPdl>
__device__ __forceinline__ void cgf_staged_tile(int tix, const Tile* tiles, const SceneDev* sds,
                                                double* partials, int pstride, BatchCounters* ctrs,
                                                unsigned char* smem) {
  using P = typename PairOf<Real>::T;
  constexpr uint32_t kSlotBytes = kSlotPairs * sizeof(P);
  const Tile t = tiles[tix];
  const SceneDev& sd = sds[t.scene];
  SceneScalars* sc = sd.sc;
  if constexpr (!kPdl) {
    if (!sc->cg_active) return;
    if constexpr (sizeof(Real) == 4) {
      if (const int ph = sc->cgf_phase) {
        cgf_verify_tile<kScaled>(ph, tix, tiles, sds, partials, pstride, ctrs);
        return;
      }
    }
  }

  // prologue: the warp's slice and its first S slots in flight (the matrix
  // does not change between iterations, so with kPdl this overlaps the
  // previous iteration's tail)
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // 32-bit shared addresses of this warp's stage ring and its mbarriers
  const uint32_t stage0 = smem_addr(smem) + (uint32_t)(warp * S) * kSlotBytes;
  const uint32_t bar0 = smem_addr(smem) + (uint32_t)((blockDim.x >> 5) * S) * kSlotBytes + (uint32_t)(warp * S) * 8u;
  const int row0 = t.begin + 32 * warp;  // first row of the warp's slice
  const int row = row0 + lane;
  const bool live = row < t.end;
  int slen = 0;
  const P* gslice = nullptr;
  if (row0 < t.end) {  // warp-uniform
    const int slice = row0 >> 5;
    const int soff = sd.slice_off[slice];
    slen = (sd.slice_off[slice + 1] - soff) >> 5;
    gslice = static_cast<const P*>(sd.ell) + 5 * (size_t)soff;  // slot k: + 160 k pairs
    if (lane == 0) {
#pragma unroll
      for (int q = 0; q < S; ++q) mbar_init(bar0 + 8u * q, 1u);
      fence_mbar_init();
      const unsigned long long pol_m = l2_matrix_policy<kKeep>();
      for (int k = 0; k < S && k < slen; ++k) {
        mbar_arrive_expect_tx(bar0 + 8u * k, kSlotBytes);
        bulk_g2s(stage0 + k * kSlotBytes, gslice + (size_t)k * kSlotPairs, kSlotBytes, bar0 + 8u * k, pol_m);
      }
    }
    __syncwarp();
  }
  if constexpr (kPdl) {
    griddep_launch_dependents();
    griddep_wait();
    int ph = 0;
    if constexpr (sizeof(Real) == 4) ph = sc->cgf_phase;
    const bool active = sc->cg_active != 0;
    if (!active || ph) {  // block-uniform
      // the prefetched slots are not needed: let them land (bounded), leave
      for (int k = 0; k < S && k < slen; ++k) mbar_wait(bar0 + 8u * k, 0u);
      __syncwarp();
      if constexpr (sizeof(Real) == 4) {
        if (active) cgf_verify_tile<kScaled>(ph, tix, tiles, sds, partials, pstride, ctrs);
      }
      return;
    }
  }
  const int it = sc->cg_iter;
  const Real a = sizeof(Real) == 4 ? Real(sc->alpha_f) : Real(sc->alpha);
  const Real b = sizeof(Real) == 4 ? Real(sc->beta_f) : Real(sc->beta);
  const Real* r_old = static_cast<const Real*>(sd.cgf_r[it & 1]);
  const Real* w_old = static_cast<const Real*>(sd.cgf_w[it & 1]);
  const Real* s_old = static_cast<const Real*>(sd.cgf_s[(it + 1) & 1]);
  Real* r_new = static_cast<Real*>(sd.cgf_r[(it + 1) & 1]);
  Real* w_new = static_cast<Real*>(sd.cgf_w[(it + 1) & 1]);
  Real* s_new = static_cast<Real*>(sd.cgf_s[it & 1]);
  Real* x = static_cast<Real*>(sd.cg_x);
  Real* u = static_cast<Real*>(sd.cg_z);
  Real* p = static_cast<Real*>(sd.cg_p[0]);
  using E = typename Ext<Real>::T;
  E dots[3] = {E(0), E(0), E(0)};  // (r,r), (r,u), (w,u) at it+1

  // own row: p, x, s, r (and u) of iteration it+1, while the first slots
  // fly.  Nothing of it stays in registers across the slot loop (the 40
  // registers of six resident blocks would spill): the dot products reload
  // r and u afterwards (their lines are still in L1).
  if (live) {
    const size_t k4 = 4 * (size_t)row;
    Real dv[3], rv[3], wv[3], sp[3], sv[3], uv[3], pv[3], xv[3], un[3], rn[3];
    if (kScaled) ld3<false>(static_cast<const Real*>(sd.dinv) + k4, dv);
    ld3<false>(r_old + k4, rv);
    ld3<false>(w_old + k4, wv);
    ld3<false>(s_old + k4, sp);
    if (kScaled) {
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        sv[c] = fma(b, sp[c], wv[c]);
        un[c] = fma(-a, sv[c], rv[c]);
        uv[c] = rv[c];  // u_i = r~_i
      }
    } else {
      cgf_next<Real>(sd, row, rv, wv, sp, a, b, sv, rn, un);
      ld3<false>(u + k4, uv);
    }
    ld3<false>(p + k4, pv);
    ld3<false>(x + k4, xv);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      pv[c] = fma(b, pv[c], uv[c]);
      xv[c] = fma(a, pv[c], xv[c]);
    }
    st3(p + k4, pv);
    st3(x + k4, xv);
    st3(s_new + k4, sv);
    if (kScaled) {
      st3(r_new + k4, un);
    } else {
      st3(r_new + k4, rn);
      st3(u + k4, un);
    }
  }

  // w_{i+1} = A u_{i+1}, out of the stage ring: U slots at a time, whose
  // gathers all go out before the first of them is consumed (the slots are
  // still accumulated in order, so every U computes the same bits)
  Real acc0 = 0, acc1 = 0, acc2 = 0;
  int k = 0;
  bool ok = true;
  const uint32_t pb = (uint32_t)sizeof(P) * 32u;
  const uint32_t lane_off = (uint32_t)lane * (uint32_t)sizeof(P);
  auto fill = [&](int j) {  // lane 0: stage of slot j - S gets slot j
    if (lane == 0 && j < slen) {
      const int q = j % S;
      fence_proxy_async_smem();
      mbar_arrive_expect_tx(bar0 + 8u * q, kSlotBytes);
      bulk_g2s(stage0 + (uint32_t)q * kSlotBytes, gslice + (size_t)j * kSlotPairs, kSlotBytes, bar0 + 8u * q,
               l2_matrix_policy<kKeep>());
    }
  };
  for (; ok && k < slen; k += U) {
    const int n = min(U, slen - k);  // warp-uniform
    P w0[U];
    Real uc[U][3];
#pragma unroll
    for (int j = 0; j < U; ++j) {
      if (j < n) {
        const int q = (k + j) % S;
        const bool got = mbar_wait(bar0 + 8u * q, (uint32_t)(((k + j) / S) & 1));
        if (!__all_sync(0xffffffffu, got)) {
          ok = false;
          break;
        }
        // the column first: the gathers go out before the other pairs are read
        w0[j] = lds_pair(stage0 + (uint32_t)q * kSlotBytes + lane_off, Real(0));
        if (live) {
          const unsigned long long pol_k = l2_evict_last();
          const size_t c4 = 4 * (size_t)pair_col(w0[j]);
          Real rc[3], wc[3], spc[3];
          ld3_keep(r_old + c4, rc, pol_k);
          ld3_keep(w_old + c4, wc, pol_k);
          ld3_keep(s_old + c4, spc, pol_k);
          if (kScaled) {
#pragma unroll
            for (int c = 0; c < 3; ++c) uc[j][c] = fma(-a, fma(b, spc[c], wc[c]), rc[c]);
          } else {
            Real sc_[3], rnc[3];
            cgf_next<Real>(sd, pair_col(w0[j]), rc, wc, spc, a, b, sc_, rnc, uc[j]);
          }
        }
      }
    }
    if (!ok) break;
#pragma unroll
    for (int j = 0; j < U; ++j) {
      if (j < n) {
        const uint32_t sp = stage0 + (uint32_t)((k + j) % S) * kSlotBytes + lane_off;
        const P w1 = lds_pair(sp + pb, Real(0)), w2 = lds_pair(sp + 2 * pb, Real(0)),
                w3 = lds_pair(sp + 3 * pb, Real(0)), w4 = lds_pair(sp + 4 * pb, Real(0));
        __syncwarp();
        fill(k + j + S);
        if (live) ell_block_fma(w0[j], w1, w2, w3, w4, uc[j], acc0, acc1, acc2);
      }
    }
  }
  if (!ok) {
    // a wait ran out: flag it, then let the copies still in flight land
    // (bounded) before the block may exit
    if (lane == 0) atomicExch(&ctrs->error, 1);
    for (int j = k; j < slen && j < k + S; ++j) mbar_wait(bar0 + 8u * (j % S), (uint32_t)((j / S) & 1));
    __syncwarp();
  }
  if (live) {
    const size_t k4 = 4 * (size_t)row;
    const Real wn[3] = {acc0, acc1, acc2};
    Real un[3], rn[3];
    if (kScaled) {
      Real dv[3];
      ld3<false>(static_cast<const Real*>(sd.dinv) + k4, dv);
      ld3<false>(r_new + k4, un);
#pragma unroll
      for (int c = 0; c < 3; ++c) rn[c] = un[c] / dv[c];
      const Real ws[3] = {dv[0] * acc0, dv[1] * acc1, dv[2] * acc2};
      st3(w_new + k4, ws);
    } else {
      ld3<false>(r_new + k4, rn);
      ld3<false>(u + k4, un);
      st3(w_new + k4, wn);
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      dots[0] = dots[0] + exact_prod(rn[c], rn[c]);
      dots[1] = dots[1] + exact_prod(rn[c], un[c]);
      dots[2] = dots[2] + exact_prod(wn[c], un[c]);
    }
  }
  cgf_finish<Real, false>(sd, ctrs, dots, partials, pstride, tix, it);
}

// Resident blocks per SM: six (40 registers) in FP32 where the stages fit
// six blocks' shared memory, five with four stages (41 KB a block), four
// (64 registers) when two slots' gathers are in flight together, two (82 KB
// of stages) with eight stages and four slots in flight: the shape for
// systems too small to fill the GPU, where each row's chain of slots, not
// the bandwidth, sets the iteration's time.
template <typename Real, int S, int U>
constexpr int cgf_staged_min_blocks() {
  return sizeof(Real) == 4 ? (U >= 4 ? 2 : (U > 1 ? 4 : (S >= 4 ? 5 : 6))) : 4;
}
template <typename Real, bool kScaled, int S, int kKeep, int U, bool kPdl>
__global__ void __launch_bounds__(kCgThreads, cgf_staged_min_blocks<Real, S, U>()) k_cgf_iter_staged(
    const Tile* tiles, const SceneDev* sds, double* partials, int pstride, BatchCounters* ctrs) {
  extern __shared__ __align__(128) unsigned char cgf_smem[];
  cgf_staged_tile<Real, kScaled, S, kKeep, U, kPdl>(blockIdx.x, tiles, sds, partials, pstride, ctrs, cgf_smem);
}

// Nanoseconds of the GPU's global timer.
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Barrier over all blocks of a cooperative launch (every block is resident).
// Arrival counter plus a generation word; the last arrival resets the
// counter and advances the generation.  Every wait is bounded: after
// kBarrierTimeoutNs (or kBarrierMaxPolls polls) the block raises
// ctrs->error and every block leaves at its next barrier.  Returns false
// when the launch must end.
constexpr unsigned long long kBarrierTimeoutNs = 2000000000ull;
constexpr unsigned int kBarrierMaxPolls = 1u << 26;

__device__ __forceinline__ bool grid_barrier(BatchCounters* ctrs) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned int* gen = &ctrs->bar_gen;
    volatile int* err = &ctrs->error;
    int ok = (*err == 0);
    if (ok) {
      const unsigned int g = *gen;
      __threadfence();
      if (atomicAdd(&ctrs->bar_count, 1u) + 1u == gridDim.x) {
        ctrs->bar_count = 0u;
        __threadfence();
        atomicAdd(&ctrs->bar_gen, 1u);
      } else {
        const unsigned long long t0 = global_ns();
        unsigned int polls = 0;
        while (*gen == g) {
          if (*err) {
            ok = 0;
            break;
          }
          if (++polls >= kBarrierMaxPolls || ((polls & 255u) == 0 && global_ns() - t0 > kBarrierTimeoutNs)) {
            atomicExch(&ctrs->error, 1);
            ok = 0;
            break;
          }
          __nanosleep(32);
        }
      }
      __threadfence();
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// The whole PCG solve of every active scene in ONE cooperative launch: the
// blocks walk the tile table in a grid-stride loop for the SpMV phase, meet
// at a grid barrier, do the update phase, meet again.  The arithmetic and
// its order are those of the two-launch form; the results are bitwise the
// same.  Six resident blocks per SM in the mixed path (912 on 152 SMs)
// cover a 1M-tet scene's 873 PCG tiles in one round.
template <typename Real>
__global__ void __launch_bounds__(kCgThreads, sizeof(Real) == 4 ? 6 : 4) k_cg_solve(
    const Tile* tiles, int ntiles, const SceneDev* sds, double* partials, int pstride,
    BatchCounters* ctrs, int max_iters) {
  for (int it = 0; it < max_iters; ++it) {
    if (*(volatile int*)&ctrs->cg_active == 0) return;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x)
      cg_spmv_tile<Real, true>(t, tiles, sds, partials, pstride);
    if (!grid_barrier(ctrs)) return;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x)
      cg_update_tile<Real, true>(t, tiles, sds, partials, pstride, ctrs);
    if (!grid_barrier(ctrs)) return;
    if (sizeof(Real) == 4 && (it + 1) % kCgReplace == 0) {
      for (int t = blockIdx.x; t < ntiles; t += gridDim.x)
        cg_replace_tile<true>(t, tiles, sds, partials, pstride, ctrs);
      if (!grid_barrier(ctrs)) return;
    }
  }
}

// steps: the call's timesteps per scene (0: the plain one-step form);
// ticked: the kernels gate on the scenes' phases.
__global__ void k_scalars_begin(const SceneDev* sds, int n, BatchCounters* ctrs, int steps, int ticked) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    SceneScalars* sc = sds[i].sc;
    reset_step_scalars(sc);
    sc->steps_target = steps;
    sc->steps_done = 0;
    sc->turn = 0;
    sc->acc_newton = 0;
    sc->acc_cg = 0;
    sc->acc_ls = 0;
    sc->acc_status = 0;
    sc->ticked = ticked;
  }
  if (threadIdx.x == 0) {
    ctrs->newton_active = n;
    ctrs->cg_active = 0;
    ctrs->ls_active = 0;
    ctrs->error = 0;
    ctrs->bar_count = 0u;
  }
}

}  // namespace

#define MFEM_LAUNCH_ROWS(kern, threads)                                                      \
  do {                                                                                       \
    if (L.ntiles == 0) return;                                                               \
    if (L.fp64)                                                                              \
      kern<double><<<L.ntiles, threads, 0, L.stream>>>(L.tiles, L.sds, L.partials, L.pstride,   \
                                                       L.counters);                          \
    else                                                                                     \
      kern<float><<<L.ntiles, threads, 0, L.stream>>>(L.tiles, L.sds, L.partials, L.pstride,    \
                                                      L.counters);                           \
  } while (0)

void launch_assemble(const Launch& L) { MFEM_LAUNCH_ROWS(k_assemble, 256); }
void launch_cg_init(const Launch& L) { MFEM_LAUNCH_ROWS(k_cg_init, kCgThreads); }
void launch_cg_spmv(const Launch& L) { MFEM_LAUNCH_ROWS(k_cg_spmv, kCgThreads); }
void launch_cg_update(const Launch& L) { MFEM_LAUNCH_ROWS(k_cg_update, kCgThreads); }
void launch_cg_replace(const Launch& L) {
  if (L.ntiles == 0 || L.fp64) return;
  k_cg_replace<<<L.ntiles, kCgThreads, 0, L.stream>>>(L.tiles, L.sds, L.partials, L.pstride, L.counters);
}
#define MFEM_LAUNCH_CGF(kern)                                                                \
  do {                                                                                       \
    if (L.ntiles == 0) return;                                                               \
    const auto args = [&](auto k) {                                                          \
      k<<<L.ntiles, kCgThreads, 0, L.stream>>>(L.tiles, L.sds, L.partials, L.pstride, L.counters); \
    };                                                                                       \
    if (L.fp64) {                                                                            \
      if (L.jacobi) args(kern<double, true>);                                                \
      else args(kern<double, false>);                                                        \
    } else {                                                                                 \
      if (L.jacobi) args(kern<float, true>);                                                 \
      else args(kern<float, false>);                                                         \
    }                                                                                        \
  } while (0)

__global__ void k_cg_continue(BatchCounters* ctrs, cudaGraphConditionalHandle h, int max_bodies) {
  const int n = ++ctrs->cg_bodies;
  const bool more = *(volatile int*)&ctrs->cg_active > 0 && *(volatile int*)&ctrs->error == 0 && n < max_bodies;
  cudaGraphSetConditional(h, more ? 1u : 0u);
}

void launch_cg_continue(const Launch& L, cudaGraphConditionalHandle h, int max_bodies) {
  k_cg_continue<<<1, 1, 0, L.stream>>>(L.counters, h, max_bodies);
}

__global__ void k_cg_enter(BatchCounters* ctrs, cudaGraphConditionalHandle h) {
  const bool go = *(volatile int*)&ctrs->cg_active > 0 && *(volatile int*)&ctrs->error == 0;
  cudaGraphSetConditional(h, go ? 1u : 0u);
}

void launch_cg_enter(const Launch& L, cudaGraphConditionalHandle h) {
  k_cg_enter<<<1, 1, 0, L.stream>>>(L.counters, h);
}

void launch_cgf_init(const Launch& L) { MFEM_LAUNCH_CGF(k_cgf_init); }
void launch_cgf_scale(const Launch& L) {
  if (L.ntiles == 0 || L.fp64) return;
  k_cgf_scale<<<L.ntiles, kCgThreads, 0, L.stream>>>(L.tiles, L.sds, L.partials, L.pstride, L.counters);
}

namespace {
template <typename Real, bool kScaled, int S, int kKeep, int U, bool kPdl>
void launch_staged(const Launch& L) {
  const size_t smem = cgf_staged_smem_bytes<Real, S>(kCgThreads / 32);
  if (smem > 48 * 1024) {  // above the default dynamic limit: opt in once
    static const cudaError_t opt = cudaFuncSetAttribute(k_cgf_iter_staged<Real, kScaled, S, kKeep, U, kPdl>,
                                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    (void)opt;
  }
  if constexpr (kPdl) {
    // the launch may start while the previous kernel of the stream runs; the
    // kernel waits for it (griddepcontrol.wait) before reading its results
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(L.ntiles);
    cfg.blockDim = dim3(kCgThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = L.stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k_cgf_iter_staged<Real, kScaled, S, kKeep, U, true>, L.tiles, L.sds, L.partials,
                       L.pstride, L.counters);
  } else {
    k_cgf_iter_staged<Real, kScaled, S, kKeep, U, false>
        <<<L.ntiles, kCgThreads, smem, L.stream>>>(L.tiles, L.sds, L.partials, L.pstride, L.counters);
  }
}
template <typename Real, bool kScaled, int kKeep, bool kPdl>
void launch_staged_s(const Launch& L, int stages, int unroll) {
  if constexpr (sizeof(Real) == 4) {
    if (unroll >= 4) launch_staged<Real, kScaled, 8, kKeep, 4, kPdl>(L);
    else if (unroll > 1) launch_staged<Real, kScaled, 4, kKeep, 2, kPdl>(L);
    else if (stages == 2) launch_staged<Real, kScaled, 2, kKeep, 1, kPdl>(L);
    else if (stages == 3) launch_staged<Real, kScaled, 3, kKeep, 1, kPdl>(L);
    else launch_staged<Real, kScaled, 4, kKeep, 1, kPdl>(L);
  } else {
    launch_staged<Real, kScaled, 2, kKeep, 1, kPdl>(L);  // 2560-byte slots: two stages
  }
}
template <typename Real, bool kScaled>
void launch_staged_k(const Launch& L, const CgfShape& sh) {
  if (sh.pdl) {
    if (sh.keep) launch_staged_s<Real, kScaled, 1, true>(L, sh.stages, sh.unroll);
    else launch_staged_s<Real, kScaled, 0, true>(L, sh.stages, sh.unroll);
  } else {
    if (sh.keep) launch_staged_s<Real, kScaled, 1, false>(L, sh.stages, sh.unroll);
    else launch_staged_s<Real, kScaled, 0, false>(L, sh.stages, sh.unroll);
  }
}
}  // namespace

void launch_cgf_iter(const Launch& L, const CgfShape& sh) {
  if (sh.stages <= 0) {
    MFEM_LAUNCH_CGF(k_cgf_iter);
    return;
  }
  if (L.ntiles == 0) return;
  if (L.fp64) {
    if (L.jacobi) launch_staged_k<double, true>(L, sh);
    else launch_staged_k<double, false>(L, sh);
  } else {
    if (L.jacobi) launch_staged_k<float, true>(L, sh);
    else launch_staged_k<float, false>(L, sh);
  }
}

// Failure-detection check of the bounded grid barrier: a cooperative launch
// of two blocks in which block 1 leaves without arriving (a lost peer), so
// block 0's wait must run out, raise ctrs->error and return.
__global__ void k_barrier_selftest(BatchCounters* ctrs) {
  if (blockIdx.x == 1) return;
  grid_barrier(ctrs);
}

cudaError_t launch_barrier_selftest(BatchCounters* ctrs, cudaStream_t st) {
  void* args[] = {&ctrs};
  return cudaLaunchCooperativeKernel((const void*)k_barrier_selftest, dim3(2), dim3(32), args, 0, st);
}

int cg_solve_blocks_per_sm(int fp64) {
  int nb = 0;
  cudaError_t e = fp64 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_cg_solve<double>, kCgThreads, 0)
                       : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_cg_solve<float>, kCgThreads, 0);
  return e == cudaSuccess ? nb : 0;
}

cudaError_t launch_cg_solve(const Launch& L, int grid, int max_iters) {
  if (L.ntiles == 0 || grid <= 0) return cudaSuccess;
  const Tile* tiles = L.tiles;
  int ntiles = L.ntiles;
  const SceneDev* sds = L.sds;
  double* partials = L.partials;
  int pstride = L.pstride;
  BatchCounters* ctrs = L.counters;
  void* args[] = {&tiles, &ntiles, &sds, &partials, &pstride, &ctrs, &max_iters};
  const void* fn = L.fp64 ? (const void*)k_cg_solve<double> : (const void*)k_cg_solve<float>;
  return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(kCgThreads), args, 0, L.stream);
}

void launch_scalars_begin(const Launch& L, int nscenes) {
  k_scalars_begin<<<1, 128, 0, L.stream>>>(L.sds, nscenes, L.counters, 0, 0);
}
void launch_scalars_begin_n(const Launch& L, int nscenes, int steps, int ticked) {
  k_scalars_begin<<<1, 128, 0, L.stream>>>(L.sds, nscenes, L.counters, steps, ticked);
}

__global__ void k_stamp(unsigned long long* ns) {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  *ns = t;
}
void launch_stamp(unsigned long long* ns, cudaStream_t st) { k_stamp<<<1, 1, 0, st>>>(ns); }

}  // namespace mfem_gpu
