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
//                Vectors are Real; every inner product is accumulated in FP64.
#include <cfloat>

#include "device_math.cuh"
#include "kernels.cuh"
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

constexpr int kAsmWindow = 64;  // block slots per warp accumulated in shared memory per pass

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
  if (!sc->newton_active) return;
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
    for (int k = ib + lane; k < ie; k += 32) {
      const int2 ic = sd.inc[k];
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
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        rhs[3 * row + c] = Real(Ext<Real>::to_real(acc[c]));
        r2 = r2 + acc[c] * acc[c];
      }
      rn2 = rn2 + r2;
    }
    // ---- block values: the warp accumulates the row's blocks in shared
    // memory, one incidence (element, local vertex i) at a time; lane l < 36
    // adds entry l % 9 of local block (i, l / 9) to that block's column slot.
    // Slots of one incidence are distinct, so the adds never collide, and
    // every entry sums its contributions in element order.
    const int slice = row >> 5, rs = row & 31;
    const int soff = sd.slice_off[slice], slen = (sd.slice_off[slice + 1] - soff) >> 5;
    Real* val = static_cast<Real*>(sd.ell_val) + (size_t)soff * 9 + rs;
    const Real* bm = static_cast<const Real*>(sd.b_mass) + rb;
    Real* acc_w = acc_s[warp];
    for (int w0 = 0; w0 < nb; w0 += kAsmWindow) {
      const int wn = min(kAsmWindow, nb - w0);
      for (int o = lane; o < 9 * wn; o += 32) acc_w[o] = Real(0);
      __syncwarp();
      for (int k = ib; k < ie; ++k) {
        const int2 ic = sd.inc[k];
        const int i = ic.y & 3;
        const Real* rp = reinterpret_cast<const Real*>(sd.rec + (size_t)ic.x * rec_bytes(RB));
#pragma unroll
        for (int pass = 0; pass < 2; ++pass) {
          const int l = lane + 32 * pass;
          if (l < 36) {
            const int j = l / 9, ent = l - 9 * j;
            const int slot = (ic.y >> (2 + 7 * j)) & 127;
            const int sl = slot - w0;
            if (slot != 127 && sl >= 0 && sl < wn) acc_w[9 * sl + ent] += rp[offtab[i][j][ent]];
          }
        }
        __syncwarp();
      }
      for (int o = lane; o < 9 * wn; o += 32) {
        const int q = o / 9, ent = o - 9 * q;
        val[(size_t)288 * (w0 + q) + 32 * ent] =
            acc_w[o] + ((ent == 0 || ent == 4 || ent == 8) ? bm[w0 + q] : Real(0));
      }
      __syncwarp();
    }
    // padding blocks of the slice beyond this row's length are zero
    for (int o = lane; o < 9 * (slen - nb); o += 32) {
      const int q = nb + o / 9, ent = o % 9;
      val[(size_t)288 * q + 32 * ent] = Real(0);
    }
    // ---- preconditioner from the diagonal block
    int qd = -1;
    for (int q0 = 0; q0 < nb; q0 += 32) {
      const bool hit = (q0 + lane < nb) && sd.b_col[rb + q0 + lane] == row;
      const unsigned bal = __ballot_sync(0xffffffffu, hit);
      if (bal && qd < 0) qd = q0 + __ffs(bal) - 1;
    }
    if (lane == 0) {
      Real* dinv = static_cast<Real*>(sd.dinv);
      Real D[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) D[k] = (qd >= 0) ? val[(size_t)288 * qd + 32 * k] : Real(0);
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
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const Real d = D[4 * c];
          dinv[3 * row + c] = d != Real(0) ? Real(1) / d : Real(1);
        }
      }
    }
  }
  }
  {
    typename Ext<Real>::T sums[1] = {rn2};
    tile_partials<typename Ext<Real>::T, 1, 0>(sums, nullptr, partials, pstride, 0, tix, 0);
  }
  if (last_tile(sd, TB_ROW, tix)) {
    const double s = scene_sum(partials, pstride, 0, sd.tile_first[TB_ROW], sd.tile_count[TB_ROW]);
    if (threadIdx.x == 0) {
      const double rn = sqrt(s);
      if (sc->newton_iter == 0) sc->rhs_norm0 = rn;
      sc->rhs_norm = rn;
      // |rhs_k| <= tol * max(|rhs_0|, |h^2 P M f|)
      if (sd.res_tol > 0 && ((sc->newton_iter > 0 && rn <= sd.res_tol * sc->rhs_norm0) ||
                             rn <= sd.res_tol * sd.load_norm)) {
        sc->converged_by_residual = 1;
        sc->newton_active = 0;
        atomicSub(&ctrs->newton_active, 1);
      }
      if (!(s == s) || isinf(s)) {
        sc->status = 4;  // MFEM_ERR_NONFINITE
        if (sc->newton_active) {
          sc->newton_active = 0;
          atomicSub(&ctrs->newton_active, 1);
        }
      }
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
#pragma unroll
    for (int c = 0; c < 3; ++c) z[c] = dinv[3 * (size_t)row + c] * r[c];
  }
}

// r = b, z = D^{-1} b, x = 0, rz; one thread per row.
template <typename Real>
__global__ void __launch_bounds__(kCgThreads) k_cg_init(const Tile* tiles, const SceneDev* sds,
                                                        double* partials, int pstride,
                                                        BatchCounters* ctrs) {
  const int tix = blockIdx.x;
  const Tile t = tiles[tix];
  const SceneDev& sd = sds[t.scene];
  SceneScalars* sc = sd.sc;
  if (!sc->newton_active) return;
  using E = typename Ext<Real>::T;
  E dots[2] = {E(0), E(0)};  // r.r, r.z
  const int row = t.begin + threadIdx.x;
  if (row < t.end) {
    const Real* b = static_cast<const Real*>(sd.rhs) + 3 * (size_t)row;
    Real r[3] = {b[0], b[1], b[2]}, z[3];
    apply_prec<Real>(sd, row, r, z);
    Real* pr = static_cast<Real*>(sd.cg_r) + 3 * (size_t)row;
    Real* pz = static_cast<Real*>(sd.cg_z) + 3 * (size_t)row;
    Real* px = static_cast<Real*>(sd.cg_x) + 3 * (size_t)row;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      pr[c] = r[c];
      pz[c] = z[c];
      px[c] = Real(0);
      dots[0] = dots[0] + exact_prod(r[c], r[c]);
      dots[1] = dots[1] + exact_prod(r[c], z[c]);
    }
  }
  tile_partials<E, 2, 0>(dots, nullptr, partials, pstride, 0, tix, 0);
  if (last_tile(sd, TB_CG, tix)) {
    const int t0 = sd.tile_first[TB_CG], tc = sd.tile_count[TB_CG];
    const double rrs = scene_sum(partials, pstride, 0, t0, tc);
    const double rzs = scene_sum(partials, pstride, 1, t0, tc);
    if (threadIdx.x == 0) {
      sc->cg_rhs_norm2 = rrs;
      sc->cg_iter = 0;
      sc->beta = 0.0;
      sc->rz = rzs;
      sc->cg_err = 0.0;
      if (rrs == 0.0) {
        sc->cg_active = 0;
      } else {
        const double thr = fmax(sd.cg_tol * sd.cg_tol * rrs, DBL_MIN);
        sc->cg_threshold = thr;
        if (rrs < thr || sd.max_cg <= 0) {
          sc->cg_active = 0;
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
// One thread per row over the sliced-ELL layout: every column and value
// load of a warp is one coalesced 128-byte access, and the block loop is
// unrolled so that several blocks' loads are in flight per thread.
template <typename Real>
__global__ void __launch_bounds__(kCgThreads) k_cg_spmv(const Tile* tiles, const SceneDev* sds,
                                                        double* partials, int pstride,
                                                        BatchCounters* ctrs) {
  const int tix = blockIdx.x;
  const Tile t = tiles[tix];
  const SceneDev& sd = sds[t.scene];
  SceneScalars* sc = sd.sc;
  if (!sc->cg_active) return;
  const int it = sc->cg_iter;
  const Real beta = Real(sc->beta);
  const bool first = (it == 0);
  const Real* z = static_cast<const Real*>(sd.cg_z);
  const Real* pin = static_cast<const Real*>(sd.cg_p[(it + 1) & 1]);
  Real* pout = static_cast<Real*>(sd.cg_p[it & 1]);
  Real* Ap = static_cast<Real*>(sd.cg_Ap);
  using E = typename Ext<Real>::T;
  E pAp[1] = {E(0)};
  const int row = t.begin + threadIdx.x;
  if (row < t.end) {
    const int slice = row >> 5, rs = row & 31;
    const int soff = sd.slice_off[slice], slen = (sd.slice_off[slice + 1] - soff) >> 5;
    const int* colp = sd.ell_col + soff + rs;
    const Real* vp = static_cast<const Real*>(sd.ell_val) + (size_t)soff * 9 + rs;
    Real acc0 = 0, acc1 = 0, acc2 = 0;
#pragma unroll 4
    for (int k = 0; k < slen; ++k) {
      const int col = colp[32 * k];
      const Real* v = vp + (size_t)288 * k;
      Real p0, p1, p2;
      if (first) {
        p0 = z[3 * col];
        p1 = z[3 * col + 1];
        p2 = z[3 * col + 2];
      } else {
        p0 = z[3 * col] + beta * pin[3 * col];
        p1 = z[3 * col + 1] + beta * pin[3 * col + 1];
        p2 = z[3 * col + 2] + beta * pin[3 * col + 2];
      }
      acc0 += v[0] * p0 + v[32] * p1 + v[64] * p2;
      acc1 += v[96] * p0 + v[128] * p1 + v[160] * p2;
      acc2 += v[192] * p0 + v[224] * p1 + v[256] * p2;
    }
    const Real acc[3] = {acc0, acc1, acc2};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const Real p = first ? z[3 * row + c] : z[3 * row + c] + beta * pin[3 * row + c];
      pout[3 * row + c] = p;
      Ap[3 * row + c] = acc[c];
      pAp[0] = pAp[0] + exact_prod(p, acc[c]);
    }
  }
  tile_partials<E, 1, 0>(pAp, nullptr, partials, pstride, 0, tix, 0);
  if (last_tile(sd, TB_CG, tix)) {
    const double s = scene_sum(partials, pstride, 0, sd.tile_first[TB_CG], sd.tile_count[TB_CG]);
    if (threadIdx.x == 0) sc->alpha = sc->rz / s;
  }
}

// x += alpha p, r -= alpha Ap, z = D^{-1} r, then beta and the stopping test.
template <typename Real>
__global__ void __launch_bounds__(kCgThreads) k_cg_update(const Tile* tiles, const SceneDev* sds,
                                                          double* partials, int pstride,
                                                          BatchCounters* ctrs) {
  const int tix = blockIdx.x;
  const Tile t = tiles[tix];
  const SceneDev& sd = sds[t.scene];
  SceneScalars* sc = sd.sc;
  if (!sc->cg_active) return;
  const int it = sc->cg_iter;
  const Real alpha = Real(sc->alpha);
  using E = typename Ext<Real>::T;
  E dots[2] = {E(0), E(0)};  // r.r, r.z
  const int row = t.begin + threadIdx.x;
  if (row < t.end) {
    const size_t k = 3 * (size_t)row;
    const Real* p = static_cast<const Real*>(sd.cg_p[it & 1]) + k;
    const Real* Ap = static_cast<const Real*>(sd.cg_Ap) + k;
    Real* x = static_cast<Real*>(sd.cg_x) + k;
    Real* r = static_cast<Real*>(sd.cg_r) + k;
    Real rv[3], z[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      x[c] += alpha * p[c];
      rv[c] = r[c] - alpha * Ap[c];
      r[c] = rv[c];
      dots[0] = dots[0] + exact_prod(rv[c], rv[c]);
    }
    apply_prec<Real>(sd, row, rv, z);
    Real* pz = static_cast<Real*>(sd.cg_z) + k;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      pz[c] = z[c];
      dots[1] = dots[1] + exact_prod(rv[c], z[c]);
    }
  }
  tile_partials<E, 2, 0>(dots, nullptr, partials, pstride, 0, tix, 0);
  if (last_tile(sd, TB_CG, tix)) {
    const int t0 = sd.tile_first[TB_CG], tc = sd.tile_count[TB_CG];
    const double rrs = scene_sum(partials, pstride, 0, t0, tc);
    const double rzs = scene_sum(partials, pstride, 1, t0, tc);
    if (threadIdx.x == 0) {
      sc->cg_err = sqrt(rrs / sc->cg_rhs_norm2);
      bool stop = false;
      if (rrs < sc->cg_threshold) {
        stop = true;
      } else {
        sc->beta = rzs / sc->rz;
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
        sc->cg_total += sc->cg_iter;
        sc->cg_active = 0;
        atomicSub(&ctrs->cg_active, 1);
      }
    }
  }
}

__global__ void k_scalars_begin(const SceneDev* sds, int n, BatchCounters* ctrs) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    SceneScalars* sc = sds[i].sc;
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
    sc->procrustes_fail = 0;
  }
  if (threadIdx.x == 0) {
    ctrs->newton_active = n;
    ctrs->cg_active = 0;
    ctrs->ls_active = 0;
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

void launch_scalars_begin(const Launch& L, int nscenes) {
  k_scalars_begin<<<1, 128, 0, L.stream>>>(L.sds, nscenes, L.counters);
}

}  // namespace mfem_gpu
