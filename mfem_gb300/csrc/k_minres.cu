// "minres-indefinite-block" (linear_solver_factory.cpp:116-133): MINRES on
// the full (x, s, lambda) Newton system of SystemMatrixIndefinite
// (linear_system.h:61-99), the product of BlockMatrix (block_matrix.h:63-126)
// applied matrix-free from each element's ds/dx and Hessian, and a
// block-diagonal preconditioner of per-element 6x6 blocks.
//
// Vectors are FP64 in both precision paths (the element data B and H are in
// the path's Real).  One KKT vector of a scene is
//   [x: 4 nf (row f: x, y, z, 0)][s: 6 ntp (i ntp + e)][lambda: 6 ntp]
// with rows in the device (sliced-ELL) numbering.
//
// Iteration (Eigen 3.4 unsupported MINRES, restated: Paige & Saunders'
// preconditioned MINRES with the stopping test |r0|^2 prod s_k^2 < tol^2 |b|^2)
// in three launches, each a pass over the scene's elements and/or vertices:
//   A1 (elements)  the pending update p_{k-1}, x of the previous iteration;
//                  v <- vn / beta, w <- wn / beta; the s and lambda rows of
//                  t = K w - beta v_old; the per-element x-row shares y
//   A2 (vertices)  the same for the x rows (mass product + gather of y);
//                  alpha = t . w
//   B  (both)      vn = t - alpha v, wn = P vn, beta' = sqrt(vn . wn); the
//                  Givens rotation and the convergence test in the finalizer
// The p / x update of iteration k needs r1 from B's reduction, so it is
// applied by the next A1/A2 (or by a final A1/A2 after the loop).
#include <cfloat>

#include "device_math.cuh"
#include "kernels.cuh"
#include "reduce.cuh"

namespace mfem_gpu {

namespace {

enum { MR_V = 0, MR_VN = 1, MR_WN = 2, MR_W = 3, MR_P0 = 4, MR_X = 7 };

__device__ __forceinline__ int sym6(int i, int j) {  // upper-triangle index, i <= j
  return i * 6 - (i * (i - 1)) / 2 + (j - i);
}
__device__ __forceinline__ double symv(int i) { return i < 3 ? 1.0 : 2.0; }

// Inverse of a symmetric positive definite 6x6 (column-major) by Cholesky;
// false if a pivot is not positive.
__device__ bool spd_inverse6(const double* A, double* Ai) {
  double L[36];
#pragma unroll
  for (int i = 0; i < 36; ++i) L[i] = A[i];
  bool ok = true;
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    double d = L[j + 6 * j];
#pragma unroll
    for (int k = 0; k < j; ++k) d -= L[j + 6 * k] * L[j + 6 * k];
    ok = ok && d > 0.0;
    const double ljj = sqrt(d > 0.0 ? d : DBL_MIN);
    L[j + 6 * j] = ljj;
#pragma unroll
    for (int i = j + 1; i < 6; ++i) {
      double v = L[i + 6 * j];
#pragma unroll
      for (int k = 0; k < j; ++k) v -= L[i + 6 * k] * L[j + 6 * k];
      L[i + 6 * j] = v / ljj;
    }
  }
  // columns of A^-1: L y = e_c, L^T z = y
#pragma unroll
  for (int c = 0; c < 6; ++c) {
    double y[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      double v = (i == c) ? 1.0 : 0.0;
#pragma unroll
      for (int k = 0; k < i; ++k) v -= L[i + 6 * k] * y[k];
      y[i] = v / L[i + 6 * i];
    }
#pragma unroll
    for (int i = 5; i >= 0; --i) {
      double v = y[i];
#pragma unroll
      for (int k = i + 1; k < 6; ++k) v -= L[k + 6 * i] * Ai[k + 6 * c];
      Ai[i + 6 * c] = v / L[i + 6 * i];
    }
  }
  return ok;
}

__device__ __forceinline__ double* mr_vec(const SceneDev& sd, int k) { return sd.mr_vec + (size_t)k * sd.mr_len; }
// slot of p_{k} for iteration k (three rotating vectors)
__device__ __forceinline__ double* mr_p(const SceneDev& sd, int k) { return mr_vec(sd, MR_P0 + (k % 3)); }

template <typename Real>
__device__ __forceinline__ void load_sym21(const void* base, int ntp, int e, double* M) {
  const Real* p = static_cast<const Real*>(base);
#pragma unroll
  for (int i = 0; i < 6; ++i)
#pragma unroll
    for (int j = i; j < 6; ++j) {
      const double v = double(p[(size_t)sym6(i, j) * ntp + e]);
      M[i + 6 * j] = v;
      M[j + 6 * i] = v;
    }
}
__device__ __forceinline__ void store_sym21(double* p, int ntp, int e, const double* M) {
#pragma unroll
  for (int i = 0; i < 6; ++i)
#pragma unroll
    for (int j = i; j < 6; ++j) p[(size_t)sym6(i, j) * ntp + e] = M[i + 6 * j];
}

// The pending p / x update of one entry: p_k = (w - r2 p_{k-1} - r3 p_{k-2}) / r1,
// x += beta_one c eta p_k (all scalars of iteration k, slot = k mod 3).
__device__ __forceinline__ void mr_pending_entry(const SceneDev& sd, const SceneScalars* sc, size_t j) {
  const int k = sc->mr_slot;
  double* p0 = mr_p(sd, k);
  const double* p1 = mr_p(sd, k + 2);
  const double* p2 = mr_p(sd, k + 1);
  const double w = mr_vec(sd, MR_W)[j];
  const double p = (w - sc->mr_r2 * p1[j] - sc->mr_r3 * p2[j]) / sc->mr_r1;
  p0[j] = p;
  mr_vec(sd, MR_X)[j] += sc->mr_coef * p;
}

// ------------------------------------------------------------------ init ---
// rhs = [-PM(x - x_tilde - h^2 f); -vol g; vol Sym (S - s)]
// (SystemMatrixIndefinite::pre_solve, linear_system.h:67-86), vn = rhs,
// wn = P rhs, every other vector 0; the per-element preconditioner blocks
// (vol H)^-1 and S_ee^-1 with
//   S_ee = Sym (vol H^-1 + sum_{a free} vol^2 / m_a B_a B_a^T) Sym,
// the element's diagonal block of Gx^T Mlump^-1 Gx + Gs Hs^-1 Gs.
template <typename Real>
__global__ void __launch_bounds__(kElemTile) k_mr_init(const Tile* tiles, const SceneDev* sds,
                                                       double* partials, int pstride,
                                                       BatchCounters* ctrs) {
  using E = typename Ext<Real>::T;
  const int tix = blockIdx.x;
  const Tile t = tiles[tix];
  const SceneDev& sd = sds[t.scene];
  SceneScalars* sc = sd.sc;
  if (!sc->newton_active) return;
  const int idx = t.begin + threadIdx.x;
  const int ntp = sd.ntp;
  const size_t XS = 4 * (size_t)sd.nf, XL = XS + 6 * (size_t)ntp;
  double sums[2] = {0.0, 0.0};
  if (t.kind == 0) {
    if (idx < t.end) {
      const int e = idx;
      const double vol = double(static_cast<const Real*>(sd.vol)[e]);
      double H[36], Hi[36], S[36];
      load_sym21<Real>(sd.mr_H, ntp, e, H);
      spd_inverse6(H, Hi);
      double Hs_inv[36];
#pragma unroll
      for (int i = 0; i < 36; ++i) Hs_inv[i] = Hi[i] / vol;
      store_sym21(sd.mr_hinv, ntp, e, Hs_inv);
      const Real* Bp = static_cast<const Real*>(sd.mr_B);
      double G[36];
#pragma unroll
      for (int i = 0; i < 36; ++i) G[i] = vol * Hi[i];
      const int4 tv = sd.tets[e];
      const int v4[4] = {tv.x, tv.y, tv.z, tv.w};
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        const int f = sd.free_map[v4[a]];
        if (f < 0) continue;
        const double w = vol * vol * sd.mr_mlinv[f];
        double Ba[18];
#pragma unroll
        for (int i = 0; i < 6; ++i)
#pragma unroll
          for (int l = 0; l < 3; ++l) Ba[3 * i + l] = double(Bp[(size_t)(12 * i + 3 * a + l) * ntp + e]);
#pragma unroll
        for (int i = 0; i < 6; ++i)
#pragma unroll
          for (int j = 0; j < 6; ++j)
            G[i + 6 * j] += w * (Ba[3 * i] * Ba[3 * j] + Ba[3 * i + 1] * Ba[3 * j + 1] + Ba[3 * i + 2] * Ba[3 * j + 2]);
      }
#pragma unroll
      for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int j = 0; j < 6; ++j) S[i + 6 * j] = symv(i) * G[i + 6 * j] * symv(j);
      double Si[36];
      spd_inverse6(S, Si);
      store_sym21(sd.mr_sinv, ntp, e, Si);
      // rhs of the element rows
      double sv[6], g[6], rs[6], rl[6];
#pragma unroll
      for (int i = 0; i < 6; ++i) sv[i] = to_double_any(Ext<Real>::ld(sd.s, (size_t)i * ntp + e));
      const double mu = double(static_cast<const Real*>(sd.mu)[e]);
      const double lam = double(static_cast<const Real*>(sd.lam)[e]);
      const int mat = sd.material_uniform >= 0 ? sd.material_uniform : int(sd.mat[e]);
      material_grad<double>(mat, mu, lam, sv, g);
      const Real* dS = static_cast<const Real*>(sd.dS);
#pragma unroll
      for (int i = 0; i < 6; ++i) {
        rs[i] = -vol * (sd.h2 * g[i]);
        rl[i] = vol * symv(i) * double(dS[(size_t)i * ntp + e]);
      }
      double* VN = mr_vec(sd, MR_VN);
      double* WN = mr_vec(sd, MR_WN);
#pragma unroll
      for (int i = 0; i < 6; ++i) {
        double ws = 0, wl = 0;
#pragma unroll
        for (int j = 0; j < 6; ++j) {
          ws += Hs_inv[i + 6 * j] * rs[j];
          wl += Si[i + 6 * j] * rl[j];
        }
        const size_t js = XS + (size_t)i * ntp + e, jl = XL + (size_t)i * ntp + e;
        VN[js] = rs[i];
        VN[jl] = rl[i];
        WN[js] = ws;
        WN[jl] = wl;
        sums[0] += rs[i] * rs[i] + rl[i] * rl[i];
        sums[1] += rs[i] * ws + rl[i] * wl;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          if (k == MR_VN || k == MR_WN) continue;
          mr_vec(sd, k)[js] = 0.0;
          mr_vec(sd, k)[jl] = 0.0;
        }
      }
    }
  } else if (idx < t.end) {
    const int a = idx;
    const int f = sd.free_map[a];
    if (f >= 0) {
      // -PM (x - x_tilde - h^2 f) of row a (Displacement::gradient, displacement.cpp:64-73)
      const Real* mval = static_cast<const Real*>(sd.m_val);
      E Md[3] = {E(0), E(0), E(0)};
      for (int q = sd.m_ptr[a]; q < sd.m_ptr[a + 1]; ++q) {
        const int b = sd.m_col[q];
        const E m = E(mval[q]);
#pragma unroll
        for (int c = 0; c < 3; ++c)
          Md[c] = Md[c] + m * (Ext<Real>::ld(sd.x, 3 * (size_t)b + c) - Ext<Real>::ld(sd.xt, 3 * (size_t)b + c));
      }
      const double ml = sd.mr_mlinv[f];
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const size_t j = 4 * (size_t)f + c;
        const double r = c < 3 ? -to_double_any(Md[c]) : 0.0;
        mr_vec(sd, MR_VN)[j] = r;
        mr_vec(sd, MR_WN)[j] = ml * r;
        sums[0] += r * r;
        sums[1] += r * ml * r;
#pragma unroll
        for (int k = 0; k < 8; ++k)
          if (k != MR_VN && k != MR_WN) mr_vec(sd, k)[j] = 0.0;
      }
    }
  }
  tile_partials<double, double, 2, 0>(sums, nullptr, partials, pstride, 0, tix);
  if (last_tile(sd, TB_EV, tix)) {
    double v[2];
    scene_sums<double, 2>(partials, pstride, 0, sd.tile_first[TB_EV], sd.tile_count[TB_EV], v);
    if (threadIdx.x == 0) {
      const double rhs2 = v[0], beta2 = v[1];
      sc->cg_iter = 0;
      sc->cg_status = 0;
      sc->mr_pending = 0;
      sc->mr_slot = 0;
      sc->cg_rhs_norm2 = rhs2;
      if (rhs2 == 0.0 || !(beta2 > 0.0)) {
        // zero right-hand side (Eigen: x = 0, no iteration)
        sc->cg_active = 0;
        sc->cg_err = 0.0;
      } else {
        const double b = sqrt(beta2);
        sc->mr_beta = b;
        sc->mr_beta_one = b;
        sc->mr_c = sc->mr_c_old = 1.0;
        sc->mr_s = sc->mr_s_old = 0.0;
        sc->mr_eta = 1.0;
        sc->mr_resid2 = rhs2;
        sc->mr_thr2 = sd.cg_tol * sd.cg_tol * rhs2;
        if (sd.max_cg > 0) {
          sc->cg_active = 1;
          atomicAdd(&ctrs->cg_active, 1);
        } else {
          sc->cg_active = 0;
          sc->cg_status = 5;  // MFEM_ERR_CG_MAXITER
          sc->cg_err = 1.0;
        }
      }
    }
  }
}

// -------------------------------------------------------------------- A1 ---
template <typename Real>
__global__ void __launch_bounds__(kElemTile) k_mr_elem(const Tile* tiles, const SceneDev* sds,
                                                       double* partials, int pstride) {
  const int tix = blockIdx.x;
  const Tile t = tiles[tix];
  const SceneDev& sd = sds[t.scene];
  const SceneScalars* sc = sd.sc;
  const bool active = sc->cg_active != 0, pending = sc->mr_pending != 0;
  if (t.kind != 0 || (!active && !pending)) return;
  const int idx = t.begin + threadIdx.x;
  const int ntp = sd.ntp;
  const size_t XS = 4 * (size_t)sd.nf, XL = XS + 6 * (size_t)ntp;
  double alpha_part = 0.0;
  if (idx < t.end) {
    const int e = idx;
    if (pending) {
#pragma unroll
      for (int i = 0; i < 6; ++i) {
        mr_pending_entry(sd, sc, XS + (size_t)i * ntp + e);
        mr_pending_entry(sd, sc, XL + (size_t)i * ntp + e);
      }
    }
    if (active) {
      const double beta = sc->mr_beta, ib = 1.0 / beta;
      double* V = mr_vec(sd, MR_V);
      double* VN = mr_vec(sd, MR_VN);
      const double* WN = mr_vec(sd, MR_WN);
      double* W = mr_vec(sd, MR_W);
      double vo[12], w[12];
#pragma unroll
      for (int i = 0; i < 12; ++i) {
        const size_t j = XS + (size_t)i * ntp + e;  // s rows then lambda rows
        vo[i] = V[j];
        const double v = VN[j] * ib;
        w[i] = WN[j] * ib;
        V[j] = v;
        W[j] = w[i];
      }
      // The element products run in the element data's precision (FP32 in
      // the mixed path: GB300's FP64 rate is 1/64 of FP32's, and these are
      // most of the iteration's arithmetic); the Lanczos vectors and the
      // inner products stay FP64.
      const Real vol = static_cast<const Real*>(sd.vol)[e];
      const Real* Hp = static_cast<const Real*>(sd.mr_H);
      Real H[36];
#pragma unroll
      for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int j = i; j < 6; ++j) {
          const Real v = Hp[(size_t)sym6(i, j) * ntp + e];
          H[i + 6 * j] = v;
          H[j + 6 * i] = v;
        }
      const Real* Bp = static_cast<const Real*>(sd.mr_B);
      const int4 tv = sd.tets[e];
      const int v4[4] = {tv.x, tv.y, tv.z, tv.w};
      Real wx[12], wr[12];
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        const int f = sd.free_map[v4[a]];
#pragma unroll
        for (int l = 0; l < 3; ++l) wx[3 * a + l] = f >= 0 ? Real(WN[4 * (size_t)f + l] * ib) : Real(0);
      }
#pragma unroll
      for (int i = 0; i < 12; ++i) wr[i] = Real(w[i]);
      double tkw[12];
#pragma unroll
      for (int i = 0; i < 6; ++i) {
        Real hs = Real(0), bw = Real(0);
#pragma unroll
        for (int j = 0; j < 6; ++j) hs += H[i + 6 * j] * wr[j];
#pragma unroll
        for (int q = 0; q < 12; ++q) bw += Bp[(size_t)(12 * i + q) * ntp + e] * wx[q];
        tkw[i] = double(vol * hs + vol * Real(symv(i)) * wr[6 + i]);
        tkw[6 + i] = double(-vol * Real(symv(i)) * bw + vol * Real(symv(i)) * wr[i]);
      }
#pragma unroll
      for (int i = 0; i < 12; ++i) {
        const double tv_ = tkw[i] - beta * vo[i];
        VN[XS + (size_t)i * ntp + e] = tv_;
        alpha_part += tv_ * w[i];
      }
      // x-row shares of this element: -vol B_a^T Sym w_lambda
#pragma unroll
      for (int q = 0; q < 12; ++q) {
        Real acc = Real(0);
#pragma unroll
        for (int i = 0; i < 6; ++i) acc += Bp[(size_t)(12 * i + q) * ntp + e] * Real(symv(i)) * wr[6 + i];
        sd.mr_y[(size_t)q * ntp + e] = double(-vol * acc);
      }
    }
  }
  if (active) tile_partials<double, double, 1, 0>(&alpha_part, nullptr, partials, pstride, 0, tix);
}

// -------------------------------------------------------------------- A2 ---
template <typename Real>
__global__ void __launch_bounds__(kElemTile) k_mr_vert(const Tile* tiles, const SceneDev* sds,
                                                       double* partials, int pstride) {
  const int tix = blockIdx.x;
  const Tile t = tiles[tix];
  const SceneDev& sd = sds[t.scene];
  SceneScalars* sc = sd.sc;
  const bool active = sc->cg_active != 0, pending = sc->mr_pending != 0;
  if (!active && !pending) return;
  const int idx = t.begin + threadIdx.x;
  double alpha_part = 0.0;
  if (t.kind == 1 && idx < t.end) {
    const int a = idx;
    const int f = sd.free_map[a];
    if (f >= 0) {
      if (pending) {
#pragma unroll
        for (int c = 0; c < 3; ++c) mr_pending_entry(sd, sc, 4 * (size_t)f + c);
      }
      if (active) {
        const double beta = sc->mr_beta, ib = 1.0 / beta;
        double* V = mr_vec(sd, MR_V);
        double* VN = mr_vec(sd, MR_VN);
        const double* WN = mr_vec(sd, MR_WN);
        double* W = mr_vec(sd, MR_W);
        const Real* mval = static_cast<const Real*>(sd.m_val);
        double kw[3] = {0.0, 0.0, 0.0};
        for (int q = sd.m_ptr[a]; q < sd.m_ptr[a + 1]; ++q) {
          const int fb = sd.free_map[sd.m_col[q]];
          if (fb < 0) continue;
          const double m = double(mval[q]);
#pragma unroll
          for (int c = 0; c < 3; ++c) kw[c] += m * (WN[4 * (size_t)fb + c] * ib);
        }
        for (int q = sd.inc_ptr[f]; q < sd.inc_ptr[f + 1]; ++q) {
          const int2 ic = sd.inc[q];
          const int li = ic.y & 3;
#pragma unroll
          for (int c = 0; c < 3; ++c) kw[c] += sd.mr_y[(size_t)(3 * li + c) * sd.ntp + ic.x];
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const size_t j = 4 * (size_t)f + c;
          const double vo = V[j];
          const double w = WN[j] * ib;
          V[j] = VN[j] * ib;
          W[j] = w;
          const double tv_ = kw[c] - beta * vo;
          VN[j] = tv_;
          alpha_part += tv_ * w;
        }
      }
    }
  }
  // element tiles keep the partials A1 wrote; vertex tiles add theirs
  if (active && t.kind == 1) tile_partials<double, double, 1, 0>(&alpha_part, nullptr, partials, pstride, 0, tix);
  if (last_tile(sd, TB_EV, tix)) {
    double v[1] = {0.0};
    if (active) scene_sums<double, 1>(partials, pstride, 0, sd.tile_first[TB_EV], sd.tile_count[TB_EV], v);
    if (threadIdx.x == 0) {
      if (active) sc->mr_alpha = v[0];
      sc->mr_pending = 0;
    }
  }
}

// --------------------------------------------------------------------- B ---
template <typename Real>
__global__ void __launch_bounds__(kElemTile) k_mr_update(const Tile* tiles, const SceneDev* sds,
                                                         double* partials, int pstride,
                                                         BatchCounters* ctrs) {
  const int tix = blockIdx.x;
  const Tile t = tiles[tix];
  const SceneDev& sd = sds[t.scene];
  SceneScalars* sc = sd.sc;
  if (!sc->cg_active) return;
  const int idx = t.begin + threadIdx.x;
  const int ntp = sd.ntp;
  const size_t XS = 4 * (size_t)sd.nf, XL = XS + 6 * (size_t)ntp;
  const double alpha = sc->mr_alpha;
  double* VN = mr_vec(sd, MR_VN);
  double* WN = mr_vec(sd, MR_WN);
  const double* V = mr_vec(sd, MR_V);
  double b2 = 0.0;
  if (t.kind == 0) {
    if (idx < t.end) {
      const int e = idx;
      double vs[6], vl[6];
#pragma unroll
      for (int i = 0; i < 6; ++i) {
        const size_t js = XS + (size_t)i * ntp + e, jl = XL + (size_t)i * ntp + e;
        vs[i] = VN[js] - alpha * V[js];
        vl[i] = VN[jl] - alpha * V[jl];
        VN[js] = vs[i];
        VN[jl] = vl[i];
      }
      double Hi[36], Si[36];
      load_sym21<double>(sd.mr_hinv, ntp, e, Hi);
      load_sym21<double>(sd.mr_sinv, ntp, e, Si);
#pragma unroll
      for (int i = 0; i < 6; ++i) {
        double ws = 0.0, wl = 0.0;
#pragma unroll
        for (int j = 0; j < 6; ++j) {
          ws += Hi[i + 6 * j] * vs[j];
          wl += Si[i + 6 * j] * vl[j];
        }
        WN[XS + (size_t)i * ntp + e] = ws;
        WN[XL + (size_t)i * ntp + e] = wl;
        b2 += vs[i] * ws + vl[i] * wl;
      }
    }
  } else if (idx < t.end) {
    const int f = sd.free_map[idx];
    if (f >= 0) {
      const double ml = sd.mr_mlinv[f];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const size_t j = 4 * (size_t)f + c;
        const double v = VN[j] - alpha * V[j];
        VN[j] = v;
        WN[j] = ml * v;
        b2 += v * ml * v;
      }
    }
  }
  tile_partials<double, double, 1, 0>(&b2, nullptr, partials, pstride, 0, tix);
  if (last_tile(sd, TB_EV, tix)) {
    double v[1];
    scene_sums<double, 1>(partials, pstride, 0, sd.tile_first[TB_EV], sd.tile_count[TB_EV], v);
    if (threadIdx.x == 0) {
      const int k = sc->cg_iter;
      const double beta = sc->mr_beta;
      const double beta_new = v[0] > 0.0 ? sqrt(v[0]) : 0.0;
      const double c = sc->mr_c, c_old = sc->mr_c_old, s = sc->mr_s, s_old = sc->mr_s_old;
      // Givens rotation
      const double r2 = s * alpha + c * c_old * beta;
      const double r3 = s_old * beta;
      const double r1_hat = c * alpha - c_old * s * beta;
      const double r1 = sqrt(r1_hat * r1_hat + beta_new * beta_new);
      bool stop = false;
      if (!(r1 > 0.0) || !isfinite(r1)) {
        // breakdown: no further direction; keep the current x
        sc->mr_pending = 0;
        sc->cg_status = isfinite(r1) ? 0 : 4;  // MFEM_ERR_NONFINITE
        sc->cg_iter = k;
        stop = true;
      } else {
        const double cn = r1_hat / r1, sn = beta_new / r1;
        sc->mr_c_old = c;
        sc->mr_s_old = s;
        sc->mr_c = cn;
        sc->mr_s = sn;
        sc->mr_r1 = r1;
        sc->mr_r2 = r2;
        sc->mr_r3 = r3;
        sc->mr_coef = sc->mr_beta_one * cn * sc->mr_eta;
        sc->mr_slot = k % 3;
        sc->mr_pending = 1;
        sc->mr_beta = beta_new;
        const double res2 = sc->mr_resid2 * sn * sn;
        sc->mr_resid2 = res2;
        if (res2 < sc->mr_thr2) {
          sc->cg_iter = k;
          stop = true;
        } else {
          sc->mr_eta = -sn * sc->mr_eta;
          sc->cg_iter = k + 1;
          if (k + 1 >= sd.max_cg) {
            sc->cg_status = 5;  // MFEM_ERR_CG_MAXITER
            stop = true;
          }
        }
      }
      if (stop) {
        sc->cg_err = sc->cg_rhs_norm2 > 0.0 ? sqrt(sc->mr_resid2 / sc->cg_rhs_norm2) : 0.0;
        sc->cg_total += sc->cg_iter;
        sc->cg_active = 0;
        atomicSub(&ctrs->cg_active, 1);
      }
    }
  }
}

// ---------------------------------------------------------------- export ---
// dx (the PCG solution vector the line search and apply read) from x.
template <typename Real>
__global__ void __launch_bounds__(kElemTile) k_mr_export(const Tile* tiles, const SceneDev* sds) {
  const Tile t = tiles[blockIdx.x];
  const SceneDev& sd = sds[t.scene];
  if (!sd.sc->newton_active || t.kind != 1) return;
  const int idx = t.begin + threadIdx.x;
  if (idx >= t.end) return;
  const int f = sd.free_map[idx];
  if (f < 0) return;
  const double* X = mr_vec(sd, MR_X);
  Real* cgx = static_cast<Real*>(sd.cg_x);
#pragma unroll
  for (int c = 0; c < 4; ++c) cgx[4 * (size_t)f + c] = c < 3 ? Real(X[4 * (size_t)f + c]) : Real(0);
}

}  // namespace

#define MFEM_LAUNCH_MR(kern, ...)                                       \
  do {                                                                  \
    if (L.ntiles == 0) return;                                          \
    if (L.fp64)                                                         \
      kern<double><<<L.ntiles, kElemTile, 0, L.stream>>>(__VA_ARGS__);  \
    else                                                                \
      kern<float><<<L.ntiles, kElemTile, 0, L.stream>>>(__VA_ARGS__);   \
  } while (0)

void launch_mr_init(const Launch& L) {
  MFEM_LAUNCH_MR(k_mr_init, L.tiles, L.sds, L.partials, L.pstride, L.counters);
}
void launch_mr_elem(const Launch& L) { MFEM_LAUNCH_MR(k_mr_elem, L.tiles, L.sds, L.partials, L.pstride); }
void launch_mr_vert(const Launch& L) { MFEM_LAUNCH_MR(k_mr_vert, L.tiles, L.sds, L.partials, L.pstride); }
void launch_mr_update(const Launch& L) {
  MFEM_LAUNCH_MR(k_mr_update, L.tiles, L.sds, L.partials, L.pstride, L.counters);
}
void launch_mr_export(const Launch& L) { MFEM_LAUNCH_MR(k_mr_export, L.tiles, L.sds); }

}  // namespace mfem_gpu
