// Element-parallel kernels of the mixed-stretch Newton step.
//
//   k_elem_init     s0 = polar(F0)                    mixed_stretch.cpp:287-303
//   k_elem_update   K1: F = J x, polar R (warm start), S, ds/dF, h^2 psi'/psi''
//                   (psd-fixed), the 12x12 element block and the element's
//                   right-hand-side share            mixed_stretch.cpp:133-226
//   k_local_solve   K5: ds, lambda and E(0)          mixed_stretch.cpp:243-259,
//                                                     newton_optimizer.cpp:34-52
//   k_ls_energy     K6: E(alpha) for the backtracking line search
//                                                     linesearch.h:80-129
//   k_apply         x += alpha dx, s += alpha ds       linesearch.h:120-125
//   k_step_begin/end  BDF x_tilde, BDF update, pins, lambda = 0
//                                                     BDF.cpp:6-27, displacement.cpp:32-50
//
// One thread per element.  Element arrays are structure-of-arrays with
// stride ntp.  Real is the working precision (float in the mixed path) and
// Ext the high precision (df64 / double) of positions, s and the residual.
#include <cfloat>

#include "device_math.cuh"
#include "kernels.cuh"
#include "reduce.cuh"

namespace mfem_gpu {

namespace {

constexpr double kPsdTol = 1e-6;         // simple_psd_fix tolerance
constexpr double kProcrustesTol = 1e-6;  // mixed_stretch.cpp:21-22
constexpr int kProcrustesIters = 100;

template <typename Real> struct ElemIn {
  int4 tv;
  Real dp[9];  // dphi_k/dX for k = 1..3: dp[3(k-1)+c]
  Real vol, mu, lam;
  int mat;
};

template <typename Real>
__device__ __forceinline__ void load_elem(const SceneDev& sd, int e, ElemIn<Real>& in) {
  const Real* dphi = static_cast<const Real*>(sd.dphi);
  const int ntp = sd.ntp;
  in.tv = sd.tets[e];
#pragma unroll
  for (int i = 0; i < 9; ++i) in.dp[i] = dphi[i * ntp + e];
  in.vol = static_cast<const Real*>(sd.vol)[e];
  in.mu = static_cast<const Real*>(sd.mu)[e];
  in.lam = static_cast<const Real*>(sd.lam)[e];
  in.mat = sd.material_uniform >= 0 ? sd.material_uniform : int(sd.mat[e]);
}

template <typename Real>
__device__ __forceinline__ void dphi12(const ElemIn<Real>& in, Real* dph) {
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    dph[3 + c] = in.dp[c];
    dph[6 + c] = in.dp[3 + c];
    dph[9 + c] = in.dp[6 + c];
    dph[c] = -(in.dp[c] + in.dp[3 + c] + in.dp[6 + c]);
  }
}

// F = sum_k (x_k - x_0) (x) dphi_k with the edge vectors in Ext (optionally
// at x + alpha dx), returned in Ext (when FE is given) and rounded to Real.
template <typename Real>
__device__ __forceinline__ void deformation_gradients(const SceneDev& sd, const ElemIn<Real>& in,
                                                      const Real* dx, typename Ext<Real>::T alpha,
                                                      typename Ext<Real>::T* FE, Real* F) {
  using E = typename Ext<Real>::T;
  const int v[4] = {in.tv.x, in.tv.y, in.tv.z, in.tv.w};
  E p[4][3];
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int d = 0; d < 3; ++d) p[k][d] = Ext<Real>::ld(sd.x, 3 * (size_t)v[k] + d);
  if (dx != nullptr) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int f = sd.free_map[v[k]];
      if (f >= 0) {
#pragma unroll
        for (int d = 0; d < 3; ++d) p[k][d] = p[k][d] + alpha * E(dx[4 * f + d]);
      }
    }
  }
  E ed[9];
#pragma unroll
  for (int k = 1; k < 4; ++k)
#pragma unroll
    for (int r = 0; r < 3; ++r) ed[3 * (k - 1) + r] = p[k][r] - p[0][r];
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      if (FE) {
        const E f = madd(madd(ed[r] * E(in.dp[c]), ed[3 + r], in.dp[3 + c]), ed[6 + r], in.dp[6 + c]);
        FE[r + 3 * c] = f;
        F[r + 3 * c] = Real(Ext<Real>::to_real(f));
      } else {
        F[r + 3 * c] = Real(Ext<Real>::to_real(ed[r])) * in.dp[c] +
                       Real(Ext<Real>::to_real(ed[3 + r])) * in.dp[3 + c] +
                       Real(Ext<Real>::to_real(ed[6 + r])) * in.dp[6 + c];
      }
    }
}

template <typename Real>
__device__ __forceinline__ void load_quat(const SceneDev& sd, int e, Real* R) {
  const Real* q = static_cast<const Real*>(sd.quat);
  Real qq[4] = {q[e], q[sd.ntp + e], q[2 * sd.ntp + e], q[3 * sd.ntp + e]};
  quat_to_rot(qq, R);
}

// Stores R as its quaternion and returns, in RE, the rotation of that
// quaternion evaluated in Ext.  In the mixed path the Real rotation is
// orthogonal only to ~1e-7 and differs from one evaluation to the next
// through the rounding of its quaternion; the polish of the residual chain
// converges the rotation's angle but cannot repair a non-orthogonal start,
// so the chain starts from the quaternion's exactly orthogonal rotation
// (quat_to_rot normalises).  Otherwise S = R^T F would carry ~1e-7 of
// evaluation-to-evaluation noise, i.e. 1e-4 of a 1e-3 strain, which floors
// the Newton residual near 1e-5.
template <typename Real>
__device__ __forceinline__ void quat_rot_ext(const Real qq[4], const Real* R, typename Ext<Real>::T* RE) {
  using E = typename Ext<Real>::T;
  if constexpr (Prec<Real>::kFP64) {
#pragma unroll
    for (int i = 0; i < 9; ++i) RE[i] = E(R[i]);
  } else {
    quat_to_rot_df(qq, RE);
  }
}

template <typename Real>
__device__ __forceinline__ void store_quat(const SceneDev& sd, int e, const Real* R,
                                           typename Ext<Real>::T* RE = nullptr) {
  Real* q = static_cast<Real*>(sd.quat);
  Real qq[4];
  rot_to_quat(R, qq);
#pragma unroll
  for (int i = 0; i < 4; ++i) q[i * sd.ntp + e] = qq[i];
  if (RE) quat_rot_ext<Real>(qq, R, RE);
}

// S(F) in Ext from a Real Procrustes rotation: the orthogonal Ext rotation
// of its quaternion, polished against the Ext F in the mixed path (the same
// construction as the residual chain of K1, so that the line-search energy
// and the energy at alpha = 0 agree).
template <typename Real>
__device__ __forceinline__ void stretch_ext(const Real* R, const typename Ext<Real>::T* FE,
                                            typename Ext<Real>::T* SE) {
  using E = typename Ext<Real>::T;
  Real qq[4];
  rot_to_quat(R, qq);
  E RE[9];
  quat_rot_ext<Real>(qq, R, RE);
  if (!Prec<Real>::kFP64) polish_rotation(RE, FE);
  stretch_vec(RE, FE, SE);
}

template <typename Real>
__device__ __forceinline__ void load6(const void* base, int ntp, int e, Real* v) {
  const Real* p = static_cast<const Real*>(base);
#pragma unroll
  for (int i = 0; i < 6; ++i) v[i] = p[i * ntp + e];
}
template <typename Real>
__device__ __forceinline__ void store6(void* base, int ntp, int e, const Real* v) {
  Real* p = static_cast<Real*>(base);
#pragma unroll
  for (int i = 0; i < 6; ++i) p[i * ntp + e] = v[i];
}
template <typename Real>
__device__ __forceinline__ void load6e(const SceneDev& sd, int e, typename Ext<Real>::T* v) {
#pragma unroll
  for (int i = 0; i < 6; ++i) v[i] = Ext<Real>::ld(sd.s, (size_t)i * sd.ntp + e);
}

// h^2 * gradient and psd-fixed h^2 * Hessian of psi at s.
template <typename Real>
__device__ __forceinline__ void material_gH(const ElemIn<Real>& in, const Real* s, Real h2,
                                            Real* g, Real* H) {
  bool psd = material_grad_hess<Real>(in.mat, in.mu, in.lam, s, g, H);
  if (psd) psd_fix(H, Real(kPsdTol));
#pragma unroll
  for (int i = 0; i < 6; ++i) g[i] *= h2;
#pragma unroll
  for (int i = 0; i < 36; ++i) H[i] *= h2;
}

// Offset of entry (l, m) of block (a, b) in the element record: upper
// blocks row-major, diagonal blocks as (xx, xy, xz, yy, yz, zz).
__host__ __device__ constexpr int rec_block_start(int a) {
  return a == 0 ? 0 : (a == 1 ? 33 : (a == 2 ? 57 : 72));
}
__host__ __device__ constexpr int sym_idx(int r, int c) { return r == 0 ? c : (r == 1 ? 2 + c : 5); }

// 32-bit-word stores into the staged element record (shared memory).
__device__ __forceinline__ void put_word(unsigned int* w, int idx, float v) { w[idx] = __float_as_uint(v); }
__device__ __forceinline__ void put_word(unsigned int* w, int idx, double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  w[idx] = (unsigned int)(b & 0xffffffffull);
  w[idx + 1] = (unsigned int)(b >> 32);
}
__device__ __forceinline__ void put_word(unsigned int* w, int idx, df64 v) {
  w[idx] = __float_as_uint(v.hi);
  w[idx + 1] = __float_as_uint(v.lo);
}

// ------------------------------------------------------------------ K0 ---
template <typename Real>
__global__ void __launch_bounds__(kElemTile) k_elem_init(const Tile* tiles, const SceneDev* sds) {
  using E = typename Ext<Real>::T;
  const Tile t = tiles[blockIdx.x];
  const SceneDev& sd = sds[t.scene];
  const int e = t.begin + threadIdx.x;
  if (e >= t.end) return;
  ElemIn<Real> in;
  load_elem(sd, e, in);
  E FE[9];
  Real F[9], R[9];
  deformation_gradients<Real>(sd, in, nullptr, E(0), FE, F);
#pragma unroll
  for (int i = 0; i < 9; ++i) R[i] = (i % 4 == 0) ? Real(1) : Real(0);
  int it = procrustes<Real>(R, F, Real(kProcrustesTol), kProcrustesIters);
  if (it < 0) atomicAdd(&sd.sc->procrustes_fail, 1);
  E RE[9], sE[6];
  store_quat(sd, e, R, RE);
  if (!Prec<Real>::kFP64) polish_rotation(RE, FE);
  stretch_vec(RE, FE, sE);
#pragma unroll
  for (int i = 0; i < 6; ++i) Ext<Real>::st(sd.s, (size_t)i * sd.ntp + e, sE[i]);
  Real z[6] = {0, 0, 0, 0, 0, 0};
  store6(sd.dS, sd.ntp, e, z);
  store6(sd.la, sd.ntp, e, z);
  store6(sd.ds, sd.ntp, e, z);
}

// ------------------------------------------------------------------ K1 ---
// The residual chain (one Ext polish of the Real rotation, S, S - s,
// h^2 psi'(s), q and the element forces) runs in Ext: in a loaded body the
// element forces are tens of times the net residual, so Real forces would
// floor the Newton residual near 1e-4.  The Hessian, ds/dF and the element
// block stay in Real.
// MB: resident blocks per SM the register allocation must allow (0: the
// compiler's own choice).  The variants differ only in register allocation
// (the autotuner picks one per batch); each one offered is tested to
// compute the same bits as the default.
template <typename Real, bool DBG, int MB = 0>
__global__ void __launch_bounds__(kElemTile, MB)
    k_elem_update(const Tile* tiles, const SceneDev* sds, ElemDebug dbg) {
  using E = typename Ext<Real>::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned int* words = reinterpret_cast<unsigned int*>(smem_raw);
  constexpr int RB = sizeof(Real);
  constexpr int kWords = rec_bytes(RB) / 4;  // words per record
  constexpr int kStride = kWords + 1;         // odd stride: no bank conflicts
  constexpr int kRhsWord = rec_rhs_offset(RB) / 4;
  const Tile t = tiles[blockIdx.x];
  const SceneDev& sd = sds[t.scene];
  if (!sd.sc->newton_active || not_my_phase(sd.sc, kPhNewton)) return;
  const int e = t.begin + threadIdx.x;
  const Real h2 = Ext<Real>::r(sd.h2, sd.h2x);
  if (e < t.end) {
    unsigned int* out = words + threadIdx.x * kStride;
    ElemIn<Real> in;
    load_elem(sd, e, in);
    E sE[6];
    load6e<Real>(sd, e, sE);
    Real sv[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) sv[i] = Real(Ext<Real>::to_real(sE[i]));
    Real g[6], H[36];
    material_gH(in, sv, h2, g, H);
    E FE[9];
    Real F[9], R[9];
    deformation_gradients<Real>(sd, in, nullptr, E(0), FE, F);
    load_quat(sd, e, R);
    int it = procrustes<Real>(R, F, Real(kProcrustesTol), kProcrustesIters);
    E RE[9];
    store_quat(sd, e, R, RE);
    Real S6[6];
    stretch_vec(R, F, S6);
    Real u[18];
    bool ok = stretch_derivative_u(S6, u);
    if (it < 0 || !ok) atomicAdd(&sd.sc->procrustes_fail, 1);
    Real dph[12];
    dphi12(in, dph);
    // ---- residual chain in Ext: S - s, q = H (S - s) + h^2 psi'(s), forces
    {
      E SE[6], dE[6], gE[6], qE[6], dphE[12], fE[12];
      if (!Prec<Real>::kFP64) polish_rotation(RE, FE);
      stretch_vec(RE, FE, SE);
      material_grad<E>(in.mat, E(in.mu), E(in.lam), sE, gE);
      const E h2E = Ext<Real>::c(sd.h2, sd.h2x);
#pragma unroll
      for (int i = 0; i < 6; ++i) dE[i] = SE[i] - sE[i];
      if constexpr (Prec<Real>::kFP64) {
#pragma unroll
        for (int i = 0; i < 6; ++i) {
          E acc = h2E * gE[i];
#pragma unroll
          for (int j = 0; j < 6; ++j) acc = acc + E(H[i + 6 * j]) * dE[j];
          qE[i] = acc;
        }
      } else {
        // H (S - s) in FP32: its rounding is relative to |S - s|, which
        // vanishes as the Newton iteration converges, so it cannot floor
        // the residual; h^2 psi'(s), an O(stress) term, stays float-float.
        Real d32[6];
#pragma unroll
        for (int j = 0; j < 6; ++j) d32[j] = Real(Ext<Real>::to_real(dE[j]));
#pragma unroll
        for (int i = 0; i < 6; ++i) {
          Real hd = 0;
#pragma unroll
          for (int j = 0; j < 6; ++j) hd += H[i + 6 * j] * d32[j];
          qE[i] = h2E * gE[i] + E(hd);
        }
      }
#pragma unroll
      for (int i = 0; i < 12; ++i) dphE[i] = E(dph[i]);
      element_force<E>(RE, SE, qE, dphE, E(in.vol), fE);
#pragma unroll
      for (int i = 0; i < 12; ++i) put_word(out, kRhsWord + 2 * i, fE[i]);
      Real dS[6];
#pragma unroll
      for (int i = 0; i < 6; ++i) dS[i] = Real(Ext<Real>::to_real(dE[i]));
      store6(sd.dS, sd.ntp, e, dS);
      if (DBG) {
        const size_t Ei = e;
        for (int i = 0; i < 9; ++i) dbg.R[9 * Ei + i] = to_double_any(RE[i]);
        for (int i = 0; i < 6; ++i) {
          dbg.S[6 * Ei + i] = to_double_any(SE[i]);
          dbg.g[6 * Ei + i] = to_double_any(h2E * gE[i]);
          dbg.gl[6 * Ei + i] = (i < 3 ? 1.0 : 0.5) * to_double_any(qE[i]);
        }
        for (int i = 0; i < 36; ++i) dbg.H[36 * Ei + i] = H[i];
      }
    }
    // ---- B[i][a][l] = ds_i / dx_{a,l} = (G_i dphi_a)_l
    Real B[72];
    {
      Real G[54];
      ds_dF(R, u, G);
#pragma unroll
      for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int l = 0; l < 3; ++l)
            B[12 * i + 3 * a + l] = G[9 * i + l] * dph[3 * a] + G[9 * i + l + 3] * dph[3 * a + 1] +
                                    G[9 * i + l + 6] * dph[3 * a + 2];
      if (DBG) {
        const double sym[6] = {1, 1, 1, 2, 2, 2};
        for (int i = 0; i < 6; ++i)
          for (int r = 0; r < 9; ++r) dbg.dSdF[54 * (size_t)e + r + 9 * i] = sym[i] * double(G[9 * i + r]);
      }
    }
    if (sd.minres) {
      // ds/dx and the Hessian for the matrix-free (x, s, lambda) product
      Real* Bo = static_cast<Real*>(sd.mr_B);
#pragma unroll
      for (int k = 0; k < 72; ++k) Bo[(size_t)k * sd.ntp + e] = B[k];
      Real* Ho = static_cast<Real*>(sd.mr_H);
      int k = 0;
#pragma unroll
      for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int j = i; j < 6; ++j, ++k) Ho[(size_t)k * sd.ntp + e] = H[i + 6 * j];
    }
    // ---- upper 3x3 blocks of Aloc = vol * B^T H B  (mixed_stretch.cpp:174-175);
    // with B_0 = -(B_1 + B_2 + B_3), block (0, 0) is -sum_b (0, b)
    Real A00[6] = {Real(0), Real(0), Real(0), Real(0), Real(0), Real(0)};
#pragma unroll
    for (int b = 1; b < 4; ++b) {
      Real HB[18];
#pragma unroll
      for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int m = 0; m < 3; ++m) {
          Real acc = 0;
#pragma unroll
          for (int j = 0; j < 6; ++j) acc += H[i + 6 * j] * B[12 * j + 3 * b + m];
          HB[3 * i + m] = acc;
        }
#pragma unroll
      for (int a = 0; a <= b; ++a) {
        const int base = rec_block_start(a) + (a == b ? 0 : 6 + 9 * (b - a - 1));
#pragma unroll
        for (int l = 0; l < 3; ++l)
#pragma unroll
          for (int m = 0; m < 3; ++m) {
            if (a == b && m < l) continue;
            Real acc = 0;
#pragma unroll
            for (int i = 0; i < 6; ++i) acc += B[12 * i + 3 * a + l] * HB[3 * i + m];
            const int k = base + (a == b ? sym_idx(l, m) : 3 * l + m);
            const Real v = in.vol * acc;
            if (a == 0 && m >= l) A00[sym_idx(l, m)] -= v;
            put_word(out, k * (RB / 4), v);
            if (DBG) {
              const size_t Ei = e;
              dbg.Aloc[144 * Ei + (3 * a + l) + 12 * (3 * b + m)] = double(v);
              dbg.Aloc[144 * Ei + (3 * b + m) + 12 * (3 * a + l)] = double(v);
            }
          }
      }
    }
#pragma unroll
    for (int l = 0; l < 3; ++l)
#pragma unroll
      for (int m = l; m < 3; ++m) {
        const Real v = A00[sym_idx(l, m)];
        put_word(out, sym_idx(l, m) * (RB / 4), v);
        if (DBG) {
          const size_t Ei = e;
          dbg.Aloc[144 * Ei + l + 12 * m] = double(v);
          dbg.Aloc[144 * Ei + m + 12 * l] = double(v);
        }
      }
  }
  __syncthreads();
  // contiguous store of the tile's records as 32-bit words
  const int n = t.end - t.begin;
  unsigned int* dst = reinterpret_cast<unsigned int*>(sd.rec + (size_t)t.begin * rec_bytes(RB));
  for (int i = threadIdx.x; i < n * kWords; i += blockDim.x) {
    const int el = i / kWords;
    dst[i] = words[el * kStride + (i - el * kWords)];
  }
}

// ------------------------------------------------------------- K1 (FEM) ---
// The standard-FEM variable (Stretch::update, src/variables/stretch.cpp:33-60):
// per element the 12x12 block h^2 vol Jloc^T d2psi/dF2 Jloc (psd-fixed:
// tolerance 0 for Stable-Neohookean, stable_neohookean.cpp:232; the default
// for Neohookean, neohookean.cpp:230) and the forces -h^2 vol Jloc^T dpsi/dF,
// in the record layout of the mixed K1 so that the assembly, the solvers and
// the line search are shared.  Forces in Ext, as in the mixed residual chain.
// The psd fix takes the closed-form eigensystem (fem_hess_projected), and
// the 9x9 Jacobi only when the SVD of F is ill-conditioned.
template <typename Real, bool DBG>
__global__ void __launch_bounds__(kElemTile)
    k_elem_fem(const Tile* tiles, const SceneDev* sds, ElemDebug dbg) {
  using E = typename Ext<Real>::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned int* words = reinterpret_cast<unsigned int*>(smem_raw);
  constexpr int RB = sizeof(Real);
  constexpr int kWords = rec_bytes(RB) / 4;
  constexpr int kStride = kWords + 1;
  constexpr int kRhsWord = rec_rhs_offset(RB) / 4;
  const Tile t = tiles[blockIdx.x];
  const SceneDev& sd = sds[t.scene];
  if (!sd.sc->newton_active || not_my_phase(sd.sc, kPhNewton)) return;
  const int e = t.begin + threadIdx.x;
  const Real h2 = Ext<Real>::r(sd.h2, sd.h2x);
  if (e < t.end) {
    unsigned int* out = words + threadIdx.x * kStride;
    ElemIn<Real> in;
    load_elem(sd, e, in);
    E FE[9];
    Real F[9];
    deformation_gradients<Real>(sd, in, nullptr, E(0), FE, F);
    Real dph[12];
    dphi12(in, dph);
    {
      E gE[9];
      fem_grad<E>(in.mat, E(in.mu), E(in.lam), FE, gE);
      const E c = E(0) - Ext<Real>::c(sd.h2, sd.h2x) * E(in.vol);
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int r = 0; r < 3; ++r) {
          const E f = c * (gE[r] * E(dph[3 * a]) + gE[r + 3] * E(dph[3 * a + 1]) + gE[r + 6] * E(dph[3 * a + 2]));
          put_word(out, kRhsWord + 2 * (3 * a + r), f);
        }
    }
    Real H[81];
    const Real tol = in.mat == kSNH ? Real(0) : Real(kPsdTol);
    if (!fem_hess_projected<Real>(in.mat, in.mu, in.lam, F, tol, H)) {
      Real g[9];
      fem_grad_hess<Real>(in.mat, in.mu, in.lam, F, g, H);
      psd_fix_n<9>(H, tol);
    }
    const Real w = h2 * in.vol;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      // HB(p, m) = sum_c' H(p, m + 3c') dphi_b[c']
      Real HB[27];
#pragma unroll
      for (int pp = 0; pp < 9; ++pp)
#pragma unroll
        for (int m = 0; m < 3; ++m)
          HB[pp + 9 * m] = H[pp + 9 * m] * dph[3 * b] + H[pp + 9 * (m + 3)] * dph[3 * b + 1] +
                           H[pp + 9 * (m + 6)] * dph[3 * b + 2];
#pragma unroll
      for (int a = 0; a <= b; ++a) {
        const int base = rec_block_start(a) + (a == b ? 0 : 6 + 9 * (b - a - 1));
#pragma unroll
        for (int l = 0; l < 3; ++l)
#pragma unroll
          for (int m = 0; m < 3; ++m) {
            if (a == b && m < l) continue;
            const Real acc = dph[3 * a] * HB[l + 9 * m] + dph[3 * a + 1] * HB[l + 3 + 9 * m] +
                             dph[3 * a + 2] * HB[l + 6 + 9 * m];
            const int k = base + (a == b ? sym_idx(l, m) : 3 * l + m);
            const Real v = w * acc;
            put_word(out, k * (RB / 4), v);
            if (DBG) {
              const size_t Ei = e;
              dbg.Aloc[144 * Ei + (3 * a + l) + 12 * (3 * b + m)] = double(v);
              dbg.Aloc[144 * Ei + (3 * b + m) + 12 * (3 * a + l)] = double(v);
            }
          }
      }
    }
  }
  __syncthreads();
  const int n = t.end - t.begin;
  unsigned int* dst = reinterpret_cast<unsigned int*>(sd.rec + (size_t)t.begin * rec_bytes(RB));
  for (int i = threadIdx.x; i < n * kWords; i += blockDim.x) {
    const int el = i / kWords;
    dst[i] = words[el * kStride + (i - el * kWords)];
  }
}

// Vertex part of the energy: 1/2 diff^T M diff with diff = x + alpha dx - xt.
template <typename Real>
__device__ __forceinline__ typename Ext<Real>::T vertex_energy(const SceneDev& sd, int a,
                                                               const Real* dx,
                                                               typename Ext<Real>::T alpha) {
  using E = typename Ext<Real>::T;
  const Real* mval = static_cast<const Real*>(sd.m_val);
  E Md[3] = {E(0), E(0), E(0)};
  for (int q = sd.m_ptr[a]; q < sd.m_ptr[a + 1]; ++q) {
    const int b = sd.m_col[q];
    const E m = E(mval[q]);
    const int fb = sd.free_map[b];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      E d = Ext<Real>::ld(sd.x, 3 * (size_t)b + c) - Ext<Real>::ld(sd.xt, 3 * (size_t)b + c);
      if (dx && fb >= 0) d = d + alpha * E(dx[4 * fb + c]);
      Md[c] = Md[c] + m * d;
    }
  }
  const int fa = sd.free_map[a];
  E e2 = E(0);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    E d = Ext<Real>::ld(sd.x, 3 * (size_t)a + c) - Ext<Real>::ld(sd.xt, 3 * (size_t)a + c);
    if (dx && fa >= 0) d = d + alpha * E(dx[4 * fa + c]);
    e2 = e2 + d * Md[c];
  }
  return E(0.5) * e2;
}

// ------------------------------------------------------------------ K5 ---
// ds = (S - s) + dS/dF : dF(dx)  (the closed form of -H^{-1}(Sym la + g),
// MixedStretch::solve), la = -Syminv (H ds + g); E(0), max |ds|, max |dx|.
// Tile partials: 0 E(0), 1 sum |terms|, 2 max|ds|, 3 max|dx|.
template <typename Real, int MB>
__global__ void __launch_bounds__(kElemTile, MB) k_local_solve(const Tile* tiles, const SceneDev* sds,
                                                           double* partials, int pstride,
                                                           BatchCounters* ctrs) {
  using E = typename Ext<Real>::T;
  const int tix = blockIdx.x;
  const Tile t = tiles[tix];
  const SceneDev& sd = sds[t.scene];
  SceneScalars* sc = sd.sc;
  if (!sc->newton_active || not_my_phase(sc, kPhLocal)) return;
  const Real h2 = Ext<Real>::r(sd.h2, sd.h2x);
  const Real* cgx = static_cast<const Real*>(sd.cg_x);
  E sums[2] = {E(0), E(0)};
  Real maxs[2] = {Real(0), Real(0)};
  const int idx = t.begin + threadIdx.x;
  if (t.kind == 0) {
    if (idx < t.end && sd.fem) {
      // standard FEM: E(0) element term h^2 vol psi(F) (Stretch::energy), no s
      ElemIn<Real> in;
      load_elem(sd, idx, in);
      E FE[9];
      Real F[9];
      deformation_gradients<Real>(sd, in, nullptr, E(0), FE, F);
      const E e1 = Ext<Real>::c(sd.h2, sd.h2x) * E(in.vol) * fem_psi<E>(in.mat, E(in.mu), E(in.lam), FE);
      sums[0] = e1;
      sums[1] = E(Real(1e-7) * Real(fabs(Ext<Real>::to_real(e1))));
    } else if (idx < t.end) {
      const int e = idx;
      ElemIn<Real> in;
      load_elem(sd, e, in);
      Real R[9], d[6], sv[6], S6[6];
      E sE[6];
      load_quat(sd, e, R);
      load6(sd.dS, sd.ntp, e, d);
      load6e<Real>(sd, e, sE);
#pragma unroll
      for (int i = 0; i < 6; ++i) {
        sv[i] = Real(Ext<Real>::to_real(sE[i]));
        S6[i] = Real(Ext<Real>::to_real(sE[i] + E(d[i])));
      }
      Real ds[6], la[6];
      if (sd.minres) {
        // MINRES solved for ds and lambda with dx (SystemMatrixIndefinite::
        // post_solve, linear_system.h:88-99)
        const double* X = sd.mr_vec + 7 * sd.mr_len + 4 * (size_t)sd.nf;
#pragma unroll
        for (int i = 0; i < 6; ++i) {
          ds[i] = Real(X[(size_t)i * sd.ntp + e]);
          la[i] = Real(X[(size_t)(6 + i) * sd.ntp + e]);
        }
      } else {
        const int v[4] = {in.tv.x, in.tv.y, in.tv.z, in.tv.w};
        Real dd[4][3];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const int f = sd.free_map[v[k]];
#pragma unroll
          for (int c = 0; c < 3; ++c) dd[k][c] = f >= 0 ? cgx[4 * f + c] : Real(0);
        }
        Real dF[9];
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
          for (int r = 0; r < 3; ++r)
            dF[r + 3 * c] = (dd[1][r] - dd[0][r]) * in.dp[c] + (dd[2][r] - dd[0][r]) * in.dp[3 + c] +
                            (dd[3][r] - dd[0][r]) * in.dp[6 + c];
        Real dFh[9];
        mulAtB(R, dF, dFh);
        Real u[18], delta[6];
        stretch_derivative_u(S6, u);
        ds_dot(u, dFh, delta);
#pragma unroll
        for (int i = 0; i < 6; ++i) ds[i] = d[i] + delta[i];
        Real g[6], H[36];
        material_gH(in, sv, h2, g, H);
#pragma unroll
        for (int i = 0; i < 6; ++i) {
          Real acc = g[i];
#pragma unroll
          for (int j = 0; j < 6; ++j) acc += H[i + 6 * j] * ds[j];
          la[i] = -(i < 3 ? Real(1) : Real(0.5)) * acc;
        }
      }
      store6(sd.ds, sd.ntp, e, ds);
      store6(sd.la, sd.ntp, e, la);
      // E(0) = h^2 vol psi(s) - vol la . Sym (S - s).  psi in Ext: near the
      // rest state a Real psi is a difference of O(1) invariants whose
      // rounding exceeds the energy changes the line search compares.
      const E psiE = material_psi<E>(in.mat, E(in.mu), E(in.lam), sE);
      Real con = 0;
#pragma unroll
      for (int i = 0; i < 6; ++i) con += la[i] * (i < 3 ? Real(1) : Real(2)) * d[i];
      const E e1 = Ext<Real>::c(sd.h2, sd.h2x) * E(in.vol) * psiE;
      const Real e2 = in.vol * con;
      sums[0] = e1 - E(e2);
      // rounding bound of the line-search comparison: e2 is a Real sum, e1
      // and the vertex energies are Ext (relative error far below 1e-7 eps)
      sums[1] = E(Real(fabs(e2))) + E(Real(1e-7) * Real(fabs(Ext<Real>::to_real(e1))));
      Real m = 0;
#pragma unroll
      for (int i = 0; i < 6; ++i) m = fmax(m, Real(fabs(ds[i])));
      maxs[0] = m;
    }
  } else if (idx < t.end) {
    const int a = idx;
    sums[0] = vertex_energy<Real>(sd, a, nullptr, E(0));
    const int f = sd.free_map[a];
    if (f >= 0) {
      Real m = 0;
#pragma unroll
      for (int c = 0; c < 3; ++c) m = fmax(m, Real(fabs(cgx[4 * f + c])));
      maxs[1] = m;
    }
  }
  tile_partials<E, Real, 2, 2>(sums, maxs, partials, pstride, 0, tix);
  if (last_tile(sd, TB_EV, tix)) {
    const int t0 = sd.tile_first[TB_EV], tc = sd.tile_count[TB_EV];
    E v[2];
    scene_sums<E, 2>(partials, pstride, 0, t0, tc, v);
    const Real ms_ = scene_max<Real>(partials, pstride, 2, t0, tc);
    const Real mx_ = scene_max<Real>(partials, pstride, 3, t0, tc);
    if (threadIdx.x == 0) {
      const double Ev = to_double_any(v[0]), ea = to_double_any(v[1]);
      const double ms = double(ms_), mx = double(mx_);
      sc->E_abs = ea;
      sc->E = Ev;
      sc->eres = fabs(Fin<Real>::div(Ev - sc->E_prev, Ev + 1e-6));
      sc->E_prev = Ev;
      sc->fx0 = Ev;
      sc->max_ds = ms;
      sc->max_dx = mx;
      sc->decrement = fmax(mx, ms);
      sc->alpha_ls = 1.0;
      sc->alpha_ls_f = 1.0f;
      sc->ls_iter = 0;
      sc->ls_ok = 0;
      if (sd.max_ls > 0) {
        sc->ls_active = 1;
        sc->nph = kPhLs;
        atomicAdd(&ctrs->ls_active, 1);
      } else {
        sc->ls_active = 0;
        sc->nph = kPhApply;
      }
    }
  }
}

// ------------------------------------------------------------------ K6 ---
// Tile partials: 0 E(alpha), 1 sum |terms|.
template <typename Real, int MB>
__global__ void __launch_bounds__(kElemTile, MB) k_ls_energy(const Tile* tiles, const SceneDev* sds,
                                                         double* partials, int pstride,
                                                         BatchCounters* ctrs) {
  using E = typename Ext<Real>::T;
  const int tix = blockIdx.x;
  const Tile t = tiles[tix];
  const SceneDev& sd = sds[t.scene];
  SceneScalars* sc = sd.sc;
  if (!sc->ls_active) return;
  const E alpha = E(sc->alpha_ls_f);
  const Real h2 = Ext<Real>::r(sd.h2, sd.h2x);
  const Real* cgx = static_cast<const Real*>(sd.cg_x);
  E sums[2] = {E(0), E(0)};
  const int idx = t.begin + threadIdx.x;
  if (t.kind == 0) {
    if (idx < t.end && sd.fem) {
      // standard FEM: h^2 vol psi(F(x + alpha dx))
      ElemIn<Real> in;
      load_elem(sd, idx, in);
      E FE[9];
      Real F[9];
      deformation_gradients<Real>(sd, in, cgx, alpha, FE, F);
      const E e1 = Ext<Real>::c(sd.h2, sd.h2x) * E(in.vol) * fem_psi<E>(in.mat, E(in.mu), E(in.lam), FE);
      sums[0] = e1;
      sums[1] = E(Real(1e-7) * Real(fabs(Ext<Real>::to_real(e1))));
    } else if (idx < t.end) {
      const int e = idx;
      ElemIn<Real> in;
      load_elem(sd, e, in);
      Real F[9], R[9];
      E FE[9];
      // x0 = x + alpha dx  (energy_func, newton_optimizer.cpp:37)
      deformation_gradients<Real>(sd, in, cgx, alpha, FE, F);
      load_quat(sd, e, R);
      procrustes<Real>(R, F, Real(kProcrustesTol), kProcrustesIters);
      E StE[6];
      stretch_ext<Real>(R, FE, StE);
      E sE[6], siE[6];
      Real dsv[6], la[6];
      load6e<Real>(sd, e, sE);
      load6(sd.ds, sd.ntp, e, dsv);
      load6(sd.la, sd.ntp, e, la);
      Real con = 0;
#pragma unroll
      for (int i = 0; i < 6; ++i) {
        siE[i] = sE[i] + alpha * E(dsv[i]);
        // S(x0) - s(alpha) formed in Ext before rounding
        const Real diff = Real(Ext<Real>::to_real(StE[i] - siE[i]));
        con += la[i] * (i < 3 ? Real(1) : Real(2)) * diff;
      }
      // psi in Ext (see K5)
      const E psiE = material_psi<E>(in.mat, E(in.mu), E(in.lam), siE);
      const E e1 = Ext<Real>::c(sd.h2, sd.h2x) * E(in.vol) * psiE;
      const Real e2 = in.vol * con;
      sums[0] = e1 - E(e2);
      // rounding bound of the line-search comparison: e2 is a Real sum, e1
      // and the vertex energies are Ext (relative error far below 1e-7 eps)
      sums[1] = E(Real(fabs(e2))) + E(Real(1e-7) * Real(fabs(Ext<Real>::to_real(e1))));
    }
  } else if (idx < t.end) {
    sums[0] = vertex_energy<Real>(sd, idx, cgx, alpha);
  }
  tile_partials<E, Real, 2, 0>(sums, nullptr, partials, pstride, 0, tix);
  if (last_tile(sd, TB_EV, tix)) {
    const int t0 = sd.tile_first[TB_EV], tc = sd.tile_count[TB_EV];
    E v[2];
    scene_sums<E, 2>(partials, pstride, 0, t0, tc, v);
    if (threadIdx.x == 0) {
      const double fx = to_double_any(v[0]), eab = to_double_any(v[1]);
      sc->E_trial = fx;
      // Armijo with c = 0 (newton_optimizer.cpp:58).  With FP32 element
      // energies a difference below their rounding bound is not a decision
      // the arithmetic can make; such a step is accepted.
      const double noise = sd.fp64 ? 0.0 : 8.0 * 1.1920929e-7 * (eab + sc->E_abs);
      // A trial point whose energy terms overflowed makes the bound
      // infinite; it is rejected, not accepted.
      if (isfinite(fx) && isfinite(noise) && fx < sc->fx0 + noise) {
        sc->ls_active = 0;
        sc->ls_ok = 1;
        sc->nph = kPhApply;
        atomicSub(&ctrs->ls_active, 1);
      } else {
        sc->alpha_ls *= 0.5;
        sc->alpha_ls_f = float(sc->alpha_ls);
        sc->ls_iter += 1;
        if (sc->ls_iter >= sd.max_ls) {
          sc->ls_active = 0;
          sc->ls_ok = 0;
          sc->nph = kPhApply;
          atomicSub(&ctrs->ls_active, 1);
        }
      }
    }
  }
}

// ---------------------------------------------------------------- apply ---
template <typename Real>
__global__ void __launch_bounds__(kElemTile) k_apply(const Tile* tiles, const SceneDev* sds,
                                                     double* partials, int pstride,
                                                     BatchCounters* ctrs) {
  using E = typename Ext<Real>::T;
  const int tix = blockIdx.x;
  const Tile t = tiles[tix];
  const SceneDev& sd = sds[t.scene];
  SceneScalars* sc = sd.sc;
  if (!sc->newton_active || not_my_phase(sc, kPhApply)) return;
  const int idx = t.begin + threadIdx.x;
  if (sc->ls_ok && idx < t.end) {
    const E alpha = E(sc->alpha_ls_f);
    if (t.kind == 0) {
      const Real* ds = static_cast<const Real*>(sd.ds);
#pragma unroll
      for (int i = 0; i < 6; ++i) {
        const size_t k = (size_t)i * sd.ntp + idx;
        Ext<Real>::st(sd.s, k, Ext<Real>::ld(sd.s, k) + alpha * E(ds[k]));
      }
    } else {
      const int f = sd.free_map[idx];
      if (f >= 0) {
        const Real* cgx = static_cast<const Real*>(sd.cg_x);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const size_t k = 3 * (size_t)idx + c;
          Ext<Real>::st(sd.x, k, Ext<Real>::ld(sd.x, k) + alpha * E(cgx[4 * f + c]));
        }
      }
    }
  }
  if (last_tile(sd, TB_EV, tix)) {
    if (threadIdx.x == 0) {
      sc->ls_total += sc->ls_iter;
      if (!sc->ls_ok && sc->status == 0) sc->status = 6;  // MFEM_ERR_LS_FAILED
      sc->newton_iter += 1;
      // In FP32 the energy-change test measures rounding, not convergence;
      // with a residual tolerance set, the mixed path stops on the residual.
      const bool eres_ok = (!sd.fp64 && sd.res_tol > 0) ? true : sc->eres > 1e-12;
      const bool go = sc->newton_iter < sd.max_newton && sc->decrement > sd.newton_tol && eres_ok;
      if (!go) end_newton_loop(sc, ctrs);
      else sc->nph = kPhNewton;
    }
  }
}

// ------------------------------------------------------------ BDF steps ---
// x_tilde + h^2 f of vertex a from the BDF ring at `head`, BDF<I>::x_tilde
// (BDF.cpp:6-9) and Displacement::gradient's target (displacement.cpp:63-73).
template <typename Real>
__device__ __forceinline__ void vertex_step_begin(const SceneDev& sd, int a, int head) {
  using E = typename Ext<Real>::T;
  const int I = sd.bdf_order;
  const size_t n3 = 3 * (size_t)sd.nv;
  const E dt = E(sd.dt), h2 = E(sd.h2);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    E wx = E(0), wv = E(0);
    for (int i = 0; i < I; ++i) {
      const size_t slot = (size_t)((head + i) % I) * n3 + 3 * (size_t)a + c;
      const E al = E(sd.bdf_alpha[i]);
      wx = wx + al * Ext<Real>::ld(sd.xhist, slot);
      wv = wv + al * Ext<Real>::ld(sd.vhist, slot);
    }
    Ext<Real>::st(sd.xt, 3 * (size_t)a + c, wx + dt * wv + h2 * E(sd.body[c]));
  }
}

// Vertex a at the end of a step: a pin moves to its post-BC-step position
// (from `pins`), BDF<I>::update (BDF.cpp:11-21) into ring slot nhead.
template <typename Real>
__device__ __forceinline__ void vertex_step_end(const SceneDev& sd, int a, int head, int nhead,
                                                const double* pins) {
  using E = typename Ext<Real>::T;
  const int I = sd.bdf_order;
  const int f = sd.free_map[a];
  const size_t n3 = 3 * (size_t)sd.nv;
  const E dt = E(sd.dt);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const size_t k = 3 * (size_t)a + c;
    const E xv = (f < 0) ? E(pins[3 * (-1 - f) + c]) : Ext<Real>::ld(sd.x, k);
    E wx = E(0);
    for (int i = 0; i < I; ++i)
      wx = wx + E(sd.bdf_alpha[i]) * Ext<Real>::ld(sd.xhist, (size_t)((head + i) % I) * n3 + k);
    const E vnew = (xv - wx) / dt;
    Ext<Real>::st(sd.x, k, xv);
    Ext<Real>::st(sd.xhist, (size_t)nhead * n3 + k, xv);
    Ext<Real>::st(sd.vhist, (size_t)nhead * n3 + k, vnew);
  }
}

template <typename Real>
__global__ void __launch_bounds__(kElemTile) k_step_begin(const Tile* tiles, const SceneDev* sds) {
  const Tile t = tiles[blockIdx.x];
  const SceneDev& sd = sds[t.scene];
  if (t.kind == 0) return;
  const int a = t.begin + threadIdx.x;
  if (a >= t.end) return;
  vertex_step_begin<Real>(sd, a, sd.sc->hist_head);
}

// Pins move to their post-BC-step positions, BDF<I>::update (BDF.cpp:11-21),
// lambda = 0 (MixedStretch::post_solve, mixed_stretch.cpp:306-309).
template <typename Real>
__global__ void __launch_bounds__(kElemTile) k_step_end(const Tile* tiles, const SceneDev* sds) {
  const int tix = blockIdx.x;
  const Tile t = tiles[tix];
  const SceneDev& sd = sds[t.scene];
  SceneScalars* sc = sd.sc;
  const int idx = t.begin + threadIdx.x;
  const int I = sd.bdf_order, head = sc->hist_head;
  const int nhead = (head + I - 1) % I;
  if (idx < t.end) {
    if (t.kind == 0) {
      Real* la = static_cast<Real*>(sd.la);
#pragma unroll
      for (int i = 0; i < 6; ++i) la[(size_t)i * sd.ntp + idx] = Real(0);
    } else {
      vertex_step_end<Real>(sd, idx, head, nhead, sd.pin_pos);
    }
  }
  if (last_tile(sd, TB_EV, tix)) {
    if (threadIdx.x == 0) sc->hist_head = nhead;
  }
}

// A step's status as the host reports it: non-finite first, then a failed
// rotation solve, then the step's own status, then the PCG's.
__device__ __forceinline__ int step_status(const SceneScalars* sc) {
  if (sc->status == 4) return 4;
  if (sc->procrustes_fail) return 7;
  if (sc->status) return sc->status;
  return sc->cg_status;
}
__device__ __forceinline__ int status_rank(int st) { return st == 4 ? 3 : st == 7 ? 2 : st ? 1 : 0; }

// Several timesteps per call (mfem_gpu_batch_step_n): a scene whose Newton
// loop has ended turns over here.  Its step ends as k_step_end
// ends it (the pins from the step's slot of the precomputed trajectory);
// unless that was its last step, the next one begins as k_step_begin begins
// it, its per-step state is reset and it joins the next round's launches
// while other scenes are still in their Newton loops.  The per-vertex work
// is the same device code as the two kernels'.  A step that ends
// non-finite or with a singular rotation solve retires the scene.
template <typename Real>
__global__ void __launch_bounds__(kElemTile) k_step_turn(const Tile* tiles, const SceneDev* sds,
                                                         BatchCounters* ctrs) {
  const int tix = blockIdx.x;
  const Tile t = tiles[tix];
  const SceneDev& sd = sds[t.scene];
  SceneScalars* sc = sd.sc;
  if (!sc->turn) return;
  const int idx = t.begin + threadIdx.x;
  const int I = sd.bdf_order, head = sc->hist_head;
  const int nhead = (head + I - 1) % I;
  const int done = sc->steps_done;
  // a step that ended non-finite or with a singular rotation solve retires
  // the scene: its state cannot give a meaningful next step
  const bool failed = status_rank(step_status(sc)) >= 2;
  const bool last = failed || done + 1 >= sc->steps_target;
  if (idx < t.end) {
    if (t.kind == 0) {
      Real* la = static_cast<Real*>(sd.la);
#pragma unroll
      for (int i = 0; i < 6; ++i) la[(size_t)i * sd.ntp + idx] = Real(0);
    } else {
      const double* pins = sd.pin_traj ? sd.pin_traj + 3 * (size_t)sd.npin * done : sd.pin_pos;
      vertex_step_end<Real>(sd, idx, head, nhead, pins);
      if (!last) vertex_step_begin<Real>(sd, idx, nhead);
    }
  }
  if (last_tile(sd, TB_EV, tix)) {
    if (threadIdx.x == 0) {
      sc->hist_head = nhead;
      const int st = step_status(sc);
      if (status_rank(st) > status_rank(sc->acc_status)) sc->acc_status = st;
      sc->acc_newton += sc->newton_iter;
      sc->acc_cg += sc->cg_total;
      sc->acc_ls += sc->ls_total;
      if (sd.step_ns) {
        unsigned long long t;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
        sd.step_ns[done] = t;
      }
      sc->steps_done = done + 1;
      sc->turn = 0;
      if (last) {
        atomicSub(&ctrs->newton_active, 1);  // the scene's last step: its stats stay
      } else {
        reset_step_scalars(sc);  // newton_active = 1: in the next round
      }
    }
  }
}

template <typename K>
void set_smem(K kernel, int bytes) {
  cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

}  // namespace

int elem_update_smem_bytes(int fp64) { return kElemTile * (rec_bytes(fp64 ? 8 : 4) / 4 + 1) * 4; }

void configure_kernels() {
  set_smem(k_elem_update<float, false>, elem_update_smem_bytes(0));
  set_smem(k_elem_update<float, false, 2>, elem_update_smem_bytes(0));
  set_smem(k_elem_update<float, true>, elem_update_smem_bytes(0));
  set_smem(k_elem_update<double, false>, elem_update_smem_bytes(1));
  set_smem(k_elem_update<double, true>, elem_update_smem_bytes(1));
  set_smem(k_elem_fem<float, false>, elem_update_smem_bytes(0));
  set_smem(k_elem_fem<float, true>, elem_update_smem_bytes(0));
  set_smem(k_elem_fem<double, false>, elem_update_smem_bytes(1));
  set_smem(k_elem_fem<double, true>, elem_update_smem_bytes(1));
}

void launch_elem_init(const Launch& L) {
  if (L.ntiles == 0) return;
  if (L.fp64)
    k_elem_init<double><<<L.ntiles, kElemTile, 0, L.stream>>>(L.tiles, L.sds);
  else
    k_elem_init<float><<<L.ntiles, kElemTile, 0, L.stream>>>(L.tiles, L.sds);
}

void launch_elem_update(const Launch& L, const ElemDebug* dbg) {
  if (L.ntiles == 0) return;
  ElemDebug d{};
  if (dbg) d = *dbg;
  const int sm = elem_update_smem_bytes(L.fp64);
  if (L.fem) {
    if (L.fp64) {
      if (dbg) k_elem_fem<double, true><<<L.ntiles, kElemTile, sm, L.stream>>>(L.tiles, L.sds, d);
      else k_elem_fem<double, false><<<L.ntiles, kElemTile, sm, L.stream>>>(L.tiles, L.sds, d);
    } else {
      if (dbg) k_elem_fem<float, true><<<L.ntiles, kElemTile, sm, L.stream>>>(L.tiles, L.sds, d);
      else k_elem_fem<float, false><<<L.ntiles, kElemTile, sm, L.stream>>>(L.tiles, L.sds, d);
    }
    return;
  }
  if (L.fp64) {
    if (dbg)
      k_elem_update<double, true><<<L.ntiles, kElemTile, sm, L.stream>>>(L.tiles, L.sds, d);
    else
      k_elem_update<double, false><<<L.ntiles, kElemTile, sm, L.stream>>>(L.tiles, L.sds, d);
  } else {
    if (dbg)
      k_elem_update<float, true><<<L.ntiles, kElemTile, sm, L.stream>>>(L.tiles, L.sds, d);
    else if (L.variant == 1)
      k_elem_update<float, false, 2><<<L.ntiles, kElemTile, sm, L.stream>>>(L.tiles, L.sds, d);
    else
      k_elem_update<float, false><<<L.ntiles, kElemTile, sm, L.stream>>>(L.tiles, L.sds, d);
  }
}

// The variants the autotuner may pick (Launch::variant; 0 is the default).
// Only register budgets whose builds were measured to give the default's
// bits are offered.
int elem_update_variants(int fp64, int fem) { return (fp64 || fem) ? 1 : 2; }
int local_solve_variants(int) { return 3; }
int ls_energy_variants(int) { return 2; }
const char* elem_update_variant_name(int v) {
  return v == 1 ? "2 blocks/SM (255 registers)" : "default (168 registers in FP32)";
}
const char* local_solve_variant_name(int v) {
  return v == 1 ? "4 blocks/SM (128 registers)" : v == 2 ? "5 blocks/SM (102 registers)" : "default";
}
const char* ls_energy_variant_name(int v) { return v == 1 ? "8 blocks/SM (64 registers)" : "default"; }

#define MFEM_LAUNCH_EV(kern, ...)                                                     \
  do {                                                                                \
    if (L.ntiles == 0) return;                                                        \
    if (L.fp64)                                                                       \
      kern<double><<<L.ntiles, kElemTile, 0, L.stream>>>(__VA_ARGS__);                \
    else                                                                              \
      kern<float><<<L.ntiles, kElemTile, 0, L.stream>>>(__VA_ARGS__);                 \
  } while (0)

// Launch of a register-budget variant: v1, v2 are the blocks per SM of
// variants 1 and 2 (0: no such variant), variant 0 the compiler's choice.
#define MFEM_LAUNCH_EV_MB(kern, v1, v2)                                                   \
  do {                                                                                  \
    if (L.ntiles == 0) return;                                                          \
    const auto go = [&](auto k) {                                                       \
      k<<<L.ntiles, kElemTile, 0, L.stream>>>(L.tiles, L.sds, L.partials, L.pstride, L.counters); \
    };                                                                                  \
    if (L.fp64) {                                                                       \
      if (L.variant == 1) go(kern<double, v1>);                                         \
      else if (L.variant == 2) go(kern<double, v2>);                                    \
      else go(kern<double, 0>);                                                         \
    } else {                                                                            \
      if (L.variant == 1) go(kern<float, v1>);                                          \
      else if (L.variant == 2) go(kern<float, v2>);                                     \
      else go(kern<float, 0>);                                                          \
    }                                                                                   \
  } while (0)

void launch_local_solve(const Launch& L) { MFEM_LAUNCH_EV_MB(k_local_solve, 4, 5); }
void launch_ls_energy(const Launch& L) { MFEM_LAUNCH_EV_MB(k_ls_energy, 8, 0); }
void launch_apply(const Launch& L) {
  MFEM_LAUNCH_EV(k_apply, L.tiles, L.sds, L.partials, L.pstride, L.counters);
}
void launch_step_begin(const Launch& L) { MFEM_LAUNCH_EV(k_step_begin, L.tiles, L.sds); }
void launch_step_end(const Launch& L) { MFEM_LAUNCH_EV(k_step_end, L.tiles, L.sds); }
void launch_step_turn(const Launch& L) { MFEM_LAUNCH_EV(k_step_turn, L.tiles, L.sds, L.counters); }

}  // namespace mfem_gpu
