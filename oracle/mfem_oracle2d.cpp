/*
 * TEST INFRASTRUCTURE ONLY — the FP64 CPU oracle of the 2-D (triangle mesh)
 * mixed-FEM Newton timestep of tytrusty/mfem.  The same rules of use as
 * mfem_oracle.cpp: only tests/, __graft_entry__.smoke() and bench.py's CPU
 * legs may load it, to check the GPU path or as the timed CPU baseline.
 *
 * It restates the DIM = 2 instantiation of the reference:
 *   Tri2DMesh            src/mesh/tri2d_mesh.cpp:11-83 (Jloc 4x6, doublearea
 *                        volumes, dphi/dX, mass)
 *   Mesh::init           src/mesh/mesh.cpp:44-75 (W, PJW, PM, PMP)
 *   polar_svd<2>         src/variables/mixed_stretch.cpp:43-78
 *   svd<double,2>        src/svd/svd_eigen.h:7-32 (sign fix: U, V rotations)
 *   dsvd, 2-D            src/svd/dsvd.cpp:140-189 (1/(s1^2 - s0^2) zeroed
 *                        below 1e-4)
 *   materials            the Vector3d sections of stable_neohookean.cpp:236-277,
 *                        arap.cpp:67-99, corotational.cpp:62-97,
 *                        fixed_corotational.cpp:93-130
 *   MixedStretch<2>, Displacement<2>, BDF<2>, NewtonOptimizer<2> and
 *   linesearch_backtracking as the 3-D oracle restates them (N = 3, M = 4,
 *   Sym = diag(1, 1, 2)).
 *
 * Parity status: the reference holds no 2-D test or output, so step-level
 * parity is "parity unpinned"; the polar derivative and every material
 * derivative are pinned by finite differences in tests/.  Two Bartels
 * functions have no source here: linear_tri2dmesh_dphi_dX, restated as the
 * rows of Dm^-1 (the construction of the tetrahedral dphi/dX), and
 * linear_tri2dmesh_mass_matrix, restated as the P1 consistent mass
 * rho*vol/12*(1+delta_ab) on the volumes it is handed (igl::doublearea, as
 * Tri2DMesh::mass_matrix passes them), which scales the mass exactly as the
 * elastic terms are scaled by the same doubled areas.  JacobiSVD's 2x2
 * factorisation is restated in closed form (the sign-fixed factors are
 * unique up to a joint half-turn of U and V, which changes neither R nor
 * dR/dF).
 */
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <deque>
#include <limits>
#include <memory>
#include <vector>

#include "mfem_oracle.h"

namespace {

using M2 = std::array<double, 4>;  // column-major: [m00, m10, m01, m11]
inline double& at(M2& m, int r, int c) { return m[r + 2 * c]; }
inline double at(const M2& m, int r, int c) { return m[r + 2 * c]; }

M2 mul(const M2& a, const M2& b) {
  M2 c{};
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) at(c, i, j) = at(a, i, 0) * at(b, 0, j) + at(a, i, 1) * at(b, 1, j);
  return c;
}
M2 transpose(const M2& a) { return {a[0], a[2], a[1], a[3]}; }
M2 rot(double th) { return {std::cos(th), std::sin(th), -std::sin(th), std::cos(th)}; }

const double kPsdTol = 1e-6;             // sim::simple_psd_fix default (as in the 3-D oracle)
const double kDsvdTol = 1e-4;            // dsvd.cpp:153
const double kSym[3] = {1, 1, 2};
const double kSymInv[3] = {1, 1, 0.5};

// svd<double,2> with the sign fix (svd_eigen.h:7-32): F = U diag(sig) V^T with
// U, V rotations and sig[0] >= |sig[1]| (sig[1] < 0 when det F < 0).
// Writing F = [[e+f, g-h], [g+h, e-f]]: sig = q +- r with q = |(e, h)|,
// r = |(f, g)|, U = rot((a2 + a1)/2), V = rot((a1 - a2)/2), a1 = atan2(g, f),
// a2 = atan2(h, e) (the closed-form 2x2 SVD).
void svd2(const M2& F, double sig[2], M2& U, M2& V) {
  const double e = 0.5 * (at(F, 0, 0) + at(F, 1, 1)), f = 0.5 * (at(F, 0, 0) - at(F, 1, 1));
  const double g = 0.5 * (at(F, 1, 0) + at(F, 0, 1)), h = 0.5 * (at(F, 1, 0) - at(F, 0, 1));
  const double q = std::sqrt(e * e + h * h), r = std::sqrt(f * f + g * g);
  sig[0] = q + r;
  sig[1] = q - r;
  const double a1 = std::atan2(g, f), a2 = std::atan2(h, e);
  U = rot(0.5 * (a2 + a1));
  V = rot(0.5 * (a1 - a2));
}

// dsvd for 2x2 (dsvd.cpp:140-189) folded into polar_svd<2>'s
// dR_dF[2c + r] = dU[r][c] V^T + U dV[r][c]^T (mixed_stretch.cpp:53-58);
// dRdF column 2c+r is vec(dR/dF_rc), column-major.
void dRdF2(const M2& U, const double sig[2], const M2& V, double dRdF[16]) {
  double d01 = sig[1] * sig[1] - sig[0] * sig[0];
  d01 = std::fabs(d01) < kDsvdTol ? 0.0 : 1.0 / d01;
  for (int r = 0; r < 2; ++r)
    for (int c = 0; c < 2; ++c) {
      M2 P;  // U.row(r)^T * V.row(c)
      for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j) at(P, i, j) = at(U, r, i) * at(V, c, j);
      at(P, 0, 0) = 0;
      at(P, 1, 1) = 0;
      const double wv = (sig[0] * at(P, 0, 1) + at(P, 1, 0) * sig[1]) * d01;
      const double wu = (at(P, 0, 1) * sig[1] + sig[0] * at(P, 1, 0)) * d01;
      const M2 Wv{0, -wv, wv, 0}, Wu{0, -wu, wu, 0};
      const M2 dV = mul(V, Wv), dU = mul(U, Wu);
      const M2 a = mul(dU, transpose(V)), b = mul(U, transpose(dV));
      for (int k = 0; k < 4; ++k) dRdF[k + 4 * (2 * c + r)] = a[k] + b[k];
    }
}

// polar_svd<2,3> (mixed_stretch.cpp:43-78): R = U V^T, S = R^T F,
// s = [S00, S11, (S10 + S01)/2] and ds/dF (3x4, column-major) from
// J = (I (x) R^T)(I - (S^T (x) I) dRdF).
int polar2(M2& R, const M2& F, bool grads, double s[3], double* dsdF) {
  double sig[2];
  M2 U, V;
  svd2(F, sig, U, V);
  R = mul(U, transpose(V));
  const M2 S = mul(transpose(R), F);
  s[0] = at(S, 0, 0);
  s[1] = at(S, 1, 1);
  s[2] = 0.5 * (at(S, 1, 0) + at(S, 0, 1));
  if (!(sig[0] + sig[1] > 0)) return MFEM_ERR_PROCRUSTES;  // F has no unique nearest rotation
  if (!grads) return MFEM_OK;
  double dRdF[16], T1[16], J[16];
  dRdF2(U, sig, V, dRdF);
  for (int col = 0; col < 4; ++col)
    for (int rr = 0; rr < 4; ++rr) {
      const int r = rr % 2, cc = rr / 2;
      double v = 0;
      for (int k = 0; k < 2; ++k) v += at(S, k, cc) * dRdF[(r + 2 * k) + 4 * col];
      T1[rr + 4 * col] = (rr == col ? 1.0 : 0.0) - v;
    }
  for (int col = 0; col < 4; ++col)
    for (int rr = 0; rr < 4; ++rr) {
      const int r = rr % 2, cc = rr / 2;
      double v = 0;
      for (int k = 0; k < 2; ++k) v += at(R, k, r) * T1[(k + 2 * cc) + 4 * col];
      J[rr + 4 * col] = v;
    }
  for (int col = 0; col < 4; ++col) {
    dsdF[0 + 3 * col] = J[0 + 4 * col];
    dsdF[1 + 3 * col] = J[3 + 4 * col];
    dsdF[2 + 3 * col] = 0.5 * (J[1 + 4 * col] + J[2 + 4 * col]);
  }
  return MFEM_OK;
}

// ---------------------------------------------------------------------------
// The 3-vector materials, each as psi = A(Q) + B(J) + C(t) with
// Q = s0^2 + s1^2 + 2 s2^2 = |S|_F^2, J = s0 s1 - s2^2 = det S, t = s0 + s1:
//   SNH   mu (1 - J) + la/2 (1 - J)^2 + mu/2 (Q - 2)     (psd-fixed Hessian)
//   Corot la/2 (t - 2)^2 + mu (Q - 2t + 2)
//   FCR   la/2 (J - 1)^2 + mu (Q - 2t + 2)
//   ARAP  mu/2 (Q - 2t + 2)
// which is the generated code of the reference expanded.
struct Coef {
  double psi, A1, B1, B2, C1, C2;
  bool psd;
  bool ok;
};

Coef coef2(int type, double mu, double la, const double* s) {
  const double Q = s[0] * s[0] + s[1] * s[1] + 2 * s[2] * s[2];
  const double J = s[0] * s[1] - s[2] * s[2];
  const double t = s[0] + s[1];
  Coef c{0, 0, 0, 0, 0, 0, false, true};
  switch (type) {
    case MFEM_MATERIAL_SNH:
      c.psi = mu * (1 - J) + 0.5 * la * (1 - J) * (1 - J) + 0.5 * mu * (Q - 2);
      c.A1 = 0.5 * mu;
      c.B1 = -mu - la * (1 - J);
      c.B2 = la;
      c.psd = true;
      break;
    case MFEM_MATERIAL_COROT:
      c.psi = 0.5 * la * (t - 2) * (t - 2) + mu * (Q - 2 * t + 2);
      c.A1 = mu;
      c.C1 = la * (t - 2) - 2 * mu;
      c.C2 = la;
      break;
    case MFEM_MATERIAL_FCR:
      c.psi = 0.5 * la * (J - 1) * (J - 1) + mu * (Q - 2 * t + 2);
      c.A1 = mu;
      c.B1 = la * (J - 1);
      c.B2 = la;
      c.C1 = -2 * mu;
      break;
    case MFEM_MATERIAL_ARAP:
      c.psi = 0.5 * mu * (Q - 2 * t + 2);
      c.A1 = 0.5 * mu;
      c.C1 = -mu;
      break;
    default:
      c.ok = false;
  }
  return c;
}

void material2(int type, double mu, double la, const double* s, double* psi, double* g,
               double* H, bool fix) {
  const Coef c = coef2(type, mu, la, s);
  if (psi) *psi = c.psi;
  const double dJ[3] = {s[1], s[0], -2 * s[2]};
  if (g)
    for (int i = 0; i < 3; ++i) g[i] = 2 * c.A1 * kSym[i] * s[i] + c.B1 * dJ[i] + (i < 2 ? c.C1 : 0.0);
  if (!H) return;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double v = c.B2 * dJ[i] * dJ[j];
      if (i == j) v += 2 * c.A1 * kSym[i];
      if (i < 2 && j < 2) v += c.C2;
      H[i + 3 * j] = v;
    }
  H[0 + 3 * 1] += c.B1;  // d2J/ds0 ds1 = 1
  H[1 + 3 * 0] += c.B1;
  H[2 + 3 * 2] += -2 * c.B1;  // d2J/ds2^2 = -2
  if (fix && c.psd) oracle_psd_fix(H, 3, kPsdTol);
}

bool inverse3(const double* A, double* Ai) {
  const double c00 = A[4] * A[8] - A[7] * A[5], c01 = A[7] * A[2] - A[1] * A[8],
               c02 = A[1] * A[5] - A[4] * A[2];
  const double det = A[0] * c00 + A[3] * c01 + A[6] * c02;
  if (!(det != 0) || !std::isfinite(det)) return false;
  const double id = 1.0 / det;
  Ai[0] = c00 * id;
  Ai[1] = c01 * id;
  Ai[2] = c02 * id;
  Ai[3] = (A[6] * A[5] - A[3] * A[8]) * id;
  Ai[4] = (A[0] * A[8] - A[6] * A[2]) * id;
  Ai[5] = (A[3] * A[2] - A[0] * A[5]) * id;
  Ai[6] = (A[3] * A[7] - A[6] * A[4]) * id;
  Ai[7] = (A[6] * A[1] - A[0] * A[7]) * id;
  Ai[8] = (A[0] * A[4] - A[3] * A[1]) * id;
  return true;
}

// ---------------------------------------------------------------------------
struct Scene2 {
  int nv = 0, nt = 0, nfree = 0;
  std::vector<double> Vref, V;  // 2 per vertex
  std::vector<int> T, mat, is_fixed, free_map;
  std::vector<double> mu, la, rho, vol, dX;  // dX[6e + 2k + c] = dphi_k/dX_c
  int bc_type = 0, bc_axis = 0;
  double bc_ratio = 0.1, bc_vel = 0.1;
  std::vector<std::vector<int>> groups;
  std::vector<std::array<double, 2>> group_center;
  std::array<double, 2> twist_center{};
  std::vector<int> m_ptr, m_col;
  std::vector<double> m_val;
  std::vector<int> b_ptr, b_col;
  std::vector<double> b_mass;
  std::vector<int> pair_elem, pair_local, pair_blk;
  std::vector<double> A, rhs;
  double h = 0.034, ext[2] = {0, -9.8};
  int bdf = 1, max_newton = 5, ls_iters = 20, cg_iters = 500;
  double cg_tol = 1e-4, newton_tol = 1e-10, res_tol = 0, load_norm = 0;
  std::vector<double> x, dx, b, fext;
  std::deque<std::vector<double>> xprev, vprev;
  std::vector<double> s, ds, lam, Rm, Sv, dSdF, g, Hm, Hinv, Htil, gl, Aloc;

  double dt() const {
    static const double beta[7] = {0, 1.0, 2.0 / 3, 6.0 / 11, 12.0 / 25, 60.0 / 137, 60.0 / 147};
    return beta[bdf] * h;
  }
  const double* alphas() const {  // BDF.cpp:50-93
    static const double a[7][6] = {
        {0},
        {1.0},
        {4.0 / 3, -1.0 / 3},
        {18.0 / 11, -9.0 / 11, 2.0 / 11},
        {48.0 / 25, -36.0 / 25, 16.0 / 25, -3.0 / 25},
        {300.0 / 137, -300.0 / 137, 200.0 / 137, -75.0 / 137, 12.0 / 137},
        {360.0 / 147, -450.0 / 147, 400.0 / 147, -225.0 / 147, 72.0 / 147, -10.0 / 147}};
    return a[bdf];
  }
  std::vector<double> weighted(const std::deque<std::vector<double>>& q) const {
    std::vector<double> w(2 * nv, 0.0);
    const double* a = alphas();
    for (size_t i = 0; i < q.size(); ++i)
      for (int k = 0; k < 2 * nv; ++k) w[k] += a[i] * q[i][k];
    return w;
  }
  std::vector<double> xtilde() const {
    std::vector<double> wx = weighted(xprev), wv = weighted(vprev);
    const double d = dt();
    for (int k = 0; k < 2 * nv; ++k) wx[k] += d * wv[k];
    return wx;
  }
  void unproject(const std::vector<double>& xf, std::vector<double>& full) const {
    full = b;
    for (int v = 0; v < nv; ++v)
      if (free_map[v] >= 0)
        for (int d = 0; d < 2; ++d) full[2 * v + d] += xf[2 * free_map[v] + d];
  }
  M2 defgrad(const std::vector<double>& full, int e) const {
    M2 F{};
    for (int k = 0; k < 3; ++k) {
      const double* xk = &full[2 * T[3 * e + k]];
      for (int r = 0; r < 2; ++r)
        for (int c = 0; c < 2; ++c) at(F, r, c) += xk[r] * dX[6 * e + 2 * k + c];
    }
    return F;
  }
};

void bbox(const Scene2& sc, const std::vector<double>& V, double lo[2], double hi[2]) {
  for (int d = 0; d < 2; ++d) {
    lo[d] = std::numeric_limits<double>::infinity();
    hi[d] = -lo[d];
  }
  for (int v = 0; v < sc.nv; ++v)
    for (int d = 0; d < 2; ++d) {
      lo[d] = std::min(lo[d], V[2 * v + d]);
      hi[d] = std::max(hi[d], V[2 * v + d]);
    }
}

// BoundaryCondition::init_boundary_groups (boundary_condition.cpp:5-21) and
// each script's init (fixed_boundary_conditions.h, stretch/twist/bend_*.h).
void bc_init(Scene2& sc, const int32_t* override_fixed) {
  double lo[2], hi[2];
  bbox(sc, sc.Vref, lo, hi);
  const int ax = sc.bc_axis;
  const double range = hi[ax] - lo[ax];
  sc.groups.assign(2, {});
  for (int v = 0; v < sc.nv; ++v) {
    const double c = sc.Vref[2 * v + ax];
    if (c < lo[ax] + range * sc.bc_ratio)
      sc.groups[0].push_back(v);
    else if (c > hi[ax] - range * sc.bc_ratio)
      sc.groups[1].push_back(v);
  }
  sc.is_fixed.assign(sc.nv, 0);
  bbox(sc, sc.V, lo, hi);
  double ctr[2] = {0.5 * (lo[0] + hi[0]), 0.5 * (lo[1] + hi[1])};
  switch (sc.bc_type) {
    case MFEM_BC_SCALEF:
      for (int v = 0; v < sc.nv; ++v)
        for (int d = 0; d < 2; ++d) sc.V[2 * v + d] = (sc.V[2 * v + d] - ctr[d]) * 1.5 + ctr[d];
      break;
    case MFEM_BC_RANDOM: {  // RandomizeBC::init with a seeded generator
      uint64_t st = 0x9E3779B97F4A7C15ull;
      for (auto& x : sc.V) {
        st = st * 6364136223846793005ull + 1442695040888963407ull;
        x = (double((st >> 11) & ((1ull << 53) - 1)) / double(1ull << 53) * 2 - 1) / 2.0;
      }
      ctr[1] += (hi[1] - lo[1]) * 0.5;
      const double r0[2] = {sc.V[0], sc.V[1]};
      for (int v = 0; v < sc.nv; ++v)
        for (int d = 0; d < 2; ++d) sc.V[2 * v + d] += ctr[d] - r0[d];
      break;
    }
    case MFEM_BC_ONEPOINT:
      sc.is_fixed[0] = 1;
      break;
    case MFEM_BC_HANG:
      for (auto& gr : sc.groups)
        if (!gr.empty()) sc.is_fixed[gr.back()] = 1;
      break;
    case MFEM_BC_HANGENDS:
      for (int v : sc.groups[1]) sc.is_fixed[v] = 1;
      break;
    case MFEM_BC_PINMIN:
      for (int v : sc.groups[0]) sc.is_fixed[v] = 1;
      break;
    case MFEM_BC_STRETCH:
    case MFEM_BC_COMPRESS:
    case MFEM_BC_TWIST:
    case MFEM_BC_BEND:
      for (auto& gr : sc.groups)
        for (int v : gr) sc.is_fixed[v] = 1;
      sc.twist_center = {ctr[0], ctr[1]};
      sc.group_center.clear();
      for (auto& gr : sc.groups) {
        const int v = gr.empty() ? 0 : gr.back();
        sc.group_center.push_back({sc.V[2 * v], sc.V[2 * v + 1]});
      }
      break;
    default:
      break;
  }
  if (override_fixed)
    for (int v = 0; v < sc.nv; ++v) sc.is_fixed[v] = override_fixed[v] ? 1 : 0;
}

void rotate2(double* p, const double* o, double ang) {
  const double q0 = p[0] - o[0], q1 = p[1] - o[1];
  const double c = std::cos(ang), s = std::sin(ang);
  p[0] = c * q0 - s * q1 + o[0];
  p[1] = s * q0 + c * q1 + o[1];
}

void bc_step(Scene2& sc, double dt) {
  switch (sc.bc_type) {
    case MFEM_BC_STRETCH:
      for (int i = 0; i < 2; ++i)
        for (int v : sc.groups[i]) sc.V[2 * v + sc.bc_axis] += (i == 0 ? 1 : -1) * sc.bc_vel * dt;
      break;
    case MFEM_BC_COMPRESS:
      for (int v : sc.groups[1]) sc.V[2 * v + sc.bc_axis] += sc.bc_vel * dt;
      break;
    case MFEM_BC_TWIST:
      for (int i = 0; i < 2; ++i) {
        const double a = (i == 0 ? 1 : -1) * sc.bc_vel * M_PI * dt;
        for (int v : sc.groups[i]) rotate2(&sc.V[2 * v], sc.twist_center.data(), a);
      }
      break;
    case MFEM_BC_BEND:
      for (int i = 0; i < 2; ++i) {
        const double a = (i == 0 ? 1 : -1) * sc.bc_vel * M_PI * dt;
        for (int v : sc.groups[i]) rotate2(&sc.V[2 * v], sc.group_center[i].data(), a);
      }
      break;
    default:
      break;
  }
}

void build_mass(Scene2& sc) {
  std::vector<std::vector<std::pair<int, double>>> rows(sc.nv);
  for (int e = 0; e < sc.nt; ++e) {
    const double m = sc.rho[e] * sc.vol[e] / 12.0;
    for (int a = 0; a < 3; ++a)
      for (int bq = 0; bq < 3; ++bq)
        rows[sc.T[3 * e + a]].push_back({sc.T[3 * e + bq], a == bq ? 2 * m : m});
  }
  sc.m_ptr.assign(sc.nv + 1, 0);
  sc.m_col.clear();
  sc.m_val.clear();
  for (int v = 0; v < sc.nv; ++v) {
    auto& r = rows[v];
    std::sort(r.begin(), r.end(), [](auto& u, auto& w) { return u.first < w.first; });
    for (size_t i = 0; i < r.size(); ++i) {
      if (i > 0 && r[i].first == r[i - 1].first) {
        sc.m_val.back() += r[i].second;
      } else {
        sc.m_col.push_back(r[i].first);
        sc.m_val.push_back(r[i].second);
      }
    }
    sc.m_ptr[v + 1] = int(sc.m_col.size());
  }
}

// Assembler<double,2,-1> (sparse_utils.cpp:19-138) on free vertex pairs.
void build_assembler(Scene2& sc) {
  struct P { int r, c, e, l; };
  std::vector<P> pairs;
  pairs.reserve(9 * size_t(sc.nt));
  for (int e = 0; e < sc.nt; ++e)
    for (int j = 0; j < 3; ++j) {
      const int a = sc.free_map[sc.T[3 * e + j]];
      if (a < 0) continue;
      for (int k = 0; k < 3; ++k) {
        const int bq = sc.free_map[sc.T[3 * e + k]];
        if (bq < 0) continue;
        pairs.push_back({a, bq, e, 3 * j + k});
      }
    }
  std::stable_sort(pairs.begin(), pairs.end(), [](const P& u, const P& w) {
    return u.r < w.r || (u.r == w.r && u.c < w.c);
  });
  sc.b_ptr.assign(sc.nfree + 1, 0);
  sc.b_col.clear();
  sc.pair_elem.resize(pairs.size());
  sc.pair_local.resize(pairs.size());
  sc.pair_blk.resize(pairs.size());
  for (size_t i = 0; i < pairs.size(); ++i) {
    if (i == 0 || pairs[i].r != pairs[i - 1].r || pairs[i].c != pairs[i - 1].c) {
      sc.b_col.push_back(pairs[i].c);
      sc.b_ptr[pairs[i].r + 1]++;
    }
    sc.pair_elem[i] = pairs[i].e;
    sc.pair_local[i] = pairs[i].l;
    sc.pair_blk[i] = int(sc.b_col.size()) - 1;
  }
  for (int r = 0; r < sc.nfree; ++r) sc.b_ptr[r + 1] += sc.b_ptr[r];
  sc.A.assign(4 * sc.b_col.size(), 0.0);
  sc.b_mass.assign(sc.b_col.size(), 0.0);
  for (int a = 0; a < sc.nv; ++a) {
    const int fa = sc.free_map[a];
    if (fa < 0) continue;
    for (int q = sc.m_ptr[a]; q < sc.m_ptr[a + 1]; ++q) {
      const int fb = sc.free_map[sc.m_col[q]];
      if (fb < 0) continue;
      const int* beg = &sc.b_col[sc.b_ptr[fa]];
      const int* end = &sc.b_col[0] + sc.b_ptr[fa + 1];
      const int* it = std::lower_bound(beg, end, fb);
      sc.b_mass[it - &sc.b_col[0]] += sc.m_val[q];
    }
  }
}

void mass_mul(const Scene2& sc, const std::vector<double>& xin, std::vector<double>& y) {
  y.assign(2 * sc.nv, 0.0);
#pragma omp parallel for schedule(static)
  for (int a = 0; a < sc.nv; ++a) {
    double acc[2] = {0, 0};
    for (int q = sc.m_ptr[a]; q < sc.m_ptr[a + 1]; ++q)
      for (int d = 0; d < 2; ++d) acc[d] += sc.m_val[q] * xin[2 * sc.m_col[q] + d];
    y[2 * a] = acc[0];
    y[2 * a + 1] = acc[1];
  }
}

// Sums f(i) over [0, n) in fixed chunks whose partials are added in order,
// so the result does not depend on the thread count or schedule.
template <typename Fn>
double det_sum(long n, Fn f) {
  const long chunk = 2048;
  const long nc = (n + chunk - 1) / chunk;
  std::vector<double> part(nc, 0.0);
#pragma omp parallel for schedule(static)
  for (long c = 0; c < nc; ++c) {
    double s = 0;
    const long e = std::min(n, (c + 1) * chunk);
    for (long i = c * chunk; i < e; ++i) s += f(i);
    part[c] = s;
  }
  double s = 0;
  for (double p : part) s += p;
  return s;
}

double dot(const std::vector<double>& a, const std::vector<double>& b) {
  return det_sum((long)a.size(), [&](long i) { return a[i] * b[i]; });
}

// MixedStretch<2>::update_rotations + update_derivatives + rhs for one
// triangle (mixed_stretch.cpp:133-226 with N = 3, M = 4).
int elem_update(Scene2& sc, int e, const std::vector<double>& full, double dt) {
  const double h2 = dt * dt;
  const M2 F = sc.defgrad(full, e);
  M2 R;
  double sv[3], dsdF[12];
  int st = polar2(R, F, true, sv, dsdF);
  std::memcpy(&sc.Rm[4 * e], R.data(), sizeof(double) * 4);
  std::memcpy(&sc.Sv[3 * e], sv, sizeof(sv));
  double* dSdF = &sc.dSdF[12 * e];  // 4x3: dSdF(r,i) = dsdF(i,r) Sym(i)
  for (int i = 0; i < 3; ++i)
    for (int r = 0; r < 4; ++r) dSdF[r + 4 * i] = dsdF[i + 3 * r] * kSym[i];
  const double* si = &sc.s[3 * e];
  const double vol = sc.vol[e];
  double* H = &sc.Hm[9 * e];
  double* g = &sc.g[3 * e];
  material2(sc.mat[e], sc.mu[e], sc.la[e], si, nullptr, g, H, true);
  for (int i = 0; i < 9; ++i) H[i] *= h2;
  for (int i = 0; i < 3; ++i) g[i] *= h2;
  if (!inverse3(H, &sc.Hinv[9 * e])) st = MFEM_ERR_NONFINITE;
  double* Ht = &sc.Htil[9 * e];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) Ht[i + 3 * j] = (1.0 / vol) * kSymInv[i] * H[i + 3 * j] * kSymInv[j];
  double d[3];
  for (int i = 0; i < 3; ++i) d[i] = kSym[i] * (sv[i] - si[i]);
  for (int i = 0; i < 3; ++i) {
    double v = 0;
    for (int j = 0; j < 3; ++j) v += Ht[i + 3 * j] * d[j];
    sc.gl[3 * e + i] = vol * v + kSymInv[i] * g[i];
  }
  // Aloc = vol^2 Jloc^T (dSdF Htil dSdF^T) Jloc
  double DH[12], K4[16];
  for (int r = 0; r < 4; ++r)
    for (int j = 0; j < 3; ++j) {
      double v = 0;
      for (int i = 0; i < 3; ++i) v += dSdF[r + 4 * i] * Ht[i + 3 * j];
      DH[r + 4 * j] = v;
    }
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) {
      double v = 0;
      for (int j = 0; j < 3; ++j) v += DH[r + 4 * j] * dSdF[c + 4 * j];
      K4[r + 4 * c] = v;
    }
  const double* dx = &sc.dX[6 * e];
  double* Al = &sc.Aloc[36 * size_t(e)];
  for (int a = 0; a < 3; ++a)
    for (int l = 0; l < 2; ++l)
      for (int bq = 0; bq < 3; ++bq)
        for (int m = 0; m < 2; ++m) {
          double v = 0;
          for (int c = 0; c < 2; ++c)
            for (int dd = 0; dd < 2; ++dd)
              v += dx[2 * a + c] * dx[2 * bq + dd] * K4[(2 * c + l) + 4 * (2 * dd + m)];
          Al[(2 * a + l) + 6 * (2 * bq + m)] = v * vol * vol;
        }
  return st;
}

int update_system(Scene2& sc, std::vector<double>& full) {
  sc.unproject(sc.x, full);
  const double dt = sc.dt();
  int status = MFEM_OK;
#pragma omp parallel for schedule(static)
  for (int e = 0; e < sc.nt; ++e) {
    const int st = elem_update(sc, e, full, dt);
    if (st != MFEM_OK) {
#pragma omp critical
      status = st;
    }
  }
  std::fill(sc.A.begin(), sc.A.end(), 0.0);
  for (size_t i = 0; i < sc.pair_elem.size(); ++i) {
    const int e = sc.pair_elem[i], j = sc.pair_local[i] / 3, k = sc.pair_local[i] % 3;
    double* blk = &sc.A[4 * size_t(sc.pair_blk[i])];
    const double* Al = &sc.Aloc[36 * size_t(e)];
    for (int rr = 0; rr < 2; ++rr)
      for (int cc = 0; cc < 2; ++cc) blk[2 * rr + cc] += Al[(2 * j + rr) + 6 * (2 * k + cc)];
  }
  for (size_t q = 0; q < sc.b_col.size(); ++q) {
    sc.A[4 * q] += sc.b_mass[q];
    sc.A[4 * q + 3] += sc.b_mass[q];
  }
  std::vector<double> xt = sc.xtilde(), diff(2 * sc.nv), Md;
  for (int i = 0; i < 2 * sc.nv; ++i) diff[i] = full[i] - xt[i] - dt * dt * sc.fext[i];
  mass_mul(sc, diff, Md);
  std::vector<double> rfull(2 * sc.nv);
  for (int i = 0; i < 2 * sc.nv; ++i) rfull[i] = -Md[i];
  for (int e = 0; e < sc.nt; ++e) {
    double tmp[4];
    const double* D = &sc.dSdF[12 * e];
    for (int r = 0; r < 4; ++r) {
      double v = 0;
      for (int i = 0; i < 3; ++i) v += D[r + 4 * i] * sc.gl[3 * e + i];
      tmp[r] = v;
    }
    for (int k = 0; k < 3; ++k)
      for (int l = 0; l < 2; ++l) {
        double o = 0;
        for (int c = 0; c < 2; ++c) o += sc.dX[6 * e + 2 * k + c] * tmp[l + 2 * c];
        rfull[2 * sc.T[3 * e + k] + l] -= sc.vol[e] * o;
      }
  }
  sc.rhs.assign(2 * sc.nfree, 0.0);
  for (int v = 0; v < sc.nv; ++v)
    if (sc.free_map[v] >= 0)
      for (int d = 0; d < 2; ++d) sc.rhs[2 * sc.free_map[v] + d] = rfull[2 * v + d];
  return status;
}

void bcsr_mul(const Scene2& sc, const std::vector<double>& p, std::vector<double>& y) {
  y.assign(2 * sc.nfree, 0.0);
#pragma omp parallel for schedule(static)
  for (int r = 0; r < sc.nfree; ++r)
    for (int i = 0; i < 2; ++i) {
      double acc = 0;
      for (int q = sc.b_ptr[r]; q < sc.b_ptr[r + 1]; ++q)
        for (int j = 0; j < 2; ++j) acc += sc.A[4 * size_t(q) + 2 * i + j] * p[2 * sc.b_col[q] + j];
      y[2 * r + i] = acc;
    }
}

// Eigen::ConjugateGradient + DiagonalPreconditioner from x = 0.
int pcg(const Scene2& sc, const std::vector<double>& rhs, std::vector<double>& x, int* iters,
        double* err) {
  const int n = 2 * sc.nfree;
  x.assign(n, 0.0);
  std::vector<double> invdiag(n);
  for (int r = 0; r < sc.nfree; ++r) {
    int q = sc.b_ptr[r];
    while (q < sc.b_ptr[r + 1] && sc.b_col[q] != r) ++q;
    for (int d = 0; d < 2; ++d) {
      const double dv = (q < sc.b_ptr[r + 1]) ? sc.A[4 * size_t(q) + 3 * d] : 0.0;
      invdiag[2 * r + d] = dv != 0 ? 1.0 / dv : 1.0;
    }
  }
  std::vector<double> r = rhs, z(n), p(n), tmp(n);
  const double rhsNorm2 = dot(rhs, rhs);
  if (rhsNorm2 == 0) {
    *iters = 0;
    *err = 0;
    return MFEM_OK;
  }
  const double threshold = std::max(sc.cg_tol * sc.cg_tol * rhsNorm2, std::numeric_limits<double>::min());
  double rn2 = rhsNorm2;
  if (rn2 < threshold) {  // Eigen's test before the first iteration
    *iters = 0;
    *err = std::sqrt(rn2 / rhsNorm2);
    return MFEM_OK;
  }
  for (int i = 0; i < n; ++i) p[i] = invdiag[i] * r[i];
  double absNew = dot(r, p);
  int it = 0;
  while (it < sc.cg_iters) {
    bcsr_mul(sc, p, tmp);
    const double alpha = absNew / dot(p, tmp);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
      x[i] += alpha * p[i];
      r[i] -= alpha * tmp[i];
    }
    rn2 = dot(r, r);
    if (rn2 < threshold) break;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) z[i] = invdiag[i] * r[i];
    const double absOld = absNew;
    absNew = dot(r, z);
    const double beta = absNew / absOld;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
    ++it;
  }
  *iters = it;
  *err = std::sqrt(rn2 / rhsNorm2);
  return it >= sc.cg_iters ? MFEM_ERR_CG_MAXITER : MFEM_OK;
}

void local_solve(Scene2& sc) {
  std::vector<double> dfull(2 * sc.nv, 0.0);
  for (int v = 0; v < sc.nv; ++v)
    if (sc.free_map[v] >= 0)
      for (int d = 0; d < 2; ++d) dfull[2 * v + d] = sc.dx[2 * sc.free_map[v] + d];
#pragma omp parallel for schedule(static)
  for (int e = 0; e < sc.nt; ++e) {
    double Jdx[4] = {0, 0, 0, 0};
    for (int k = 0; k < 3; ++k)
      for (int c = 0; c < 2; ++c)
        for (int r = 0; r < 2; ++r)
          Jdx[2 * c + r] -= sc.vol[e] * sc.dX[6 * e + 2 * k + c] * dfull[2 * sc.T[3 * e + k] + r];
    const double* D = &sc.dSdF[12 * e];
    double DtJ[3];
    for (int i = 0; i < 3; ++i) {
      double v = 0;
      for (int r = 0; r < 4; ++r) v += D[r + 4 * i] * Jdx[r];
      DtJ[i] = v;
    }
    const double* Ht = &sc.Htil[9 * e];
    double w[3];
    for (int i = 0; i < 3; ++i) {
      double v = 0;
      for (int j = 0; j < 3; ++j) v += Ht[i + 3 * j] * DtJ[j];
      sc.lam[3 * e + i] = -sc.gl[3 * e + i] + v;
    }
    for (int i = 0; i < 3; ++i) w[i] = kSym[i] * sc.lam[3 * e + i] + sc.g[3 * e + i];
    const double* Hi = &sc.Hinv[9 * e];
    for (int i = 0; i < 3; ++i) {
      double v = 0;
      for (int j = 0; j < 3; ++j) v += Hi[i + 3 * j] * w[j];
      sc.ds[3 * e + i] = -v;
    }
  }
}

double energy(Scene2& sc, double a) {
  const double dt = sc.dt(), h2 = dt * dt;
  std::vector<double> x0(sc.x.size());
  for (size_t i = 0; i < x0.size(); ++i) x0[i] = sc.x[i] + a * sc.dx[i];
  std::vector<double> full;
  sc.unproject(x0, full);
  std::vector<double> xt = sc.xtilde(), diff(2 * sc.nv), Md;
  for (int i = 0; i < 2 * sc.nv; ++i) diff[i] = full[i] - xt[i] - h2 * sc.fext[i];
  mass_mul(sc, diff, Md);
  const double val = 0.5 * dot(diff, Md);
  std::vector<double> epsi(sc.nt), econ(sc.nt);
#pragma omp parallel for schedule(static)
  for (int e = 0; e < sc.nt; ++e) {
    double si[3];
    for (int i = 0; i < 3; ++i) si[i] = sc.s[3 * e + i] + a * sc.ds[3 * e + i];
    epsi[e] = coef2(sc.mat[e], sc.mu[e], sc.la[e], si).psi * sc.vol[e];
    M2 R;
    double st[3];
    polar2(R, sc.defgrad(full, e), false, st, nullptr);
    double c = 0;
    for (int i = 0; i < 3; ++i) c += sc.lam[3 * e + i] * kSym[i] * (st[i] - si[i]);
    econ[e] = c * sc.vol[e];
  }
  const double sp = det_sum(sc.nt, [&](long e) { return epsi[e]; });
  const double sq = det_sum(sc.nt, [&](long e) { return econ[e]; });
  return val + h2 * sp - sq;
}

double inf_norm(const std::vector<double>& v) {
  double m = 0;
  for (double x : v) m = std::max(m, std::fabs(x));
  return m;
}

int step(Scene2& sc, mfem_step_stats* stats) {
  mfem_step_stats st{};
  int status = MFEM_OK;
  int i = 0;
  double E = 0, E_prev = 0, res = 0, decrement = 0;
  std::vector<double> full;
  do {
    const int s1 = update_system(sc, full);
    if (s1 != MFEM_OK) status = s1;
    const double rn = std::sqrt(dot(sc.rhs, sc.rhs));
    if (i == 0) st.residual0 = rn;
    st.residual = rn;
    if (sc.res_tol > 0 && ((i > 0 && rn <= sc.res_tol * st.residual0) ||
                           rn <= sc.res_tol * sc.load_norm))
      break;
    int iters = 0;
    double err = 0;
    const int s2 = pcg(sc, sc.rhs, sc.dx, &iters, &err);
    if (s2 != MFEM_OK && status == MFEM_OK) status = s2;
    local_solve(sc);
    st.cg_iterations += iters;
    st.cg_error = err;
    decrement = std::max(inf_norm(sc.dx), inf_norm(sc.ds));
    E = energy(sc, 0.0);
    res = std::fabs((E - E_prev) / (E + 1e-6));
    E_prev = E;
    double alpha = 1.0;
    const double fx0 = E;
    int it = 0;
    while (it < sc.ls_iters) {
      const double fx = energy(sc, alpha);
      if (fx < fx0) break;
      alpha *= 0.5;
      ++it;
    }
    st.ls_iterations += it;
    if (it < sc.ls_iters) {
      for (size_t k = 0; k < sc.x.size(); ++k) sc.x[k] += alpha * sc.dx[k];
      for (size_t k = 0; k < sc.s.size(); ++k) sc.s[k] += alpha * sc.ds[k];
    } else if (status == MFEM_OK) {
      status = MFEM_ERR_LS_FAILED;
    }
    st.alpha = alpha;
    ++i;
  } while (i < sc.max_newton && decrement > sc.newton_tol && res > 1e-12);
  st.newton_iterations = i;
  st.energy = E;
  st.energy_residual = res;
  st.decrement = decrement;
  bc_step(sc, sc.h);
  for (int v = 0; v < sc.nv; ++v)
    if (sc.is_fixed[v])
      for (int d = 0; d < 2; ++d) sc.b[2 * v + d] = sc.V[2 * v + d];
  sc.unproject(sc.x, full);
  std::vector<double> wx = sc.weighted(sc.xprev), vnew(2 * sc.nv);
  for (int k = 0; k < 2 * sc.nv; ++k) vnew[k] = (full[k] - wx[k]) / sc.dt();
  sc.xprev.push_front(full);
  sc.vprev.push_front(vnew);
  if ((int)sc.xprev.size() > sc.bdf) {
    sc.xprev.pop_back();
    sc.vprev.pop_back();
  }
  sc.V = full;
  std::fill(sc.lam.begin(), sc.lam.end(), 0.0);
  for (double v : sc.x)
    if (!std::isfinite(v)) status = MFEM_ERR_NONFINITE;
  st.status = status;
  if (stats) *stats = st;
  return status;
}

Scene2* create(const mfem_tri2d_desc* d, int* status) {
  *status = MFEM_ERR_INVALID;
  if (!d || d->n_vertices <= 0 || d->n_tris <= 0 || !d->V_rest || !d->tris || !d->mu ||
      !d->lambda || d->bdf_order < 1 || d->bdf_order > 6 || d->bc_axis < 0 || d->bc_axis > 1)
    return nullptr;
  if (d->linear_solver != MFEM_SOLVER_EIGEN_CG_DIAG) {
    *status = MFEM_ERR_UNSUPPORTED;
    return nullptr;
  }
  auto sc = std::make_unique<Scene2>();
  sc->nv = d->n_vertices;
  sc->nt = d->n_tris;
  sc->mat = d->material ? std::vector<int>(d->material, d->material + sc->nt)
                        : std::vector<int>(sc->nt, MFEM_MATERIAL_SNH);
  for (int m : sc->mat)
    if (!coef2(m, 1, 1, std::array<double, 3>{1, 1, 0}.data()).ok) {
      *status = MFEM_ERR_UNSUPPORTED;
      return nullptr;
    }
  sc->Vref.assign(d->V_rest, d->V_rest + 2 * sc->nv);
  sc->V = d->V_init ? std::vector<double>(d->V_init, d->V_init + 2 * sc->nv) : sc->Vref;
  sc->T.assign(d->tris, d->tris + 3 * sc->nt);
  for (int v : sc->T)
    if (v < 0 || v >= sc->nv) return nullptr;
  sc->mu.assign(d->mu, d->mu + sc->nt);
  sc->la.assign(d->lambda, d->lambda + sc->nt);
  sc->rho = d->density ? std::vector<double>(d->density, d->density + sc->nt)
                       : std::vector<double>(sc->nt, d->density_const);
  sc->bc_type = d->bc_type;
  sc->bc_axis = d->bc_axis;
  sc->bc_ratio = d->bc_ratio;
  sc->bc_vel = d->bc_velocity;
  sc->h = d->dt;
  sc->ext[0] = d->body_force[0];
  sc->ext[1] = d->body_force[1];
  sc->bdf = d->bdf_order;
  sc->max_newton = d->max_newton_iterations;
  sc->ls_iters = d->max_linesearch_iterations;
  sc->cg_iters = d->max_iterative_solver_iters;
  sc->cg_tol = d->iterative_solver_tolerance;
  sc->newton_tol = d->newton_tol;
  sc->res_tol = d->newton_residual_tolerance;
  bc_init(*sc, d->is_fixed);
  sc->free_map.assign(sc->nv, -1);
  for (int v = 0; v < sc->nv; ++v)
    if (!sc->is_fixed[v]) sc->free_map[v] = sc->nfree++;
  // doublearea volumes and dphi/dX (rows of Dm^-1; phi_0 = 1 - phi_1 - phi_2)
  sc->vol.resize(sc->nt);
  sc->dX.resize(6 * size_t(sc->nt));
  for (int e = 0; e < sc->nt; ++e) {
    const double* X0 = &sc->Vref[2 * sc->T[3 * e]];
    const double* X1 = &sc->Vref[2 * sc->T[3 * e + 1]];
    const double* X2 = &sc->Vref[2 * sc->T[3 * e + 2]];
    const double m00 = X1[0] - X0[0], m10 = X1[1] - X0[1];
    const double m01 = X2[0] - X0[0], m11 = X2[1] - X0[1];
    const double det = m00 * m11 - m01 * m10;
    if (!(det > 0) || !std::isfinite(det)) return nullptr;  // clockwise or degenerate
    sc->vol[e] = det;
    const double i00 = m11 / det, i01 = -m01 / det, i10 = -m10 / det, i11 = m00 / det;
    double* dx = &sc->dX[6 * size_t(e)];
    dx[2 * 1 + 0] = i00;
    dx[2 * 1 + 1] = i01;
    dx[2 * 2 + 0] = i10;
    dx[2 * 2 + 1] = i11;
    dx[0] = -(i00 + i10);
    dx[1] = -(i01 + i11);
  }
  build_mass(*sc);
  build_assembler(*sc);
  std::vector<double> x0 = sc->V;
  std::vector<double> v0 = d->v_init ? std::vector<double>(d->v_init, d->v_init + 2 * sc->nv)
                                     : std::vector<double>(2 * sc->nv, 0.0);
  for (int i = 0; i < sc->bdf; ++i) {
    sc->xprev.push_front(x0);
    sc->vprev.push_front(v0);
  }
  sc->b.assign(2 * sc->nv, 0.0);
  sc->x.assign(2 * sc->nfree, 0.0);
  for (int v = 0; v < sc->nv; ++v) {
    if (sc->is_fixed[v])
      for (int k = 0; k < 2; ++k) sc->b[2 * v + k] = x0[2 * v + k];
    else
      for (int k = 0; k < 2; ++k) sc->x[2 * sc->free_map[v] + k] = x0[2 * v + k];
  }
  sc->dx.assign(2 * sc->nfree, 0.0);
  sc->fext.resize(2 * sc->nv);
  for (int v = 0; v < sc->nv; ++v)
    for (int k = 0; k < 2; ++k) sc->fext[2 * v + k] = float(sc->ext[k]);
  {
    double acc = 0;
    const double dt2 = sc->dt() * sc->dt();
    for (int v = 0; v < sc->nv; ++v) {
      if (sc->free_map[v] < 0) continue;
      double m = 0;
      for (int q = sc->m_ptr[v]; q < sc->m_ptr[v + 1]; ++q) m += sc->m_val[q];
      for (int k = 0; k < 2; ++k) acc += (dt2 * m * sc->fext[2 * v + k]) * (dt2 * m * sc->fext[2 * v + k]);
    }
    sc->load_norm = std::sqrt(acc);
  }
  const size_t nt = sc->nt;
  sc->s.assign(3 * nt, 0);
  sc->ds.assign(3 * nt, 0);
  sc->lam.assign(3 * nt, 0);
  sc->Rm.assign(4 * nt, 0);
  sc->Sv.assign(3 * nt, 0);
  sc->dSdF.assign(12 * nt, 0);
  sc->g.assign(3 * nt, 0);
  sc->Hm.assign(9 * nt, 0);
  sc->Hinv.assign(9 * nt, 0);
  sc->Htil.assign(9 * nt, 0);
  sc->gl.assign(3 * nt, 0);
  sc->Aloc.assign(36 * nt, 0);
  int st = MFEM_OK;
  for (int e = 0; e < sc->nt; ++e) {
    M2 R;
    double sv[3];
    const int r = polar2(R, sc->defgrad(x0, e), false, sv, nullptr);
    if (r != MFEM_OK) st = r;
    std::memcpy(&sc->Rm[4 * e], R.data(), sizeof(double) * 4);
    for (int i = 0; i < 3; ++i) sc->s[3 * e + i] = sc->Sv[3 * e + i] = sv[i];
    for (int i = 0; i < 9; ++i) sc->Hm[9 * e + i] = sc->Hinv[9 * e + i] = (i % 4 == 0);
  }
  *status = st;
  return sc.release();
}

}  // namespace

extern "C" {

int oracle2d_polar(double* R, const double* F, double* s, double* dsdF) {
  M2 Fm, Rm;
  std::memcpy(Fm.data(), F, sizeof(double) * 4);
  const int st = polar2(Rm, Fm, dsdF != nullptr, s, dsdF);
  std::memcpy(R, Rm.data(), sizeof(double) * 4);
  return st;
}

int oracle2d_svd(const double* F, double* sig, double* U, double* V) {
  M2 Fm, Um, Vm;
  std::memcpy(Fm.data(), F, sizeof(double) * 4);
  svd2(Fm, sig, Um, Vm);
  std::memcpy(U, Um.data(), sizeof(double) * 4);
  std::memcpy(V, Vm.data(), sizeof(double) * 4);
  return MFEM_OK;
}

double oracle2d_material(int type, double mu, double la, const double* s, double* g, double* H,
                         int fix) {
  double psi = 0;
  material2(type, mu, la, s, &psi, g, H, fix != 0);
  return psi;
}

void* oracle2d_create(const mfem_tri2d_desc* desc, int* status) {
  int st = MFEM_OK;
  Scene2* sc = create(desc, &st);
  if (status) *status = st;
  return sc;
}
void oracle2d_destroy(void* scene) { delete static_cast<Scene2*>(scene); }
int oracle2d_step(void* scene, mfem_step_stats* stats) {
  return step(*static_cast<Scene2*>(scene), stats);
}
int oracle2d_sizes(void* scene, int* nv, int* nt, int* nfree, int* nnzb) {
  const Scene2& sc = *static_cast<Scene2*>(scene);
  if (nv) *nv = sc.nv;
  if (nt) *nt = sc.nt;
  if (nfree) *nfree = sc.nfree;
  if (nnzb) *nnzb = int(sc.b_col.size());
  return MFEM_OK;
}
int oracle2d_get_state(void* scene, double* x, double* v, double* s, double* R, double* la) {
  Scene2& sc = *static_cast<Scene2*>(scene);
  if (x) {
    std::vector<double> full;
    sc.unproject(sc.x, full);
    std::memcpy(x, full.data(), 8 * full.size());
  }
  if (v) std::memcpy(v, sc.vprev.front().data(), 8 * 2 * size_t(sc.nv));
  if (s) std::memcpy(s, sc.s.data(), 8 * sc.s.size());
  if (R) std::memcpy(R, sc.Rm.data(), 8 * sc.Rm.size());
  if (la) std::memcpy(la, sc.lam.data(), 8 * sc.lam.size());
  return MFEM_OK;
}
int oracle2d_elem_update(void* scene, const double* x, double h, double* R, double* S,
                         double* dSdF, double* g, double* H, double* Hinv, double* Aloc,
                         double* gl) {
  Scene2& sc = *static_cast<Scene2*>(scene);
  const std::vector<double> full(x, x + 2 * sc.nv);
  int status = MFEM_OK;
  for (int e = 0; e < sc.nt; ++e) {
    const int st = elem_update(sc, e, full, h);
    if (st != MFEM_OK) status = st;
  }
  const size_t nt = sc.nt;
  if (R) std::memcpy(R, sc.Rm.data(), 8 * 4 * nt);
  if (S) std::memcpy(S, sc.Sv.data(), 8 * 3 * nt);
  if (dSdF) std::memcpy(dSdF, sc.dSdF.data(), 8 * 12 * nt);
  if (g) std::memcpy(g, sc.g.data(), 8 * 3 * nt);
  if (H) std::memcpy(H, sc.Hm.data(), 8 * 9 * nt);
  if (Hinv) std::memcpy(Hinv, sc.Hinv.data(), 8 * 9 * nt);
  if (Aloc) std::memcpy(Aloc, sc.Aloc.data(), 8 * 36 * nt);
  if (gl) std::memcpy(gl, sc.gl.data(), 8 * 3 * nt);
  return status;
}
int oracle2d_get_system(void* scene, int* row_ptr, int* col, double* val, double* rhs) {
  Scene2& sc = *static_cast<Scene2*>(scene);
  std::vector<double> full;
  const int st = update_system(sc, full);
  if (row_ptr) std::memcpy(row_ptr, sc.b_ptr.data(), 4 * sc.b_ptr.size());
  if (col) std::memcpy(col, sc.b_col.data(), 4 * sc.b_col.size());
  if (val) std::memcpy(val, sc.A.data(), 8 * sc.A.size());
  if (rhs) std::memcpy(rhs, sc.rhs.data(), 8 * sc.rhs.size());
  return st;
}
double oracle2d_energy(void* scene, double alpha) {
  return energy(*static_cast<Scene2*>(scene), alpha);
}
int oracle2d_direction(void* scene, double* dx, double* ds, double* la, int* iters) {
  Scene2& sc = *static_cast<Scene2*>(scene);
  std::vector<double> full;
  int st = update_system(sc, full);
  int it = 0;
  double err = 0;
  const int s2 = pcg(sc, sc.rhs, sc.dx, &it, &err);
  if (st == MFEM_OK) st = s2;
  local_solve(sc);
  if (dx)
    for (int v = 0; v < sc.nv; ++v)
      for (int d = 0; d < 2; ++d)
        dx[2 * v + d] = sc.free_map[v] >= 0 ? sc.dx[2 * sc.free_map[v] + d] : 0.0;
  if (ds) std::memcpy(ds, sc.ds.data(), 8 * sc.ds.size());
  if (la) std::memcpy(la, sc.lam.data(), 8 * sc.lam.size());
  if (iters) *iters = it;
  return st;
}

}  // extern "C"
