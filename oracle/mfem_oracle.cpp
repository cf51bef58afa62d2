// TEST INFRASTRUCTURE ONLY.  FP64 CPU oracle of the mixed-FEM Newton
// timestep of tytrusty/mfem (see mfem_oracle.h for its parity status).
// Every function restates the reference routine named in its comment; file
// paths are relative to the reference project.  Only tests/, the smoke check
// and bench.py's CPU-baseline legs may load this library.
//
// Conventions: 3x3 matrices are column-major (Eigen's default), index r+3c;
// vec(F) is column-major as in TetrahedralMesh::local_jacobian
// (src/mesh/tet_mesh.cpp:17-27).  The 6-vector s is
// [S00, S11, S22, S01, S02, S12] (mixed_stretch.cpp:26-29).
#include "mfem_oracle.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <deque>
#include <limits>
#include <memory>
#include <numeric>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

using M3 = std::array<double, 9>;

inline double& at(M3& m, int r, int c) { return m[r + 3 * c]; }
inline double at(const M3& m, int r, int c) { return m[r + 3 * c]; }

M3 mul(const M3& a, const M3& b) {
  M3 c{};
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0;
      for (int k = 0; k < 3; ++k) s += at(a, i, k) * at(b, k, j);
      at(c, i, j) = s;
    }
  return c;
}
M3 transpose(const M3& a) {
  M3 t{};
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) at(t, i, j) = at(a, j, i);
  return t;
}
M3 eye3() {
  M3 m{};
  m[0] = m[4] = m[8] = 1.0;
  return m;
}
double trace(const M3& a) { return a[0] + a[4] + a[8]; }
M3 skew(const double w[3]) {  // [w]x ; Skew_To_Full newton_procrustes.h:69-85
  M3 k{};
  at(k, 0, 1) = -w[2];
  at(k, 0, 2) = w[1];
  at(k, 1, 0) = w[2];
  at(k, 1, 2) = -w[0];
  at(k, 2, 0) = -w[1];
  at(k, 2, 1) = w[0];
  return k;
}

// Dense n x n solve with full pivoting, columns of B overwritten by A^{-1}B.
// Stands in for Eigen's colPivHouseholderQr().solve (newton_procrustes.h:141,186)
// and PartialPivLU inverse (mixed_stretch.cpp:162): equal up to rounding for
// a non-singular matrix.  Returns false if singular.
bool dense_solve(int n, double* A, int nrhs, double* B) {
  std::vector<int> colperm(n);
  std::iota(colperm.begin(), colperm.end(), 0);
  for (int k = 0; k < n; ++k) {
    int pr = k, pc = k;
    double best = 0;
    for (int i = k; i < n; ++i)
      for (int j = k; j < n; ++j)
        if (std::fabs(A[i + n * j]) > best) {
          best = std::fabs(A[i + n * j]);
          pr = i;
          pc = j;
        }
    if (best == 0.0) return false;
    if (pr != k) {
      for (int j = 0; j < n; ++j) std::swap(A[k + n * j], A[pr + n * j]);
      for (int j = 0; j < nrhs; ++j) std::swap(B[k + n * j], B[pr + n * j]);
    }
    if (pc != k) {
      for (int i = 0; i < n; ++i) std::swap(A[i + n * k], A[i + n * pc]);
      std::swap(colperm[k], colperm[pc]);
    }
    double piv = A[k + n * k];
    for (int i = k + 1; i < n; ++i) {
      double f = A[i + n * k] / piv;
      if (f == 0.0) continue;
      for (int j = k; j < n; ++j) A[i + n * j] -= f * A[k + n * j];
      for (int j = 0; j < nrhs; ++j) B[i + n * j] -= f * B[k + n * j];
    }
  }
  std::vector<double> y(n);
  for (int c = 0; c < nrhs; ++c) {
    for (int i = n - 1; i >= 0; --i) {
      double s = B[i + n * c];
      for (int j = i + 1; j < n; ++j) s -= A[i + n * j] * y[j];
      y[i] = s / A[i + n * i];
    }
    for (int i = 0; i < n; ++i) B[colperm[i] + n * c] = y[i];
  }
  return true;
}

bool inverse(int n, const double* A, double* Ainv) {
  std::vector<double> a(A, A + n * n);
  for (int i = 0; i < n * n; ++i) Ainv[i] = 0;
  for (int i = 0; i < n; ++i) Ainv[i + n * i] = 1;
  return dense_solve(n, a.data(), n, Ainv);
}

// rodrigues, src/svd/newton_procrustes.h:87-106
M3 rodrigues(const double w[3]) {
  double angle = std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
  if (std::fabs(angle) < 1e-8) return eye3();
  double ax[3] = {w[0] / angle, w[1] / angle, w[2] / angle};
  M3 K = skew(ax);
  M3 K2 = mul(K, K);
  M3 R = eye3();
  double sa = std::sin(angle), ca = 1 - std::cos(angle);
  for (int i = 0; i < 9; ++i) R[i] += sa * K[i] + ca * K2[i];
  return R;
}

// -tr(cp_k Y) and -tr(cp_kl Y) of newton_procrustes.h:128,136-138 written
// out: g = axial part of Y, H = tr(sym Y) I - sym Y.
void procrustes_gH(const M3& Y, double g[3], double H[9]) {
  g[0] = at(Y, 2, 1) - at(Y, 1, 2);
  g[1] = at(Y, 0, 2) - at(Y, 2, 0);
  g[2] = at(Y, 1, 0) - at(Y, 0, 1);
  double tr = trace(Y);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      H[i + 3 * j] = (i == j ? tr : 0.0) - 0.5 * (at(Y, i, j) + at(Y, j, i));
}

// newton_procrustes, src/svd/newton_procrustes.h:108-189: R minimising
// |R A - B|_F by Newton on SO(3) with 0.6 backtracking.
int procrustes(M3& R, const M3& A, const M3& B, bool grads, double* dRdF,
               double tol, int max_iter, int* iters) {
  M3 Y = mul(mul(R, A), transpose(B));
  double g[3], H[9], omega[3];
  int itr = 0;
  do {
    double Hm[9];
    procrustes_gH(Y, g, Hm);
    if (std::sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]) < tol) break;
    std::memcpy(H, Hm, sizeof(H));
    double rhs[3] = {g[0], g[1], g[2]};
    if (!dense_solve(3, H, 1, rhs)) { rhs[0] = rhs[1] = rhs[2] = 0; }
    omega[0] = -rhs[0];
    omega[1] = -rhs[1];
    omega[2] = -rhs[2];
    // E0 uses R*Y exactly as newton_procrustes.h:142 does.
    double E0 = -trace(mul(R, Y));
    double E1;
    M3 dR;
    do {
      dR = rodrigues(omega);
      E1 = -trace(mul(dR, Y));
      for (double& w : omega) w *= 0.6;
    } while (E1 > E0 &&
             std::sqrt(omega[0] * omega[0] + omega[1] * omega[1] +
                       omega[2] * omega[2]) > tol);
    R = mul(dR, R);
    Y = mul(dR, Y);
    ++itr;
  } while (itr < max_iter);
  if (iters) *iters = itr;
  if (grads) {
    procrustes_gH(Y, g, H);
    double hn = 0;
    for (double h : H) hn += h * h;
    if (std::sqrt(hn) < 1e-6) return MFEM_ERR_PROCRUSTES;
    M3 Y2 = mul(R, A);
    // dF rows (newton_procrustes.h:179-181): vec(-cp_k * Y2); X = H^{-1} dF.
    double X[27];
    for (int k = 0; k < 3; ++k) {
      double e[3] = {0, 0, 0};
      e[k] = 1;
      M3 cpY = mul(skew(e), Y2);
      for (int j = 0; j < 9; ++j) X[k + 3 * j] = -cpY[j];
    }
    double Hc[9];
    std::memcpy(Hc, H, sizeof(H));
    if (!dense_solve(3, Hc, 9, X)) return MFEM_ERR_PROCRUSTES;
    // dRdF(:,j) = -vec([X_j]x R)  (newton_procrustes.h:186)
    for (int j = 0; j < 9; ++j) {
      double w[3] = {X[0 + 3 * j], X[1 + 3 * j], X[2 + 3 * j]};
      M3 KR = mul(skew(w), R);
      for (int i = 0; i < 9; ++i) dRdF[i + 9 * j] = -KR[i];
    }
  }
  return MFEM_OK;
}

// polar_svd<3,6>, src/variables/mixed_stretch.cpp:14-42.
int polar(M3& R, const M3& F, bool grads, double s[6], double* dsdF /*6x9*/) {
  double dRdF[81];
  int st = procrustes(R, eye3(), F, grads, dRdF, 1e-6, 100, nullptr);
  M3 S = mul(transpose(R), F);
  s[0] = at(S, 0, 0);
  s[1] = at(S, 1, 1);
  s[2] = at(S, 2, 2);
  s[3] = 0.5 * (at(S, 1, 0) + at(S, 0, 1));
  s[4] = 0.5 * (at(S, 2, 0) + at(S, 0, 2));
  s[5] = 0.5 * (at(S, 2, 1) + at(S, 1, 2));
  if (!grads || st != MFEM_OK) return st;
  // J = (I (x) R^T)(I - (S^T (x) I) dRdF)   (mixed_stretch.cpp:32-33)
  double T1[81];  // I - (S^T(x)I) dRdF
  for (int c = 0; c < 9; ++c)
    for (int rr = 0; rr < 9; ++rr) {
      int r = rr % 3, cc = rr / 3;  // row index = r + 3*cc
      double v = 0;
      for (int k = 0; k < 3; ++k) v += at(S, k, cc) * dRdF[(r + 3 * k) + 9 * c];
      T1[rr + 9 * c] = (rr == c ? 1.0 : 0.0) - v;
    }
  double J[81];
  for (int c = 0; c < 9; ++c)
    for (int rr = 0; rr < 9; ++rr) {
      int r = rr % 3, cc = rr / 3;
      double v = 0;
      for (int k = 0; k < 3; ++k) v += at(R, k, r) * T1[(k + 3 * cc) + 9 * c];
      J[rr + 9 * c] = v;
    }
  for (int c = 0; c < 9; ++c) {
    dsdF[0 + 6 * c] = J[0 + 9 * c];
    dsdF[1 + 6 * c] = J[4 + 9 * c];
    dsdF[2 + 6 * c] = J[8 + 9 * c];
    dsdF[3 + 6 * c] = 0.5 * (J[1 + 9 * c] + J[3 + 9 * c]);
    dsdF[4 + 6 * c] = 0.5 * (J[2 + 9 * c] + J[6 + 9 * c]);
    dsdF[5 + 6 * c] = 0.5 * (J[5 + 9 * c] + J[7 + 9 * c]);
  }
  return MFEM_OK;
}

// ---------------------------------------------------------------------------
// Materials: psi(s), grad, hess on the 6-vector (src/energies/*.cpp, the
// Vector6d sections).  Each material is written as
//   psi = A(Q) + B(J) + C(t),  Q = |S|_F^2, J = det S, t = tr S,
// which is the same expression as the generated code (scripts/derivs.m).
struct MatCoef {
  double psi, A1, A2, B1, B2, C1, C2;
  bool psd;
};

void invariants(const double* s, double& Q, double& J, double& t, double dJ[6]) {
  Q = s[0] * s[0] + s[1] * s[1] + s[2] * s[2] +
      2 * (s[3] * s[3] + s[4] * s[4] + s[5] * s[5]);
  J = s[0] * s[1] * s[2] + 2 * s[3] * s[4] * s[5] - s[0] * s[5] * s[5] -
      s[1] * s[4] * s[4] - s[2] * s[3] * s[3];
  t = s[0] + s[1] + s[2];
  dJ[0] = s[1] * s[2] - s[5] * s[5];
  dJ[1] = s[0] * s[2] - s[4] * s[4];
  dJ[2] = s[0] * s[1] - s[3] * s[3];
  dJ[3] = 2 * (s[4] * s[5] - s[2] * s[3]);
  dJ[4] = 2 * (s[3] * s[5] - s[1] * s[4]);
  dJ[5] = 2 * (s[3] * s[4] - s[0] * s[5]);
}

MatCoef material_coef_qjt(int type, double mu, double la, double Q, double J, double t) {
  MatCoef c{0, 0, 0, 0, 0, 0, 0, false};
  switch (type) {
    case MFEM_MATERIAL_SNH:  // stable_neohookean.cpp:8-95
      c.psi = mu * (1 - J) + 0.5 * la * (1 - J) * (1 - J) + 0.5 * mu * (Q - 3);
      c.A1 = 0.5 * mu;
      c.B1 = -mu - la * (1 - J);
      c.B2 = la;
      c.psd = true;
      break;
    case MFEM_MATERIAL_NH: {  // neohookean.cpp:8-94
      double lj = std::log(J);
      c.psi = -mu * lj + 0.5 * la * lj * lj + 0.5 * mu * (Q - 3);
      c.A1 = 0.5 * mu;
      c.B1 = (-mu + la * lj) / J;
      c.B2 = (mu + la * (1 - lj)) / (J * J);
      c.psd = true;
      break;
    }
    case MFEM_MATERIAL_COROT:  // corotational.cpp:8-60
      c.psi = 0.5 * la * (t - 3) * (t - 3) + mu * (Q - 2 * t + 3);
      c.A1 = mu;
      c.C1 = la * (t - 3) - 2 * mu;
      c.C2 = la;
      break;
    case MFEM_MATERIAL_FCR:  // fixed_corotational.cpp:8-…
      c.psi = 0.5 * la * (J - 1) * (J - 1) + mu * (Q - 2 * t + 3);
      c.A1 = mu;
      c.B1 = la * (J - 1);
      c.B2 = la;
      c.C1 = -2 * mu;
      break;
    case MFEM_MATERIAL_ARAP:  // arap.cpp:7-65
      c.psi = 0.5 * mu * (Q - 2 * t + 3);
      c.A1 = 0.5 * mu;
      c.C1 = -mu;
      break;
    case MFEM_MATERIAL_FUNG: {  // fung.cpp:8-97, c = 4
      const double cf = 4.0;
      double e = std::exp(cf * (Q - 3) / 2);
      double k = (mu + cf * mu) / la;
      c.psi = 0.5 * mu * (e - 1) + 0.5 * mu * (Q - 3) +
              0.5 * la * (k + 1 - J) * (k + 1 - J);
      c.A1 = mu * cf * e / 4 + 0.5 * mu;
      c.A2 = mu * cf * cf * e / 8;
      c.B1 = -la * (k + 1 - J);
      c.B2 = la;
      c.psd = true;
      break;
    }
    default:
      break;
  }
  return c;
}

MatCoef material_coef(int type, double mu, double la, const double* s) {
  double Q, J, t, dJ[6];
  invariants(s, Q, J, t, dJ);
  return material_coef_qjt(type, mu, la, Q, J, t);
}

void material_gradient(int type, double mu, double la, const double* s, double* g) {
  double Q, J, t, dJ[6];
  invariants(s, Q, J, t, dJ);
  MatCoef c = material_coef(type, mu, la, s);
  const double w[6] = {1, 1, 1, 2, 2, 2};
  for (int i = 0; i < 6; ++i)
    g[i] = c.A1 * 2 * w[i] * s[i] + c.B1 * dJ[i] + (i < 3 ? c.C1 : 0.0);
}

// sim::simple_psd_fix (Bartels, not in this snapshot): eigenvalues of the
// symmetric matrix below tol are raised to tol; unchanged if all are >= tol.
// Cyclic Jacobi eigen-decomposition stands in for SelfAdjointEigenSolver.
void psd_fix(double* H, int n, double tol) {
  std::vector<double> a(H, H + n * n), V(n * n, 0.0);
  for (int i = 0; i < n; ++i) V[i + n * i] = 1;
  for (int sweep = 0; sweep < 64; ++sweep) {
    double off = 0, tot = 0;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        tot += a[i + n * j] * a[i + n * j];
        if (i != j) off += a[i + n * j] * a[i + n * j];
      }
    if (off <= 1e-30 * tot || off == 0) break;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) {
        double apq = a[p + n * q];
        if (apq == 0) continue;
        double theta = (a[q + n * q] - a[p + n * p]) / (2 * apq);
        double tt = (theta >= 0 ? 1.0 : -1.0) /
                    (std::fabs(theta) + std::sqrt(theta * theta + 1));
        double c = 1 / std::sqrt(tt * tt + 1), sn = tt * c;
        for (int k = 0; k < n; ++k) {  // columns p,q
          double akp = a[k + n * p], akq = a[k + n * q];
          a[k + n * p] = c * akp - sn * akq;
          a[k + n * q] = sn * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {  // rows p,q
          double apk = a[p + n * k], aqk = a[q + n * k];
          a[p + n * k] = c * apk - sn * aqk;
          a[q + n * k] = sn * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          double vkp = V[k + n * p], vkq = V[k + n * q];
          V[k + n * p] = c * vkp - sn * vkq;
          V[k + n * q] = sn * vkp + c * vkq;
        }
      }
  }
  double mn = a[0];
  for (int i = 1; i < n; ++i) mn = std::min(mn, a[i + n * i]);
  if (mn >= tol) return;
  std::vector<double> d(n);
  for (int i = 0; i < n; ++i) d[i] = std::max(a[i + n * i], tol);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double v = 0;
      for (int k = 0; k < n; ++k) v += V[i + n * k] * d[k] * V[j + n * k];
      H[i + n * j] = v;
    }
}

const double kPsdTol = 1e-6;

void material_hessian(int type, double mu, double la, const double* s, bool fix,
                      double* H) {
  double Q, J, t, dJ[6];
  invariants(s, Q, J, t, dJ);
  MatCoef c = material_coef(type, mu, la, s);
  const double w[6] = {1, 1, 1, 2, 2, 2};
  double dQ[6], d2J[36] = {0};
  for (int i = 0; i < 6; ++i) dQ[i] = 2 * w[i] * s[i];
  auto set = [&](int i, int j, double v) {
    d2J[i + 6 * j] = v;
    d2J[j + 6 * i] = v;
  };
  set(0, 1, s[2]);
  set(0, 2, s[1]);
  set(0, 5, -2 * s[5]);
  set(1, 2, s[0]);
  set(1, 4, -2 * s[4]);
  set(2, 3, -2 * s[3]);
  set(3, 3, -2 * s[2]);
  set(3, 4, 2 * s[5]);
  set(3, 5, 2 * s[4]);
  set(4, 4, -2 * s[1]);
  set(4, 5, 2 * s[3]);
  set(5, 5, -2 * s[0]);
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) {
      double v = c.A2 * dQ[i] * dQ[j] + c.B2 * dJ[i] * dJ[j] + c.B1 * d2J[i + 6 * j];
      if (i == j) v += 2 * c.A1 * w[i];
      if (i < 3 && j < 3) v += c.C2;
      H[i + 6 * j] = v;
    }
  if (fix && c.psd) psd_fix(H, 6, kPsdTol);
}

// MaterialModel's Vector9d forms (the standard-FEM "stretch" variable) for
// the two materials that define them: Stable-Neohookean
// (stable_neohookean.cpp:97-234) psi = mu (1 - J) + la/2 (1 - J)^2 +
// mu/2 (|F|^2 - 3), and Neohookean (neohookean.cpp:96-231) psi =
// la/2 log(J)^2 - mu log J + mu/2 (|F|^2 - 3), J = det F, F flattened
// column-major.  Derivatives by the chain rule through |F|^2 and det F
// (the reference's are generated code; FD-checked in the tests).  The
// Hessian's psd fix uses tolerance 0 for SNH (stable_neohookean.cpp:232)
// and the default for NH (neohookean.cpp:230).
void material9(int type, double mu, double la, const double* F, double* psi, double* g, double* H,
               bool fix) {
  double cof[9];
  cof[0] = F[4] * F[8] - F[7] * F[5];
  cof[1] = F[6] * F[5] - F[3] * F[8];
  cof[2] = F[3] * F[7] - F[6] * F[4];
  cof[3] = F[7] * F[2] - F[1] * F[8];
  cof[4] = F[0] * F[8] - F[6] * F[2];
  cof[5] = F[6] * F[1] - F[0] * F[7];
  cof[6] = F[1] * F[5] - F[4] * F[2];
  cof[7] = F[3] * F[2] - F[0] * F[5];
  cof[8] = F[0] * F[4] - F[3] * F[1];
  const double J = F[0] * cof[0] + F[1] * cof[1] + F[2] * cof[2];
  double Q = 0;
  for (int i = 0; i < 9; ++i) Q += F[i] * F[i];
  const MatCoef c = material_coef_qjt(type, mu, la, Q, J, 0.0);
  if (psi) *psi = c.psi;
  if (g)
    for (int i = 0; i < 9; ++i) g[i] = 2 * c.A1 * F[i] + c.B1 * cof[i];
  if (!H) return;
  static const int eps[3][3][3] = {{{0, 0, 0}, {0, 0, 1}, {0, -1, 0}},
                                   {{0, 0, -1}, {0, 0, 0}, {1, 0, 0}},
                                   {{0, 1, 0}, {-1, 0, 0}, {0, 0, 0}}};
  for (int a = 0; a < 9; ++a)
    for (int b = 0; b < 9; ++b) {
      const int i = a % 3, j = a / 3, k = b % 3, l = b / 3;
      double d2 = 0;  // d2 det / dF_ij dF_kl = sum_mn eps_ikm eps_jln F_mn
      for (int m = 0; m < 3; ++m)
        for (int n = 0; n < 3; ++n) d2 += eps[i][k][m] * eps[j][l][n] * F[m + 3 * n];
      H[a + 9 * b] = c.B2 * cof[a] * cof[b] + c.B1 * d2 + (a == b ? 2 * c.A1 : 0.0);
    }
  if (fix) psd_fix(H, 9, type == MFEM_MATERIAL_SNH ? 0.0 : kPsdTol);
}

// ---------------------------------------------------------------------------
// Scene: Mesh::init (src/mesh/mesh.cpp:124-175), Displacement
// (src/variables/displacement.cpp), MixedStretch (mixed_stretch.cpp),
// Assembler (src/utils/sparse_utils.cpp:19-203), BDF (src/time_integrators/BDF.cpp),
// NewtonOptimizer (src/optimizers/newton_optimizer.cpp), linesearch
// (src/linesearch.h:80-129), boundary conditions (src/boundary_conditions/*).

const double kSym[6] = {1, 1, 1, 2, 2, 2};
const double kSymInv[6] = {1, 1, 1, 0.5, 0.5, 0.5};

struct Scene {
  int nv = 0, nt = 0, nfree = 0;
  std::vector<double> Vref, V;  // V: mesh V_ (current)
  std::vector<int> T, mat, is_fixed, free_map;
  std::vector<double> mu, la, rho, vol, dX;  // dX: 12 per tet, dX[12e+3k+c]
  // BCs
  int bc_type = 0, bc_axis = 0;
  double bc_ratio = 0.1, bc_vel = 0.1;
  std::vector<std::vector<int>> groups;
  std::vector<std::array<double, 3>> group_center;
  std::array<double, 3> twist_center{};
  // mass (full vertex adjacency, scalar), CSR over all vertices
  std::vector<int> m_ptr, m_col;
  std::vector<double> m_val;
  // BCSR pattern over free vertices + assembler pairs
  std::vector<int> b_ptr, b_col;
  std::vector<double> b_mass;  // m_ab for each block
  std::vector<int> pair_elem, pair_local, pair_blk;  // sorted contributions
  std::vector<double> A;       // 9*nnzb assembled LHS
  std::vector<double> rhs;     // 3*nfree
  // config
  double h = 0.034, ext[3] = {0, -9.8, 0};
  int bdf = 1, max_newton = 5, ls_iters = 20, cg_iters = 500, solver = 5;
  int fem = 0;  // the standard-FEM "stretch" variable instead of MixedStretch
  std::vector<double> fforce;  // fem: per element 12 forces -h^2 vol Jloc^T dpsi/dF
  double cg_tol = 1e-4, newton_tol = 1e-10, res_tol = 0, load_norm = 0;
  // state
  std::vector<double> x, dx, b, fext;  // x, dx: free (3*nfree); b, fext: full
  std::deque<std::vector<double>> xprev, vprev;
  std::vector<double> s, ds, lam, Rm, Sv, dSdF, g, Hm, Hinv, Htil, gl;
  int last_cg_iters = 0;
  double last_cg_err = 0;

  double dt() const {
    static const double beta[7] = {0, 1.0, 2.0 / 3, 6.0 / 11, 12.0 / 25, 60.0 / 137, 60.0 / 147};
    return beta[bdf] * h;
  }
  const double* alphas() const {
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
    std::vector<double> w(3 * nv, 0.0);
    const double* a = alphas();
    for (size_t i = 0; i < q.size(); ++i)
      for (int k = 0; k < 3 * nv; ++k) w[k] += a[i] * q[i][k];
    return w;
  }
  std::vector<double> xtilde() const {  // BDF<I>::x_tilde, BDF.cpp:6-9
    std::vector<double> wx = weighted(xprev), wv = weighted(vprev);
    double d = dt();
    for (int k = 0; k < 3 * nv; ++k) wx[k] += d * wv[k];
    return wx;
  }
  void unproject(const std::vector<double>& xf, std::vector<double>& full) const {
    full = b;
    for (int v = 0; v < nv; ++v)
      if (free_map[v] >= 0)
        for (int d = 0; d < 3; ++d) full[3 * v + d] += xf[3 * free_map[v] + d];
  }
  M3 defgrad(const std::vector<double>& full, int e) const {
    M3 F{};
    for (int k = 0; k < 4; ++k) {
      const double* xk = &full[3 * T[4 * e + k]];
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) at(F, r, c) += xk[r] * dX[12 * e + 3 * k + c];
    }
    return F;
  }
};

// BoundaryCondition::init_boundary_groups, src/boundary_conditions/boundary_condition.cpp:5-21
void boundary_groups(Scene& sc, const std::vector<double>& V) {
  double lo[3], hi[3];
  for (int d = 0; d < 3; ++d) {
    lo[d] = std::numeric_limits<double>::infinity();
    hi[d] = -lo[d];
  }
  for (int v = 0; v < sc.nv; ++v)
    for (int d = 0; d < 3; ++d) {
      lo[d] = std::min(lo[d], V[3 * v + d]);
      hi[d] = std::max(hi[d], V[3 * v + d]);
    }
  int ax = sc.bc_axis;
  double range = hi[ax] - lo[ax];
  sc.groups.assign(2, {});
  for (int v = 0; v < sc.nv; ++v) {
    double c = V[3 * v + ax];
    if (c < lo[ax] + range * sc.bc_ratio)
      sc.groups[0].push_back(v);
    else if (c > hi[ax] - range * sc.bc_ratio)
      sc.groups[1].push_back(v);
  }
}

void bbox_center(const Scene& sc, const std::vector<double>& V, double c[3]) {
  for (int d = 0; d < 3; ++d) {
    double lo = 1e300, hi = -1e300;
    for (int v = 0; v < sc.nv; ++v) {
      lo = std::min(lo, V[3 * v + d]);
      hi = std::max(hi, V[3 * v + d]);
    }
    c[d] = 0.5 * (lo + hi);
  }
}

// Fixed set and init-time motion of each BC (fixed_boundary_conditions.h,
// stretch/twist/bend_boundary_condition.h).
void bc_init(Scene& sc, const int32_t* override_fixed) {
  boundary_groups(sc, sc.Vref);
  sc.is_fixed.assign(sc.nv, 0);
  switch (sc.bc_type) {
    case MFEM_BC_SCALEF: {  // ScaleBC::init
      double c[3];
      bbox_center(sc, sc.V, c);
      for (int v = 0; v < sc.nv; ++v)
        for (int d = 0; d < 3; ++d) sc.V[3 * v + d] = (sc.V[3 * v + d] - c[d]) * 1.5 + c[d];
      break;
    }
    case MFEM_BC_RANDOM: {  // RandomizeBC::init with a seeded generator
      double c[3], lo[3], hi[3];
      bbox_center(sc, sc.V, c);
      for (int d = 0; d < 3; ++d) {
        lo[d] = 1e300;
        hi[d] = -1e300;
        for (int v = 0; v < sc.nv; ++v) {
          lo[d] = std::min(lo[d], sc.V[3 * v + d]);
          hi[d] = std::max(hi[d], sc.V[3 * v + d]);
        }
      }
      uint64_t st = 0x9E3779B97F4A7C15ull;
      for (auto& x : sc.V) {
        st = st * 6364136223846793005ull + 1442695040888963407ull;
        x = (double((st >> 11) & ((1ull << 53) - 1)) / double(1ull << 53) * 2 - 1) / 2.0;
      }
      c[1] += (hi[1] - lo[1]) * 0.5;
      double r0[3] = {sc.V[0], sc.V[1], sc.V[2]};
      for (int v = 0; v < sc.nv; ++v)
        for (int d = 0; d < 3; ++d) sc.V[3 * v + d] += c[d] - r0[d];
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
      if (sc.bc_type == MFEM_BC_TWIST) {
        double c[3];
        bbox_center(sc, sc.V, c);
        sc.twist_center = {c[0], c[1], c[2]};
      }
      if (sc.bc_type == MFEM_BC_BEND) {
        sc.group_center.clear();
        for (auto& gr : sc.groups) {
          int v = gr.empty() ? 0 : gr.back();
          sc.group_center.push_back({sc.V[3 * v], sc.V[3 * v + 1], sc.V[3 * v + 2]});
        }
      }
      break;
    default:
      break;
  }
  if (override_fixed)
    for (int v = 0; v < sc.nv; ++v) sc.is_fixed[v] = override_fixed[v] ? 1 : 0;
}

void rotate_about(double* p, const double* o, int axis, double ang) {
  double q[3] = {p[0] - o[0], p[1] - o[1], p[2] - o[2]};
  double c = std::cos(ang), s = std::sin(ang);
  int i = (axis + 1) % 3, j = (axis + 2) % 3;
  double qi = c * q[i] - s * q[j], qj = s * q[i] + c * q[j];
  q[i] = qi;
  q[j] = qj;
  for (int d = 0; d < 3; ++d) p[d] = q[d] + o[d];
}

// BoundaryCondition::step for the scripted BCs (Meshes::update_bcs, meshes.cpp:156-167).
void bc_step(Scene& sc, double dt) {
  switch (sc.bc_type) {
    case MFEM_BC_STRETCH:  // StretchBC::step: group i moves (-1)^i * velocity
      for (int i = 0; i < 2; ++i)
        for (int v : sc.groups[i]) sc.V[3 * v + sc.bc_axis] += (i == 0 ? 1 : -1) * sc.bc_vel * dt;
      break;
    case MFEM_BC_COMPRESS:
      for (int v : sc.groups[1]) sc.V[3 * v + sc.bc_axis] += sc.bc_vel * dt;
      break;
    case MFEM_BC_TWIST:  // TwistBC::step: rotation about +x through the bbox centre
      for (int i = 0; i < 2; ++i) {
        double a = (i == 0 ? 1 : -1) * sc.bc_vel * M_PI * dt;
        for (int v : sc.groups[i]) rotate_about(&sc.V[3 * v], sc.twist_center.data(), 0, a);
      }
      break;
    case MFEM_BC_BEND:  // BendBC::step: rotation about +z through the group's last vertex
      for (int i = 0; i < 2; ++i) {
        double a = (i == 0 ? 1 : -1) * sc.bc_vel * M_PI * dt;
        for (int v : sc.groups[i]) rotate_about(&sc.V[3 * v], sc.group_center[i].data(), 2, a);
      }
      break;
    default:
      break;
  }
}

// Assembler constructor (sparse_utils.cpp:19-138): all (element, local j,k)
// pairs of free vertices, sorted row-major by global free ids.
void build_assembler(Scene& sc) {
  struct P { int r, c, e, l; };
  std::vector<P> pairs;
  pairs.reserve(16 * size_t(sc.nt));
  for (int e = 0; e < sc.nt; ++e)
    for (int j = 0; j < 4; ++j) {
      int a = sc.free_map[sc.T[4 * e + j]];
      if (a < 0) continue;
      for (int k = 0; k < 4; ++k) {
        int bq = sc.free_map[sc.T[4 * e + k]];
        if (bq < 0) continue;
        pairs.push_back({a, bq, e, 4 * j + k});
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
  sc.A.assign(9 * sc.b_col.size(), 0.0);
  // free-free mass entries per block (PMP of mesh.cpp:147-148)
  sc.b_mass.assign(sc.b_col.size(), 0.0);
  for (int a = 0; a < sc.nv; ++a) {
    int fa = sc.free_map[a];
    if (fa < 0) continue;
    for (int q = sc.m_ptr[a]; q < sc.m_ptr[a + 1]; ++q) {
      int fb = sc.free_map[sc.m_col[q]];
      if (fb < 0) continue;
      int* beg = &sc.b_col[sc.b_ptr[fa]];
      int* end = &sc.b_col[sc.b_ptr[fa + 1]];
      int* it = std::lower_bound(beg, end, fb);
      sc.b_mass[it - &sc.b_col[0]] += sc.m_val[q];
    }
  }
}

// Consistent P1 mass (sim::linear_tetmesh_mass_matrix, tet_mesh.cpp:36-41):
// rho*vol/20*(1+delta_ab) per element vertex pair, as a scalar vertex matrix.
void build_mass(Scene& sc) {
  std::vector<std::vector<std::pair<int, double>>> rows(sc.nv);
  for (int e = 0; e < sc.nt; ++e) {
    double m = sc.rho[e] * sc.vol[e] / 20.0;
    for (int a = 0; a < 4; ++a)
      for (int bq = 0; bq < 4; ++bq)
        rows[sc.T[4 * e + a]].push_back({sc.T[4 * e + bq], a == bq ? 2 * m : m});
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

// y = M x over all vertices (3 components each).
void mass_mul(const Scene& sc, const std::vector<double>& xin, std::vector<double>& y) {
  y.assign(3 * sc.nv, 0.0);
#pragma omp parallel for schedule(static)
  for (int a = 0; a < sc.nv; ++a) {
    double acc[3] = {0, 0, 0};
    for (int q = sc.m_ptr[a]; q < sc.m_ptr[a + 1]; ++q)
      for (int d = 0; d < 3; ++d) acc[d] += sc.m_val[q] * xin[3 * sc.m_col[q] + d];
    for (int d = 0; d < 3; ++d) y[3 * a + d] = acc[d];
  }
}

// Jloc^T v for local vertex k: the 3-vector sum_c dX(k,c) v(3c+r).
inline void jloc_t(const double* dX, int k, const double* v9, double out[3]) {
  for (int r = 0; r < 3; ++r) {
    double s = 0;
    for (int c = 0; c < 3; ++c) s += dX[3 * k + c] * v9[3 * c + r];
    out[r] = s;
  }
}

// MixedStretch::update_rotations + update_derivatives + rhs for one element
// (mixed_stretch.cpp:133-226).  Writes R, S, dSdF (9x6 col-major, Js^T Sym),
// g, H, Hinv, Htil, gl and the 12x12 Aloc (col-major).
int elem_update(Scene& sc, int e, const std::vector<double>& full, double dt,
                double* Aloc) {
  double h2 = dt * dt;
  M3 F = sc.defgrad(full, e);
  M3 R;
  std::memcpy(R.data(), &sc.Rm[9 * e], sizeof(double) * 9);
  double svec[6], dsdF[54];
  int st = polar(R, F, true, svec, dsdF);
  std::memcpy(&sc.Rm[9 * e], R.data(), sizeof(double) * 9);
  std::memcpy(&sc.Sv[6 * e], svec, sizeof(svec));
  double* dSdF = &sc.dSdF[54 * e];  // 9x6: dSdF(r,i) = dsdF(i,r)*Sym(i)
  for (int i = 0; i < 6; ++i)
    for (int r = 0; r < 9; ++r) dSdF[r + 9 * i] = dsdF[i + 6 * r] * kSym[i];
  const double* si = &sc.s[6 * e];
  double vol = sc.vol[e];
  double* H = &sc.Hm[36 * e];
  material_hessian(sc.mat[e], sc.mu[e], sc.la[e], si, true, H);
  for (int i = 0; i < 36; ++i) H[i] *= h2;
  if (!inverse(6, H, &sc.Hinv[36 * e])) st = MFEM_ERR_NONFINITE;
  double* g = &sc.g[6 * e];
  material_gradient(sc.mat[e], sc.mu[e], sc.la[e], si, g);
  for (int i = 0; i < 6; ++i) g[i] *= h2;
  double* Ht = &sc.Htil[36 * e];
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) Ht[i + 6 * j] = (1.0 / vol) * kSymInv[i] * H[i + 6 * j] * kSymInv[j];
  // gl = vol*Htil*Sym*(S - s) + Syminv*g    (mixed_stretch.cpp:219-220)
  double d[6];
  for (int i = 0; i < 6; ++i) d[i] = kSym[i] * (svec[i] - si[i]);
  for (int i = 0; i < 6; ++i) {
    double v = 0;
    for (int j = 0; j < 6; ++j) v += Ht[i + 6 * j] * d[j];
    sc.gl[6 * e + i] = vol * v + kSymInv[i] * g[i];
  }
  if (Aloc) {
    // Aloc = vol^2 Jloc^T (dSdF Htil dSdF^T) Jloc   (mixed_stretch.cpp:174-175)
    double DH[54], K9[81];
    for (int r = 0; r < 9; ++r)
      for (int j = 0; j < 6; ++j) {
        double v = 0;
        for (int i = 0; i < 6; ++i) v += dSdF[r + 9 * i] * Ht[i + 6 * j];
        DH[r + 9 * j] = v;
      }
    for (int r = 0; r < 9; ++r)
      for (int c = 0; c < 9; ++c) {
        double v = 0;
        for (int j = 0; j < 6; ++j) v += DH[r + 9 * j] * dSdF[c + 9 * j];
        K9[r + 9 * c] = v;
      }
    const double* dx = &sc.dX[12 * e];
    for (int a = 0; a < 4; ++a)
      for (int l = 0; l < 3; ++l)
        for (int bq = 0; bq < 4; ++bq)
          for (int m = 0; m < 3; ++m) {
            double v = 0;
            for (int c = 0; c < 3; ++c)
              for (int dd = 0; dd < 3; ++dd)
                v += dx[3 * a + c] * dx[3 * bq + dd] * K9[(3 * c + l) + 9 * (3 * dd + m)];
            Aloc[(3 * a + l) + 12 * (3 * bq + m)] = v * vol * vol;
          }
  }
  return st;
}

int update_system(Scene& sc, std::vector<double>& full) {
  sc.unproject(sc.x, full);
  double dt = sc.dt();
  int status = MFEM_OK;
  std::vector<double> Aloc(144 * size_t(sc.nt));
  if (sc.fem) {
    // Stretch::update (stretch.cpp:33-60): Jloc^T H Jloc vol h^2 and the forces
    sc.fforce.assign(12 * size_t(sc.nt), 0.0);
#pragma omp parallel for schedule(static)
    for (int e = 0; e < sc.nt; ++e) {
      const M3 F = sc.defgrad(full, e);
      double g[9], H[81];
      material9(sc.mat[e], sc.mu[e], sc.la[e], F.data(), nullptr, g, H, true);
      const double w = dt * dt * sc.vol[e];
      const double* dX = &sc.dX[12 * size_t(e)];
      for (int a = 0; a < 4; ++a)
        for (int l = 0; l < 3; ++l) {
          double f = 0;
          for (int c = 0; c < 3; ++c) f += dX[3 * a + c] * g[l + 3 * c];
          sc.fforce[12 * size_t(e) + 3 * a + l] = -w * f;
          for (int b = 0; b < 4; ++b)
            for (int m = 0; m < 3; ++m) {
              double v = 0;
              for (int c = 0; c < 3; ++c)
                for (int cc = 0; cc < 3; ++cc) v += dX[3 * a + c] * dX[3 * b + cc] * H[(l + 3 * c) + 9 * (m + 3 * cc)];
              Aloc[144 * size_t(e) + (3 * a + l) + 12 * (3 * b + m)] = w * v;
            }
        }
    }
  } else {
#pragma omp parallel for schedule(static)
  for (int e = 0; e < sc.nt; ++e) {
    int st = elem_update(sc, e, full, dt, &Aloc[144 * size_t(e)]);
    if (st != MFEM_OK) {
#pragma omp critical
      status = st;
    }
  }
  }
  // Assembler::update_matrix: gather each block's contributions in sorted order.
  std::fill(sc.A.begin(), sc.A.end(), 0.0);
  size_t np = sc.pair_elem.size();
  // contributions are grouped by block (sorted); summed in that order
  for (size_t i = 0; i < np; ++i) {
    int e = sc.pair_elem[i], j = sc.pair_local[i] / 4, k = sc.pair_local[i] % 4;
    double* blk = &sc.A[9 * size_t(sc.pair_blk[i])];
    const double* Al = &Aloc[144 * size_t(e)];
    for (int rr = 0; rr < 3; ++rr)
      for (int cc = 0; cc < 3; ++cc) blk[3 * rr + cc] += Al[(3 * j + rr) + 12 * (3 * k + cc)];
  }
  // LHS = PMP + A (SystemMatrixPD::pre_solve, linear_system.h:18-31)
  for (size_t q = 0; q < sc.b_col.size(); ++q)
    for (int d = 0; d < 3; ++d) sc.A[9 * q + 4 * d] += sc.b_mass[q];
  // RHS = -PM(x - xtilde - h^2 f) - PJW (dSdF gl)
  std::vector<double> xt = sc.xtilde(), diff(3 * sc.nv), Md;
  for (int i = 0; i < 3 * sc.nv; ++i) diff[i] = full[i] - xt[i] - dt * dt * sc.fext[i];
  mass_mul(sc, diff, Md);
  std::vector<double> rfull(3 * sc.nv);
  for (int i = 0; i < 3 * sc.nv; ++i) rfull[i] = -Md[i];
  for (int e = 0; e < sc.nt; ++e) {
    if (sc.fem) {
      for (int k = 0; k < 4; ++k)
        for (int d = 0; d < 3; ++d) rfull[3 * sc.T[4 * e + k] + d] += sc.fforce[12 * size_t(e) + 3 * k + d];
      continue;
    }
    double tmp[9];
    const double* D = &sc.dSdF[54 * e];
    for (int r = 0; r < 9; ++r) {
      double v = 0;
      for (int i = 0; i < 6; ++i) v += D[r + 9 * i] * sc.gl[6 * e + i];
      tmp[r] = v;
    }
    for (int k = 0; k < 4; ++k) {
      double o[3];
      jloc_t(&sc.dX[12 * e], k, tmp, o);
      for (int d = 0; d < 3; ++d) rfull[3 * sc.T[4 * e + k] + d] -= sc.vol[e] * o[d];
    }
  }
  sc.rhs.assign(3 * sc.nfree, 0.0);
  for (int v = 0; v < sc.nv; ++v)
    if (sc.free_map[v] >= 0)
      for (int d = 0; d < 3; ++d) sc.rhs[3 * sc.free_map[v] + d] = rfull[3 * v + d];
  return status;
}

void bcsr_mul(const Scene& sc, const std::vector<double>& p, std::vector<double>& y) {
  y.assign(3 * sc.nfree, 0.0);
#pragma omp parallel for schedule(static)
  for (int r = 0; r < sc.nfree; ++r) {
    for (int i = 0; i < 3; ++i) {
      double acc = 0;
      for (int q = sc.b_ptr[r]; q < sc.b_ptr[r + 1]; ++q)
        for (int j = 0; j < 3; ++j) acc += sc.A[9 * size_t(q) + 3 * i + j] * p[3 * sc.b_col[q] + j];
      y[3 * r + i] = acc;
    }
  }
}

// Sums f(i) over [0, n) in fixed chunks whose partials are added in order,
// so the result does not depend on the thread count or schedule.
template <typename Fn>
double det_sum(long n, Fn f) {
  const long chunk = 4096;
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

// Eigen::ConjugateGradient with DiagonalPreconditioner, zero initial guess
// (the "eigen-pcg-diag" solver of linear_solver_factory.cpp:74-84).
int pcg(const Scene& sc, const std::vector<double>& rhs, std::vector<double>& x,
        int max_iter, double tol, int* iters, double* err) {
  int n = 3 * sc.nfree;
  x.assign(n, 0.0);
  std::vector<double> invdiag(n);
  for (int r = 0; r < sc.nfree; ++r) {
    int q = sc.b_ptr[r];
    while (q < sc.b_ptr[r + 1] && sc.b_col[q] != r) ++q;
    for (int d = 0; d < 3; ++d) {
      double dv = (q < sc.b_ptr[r + 1]) ? sc.A[9 * size_t(q) + 4 * d] : 0.0;
      invdiag[3 * r + d] = dv != 0 ? 1.0 / dv : 1.0;
    }
  }
  std::vector<double> r = rhs, z(n), p(n), tmp(n);
  double rhsNorm2 = dot(rhs, rhs);
  if (rhsNorm2 == 0) {
    *iters = 0;
    *err = 0;
    return MFEM_OK;
  }
  double threshold = std::max(tol * tol * rhsNorm2, std::numeric_limits<double>::min());
  double rn2 = rhsNorm2;
  if (rn2 < threshold) {
    *iters = 0;
    *err = std::sqrt(rn2 / rhsNorm2);
    return MFEM_OK;
  }
  for (int i = 0; i < n; ++i) p[i] = invdiag[i] * r[i];
  double absNew = dot(r, p);
  int it = 0;
  while (it < max_iter) {
    bcsr_mul(sc, p, tmp);
    double alpha = absNew / dot(p, tmp);
    for (int i = 0; i < n; ++i) {
      x[i] += alpha * p[i];
      r[i] -= alpha * tmp[i];
    }
    rn2 = dot(r, r);
    if (rn2 < threshold) break;
    for (int i = 0; i < n; ++i) z[i] = invdiag[i] * r[i];
    double absOld = absNew;
    absNew = dot(r, z);
    double beta = absNew / absOld;
    for (int i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
    ++it;
  }
  *iters = it;
  *err = std::sqrt(rn2 / rhsNorm2);
  return it >= max_iter ? MFEM_ERR_CG_MAXITER : MFEM_OK;
}

// MixedStretch::solve (mixed_stretch.cpp:243-259).
void local_solve(Scene& sc) {
  std::vector<double> dfull(3 * sc.nv, 0.0);
  for (int v = 0; v < sc.nv; ++v)
    if (sc.free_map[v] >= 0)
      for (int d = 0; d < 3; ++d) dfull[3 * v + d] = sc.dx[3 * sc.free_map[v] + d];
#pragma omp parallel for schedule(static)
  for (int e = 0; e < sc.nt; ++e) {
    double Jdx[9] = {0};
    for (int k = 0; k < 4; ++k)
      for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r)
          Jdx[3 * c + r] -= sc.vol[e] * sc.dX[12 * e + 3 * k + c] * dfull[3 * sc.T[4 * e + k] + r];
    const double* D = &sc.dSdF[54 * e];
    double DtJ[6];
    for (int i = 0; i < 6; ++i) {
      double v = 0;
      for (int r = 0; r < 9; ++r) v += D[r + 9 * i] * Jdx[r];
      DtJ[i] = v;
    }
    const double* Ht = &sc.Htil[36 * e];
    double la[6], w[6];
    for (int i = 0; i < 6; ++i) {
      double v = 0;
      for (int j = 0; j < 6; ++j) v += Ht[i + 6 * j] * DtJ[j];
      la[i] = -sc.gl[6 * e + i] + v;
      sc.lam[6 * e + i] = la[i];
    }
    for (int i = 0; i < 6; ++i) w[i] = kSym[i] * la[i] + sc.g[6 * e + i];
    const double* Hi = &sc.Hinv[36 * e];
    for (int i = 0; i < 6; ++i) {
      double v = 0;
      for (int j = 0; j < 6; ++j) v += Hi[i + 6 * j] * w[j];
      sc.ds[6 * e + i] = -v;
    }
  }
}

// ---------------------------------------------------------------------------
// "minres-indefinite-block" (linear_solver_factory.cpp:116-133): MINRES on the
// full (x, s, lambda) system of SystemMatrixIndefinite (linear_system.h:61-99)
// whose product is BlockMatrix (block_matrix.h:63-126).  KKT vectors are
// [x: 3 nfree (free order)][s: 6 nt][lambda: 6 nt], 6-vectors per element.
inline int kkt_size(const Scene& sc) { return 3 * sc.nfree + 12 * sc.nt; }

// K w: x rows PMP w_x - PJW (dSdF w_la); s rows vol H w_s + vol Sym w_la;
// lambda rows -dSdF^T (PJW^T w_x) + vol Sym w_s  (Displacement::product_hessian,
// MixedStretch::product_hessian / product_jacobian_x / product_jacobian_mixed,
// mixed_stretch.cpp:373-435).
void kkt_mul(const Scene& sc, const std::vector<double>& w, std::vector<double>& out) {
  const int nx = 3 * sc.nfree, ns = 6 * sc.nt;
  out.assign(kkt_size(sc), 0.0);
  for (int r = 0; r < sc.nfree; ++r)
    for (int d = 0; d < 3; ++d) {
      double acc = 0;
      for (int q = sc.b_ptr[r]; q < sc.b_ptr[r + 1]; ++q) acc += sc.b_mass[q] * w[3 * sc.b_col[q] + d];
      out[3 * r + d] = acc;
    }
  std::vector<double> xs(12 * size_t(sc.nt));  // per element: vol Jloc^T dSdF w_la, 4 vertices x 3
#pragma omp parallel for schedule(static)
  for (int e = 0; e < sc.nt; ++e) {
    const double vol = sc.vol[e];
    const double* D = &sc.dSdF[54 * size_t(e)];
    const double* H = &sc.Hm[36 * size_t(e)];
    const double* ws = &w[nx + 6 * size_t(e)];
    const double* wl = &w[nx + ns + 6 * size_t(e)];
    double Jw[9] = {0};
    for (int k = 0; k < 4; ++k) {
      const int f = sc.free_map[sc.T[4 * e + k]];
      if (f < 0) continue;
      for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) Jw[3 * c + r] += vol * sc.dX[12 * e + 3 * k + c] * w[3 * f + r];
    }
    for (int i = 0; i < 6; ++i) {
      double hs = 0, dj = 0;
      for (int j = 0; j < 6; ++j) hs += H[i + 6 * j] * ws[j];
      for (int r = 0; r < 9; ++r) dj += D[r + 9 * i] * Jw[r];
      out[nx + 6 * size_t(e) + i] = vol * hs + vol * kSym[i] * wl[i];
      out[nx + ns + 6 * size_t(e) + i] = -dj + vol * kSym[i] * ws[i];
    }
    double t9[9];
    for (int r = 0; r < 9; ++r) {
      double v = 0;
      for (int i = 0; i < 6; ++i) v += D[r + 9 * i] * wl[i];
      t9[r] = v;
    }
    for (int k = 0; k < 4; ++k) {
      double o[3];
      jloc_t(&sc.dX[12 * e], k, t9, o);
      for (int d = 0; d < 3; ++d) xs[12 * size_t(e) + 3 * k + d] = vol * o[d];
    }
  }
  for (int e = 0; e < sc.nt; ++e)
    for (int k = 0; k < 4; ++k) {
      const int f = sc.free_map[sc.T[4 * e + k]];
      if (f < 0) continue;
      for (int d = 0; d < 3; ++d) out[3 * f + d] -= xs[12 * size_t(e) + 3 * k + d];
    }
}

// Block-diagonal preconditioner P = diag(A^-1, S^-1) with A = diag(PMP, Hs)
// the (x, s) block and S = Gx^T PMP^-1 Gx + Gs Hs^-1 Gs its Schur complement
// (Hs = vol H, Gs = vol Sym, Gx = jacobian_x = -PJW C, mixed_stretch.cpp:335-371),
// each block reduced to what is local: PMP by its lumped (row-sum)
// diagonal, S by its 6x6 diagonal block per element.  The reference's
// BlockDiagonalPreconditioner (preconditioners.h:64-208) factors PMP and
// L = Gx^T Mlump^-1 Gx + 1e-8 I with sparse direct solvers, scales the s
// block as vol Hinv, and leaves out Gs Hs^-1 Gs; with those blocks MINRES's
// recursive estimate falls below 1e-4 while the direction is still wrong
// (a 6x3x3 beam: 17 iterations, dx 100% off; 7949 iterations to 1e-8),
// whereas this one reaches 1e-4 with dx within 1e-4 in a few hundred.
struct MinresPrecond {
  std::vector<double> mlinv;  // 3 per free vertex
  std::vector<double> sinv;   // 36 per element
};

void minres_precond_build(const Scene& sc, MinresPrecond& P) {
  P.mlinv.assign(3 * size_t(sc.nfree), 0.0);
  for (int r = 0; r < sc.nfree; ++r) {
    double m = 0;
    for (int q = sc.b_ptr[r]; q < sc.b_ptr[r + 1]; ++q) m += sc.b_mass[q];
    for (int d = 0; d < 3; ++d) P.mlinv[3 * r + d] = 1.0 / m;
  }
  P.sinv.assign(36 * size_t(sc.nt), 0.0);
#pragma omp parallel for schedule(static)
  for (int e = 0; e < sc.nt; ++e) {
    const double vol = sc.vol[e];
    const double* D = &sc.dSdF[54 * size_t(e)];
    const double* Hi = &sc.Hinv[36 * size_t(e)];
    double S[36];
    for (int i = 0; i < 6; ++i)
      for (int j = 0; j < 6; ++j) S[i + 6 * j] = vol * kSym[i] * Hi[i + 6 * j] * kSym[j];
    for (int k = 0; k < 4; ++k) {
      const int f = sc.free_map[sc.T[4 * e + k]];
      if (f < 0) continue;
      double G[18];  // G(:, i) = vol Jloc_k^T dSdF(:, i)
      for (int i = 0; i < 6; ++i) jloc_t(&sc.dX[12 * e], k, &D[9 * i], &G[3 * i]);
      for (int i = 0; i < 18; ++i) G[i] *= vol;
      const double mi = P.mlinv[3 * f];
      for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j)
          S[i + 6 * j] += mi * (G[3 * i] * G[3 * j] + G[3 * i + 1] * G[3 * j + 1] + G[3 * i + 2] * G[3 * j + 2]);
    }
    inverse(6, S, &P.sinv[36 * size_t(e)]);
  }
}

void minres_precond_apply(const Scene& sc, const MinresPrecond& P, const std::vector<double>& b,
                          std::vector<double>& x) {
  const int nx = 3 * sc.nfree, ns = 6 * sc.nt;
  x.assign(b.size(), 0.0);
  for (int i = 0; i < nx; ++i) x[i] = P.mlinv[i] * b[i];
#pragma omp parallel for schedule(static)
  for (int e = 0; e < sc.nt; ++e) {
    const double* Hi = &sc.Hinv[36 * size_t(e)];
    const double* Si = &P.sinv[36 * size_t(e)];
    for (int i = 0; i < 6; ++i) {
      double a = 0, c = 0;
      for (int j = 0; j < 6; ++j) {
        a += Hi[i + 6 * j] * b[nx + 6 * size_t(e) + j];
        c += Si[i + 6 * j] * b[nx + ns + 6 * size_t(e) + j];
      }
      x[nx + 6 * size_t(e) + i] = a / sc.vol[e];
      x[nx + ns + 6 * size_t(e) + i] = c;
    }
  }
}

// Preconditioned MINRES (Paige & Saunders 1975) in the form of Eigen 3.4's
// unsupported MINRES (Eigen/src/IterativeSolvers/MINRES.h, no source here):
// zero initial guess, Lanczos on the preconditioned operator, Givens
// updates, and the stopping test on the recursive estimate
// |r0|^2 prod s_k^2 < tol^2 |b|^2 with |r0| the unpreconditioned norm.
int minres(const Scene& sc, const MinresPrecond& P, const std::vector<double>& rhs,
           std::vector<double>& x, int max_iter, double tol, int* iters, double* err) {
  const int n = kkt_size(sc);
  x.assign(n, 0.0);
  const double rhsNorm2 = dot(rhs, rhs);
  if (rhsNorm2 == 0) {
    *iters = 0;
    *err = 0;
    return MFEM_OK;
  }
  const double threshold2 = tol * tol * rhsNorm2;
  std::vector<double> v_old(n), v(n, 0.0), v_new = rhs, w(n), w_new, p_oold(n), p_old(n, 0.0),
      p(n, 0.0), Kw;
  double residualNorm2 = rhsNorm2;
  minres_precond_apply(sc, P, v_new, w_new);
  double beta_new2 = dot(v_new, w_new);
  double beta_new = std::sqrt(beta_new2);
  const double beta_one = beta_new;
  double c = 1.0, c_old = 1.0, s = 0.0, s_old = 0.0, eta = 1.0;
  int it = 0;
  while (it < max_iter) {
    const double beta = beta_new;
    v_old = v;
    for (int i = 0; i < n; ++i) {
      v_new[i] /= beta_new;
      w_new[i] /= beta_new;
    }
    v = v_new;
    w = w_new;
    kkt_mul(sc, w, Kw);
    for (int i = 0; i < n; ++i) v_new[i] = Kw[i] - beta * v_old[i];
    const double alpha = dot(v_new, w);
    for (int i = 0; i < n; ++i) v_new[i] -= alpha * v[i];
    minres_precond_apply(sc, P, v_new, w_new);
    beta_new2 = dot(v_new, w_new);
    beta_new = std::sqrt(beta_new2);
    const double r2 = s * alpha + c * c_old * beta;
    const double r3 = s_old * beta;
    const double r1_hat = c * alpha - c_old * s * beta;
    const double r1 = std::sqrt(r1_hat * r1_hat + beta_new * beta_new);
    c_old = c;
    s_old = s;
    c = r1_hat / r1;
    s = beta_new / r1;
    p_oold = p_old;
    p_old = p;
    for (int i = 0; i < n; ++i) p[i] = (w[i] - r2 * p_old[i] - r3 * p_oold[i]) / r1;
    for (int i = 0; i < n; ++i) x[i] += beta_one * c * eta * p[i];
    residualNorm2 *= s * s;
    if (residualNorm2 < threshold2) break;
    eta = -s * eta;
    ++it;
  }
  *iters = it;
  *err = std::sqrt(residualNorm2 / rhsNorm2);
  return it >= max_iter ? MFEM_ERR_CG_MAXITER : MFEM_OK;
}

// SystemMatrixIndefinite::pre_solve (linear_system.h:67-86): rhs =
// [-grad_x of Displacement; -vol g; vol Sym (S - s)], the last being
// -gradient_dual = evaluate_constraint (mixed_stretch.cpp:126-131, 306-333).
void kkt_rhs(Scene& sc, std::vector<double>& rhs) {
  const int nx = 3 * sc.nfree, ns = 6 * sc.nt;
  rhs.assign(kkt_size(sc), 0.0);
  std::vector<double> full;
  sc.unproject(sc.x, full);
  const double dt = sc.dt();
  std::vector<double> xt = sc.xtilde(), diff(3 * sc.nv), Md;
  for (int i = 0; i < 3 * sc.nv; ++i) diff[i] = full[i] - xt[i] - dt * dt * sc.fext[i];
  mass_mul(sc, diff, Md);
  for (int v = 0; v < sc.nv; ++v)
    if (sc.free_map[v] >= 0)
      for (int d = 0; d < 3; ++d) rhs[3 * sc.free_map[v] + d] = -Md[3 * v + d];
  for (int e = 0; e < sc.nt; ++e)
    for (int i = 0; i < 6; ++i) {
      rhs[nx + 6 * size_t(e) + i] = -sc.vol[e] * sc.g[6 * e + i];
      rhs[nx + ns + 6 * size_t(e) + i] = sc.vol[e] * kSym[i] * (sc.Sv[6 * e + i] - sc.s[6 * e + i]);
    }
}

// SystemMatrixIndefinite::post_solve (linear_system.h:88-99): dx, ds and
// lambda straight from the solution.
int minres_solve(Scene& sc, int* iters, double* err) {
  MinresPrecond P;
  minres_precond_build(sc, P);
  std::vector<double> rhs, sol;
  kkt_rhs(sc, rhs);
  const int st = minres(sc, P, rhs, sol, sc.cg_iters, sc.cg_tol, iters, err);
  const int nx = 3 * sc.nfree, ns = 6 * sc.nt;
  sc.dx.assign(sol.begin(), sol.begin() + nx);
  for (int i = 0; i < ns; ++i) {
    sc.ds[i] = sol[nx + i];
    sc.lam[i] = sol[nx + ns + i];
  }
  return st;
}

// energy_func(alpha) of newton_optimizer.cpp:34-49.
double energy(Scene& sc, double a) {
  double dt = sc.dt(), h2 = dt * dt;
  std::vector<double> x0(sc.x.size());
  for (size_t i = 0; i < x0.size(); ++i) x0[i] = sc.x[i] + a * sc.dx[i];
  std::vector<double> full;
  sc.unproject(x0, full);
  std::vector<double> xt = sc.xtilde(), diff(3 * sc.nv), Md;
  for (int i = 0; i < 3 * sc.nv; ++i) diff[i] = full[i] - xt[i] - h2 * sc.fext[i];
  mass_mul(sc, diff, Md);
  double val = 0.5 * dot(diff, Md);
  std::vector<double> epsi(sc.nt), econ(sc.nt);
  if (sc.fem) {  // Stretch::energy (stretch.cpp:15-28), weighted by h^2 in energy_func
#pragma omp parallel for schedule(static)
    for (int e = 0; e < sc.nt; ++e) {
      double psi;
      const M3 F = sc.defgrad(full, e);
      material9(sc.mat[e], sc.mu[e], sc.la[e], F.data(), &psi, nullptr, nullptr, false);
      epsi[e] = psi * sc.vol[e];
    }
    return val + h2 * det_sum(sc.nt, [&](long e) { return epsi[e]; });
  }
#pragma omp parallel for schedule(static)
  for (int e = 0; e < sc.nt; ++e) {
    double si[6];
    for (int i = 0; i < 6; ++i) si[i] = sc.s[6 * e + i] + a * sc.ds[6 * e + i];
    epsi[e] = material_coef(sc.mat[e], sc.mu[e], sc.la[e], si).psi * sc.vol[e];
    M3 R;
    std::memcpy(R.data(), &sc.Rm[9 * e], sizeof(double) * 9);
    double st[6];
    polar(R, sc.defgrad(full, e), false, st, nullptr);
    double c = 0;
    for (int i = 0; i < 6; ++i) c += sc.lam[6 * e + i] * kSym[i] * (st[i] - si[i]);
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

int step(Scene& sc, mfem_step_stats* stats) {
  mfem_step_stats st{};
  int status = MFEM_OK;
  int i = 0;
  double E = 0, E_prev = 0, res = 0, decrement = 0;
  std::vector<double> full;
  do {
    int s1 = update_system(sc, full);
    if (s1 != MFEM_OK) status = s1;
    double rn = std::sqrt(dot(sc.rhs, sc.rhs));
    if (i == 0) st.residual0 = rn;
    st.residual = rn;
    // Newton residual test: |rhs_k| <= tol * max(|rhs_0|, |h^2 P M f|)
    if (sc.res_tol > 0 && ((i > 0 && rn <= sc.res_tol * st.residual0) ||
                           rn <= sc.res_tol * sc.load_norm))
      break;
    int iters = 0;
    double err = 0;
    if (sc.solver == MFEM_SOLVER_MINRES_ID) {
      int s2 = minres_solve(sc, &iters, &err);
      if (s2 != MFEM_OK && status == MFEM_OK) status = s2;
    } else {
      int s2 = pcg(sc, sc.rhs, sc.dx, sc.cg_iters, sc.cg_tol, &iters, &err);
      if (s2 != MFEM_OK && status == MFEM_OK) status = s2;
      if (!sc.fem) local_solve(sc);
    }
    st.cg_iterations += iters;
    st.cg_error = err;
    decrement = std::max(inf_norm(sc.dx), inf_norm(sc.ds));
    E = energy(sc, 0.0);
    res = std::fabs((E - E_prev) / (E + 1e-6));
    E_prev = E;
    // linesearch_backtracking with c = 0, p = 0.5 (linesearch.h:80-129)
    double alpha = 1.0, fx0 = E;
    int it = 0;
    while (it < sc.ls_iters) {
      double fx = energy(sc, alpha);
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
  // update_bcs, Displacement::post_solve, MixedStretch::post_solve
  bc_step(sc, sc.h);
  for (int v = 0; v < sc.nv; ++v)
    if (sc.is_fixed[v])
      for (int d = 0; d < 3; ++d) sc.b[3 * v + d] = sc.V[3 * v + d];
  sc.unproject(sc.x, full);
  std::vector<double> wx = sc.weighted(sc.xprev), vnew(3 * sc.nv);
  for (int k = 0; k < 3 * sc.nv; ++k) vnew[k] = (full[k] - wx[k]) / sc.dt();
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

Scene* create(const mfem_scene_desc* d, int* status) {
  if (!d || d->n_vertices <= 0 || d->n_tets <= 0 || !d->V_rest || !d->tets ||
      !d->mu || !d->lambda || d->bdf_order < 1 || d->bdf_order > 6) {
    *status = MFEM_ERR_INVALID;
    return nullptr;
  }
  if (d->formulation == MFEM_FORMULATION_STRETCH) {
    // Stretch has no MINRES form, and only SNH and NH define the 9-vector
    // energy (MaterialModel's default prints "unimplemented")
    bool ok = d->linear_solver != MFEM_SOLVER_MINRES_ID;
    if (d->material)
      for (int e = 0; e < d->n_tets && ok; ++e)
        ok = d->material[e] == MFEM_MATERIAL_SNH || d->material[e] == MFEM_MATERIAL_NH;
    if (!ok) {
      *status = MFEM_ERR_UNSUPPORTED;
      return nullptr;
    }
  }
  auto sc = std::make_unique<Scene>();
  sc->nv = d->n_vertices;
  sc->nt = d->n_tets;
  sc->Vref.assign(d->V_rest, d->V_rest + 3 * sc->nv);
  sc->V = d->V_init ? std::vector<double>(d->V_init, d->V_init + 3 * sc->nv) : sc->Vref;
  sc->T.assign(d->tets, d->tets + 4 * sc->nt);
  for (int v : sc->T)
    if (v < 0 || v >= sc->nv) {
      *status = MFEM_ERR_INVALID;
      return nullptr;
    }
  sc->mu.assign(d->mu, d->mu + sc->nt);
  sc->la.assign(d->lambda, d->lambda + sc->nt);
  sc->mat = d->material ? std::vector<int>(d->material, d->material + sc->nt)
                        : std::vector<int>(sc->nt, MFEM_MATERIAL_SNH);
  sc->rho = d->density ? std::vector<double>(d->density, d->density + sc->nt)
                       : std::vector<double>(sc->nt, d->density_const);
  sc->bc_type = d->bc_type;
  sc->bc_axis = d->bc_axis;
  sc->bc_ratio = d->bc_ratio;
  sc->bc_vel = d->bc_velocity;
  sc->h = d->dt;
  for (int k = 0; k < 3; ++k) sc->ext[k] = d->body_force[k];
  sc->bdf = d->bdf_order;
  sc->max_newton = d->max_newton_iterations;
  sc->ls_iters = d->max_linesearch_iterations;
  sc->cg_iters = d->max_iterative_solver_iters;
  sc->cg_tol = d->iterative_solver_tolerance;
  sc->newton_tol = d->newton_tol;
  sc->res_tol = d->newton_residual_tolerance;
  sc->solver = d->linear_solver;
  sc->fem = d->formulation == MFEM_FORMULATION_STRETCH ? 1 : 0;
  // Mesh::init_bcs
  bc_init(*sc, d->is_fixed);
  sc->free_map.assign(sc->nv, -1);
  for (int v = 0; v < sc->nv; ++v)
    if (!sc->is_fixed[v]) sc->free_map[v] = sc->nfree++;
  // volumes, dphi/dX (igl::volume, sim::linear_tetmesh_dphi_dX)
  sc->vol.resize(sc->nt);
  sc->dX.resize(12 * size_t(sc->nt));
  for (int e = 0; e < sc->nt; ++e) {
    const double* X0 = &sc->Vref[3 * sc->T[4 * e]];
    double Dm[9];
    for (int k = 1; k < 4; ++k) {
      const double* Xk = &sc->Vref[3 * sc->T[4 * e + k]];
      for (int r = 0; r < 3; ++r) Dm[r + 3 * (k - 1)] = Xk[r] - X0[r];
    }
    double Di[9];
    if (!inverse(3, Dm, Di)) {
      *status = MFEM_ERR_INVALID;
      return nullptr;
    }
    double det = Dm[0] * (Dm[4] * Dm[8] - Dm[7] * Dm[5]) - Dm[3] * (Dm[1] * Dm[8] - Dm[7] * Dm[2]) +
                 Dm[6] * (Dm[1] * Dm[5] - Dm[4] * Dm[2]);
    sc->vol[e] = std::fabs(det) / 6.0;
    for (int c = 0; c < 3; ++c) {
      double sum = 0;
      for (int k = 1; k < 4; ++k) {
        double v = Di[(k - 1) + 3 * c];  // row k-1 of Dm^{-1}
        sc->dX[12 * e + 3 * k + c] = v;
        sum += v;
      }
      sc->dX[12 * e + 0 + c] = -sum;
    }
  }
  build_mass(*sc);
  build_assembler(*sc);
  // Displacement::reset (displacement.cpp:75-98)
  std::vector<double> x0 = sc->V;
  std::vector<double> v0 = d->v_init ? std::vector<double>(d->v_init, d->v_init + 3 * sc->nv)
                                     : std::vector<double>(3 * sc->nv, 0.0);
  for (int i = 0; i < sc->bdf; ++i) {
    sc->xprev.push_front(x0);
    sc->vprev.push_front(v0);
  }
  sc->b.assign(3 * sc->nv, 0.0);
  sc->x.assign(3 * sc->nfree, 0.0);
  for (int v = 0; v < sc->nv; ++v) {
    if (sc->is_fixed[v])
      for (int k = 0; k < 3; ++k) sc->b[3 * v + k] = x0[3 * v + k];
    else
      for (int k = 0; k < 3; ++k) sc->x[3 * sc->free_map[v] + k] = x0[3 * v + k];
  }
  sc->dx.assign(3 * sc->nfree, 0.0);
  sc->fext.resize(3 * sc->nv);
  for (int v = 0; v < sc->nv; ++v)
    for (int k = 0; k < 3; ++k) sc->fext[3 * v + k] = float(sc->ext[k]);
  // |h^2 P M f|: the gravity load on the free vertices (scale of the residual test)
  {
    double acc = 0, dt2 = sc->dt() * sc->dt();
    for (int v = 0; v < sc->nv; ++v) {
      if (sc->free_map[v] < 0) continue;
      double m = 0;
      for (int q = sc->m_ptr[v]; q < sc->m_ptr[v + 1]; ++q) m += sc->m_val[q];
      for (int k = 0; k < 3; ++k) acc += (dt2 * m * sc->fext[3 * v + k]) * (dt2 * m * sc->fext[3 * v + k]);
    }
    sc->load_norm = std::sqrt(acc);
  }
  // MixedStretch::reset (mixed_stretch.cpp:261-304)
  size_t nt = sc->nt;
  sc->s.assign(6 * nt, 0);
  sc->ds.assign(6 * nt, 0);
  sc->lam.assign(6 * nt, 0);
  sc->Rm.assign(9 * nt, 0);
  sc->Sv.assign(6 * nt, 0);
  sc->dSdF.assign(54 * nt, 0);
  sc->g.assign(6 * nt, 0);
  sc->Hm.assign(36 * nt, 0);
  sc->Hinv.assign(36 * nt, 0);
  sc->Htil.assign(36 * nt, 0);
  sc->gl.assign(6 * nt, 0);
  int st = MFEM_OK;
  for (int e = 0; e < sc->nt; ++e) {
    M3 R = eye3();
    double sv[6], dsdF[54];
    int r = polar(R, sc->defgrad(x0, e), true, sv, dsdF);
    if (r != MFEM_OK) st = r;
    std::memcpy(&sc->Rm[9 * e], R.data(), sizeof(double) * 9);
    for (int i = 0; i < 6; ++i) sc->s[6 * e + i] = sc->Sv[6 * e + i] = sv[i];
    for (int i = 0; i < 36; ++i) sc->Hm[36 * e + i] = sc->Hinv[36 * e + i] = (i % 7 == 0);
  }
  *status = st;
  return sc.release();
}

}  // namespace

extern "C" {

int oracle_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}
int oracle_get_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

int oracle_procrustes(double* R, const double* A, const double* B,
                      int compute_gradients, double* dRdF, double tol,
                      int max_iter, int* iterations) {
  M3 Rm, Am, Bm;
  std::memcpy(Rm.data(), R, 72);
  std::memcpy(Am.data(), A, 72);
  std::memcpy(Bm.data(), B, 72);
  double tmp[81];
  int st = procrustes(Rm, Am, Bm, compute_gradients != 0, dRdF ? dRdF : tmp, tol,
                      max_iter, iterations);
  std::memcpy(R, Rm.data(), 72);
  return st;
}

int oracle_polar(double* R, const double* F, int compute_gradients, double* s,
                 double* dsdF) {
  M3 Rm, Fm;
  std::memcpy(Rm.data(), R, 72);
  std::memcpy(Fm.data(), F, 72);
  double tmp[54];
  int st = polar(Rm, Fm, compute_gradients != 0, s, dsdF ? dsdF : tmp);
  std::memcpy(R, Rm.data(), 72);
  return st;
}

// SVD by the symmetric eigen-decomposition of F^T F (Jacobi), then dR/dF as
// in dsvd (src/svd/dsvd.cpp:69-138): d_ij = 1/(s_j^2 - s_i^2), set to 0 when
// |s_j^2 - s_i^2| < 1e-5.  (The reference perturbs F randomly when two
// singular values are within 1e-5; that branch is not restated.)
int oracle_dsvd_dRdF(const double* Fp, double* dRdF) {
  M3 F;
  std::memcpy(F.data(), Fp, 72);
  M3 C = mul(transpose(F), F);
  double a[9], V[9];
  std::memcpy(a, C.data(), 72);
  // Jacobi eigen of the 3x3 symmetric C with vectors in V
  for (int i = 0; i < 9; ++i) V[i] = (i % 4 == 0);
  for (int sweep = 0; sweep < 64; ++sweep) {
    double off = a[3] * a[3] + a[6] * a[6] + a[7] * a[7];
    if (off < 1e-32) break;
    for (int p = 0; p < 3; ++p)
      for (int q = p + 1; q < 3; ++q) {
        double apq = a[p + 3 * q];
        if (apq == 0) continue;
        double theta = (a[q + 3 * q] - a[p + 3 * p]) / (2 * apq);
        double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1));
        double c = 1 / std::sqrt(t * t + 1), sn = t * c;
        for (int k = 0; k < 3; ++k) {
          double akp = a[k + 3 * p], akq = a[k + 3 * q];
          a[k + 3 * p] = c * akp - sn * akq;
          a[k + 3 * q] = sn * akp + c * akq;
        }
        for (int k = 0; k < 3; ++k) {
          double apk = a[p + 3 * k], aqk = a[q + 3 * k];
          a[p + 3 * k] = c * apk - sn * aqk;
          a[q + 3 * k] = sn * apk + c * aqk;
        }
        for (int k = 0; k < 3; ++k) {
          double vkp = V[k + 3 * p], vkq = V[k + 3 * q];
          V[k + 3 * p] = c * vkp - sn * vkq;
          V[k + 3 * q] = sn * vkp + c * vkq;
        }
      }
  }
  // sort descending (JacobiSVD order)
  int idx[3] = {0, 1, 2};
  std::sort(idx, idx + 3, [&](int u, int w) { return a[u * 4] > a[w * 4]; });
  M3 Vm, U;
  double S[3];
  for (int j = 0; j < 3; ++j) {
    S[j] = std::sqrt(std::max(a[idx[j] * 4], 0.0));
    for (int r = 0; r < 3; ++r) at(Vm, r, j) = V[r + 3 * idx[j]];
  }
  M3 FV = mul(F, Vm);
  for (int j = 0; j < 3; ++j)
    for (int r = 0; r < 3; ++r) at(U, r, j) = at(FV, r, j) / S[j];
  const double tol = 1e-5;
  double d01 = S[1] * S[1] - S[0] * S[0], d02 = S[2] * S[2] - S[0] * S[0],
         d12 = S[2] * S[2] - S[1] * S[1];
  d01 = std::fabs(d01) < tol ? 0.0 : 1.0 / d01;
  d02 = std::fabs(d02) < tol ? 0.0 : 1.0 / d02;
  d12 = std::fabs(d12) < tol ? 0.0 : 1.0 / d12;
  for (int r = 0; r < 3; ++r)
    for (int s = 0; s < 3; ++s) {
      M3 UVT{};
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) at(UVT, i, j) = at(U, r, i) * at(Vm, s, j);
      for (int i = 0; i < 3; ++i) at(UVT, i, i) = 0;
      M3 t1{}, t2{};
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          at(t1, i, j) = S[i] * at(UVT, i, j) + at(UVT, j, i) * S[j];
          at(t2, i, j) = at(UVT, i, j) * S[j] + S[i] * at(UVT, j, i);
        }
      double w01 = at(t1, 0, 1) * d01, w02 = at(t1, 0, 2) * d02, w12 = at(t1, 1, 2) * d12;
      M3 Wv{};
      at(Wv, 0, 1) = w01; at(Wv, 0, 2) = w02; at(Wv, 1, 2) = w12;
      at(Wv, 1, 0) = -w01; at(Wv, 2, 0) = -w02; at(Wv, 2, 1) = -w12;
      M3 dV = mul(Vm, Wv);
      w01 = at(t2, 0, 1) * d01; w02 = at(t2, 0, 2) * d02; w12 = at(t2, 1, 2) * d12;
      M3 Wu{};
      at(Wu, 0, 1) = w01; at(Wu, 0, 2) = w02; at(Wu, 1, 2) = w12;
      at(Wu, 1, 0) = -w01; at(Wu, 2, 0) = -w02; at(Wu, 2, 1) = -w12;
      M3 dU = mul(U, Wu);
      M3 dR = mul(dU, transpose(Vm)), t3 = mul(U, transpose(dV));
      for (int i = 0; i < 9; ++i) dRdF[i + 9 * (3 * s + r)] = dR[i] + t3[i];
    }
  return MFEM_OK;
}

double oracle_material_energy(int type, double mu, double la, const double* s) {
  return material_coef(type, mu, la, s).psi;
}
void oracle_material_gradient(int type, double mu, double la, const double* s, double* g) {
  material_gradient(type, mu, la, s, g);
}
void oracle_material_hessian(int type, double mu, double la, const double* s, int fix, double* H) {
  material_hessian(type, mu, la, s, fix != 0, H);
}
void oracle_psd_fix(double* H, int n, double tol) { psd_fix(H, n, tol); }
double oracle_material9(int type, double mu, double la, const double* F, double* g, double* H, int fix) {
  double psi = 0;
  material9(type, mu, la, F, &psi, g, H, fix != 0);
  return psi;
}

void* oracle_scene_create(const mfem_scene_desc* desc, int* status) {
  int st = MFEM_OK;
  Scene* s = create(desc, &st);
  if (status) *status = st;
  return s;
}
void oracle_scene_destroy(void* scene) { delete static_cast<Scene*>(scene); }
int oracle_scene_step(void* scene, mfem_step_stats* stats) {
  return step(*static_cast<Scene*>(scene), stats);
}
int oracle_scene_sizes(void* scene, int* nv, int* nt, int* nfree, int* nnzb) {
  Scene& sc = *static_cast<Scene*>(scene);
  if (nv) *nv = sc.nv;
  if (nt) *nt = sc.nt;
  if (nfree) *nfree = sc.nfree;
  if (nnzb) *nnzb = int(sc.b_col.size());
  return MFEM_OK;
}
int oracle_scene_get_state(void* scene, double* x, double* v, double* s, double* R,
                           double* la) {
  Scene& sc = *static_cast<Scene*>(scene);
  if (x) {
    std::vector<double> full;
    sc.unproject(sc.x, full);
    std::memcpy(x, full.data(), 8 * full.size());
  }
  if (v) std::memcpy(v, sc.vprev.front().data(), 8 * 3 * size_t(sc.nv));
  if (s) std::memcpy(s, sc.s.data(), 8 * sc.s.size());
  if (R) std::memcpy(R, sc.Rm.data(), 8 * sc.Rm.size());
  if (la) std::memcpy(la, sc.lam.data(), 8 * sc.lam.size());
  return MFEM_OK;
}
int oracle_scene_set_state(void* scene, const double* x, const double* v,
                           const double* s, const double* R, const double* la) {
  Scene& sc = *static_cast<Scene*>(scene);
  if (x) {
    for (int vv = 0; vv < sc.nv; ++vv)
      for (int d = 0; d < 3; ++d) {
        if (sc.free_map[vv] >= 0)
          sc.x[3 * sc.free_map[vv] + d] = x[3 * vv + d];
        else
          sc.b[3 * vv + d] = x[3 * vv + d];
      }
    sc.V.assign(x, x + 3 * sc.nv);
    sc.xprev.front().assign(x, x + 3 * sc.nv);
  }
  if (v) sc.vprev.front().assign(v, v + 3 * sc.nv);
  if (s) sc.s.assign(s, s + sc.s.size());
  if (R) sc.Rm.assign(R, R + sc.Rm.size());
  if (la) sc.lam.assign(la, la + sc.lam.size());
  return MFEM_OK;
}
int oracle_scene_set_positions(void* scene, const double* x) {
  Scene& sc = *static_cast<Scene*>(scene);
  for (int vv = 0; vv < sc.nv; ++vv)
    for (int d = 0; d < 3; ++d) {
      if (sc.free_map[vv] >= 0)
        sc.x[3 * sc.free_map[vv] + d] = x[3 * vv + d];
      else
        sc.b[3 * vv + d] = x[3 * vv + d];
    }
  return MFEM_OK;
}
int oracle_scene_elem_update(void* scene, const double* x, double h, double* R,
                             double* S, double* dSdF, double* g, double* H,
                             double* Hinv, double* Aloc, double* gl) {
  Scene& sc = *static_cast<Scene*>(scene);
  std::vector<double> full(x, x + 3 * sc.nv);
  std::vector<double> Al(144 * size_t(sc.nt));
  int status = MFEM_OK;
  for (int e = 0; e < sc.nt; ++e) {
    int st = elem_update(sc, e, full, h, &Al[144 * size_t(e)]);
    if (st != MFEM_OK) status = st;
  }
  size_t nt = sc.nt;
  if (R) std::memcpy(R, sc.Rm.data(), 8 * 9 * nt);
  if (S) std::memcpy(S, sc.Sv.data(), 8 * 6 * nt);
  if (dSdF) std::memcpy(dSdF, sc.dSdF.data(), 8 * 54 * nt);
  if (g) std::memcpy(g, sc.g.data(), 8 * 6 * nt);
  if (H) std::memcpy(H, sc.Hm.data(), 8 * 36 * nt);
  if (Hinv) std::memcpy(Hinv, sc.Hinv.data(), 8 * 36 * nt);
  if (Aloc) std::memcpy(Aloc, Al.data(), 8 * 144 * nt);
  if (gl) std::memcpy(gl, sc.gl.data(), 8 * 6 * nt);
  return status;
}
int oracle_scene_get_system(void* scene, int* row_ptr, int* col, double* val,
                            double* rhs) {
  Scene& sc = *static_cast<Scene*>(scene);
  std::vector<double> full;
  update_system(sc, full);
  if (row_ptr) std::memcpy(row_ptr, sc.b_ptr.data(), 4 * sc.b_ptr.size());
  if (col) std::memcpy(col, sc.b_col.data(), 4 * sc.b_col.size());
  if (val) std::memcpy(val, sc.A.data(), 8 * sc.A.size());
  if (rhs) std::memcpy(rhs, sc.rhs.data(), 8 * sc.rhs.size());
  return MFEM_OK;
}
double oracle_scene_energy(void* scene, double alpha) {
  return energy(*static_cast<Scene*>(scene), alpha);
}
int oracle_scene_pcg(void* scene, const double* b, double* x, int* iters,
                     double* rel_residual) {
  Scene& sc = *static_cast<Scene*>(scene);
  std::vector<double> rhs(b, b + 3 * sc.nfree), xo;
  int st = pcg(sc, rhs, xo, sc.cg_iters, sc.cg_tol, iters, rel_residual);
  std::memcpy(x, xo.data(), 8 * xo.size());
  return st;
}

// The (x, s, lambda) system of "minres-indefinite-block" at the state of the
// last update_system / elem_update: rhs (kkt_size), and out = K w.
int oracle_scene_kkt_size(void* scene) { return kkt_size(*static_cast<Scene*>(scene)); }
int oracle_scene_kkt_rhs(void* scene, double* rhs) {
  Scene& sc = *static_cast<Scene*>(scene);
  std::vector<double> r;
  kkt_rhs(sc, r);
  std::memcpy(rhs, r.data(), 8 * r.size());
  return MFEM_OK;
}
int oracle_scene_kkt_mul(void* scene, const double* w, double* out) {
  Scene& sc = *static_cast<Scene*>(scene);
  std::vector<double> wi(w, w + kkt_size(sc)), o;
  kkt_mul(sc, wi, o);
  std::memcpy(out, o.data(), 8 * o.size());
  return MFEM_OK;
}
// MINRES on that system; x = [dx; ds; lambda].
int oracle_scene_minres(void* scene, const double* b, double* x, int* iters, double* rel) {
  Scene& sc = *static_cast<Scene*>(scene);
  MinresPrecond P;
  minres_precond_build(sc, P);
  std::vector<double> rhs(b, b + kkt_size(sc)), xo;
  int st = minres(sc, P, rhs, xo, sc.cg_iters, sc.cg_tol, iters, rel);
  std::memcpy(x, xo.data(), 8 * xo.size());
  return st;
}
// The reduced path on the same state: PCG on the Schur system then
// MixedStretch::solve; x = [dx; ds; lambda].
int oracle_scene_schur_solve(void* scene, double* x, int* iters, double* rel) {
  Scene& sc = *static_cast<Scene*>(scene);
  int st = pcg(sc, sc.rhs, sc.dx, sc.cg_iters, sc.cg_tol, iters, rel);
  local_solve(sc);
  const int nx = 3 * sc.nfree, ns = 6 * sc.nt;
  std::memcpy(x, sc.dx.data(), 8 * nx);
  std::memcpy(x + nx, sc.ds.data(), 8 * ns);
  std::memcpy(x + nx + ns, sc.lam.data(), 8 * ns);
  return st;
}
// update_system at the current positions (K1-K3 of one Newton iteration).
int oracle_scene_update_system(void* scene) {
  Scene& sc = *static_cast<Scene*>(scene);
  std::vector<double> full;
  return update_system(sc, full);
}

}  // extern "C"
