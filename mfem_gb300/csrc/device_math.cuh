// Per-element device math for the mixed-stretch Newton step: 3x3 polar
// rotation by Newton on SO(3), the closed-form derivative of the stretch s
// with respect to F, the six material models on the 6-vector s, and the
// positive-semidefinite projection of their Hessians.  Every routine is
// templated on Real (float for the mixed-precision path, double for the
// all-FP64 path) and keeps its small matrices in registers.
//
// Conventions (those of the reference): 3x3 matrices column-major, m[r+3c];
// s = [S00, S11, S22, S01, S02, S12] (src/variables/mixed_stretch.cpp:26-29);
// Sym = diag(1,1,1,2,2,2), Syminv = diag(1,1,1,.5,.5,.5) (mixed_stretch.h:120-138).
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "df64.cuh"

namespace mfem_gpu {

template <typename T> struct Prec;
template <> struct Prec<float> {
  static constexpr bool kFP64 = false;
  __device__ static float sqrt_(float x) { return sqrtf(x); }
  __device__ static float rsqrt_(float x) { return rsqrtf(x); }
  __device__ static void sincos_(float x, float* s, float* c) { sincosf(x, s, c); }
  __device__ static float log_(float x) { return logf(x); }
  __device__ static float exp_(float x) { return expf(x); }
};
template <> struct Prec<double> {
  static constexpr bool kFP64 = true;
  __device__ static double sqrt_(double x) { return sqrt(x); }
  __device__ static double rsqrt_(double x) { return rsqrt(x); }
  __device__ static void sincos_(double x, double* s, double* c) { sincos(x, s, c); }
  __device__ static double log_(double x) { return log(x); }
  __device__ static double exp_(double x) { return exp(x); }
};

template <> struct Prec<df64> {
  static constexpr bool kFP64 = true;
  __device__ static df64 sqrt_(df64 x) {
    const float s = sqrtf(x.hi);
    if (s == 0.f) return df64(0.f);
    return df64(s) + (x - two_prod(s, s)) / df64(2.f * s);
  }
  __device__ static df64 log_(df64 x) { return df64(log(x.to_double())); }
  __device__ static df64 exp_(df64 x) { return df64(exp(x.to_double())); }
};

#define MI __device__ __forceinline__

// acc + a b; float-float has its own one-pass form (df64.cuh).
template <typename T> MI T madd(T acc, T a, T b) { return acc + a * b; }

// ---------------------------------------------------------------- 3x3 ----
template <typename T> MI T tr_AB(const T* A, const T* B) {  // tr(A*B)
  T s = 0;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) s += A[i + 3 * j] * B[j + 3 * i];
  return s;
}
template <typename T> MI void mul33(const T* A, const T* B, T* C) {  // C = A*B
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      C[i + 3 * j] = madd(madd(A[i] * B[3 * j], A[i + 3], B[1 + 3 * j]), A[i + 6], B[2 + 3 * j]);
}
template <typename T> MI void mulAtB(const T* A, const T* B, T* C) {  // C = A^T*B
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      C[i + 3 * j] = madd(madd(A[3 * i] * B[3 * j], A[1 + 3 * i], B[1 + 3 * j]), A[2 + 3 * i], B[2 + 3 * j]);
}
template <typename T> MI void mulABt(const T* A, const T* B, T* C) {  // C = A*B^T
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      C[i + 3 * j] = madd(madd(A[i] * B[j], A[i + 3], B[j + 3]), A[i + 6], B[j + 6]);
}

// Rotation <-> unit quaternion (w, x, y, z).  Rotations are stored as
// quaternions so that every reload is exactly orthonormal.
template <typename T> MI void quat_to_rot(const T q_in[4], T* R) {
  T w = q_in[0], x = q_in[1], y = q_in[2], z = q_in[3];
  T n = w * w + x * x + y * y + z * z;
  T s = n > T(0) ? T(2) / n : T(0);
  R[0] = T(1) - s * (y * y + z * z);
  R[3] = s * (x * y - w * z);
  R[6] = s * (x * z + w * y);
  R[1] = s * (x * y + w * z);
  R[4] = T(1) - s * (x * x + z * z);
  R[7] = s * (y * z - w * x);
  R[2] = s * (x * z - w * y);
  R[5] = s * (y * z + w * x);
  R[8] = T(1) - s * (x * x + y * y);
}
// The rotation of a float quaternion in float-float: the ten products of its
// components are exact (TwoProduct), so only the normalisation 2 / |q|^2 and
// the combinations round -- the same entries as quat_to_rot on the
// float-float quaternion, without its products of zero low parts.
MI void quat_to_rot_df(const float q[4], df64* R) {
  const float w = q[0], x = q[1], y = q[2], z = q[3];
  const df64 ww = two_prod(w, w), xx = two_prod(x, x), yy = two_prod(y, y), zz = two_prod(z, z);
  const df64 xy = two_prod(x, y), xz = two_prod(x, z), yz = two_prod(y, z);
  const df64 wx = two_prod(w, x), wy = two_prod(w, y), wz = two_prod(w, z);
  const df64 n = ww + xx + yy + zz;
  const df64 s = n.hi > 0.f ? df64(2.f) / n : df64(0.f);
  R[0] = df64(1.f) - s * (yy + zz);
  R[3] = s * (xy - wz);
  R[6] = s * (xz + wy);
  R[1] = s * (xy + wz);
  R[4] = df64(1.f) - s * (xx + zz);
  R[7] = s * (yz - wx);
  R[2] = s * (xz - wy);
  R[5] = s * (yz + wx);
  R[8] = df64(1.f) - s * (xx + yy);
}
template <typename T> MI void rot_to_quat(const T* R, T q[4]) {
  T t = R[0] + R[4] + R[8];
  if (t > T(0)) {
    T s = Prec<T>::sqrt_(t + T(1)) * T(2);
    q[0] = T(0.25) * s;
    q[1] = (R[5] - R[7]) / s;
    q[2] = (R[6] - R[2]) / s;
    q[3] = (R[1] - R[3]) / s;
  } else if (R[0] > R[4] && R[0] > R[8]) {
    T s = Prec<T>::sqrt_(T(1) + R[0] - R[4] - R[8]) * T(2);
    q[0] = (R[5] - R[7]) / s;
    q[1] = T(0.25) * s;
    q[2] = (R[3] + R[1]) / s;
    q[3] = (R[6] + R[2]) / s;
  } else if (R[4] > R[8]) {
    T s = Prec<T>::sqrt_(T(1) + R[4] - R[0] - R[8]) * T(2);
    q[0] = (R[6] - R[2]) / s;
    q[1] = (R[3] + R[1]) / s;
    q[2] = T(0.25) * s;
    q[3] = (R[7] + R[5]) / s;
  } else {
    T s = Prec<T>::sqrt_(T(1) + R[8] - R[0] - R[4]) * T(2);
    q[0] = (R[1] - R[3]) / s;
    q[1] = (R[6] + R[2]) / s;
    q[2] = (R[7] + R[5]) / s;
    q[3] = T(0.25) * s;
  }
  T n = Prec<T>::rsqrt_(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
#pragma unroll
  for (int i = 0; i < 4; ++i) q[i] *= n;
}

// rodrigues (src/svd/newton_procrustes.h:87-106): R = I + sin|w| K + (1-cos|w|) K^2.
template <typename T> MI void rodrigues(const T w[3], T* R) {
  T a2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
  T angle = Prec<T>::sqrt_(a2);
#pragma unroll
  for (int i = 0; i < 9; ++i) R[i] = (i % 4 == 0) ? T(1) : T(0);
  if (angle < T(1e-8)) return;
  T inv = T(1) / angle;
  T k0 = w[0] * inv, k1 = w[1] * inv, k2 = w[2] * inv;
  T sa, ca;
  Prec<T>::sincos_(angle, &sa, &ca);
  T c1 = T(1) - ca;
  // K = [k]x ; K^2 = k k^T - I
  R[0] += c1 * (k0 * k0 - T(1));
  R[4] += c1 * (k1 * k1 - T(1));
  R[8] += c1 * (k2 * k2 - T(1));
  R[3] += -sa * k2 + c1 * k0 * k1;  // (0,1)
  R[1] += sa * k2 + c1 * k0 * k1;   // (1,0)
  R[6] += sa * k1 + c1 * k0 * k2;   // (0,2)
  R[2] += -sa * k1 + c1 * k0 * k2;  // (2,0)
  R[7] += -sa * k0 + c1 * k1 * k2;  // (1,2)
  R[5] += sa * k0 + c1 * k1 * k2;   // (2,1)
}

// Solve the symmetric 3x3 system H x = b (H given as xx,yy,zz,xy,xz,yz) by
// its adjugate; returns false when H is numerically singular.
template <typename T> MI bool solve_sym3(const T h[6], const T b[3], T x[3]) {
  T a00 = h[1] * h[2] - h[5] * h[5];
  T a01 = h[4] * h[5] - h[3] * h[2];
  T a02 = h[3] * h[5] - h[4] * h[1];
  T a11 = h[0] * h[2] - h[4] * h[4];
  T a12 = h[3] * h[4] - h[0] * h[5];
  T a22 = h[0] * h[1] - h[3] * h[3];
  T det = h[0] * a00 + h[3] * a01 + h[4] * a02;
  T scale = fabs(h[0]) + fabs(h[1]) + fabs(h[2]) + T(2) * (fabs(h[3]) + fabs(h[4]) + fabs(h[5]));
  T tiny = (Prec<T>::kFP64 ? T(1e-14) : T(1e-6)) * scale * scale * scale;
  if (!(fabs(det) > tiny)) return false;
  T id = T(1) / det;
  x[0] = (a00 * b[0] + a01 * b[1] + a02 * b[2]) * id;
  x[1] = (a01 * b[0] + a11 * b[1] + a12 * b[2]) * id;
  x[2] = (a02 * b[0] + a12 * b[1] + a22 * b[2]) * id;
  return true;
}

// The same solve in float-float: an FP32 solve and one correction from the
// float-float residual b - h x0 (one step of iterative refinement).  With
// h = tr(S) I - S (condition number the ratio of the largest to the
// smallest sum of two principal stretches) the error after it is about the
// square of FP32's, below the float-float resolution of what it feeds.
MI bool solve_sym3(const df64 h[6], const df64 b[3], df64 x[3]) {
  const float hf[6] = {h[0].hi, h[1].hi, h[2].hi, h[3].hi, h[4].hi, h[5].hi};
  const float bf[3] = {b[0].hi, b[1].hi, b[2].hi};
  float x0[3], dx[3];
  if (!solve_sym3(hf, bf, x0)) return false;
  const df64 r[3] = {b[0] - (h[0] * df64(x0[0]) + h[3] * df64(x0[1]) + h[4] * df64(x0[2])),
                     b[1] - (h[3] * df64(x0[0]) + h[1] * df64(x0[1]) + h[5] * df64(x0[2])),
                     b[2] - (h[4] * df64(x0[0]) + h[5] * df64(x0[1]) + h[2] * df64(x0[2]))};
  const float rf[3] = {r[0].hi, r[1].hi, r[2].hi};
  solve_sym3(hf, rf, dx);
#pragma unroll
  for (int i = 0; i < 3; ++i) x[i] = two_sum(x0[i], dx[i]);
  return true;
}

// Gradient g_k = -tr(cp_k Y) and Hessian H_kl = -tr(cp_kl Y) of the
// Procrustes energy (newton_procrustes.h:128,136-138), written out:
// g is the axial part of Y and H = tr(sym Y) I - sym Y.
template <typename T> MI void procrustes_gH(const T* Y, T g[3], T h[6]) {
  g[0] = Y[5] - Y[7];  // Y21 - Y12
  g[1] = Y[6] - Y[2];  // Y02 - Y20
  g[2] = Y[1] - Y[3];  // Y10 - Y01
  T t = Y[0] + Y[4] + Y[8];
  h[0] = t - Y[0];
  h[1] = t - Y[4];
  h[2] = t - Y[8];
  h[3] = T(-0.5) * (Y[3] + Y[1]);
  h[4] = T(-0.5) * (Y[6] + Y[2]);
  h[5] = T(-0.5) * (Y[7] + Y[5]);
}

// newton_procrustes with A = I, B = F (src/svd/newton_procrustes.h:108-159):
// R (warm start in, rotation out) minimising |R - F|_F.  tol is the
// reference's 1e-6 on |g| (mixed_stretch.cpp:21-22); in FP32 it is raised to
// the rounding floor of |g|, and the 0.6-backtracking energy test is skipped
// once |omega| < 4e-3, where a Newton step on this convex problem always
// decreases the energy and the FP32 energy difference is below rounding.
// Returns the iteration count, or -1 if the rotation Hessian was singular.
template <typename T> MI int procrustes(T* R, const T* F, T tol, int max_iter) {
  T Y[9];
  mulABt(R, F, Y);  // Y = R*A*B^T with A = I
  if (!Prec<T>::kFP64) {
    T fn = 0;
#pragma unroll
    for (int i = 0; i < 9; ++i) fn += F[i] * F[i];
    T floor_ = T(8) * T(1.1920929e-7) * Prec<T>::sqrt_(fn);
    tol = tol > floor_ ? tol : floor_;
  }
  int it = 0;
  bool singular = false;
  for (; it < max_iter;) {
    T g[3], h[6];
    procrustes_gH(Y, g, h);
    T gn2 = g[0] * g[0] + g[1] * g[1] + g[2] * g[2];
    if (gn2 < tol * tol) break;
    T om[3];
    if (!solve_sym3(h, g, om)) {
      singular = true;
      T tr = h[0] + h[1] + h[2];
      T inv = T(1) / (fabs(tr) + T(1));
      om[0] = g[0] * inv;
      om[1] = g[1] * inv;
      om[2] = g[2] * inv;
    }
    om[0] = -om[0];
    om[1] = -om[1];
    om[2] = -om[2];
    T dR[9];
    T on2 = om[0] * om[0] + om[1] * om[1] + om[2] * om[2];
    if (!Prec<T>::kFP64 && on2 < T(1.6e-5)) {
      rodrigues(om, dR);
    } else {
      T E0 = -tr_AB(R, Y);  // as newton_procrustes.h:142
      T E1;
      do {
        rodrigues(om, dR);
        E1 = -tr_AB(dR, Y);
        om[0] *= T(0.6);
        om[1] *= T(0.6);
        om[2] *= T(0.6);
        on2 = om[0] * om[0] + om[1] * om[1] + om[2] * om[2];
      } while (E1 > E0 && on2 > tol * tol);
    }
    T tmp[9];
    mul33(dR, R, tmp);
#pragma unroll
    for (int i = 0; i < 9; ++i) R[i] = tmp[i];
    mul33(dR, Y, tmp);
#pragma unroll
    for (int i = 0; i < 9; ++i) Y[i] = tmp[i];
    ++it;
  }
  return singular ? -1 : it;
}

// s-vector of S = R^T F (mixed_stretch.cpp:25-29).
template <typename T> MI void stretch_vec(const T* R, const T* F, T s[6]) {
  T S[9];
  mulAtB(R, F, S);
  s[0] = S[0];
  s[1] = S[4];
  s[2] = S[8];
  s[3] = T(0.5) * (S[1] + S[3]);
  s[4] = T(0.5) * (S[2] + S[6]);
  s[5] = T(0.5) * (S[5] + S[7]);
}

// Closed-form ds/dF at the polar optimum.  With S symmetric, F = R S and
// W = (tr(S) I - S)^{-1}, the derivative of s_i with respect to F is
//   ds_i/dF = R (E_i - [u_i]x),  u_i = W c_i,  c_{i,m} = <E_i, [e_m]x S>,
// E_i the selector of s_i.  This is the product
// (I(x)R^T)(I - (S^T(x)I) dR/dF) of mixed_stretch.cpp:32-41 with dR/dF of
// newton_procrustes.h:161-187 evaluated analytically.  Output: u[6][3];
// returns false if tr(S) I - S is singular (the reference exits there).
template <typename T> MI bool stretch_derivative_u(const T s[6], T u[18]) {
  // M = tr(S) I - S (symmetric)
  T t = s[0] + s[1] + s[2];
  T m[6] = {t - s[0], t - s[1], t - s[2], -s[3], -s[4], -s[5]};
  // c_i vectors (rows), from S entries: S00=s0, S11=s1, S22=s2, S01=s3, S02=s4, S12=s5
  T c[18] = {T(0), s[4], -s[3],                                  // i=0
             -s[5], T(0), s[3],                                  // i=1
             s[5], -s[4], T(0),                                  // i=2
             T(-0.5) * s[4], T(0.5) * s[5], T(0.5) * (s[0] - s[1]),  // i=3
             T(0.5) * s[3], T(0.5) * (s[2] - s[0]), T(-0.5) * s[5],  // i=4
             T(0.5) * (s[1] - s[2]), T(-0.5) * s[3], T(0.5) * s[4]}; // i=5
  bool ok = true;
#pragma unroll
  for (int i = 0; i < 6; ++i) ok = solve_sym3(m, &c[3 * i], &u[3 * i]) && ok;
  if (!ok) {
#pragma unroll
    for (int i = 0; i < 18; ++i) u[i] = T(0);
  }
  return ok;
}

// <E_i - [u_i]x, M> for all six i, M a 3x3 matrix in the rotated frame.
template <typename T> MI void ds_dot(const T u[18], const T* M, T out[6]) {
  T a0 = M[5] - M[7], a1 = M[6] - M[2], a2 = M[1] - M[3];  // axial part
  T e[6] = {M[0], M[4], M[8], T(0.5) * (M[1] + M[3]), T(0.5) * (M[2] + M[6]),
            T(0.5) * (M[5] + M[7])};
#pragma unroll
  for (int i = 0; i < 6; ++i) out[i] = e[i] - (u[3 * i] * a0 + u[3 * i + 1] * a1 + u[3 * i + 2] * a2);
}

// G_i = ds_i/dF = R (E_i - [u_i]x), 3x3 column-major each (G[9*i + r + 3c]).
template <typename T> MI void ds_dF(const T* R, const T u[18], T G[54]) {
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    T D[9];
    const T u0 = u[3 * i], u1 = u[3 * i + 1], u2 = u[3 * i + 2];
    // -[u]x
    D[0] = 0; D[4] = 0; D[8] = 0;
    D[3] = u2;  D[6] = -u1;  // (0,1), (0,2)
    D[1] = -u2; D[7] = u0;   // (1,0), (1,2)
    D[2] = u1;  D[5] = -u0;  // (2,0), (2,1)
    if (i < 3) {
      D[4 * i] += T(1);
    } else {
      int p = (i == 5) ? 1 : 0, q = (i == 3) ? 1 : 2;
      D[p + 3 * q] += T(0.5);
      D[q + 3 * p] += T(0.5);
    }
    mul33(R, D, &G[9 * i]);
  }
}

// ------------------------------------------------------------ materials ---
// psi = A(Q) + B(J) + C(t) with Q = |S|_F^2, J = det S, t = tr S; this is
// the expression of every Vector6d energy of src/energies/*.cpp.
enum { kSNH = 0, kNH = 1, kCOROT = 2, kFCR = 3, kARAP = 4, kFUNG = 5 };

template <typename T> struct MatCoef {
  T psi, A1, A2, B1, B2, C1, C2;
  bool psd;
};

template <typename T> MI void invariants(const T* s, T& Q, T& J, T& t, T dJ[6]) {
  Q = madd(madd(s[0] * s[0], s[1], s[1]), s[2], s[2]) +
      T(2) * madd(madd(s[3] * s[3], s[4], s[4]), s[5], s[5]);
  t = s[0] + s[1] + s[2];
  const T c0 = madd(s[1] * s[2], -s[5], s[5]), c3 = madd(s[4] * s[5], -s[2], s[3]),
          c4 = madd(s[3] * s[5], -s[1], s[4]);
  dJ[0] = c0;
  dJ[1] = madd(s[0] * s[2], -s[4], s[4]);
  dJ[2] = madd(s[0] * s[1], -s[3], s[3]);
  dJ[3] = T(2) * c3;
  dJ[4] = T(2) * c4;
  dJ[5] = T(2) * madd(s[3] * s[4], -s[0], s[5]);
  // det S by cofactors of its first row
  J = madd(madd(s[0] * c0, s[3], c3), s[4], c4);
}

template <typename T>
MI MatCoef<T> material_coef(int type, T mu, T la, T Q, T J, T t, bool need_psi) {
  MatCoef<T> c{T(0), T(0), T(0), T(0), T(0), T(0), T(0), false};
  switch (type) {
    case kNH: {  // neohookean.cpp:8-94
      T lj = Prec<T>::log_(J);
      if (need_psi) c.psi = -mu * lj + T(0.5) * la * lj * lj + T(0.5) * mu * (Q - T(3));
      c.A1 = T(0.5) * mu;
      c.B1 = (-mu + la * lj) / J;
      c.B2 = (mu + la * (T(1) - lj)) / (J * J);
      c.psd = true;
      break;
    }
    case kCOROT:  // corotational.cpp:8-60
      if (need_psi) c.psi = T(0.5) * la * (t - T(3)) * (t - T(3)) + mu * (Q - T(2) * t + T(3));
      c.A1 = mu;
      c.C1 = la * (t - T(3)) - T(2) * mu;
      c.C2 = la;
      break;
    case kFCR:  // fixed_corotational.cpp:8-…
      if (need_psi) c.psi = T(0.5) * la * (J - T(1)) * (J - T(1)) + mu * (Q - T(2) * t + T(3));
      c.A1 = mu;
      c.B1 = la * (J - T(1));
      c.B2 = la;
      c.C1 = T(-2) * mu;
      break;
    case kARAP:  // arap.cpp:7-65
      if (need_psi) c.psi = T(0.5) * mu * (Q - T(2) * t + T(3));
      c.A1 = T(0.5) * mu;
      c.C1 = -mu;
      break;
    case kFUNG: {  // fung.cpp:8-97 with c = 4
      const T cf = T(4);
      T e = Prec<T>::exp_(cf * (Q - T(3)) * T(0.5));
      T k = (mu + cf * mu) / la;
      if (need_psi)
        c.psi = T(0.5) * mu * (e - T(1)) + T(0.5) * mu * (Q - T(3)) +
                T(0.5) * la * (k + T(1) - J) * (k + T(1) - J);
      c.A1 = mu * cf * e * T(0.25) + T(0.5) * mu;
      c.A2 = mu * cf * cf * e * T(0.125);
      c.B1 = -la * (k + T(1) - J);
      c.B2 = la;
      c.psd = true;
      break;
    }
    default: {  // kSNH, stable_neohookean.cpp:8-95
      T omj = T(1) - J;
      if (need_psi) c.psi = mu * omj + T(0.5) * la * omj * omj + T(0.5) * mu * (Q - T(3));
      c.A1 = T(0.5) * mu;
      c.B1 = -mu - la * omj;
      c.B2 = la;
      c.psd = true;
      break;
    }
  }
  return c;
}

template <typename T> MI T material_psi(int type, T mu, T la, const T* s) {
  T Q, J, t, dJ[6];
  invariants(s, Q, J, t, dJ);
  return material_coef<T>(type, mu, la, Q, J, t, true).psi;
}

// Gradient of psi on the 6-vector.
template <typename T> MI void material_grad(int type, T mu, T la, const T* s, T g[6]) {
  T Q, J, t, dJ[6];
  invariants(s, Q, J, t, dJ);
  MatCoef<T> c = material_coef<T>(type, mu, la, Q, J, t, false);
#pragma unroll
  for (int i = 0; i < 6; ++i)
    g[i] = madd(c.A1 * T(2) * (i < 3 ? T(1) : T(2)) * s[i], c.B1, dJ[i]) + (i < 3 ? c.C1 : T(0));
}

// Gradient and (unfixed) Hessian of psi on the 6-vector; H full 6x6 column-major.
template <typename T>
MI bool material_grad_hess(int type, T mu, T la, const T* s, T g[6], T H[36]) {
  T Q, J, t, dJ[6];
  invariants(s, Q, J, t, dJ);
  MatCoef<T> c = material_coef<T>(type, mu, la, Q, J, t, false);
  const T w[6] = {T(1), T(1), T(1), T(2), T(2), T(2)};
  T dQ[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    dQ[i] = T(2) * w[i] * s[i];
    g[i] = c.A1 * dQ[i] + c.B1 * dJ[i] + (i < 3 ? c.C1 : T(0));
  }
#pragma unroll
  for (int j = 0; j < 6; ++j)
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      T v = c.A2 * dQ[i] * dQ[j] + c.B2 * dJ[i] * dJ[j];
      if (i == j) v += T(2) * c.A1 * w[i];
      if (i < 3 && j < 3) v += c.C2;
      H[i + 6 * j] = v;
    }
  // + B1 * d2J/ds2 (symmetric pattern)
  const T b = c.B1;
  H[0 + 6 * 1] += b * s[2]; H[1 + 6 * 0] += b * s[2];
  H[0 + 6 * 2] += b * s[1]; H[2 + 6 * 0] += b * s[1];
  H[0 + 6 * 5] += b * T(-2) * s[5]; H[5 + 6 * 0] += b * T(-2) * s[5];
  H[1 + 6 * 2] += b * s[0]; H[2 + 6 * 1] += b * s[0];
  H[1 + 6 * 4] += b * T(-2) * s[4]; H[4 + 6 * 1] += b * T(-2) * s[4];
  H[2 + 6 * 3] += b * T(-2) * s[3]; H[3 + 6 * 2] += b * T(-2) * s[3];
  H[3 + 6 * 3] += b * T(-2) * s[2];
  H[3 + 6 * 4] += b * T(2) * s[5]; H[4 + 6 * 3] += b * T(2) * s[5];
  H[3 + 6 * 5] += b * T(2) * s[4]; H[5 + 6 * 3] += b * T(2) * s[4];
  H[4 + 6 * 4] += b * T(-2) * s[1];
  H[4 + 6 * 5] += b * T(2) * s[3]; H[5 + 6 * 4] += b * T(2) * s[3];
  H[5 + 6 * 5] += b * T(-2) * s[0];
  return c.psd;
}

// In-place lower Cholesky of the symmetric 6x6 H (column-major, lower part
// used); succeeds only if every pivot exceeds `floor_`.  In FP32, where it
// only tests definiteness, the diagonal is left holding 1/L_jj (one rsqrt
// instead of a square root and a division).
template <typename T> MI bool cholesky6(T* A, T floor_) {
  bool ok = true;
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    T d = A[j + 6 * j];
#pragma unroll
    for (int k = 0; k < j; ++k) d -= A[j + 6 * k] * A[j + 6 * k];
    ok = ok && (d > floor_);
    T inv;
    if constexpr (Prec<T>::kFP64) {
      const T ljj = Prec<T>::sqrt_(d > floor_ ? d : floor_);
      A[j + 6 * j] = ljj;
      inv = T(1) / ljj;
    } else {
      inv = Prec<T>::rsqrt_(d > floor_ ? d : floor_);
      A[j + 6 * j] = inv;
    }
#pragma unroll
    for (int i = j + 1; i < 6; ++i) {
      T v = A[i + 6 * j];
#pragma unroll
      for (int k = 0; k < j; ++k) v -= A[i + 6 * k] * A[j + 6 * k];
      A[i + 6 * j] = v * inv;
    }
  }
  return ok;
}

// Cyclic Jacobi eigen-decomposition of the symmetric 6x6 A: on return the
// diagonal of A holds the eigenvalues and V (column-major) the eigenvectors.
template <typename T> MI void jacobi_eig6(T* A, T* V) {
#pragma unroll
  for (int i = 0; i < 36; ++i) V[i] = (i % 7 == 0) ? T(1) : T(0);
  for (int sweep = 0; sweep < 12; ++sweep) {
    T off = 0, tot = 0;
#pragma unroll
    for (int j = 0; j < 6; ++j)
#pragma unroll
      for (int i = 0; i < 6; ++i) {
        T a = A[i + 6 * j] * A[i + 6 * j];
        tot += a;
        if (i != j) off += a;
      }
    if (!(off > (Prec<T>::kFP64 ? T(1e-30) : T(1e-14)) * tot)) break;
#pragma unroll
    for (int p = 0; p < 5; ++p)
#pragma unroll
      for (int q = p + 1; q < 6; ++q) {
        T apq = A[p + 6 * q];
        if (apq != T(0)) {
          T theta = (A[q + 6 * q] - A[p + 6 * p]) / (T(2) * apq);
          T tt = (theta >= T(0) ? T(1) : T(-1)) /
                 (fabs(theta) + Prec<T>::sqrt_(theta * theta + T(1)));
          T c = Prec<T>::rsqrt_(tt * tt + T(1)), sn = tt * c;
#pragma unroll
          for (int k = 0; k < 6; ++k) {
            T akp = A[k + 6 * p], akq = A[k + 6 * q];
            A[k + 6 * p] = c * akp - sn * akq;
            A[k + 6 * q] = sn * akp + c * akq;
          }
#pragma unroll
          for (int k = 0; k < 6; ++k) {
            T apk = A[p + 6 * k], aqk = A[q + 6 * k];
            A[p + 6 * k] = c * apk - sn * aqk;
            A[q + 6 * k] = sn * apk + c * aqk;
          }
#pragma unroll
          for (int k = 0; k < 6; ++k) {
            T vkp = V[k + 6 * p], vkq = V[k + 6 * q];
            V[k + 6 * p] = c * vkp - sn * vkq;
            V[k + 6 * q] = sn * vkp + c * vkq;
          }
        }
      }
  }
}

// sim::simple_psd_fix with tol 1e-6 (stable_neohookean.cpp:91-93, Bartels):
// eigenvalues below tol are raised to tol and H rebuilt; H is unchanged when
// it is already positive definite.  The Cholesky test (pivots above tol)
// decides the common case; only a failing H pays for the Jacobi
// eigen-decomposition.  Returns true if H was modified.
template <typename T> MI bool psd_fix(T* H, T tol) {
  T L[36];
#pragma unroll
  for (int i = 0; i < 36; ++i) L[i] = H[i];
  if (cholesky6(L, tol)) return false;
  T V[36];
#pragma unroll
  for (int i = 0; i < 36; ++i) L[i] = H[i];
  jacobi_eig6(L, V);
  T lam[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) lam[k] = L[k + 6 * k] < tol ? tol : L[k + 6 * k];
#pragma unroll
  for (int j = 0; j < 6; ++j)
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      T v = 0;
#pragma unroll
      for (int k = 0; k < 6; ++k) v += V[i + 6 * k] * lam[k] * V[j + 6 * k];
      H[i + 6 * j] = v;
    }
  return true;
}

// ---------------------------------------------------------------------------
// Standard FEM (the "stretch" variable, src/variables/stretch.cpp:33-60):
// psi on the flattened deformation gradient F (9, column-major, index r + 3c;
// MaterialModel's Vector9d forms, stable_neohookean.cpp:97-234,
// neohookean.cpp:96-231).  Both are psi = A(|F|^2) + B(det F), so with the
// invariant coefficients of material_coef (A1 = dA/dQ, B1 = dB/dJ, B2 =
// d2B/dJ2; A2 = 0 for both):
//   d psi / dF   = 2 A1 F + B1 cof F
//   d2 psi / dF2 = 2 A1 I + B2 cof cof^T + B1 d2J/dF2,
//   d2J / dF_ij dF_kl = sum_mn eps_ikm eps_jln F_mn.
template <typename T> MI void det_cof3(const T* F, T& J, T cof[9]) {
  // cof(r, c) = dJ / dF(r, c), column-major
  cof[0] = F[4] * F[8] - F[7] * F[5];
  cof[1] = F[6] * F[5] - F[3] * F[8];
  cof[2] = F[3] * F[7] - F[6] * F[4];
  cof[3] = F[7] * F[2] - F[1] * F[8];
  cof[4] = F[0] * F[8] - F[6] * F[2];
  cof[5] = F[6] * F[1] - F[0] * F[7];
  cof[6] = F[1] * F[5] - F[4] * F[2];
  cof[7] = F[3] * F[2] - F[0] * F[5];
  cof[8] = F[0] * F[4] - F[3] * F[1];
  J = F[0] * cof[0] + F[1] * cof[1] + F[2] * cof[2];
}

template <typename T> MI T fem_psi(int type, T mu, T la, const T* F) {
  T J, cof[9], Q = T(0);
#pragma unroll
  for (int i = 0; i < 9; ++i) Q = Q + F[i] * F[i];
  det_cof3(F, J, cof);
  return material_coef<T>(type, mu, la, Q, J, T(0), true).psi;
}

template <typename T> MI void fem_grad(int type, T mu, T la, const T* F, T g[9]) {
  T J, cof[9], Q = T(0);
#pragma unroll
  for (int i = 0; i < 9; ++i) Q = Q + F[i] * F[i];
  det_cof3(F, J, cof);
  const MatCoef<T> c = material_coef<T>(type, mu, la, Q, J, T(0), false);
#pragma unroll
  for (int i = 0; i < 9; ++i) g[i] = T(2) * c.A1 * F[i] + c.B1 * cof[i];
}

// Gradient and Hessian (full 9x9, column-major; not psd-fixed).
template <typename T> MI void fem_grad_hess(int type, T mu, T la, const T* F, T g[9], T H[81]) {
  T J, cof[9], Q = T(0);
#pragma unroll
  for (int i = 0; i < 9; ++i) Q = Q + F[i] * F[i];
  det_cof3(F, J, cof);
  const MatCoef<T> c = material_coef<T>(type, mu, la, Q, J, T(0), false);
#pragma unroll
  for (int i = 0; i < 9; ++i) g[i] = T(2) * c.A1 * F[i] + c.B1 * cof[i];
#pragma unroll
  for (int a = 0; a < 9; ++a)
#pragma unroll
    for (int b = 0; b < 9; ++b) H[a + 9 * b] = c.B2 * cof[a] * cof[b] + (a == b ? T(2) * c.A1 : T(0));
  // B1 d2J/dF2: for (i, j) = (a % 3, a / 3), (k, l) = (b % 3, b / 3), nonzero
  // only for i != k and j != l, = +-F(m, n) with m, n the remaining indices
#pragma unroll
  for (int a = 0; a < 9; ++a)
#pragma unroll
    for (int b = 0; b < 9; ++b) {
      const int i = a % 3, j = a / 3, k = b % 3, l = b / 3;
      if (i == k || j == l) continue;
      const int m = 3 - i - k, n = 3 - j - l;
      // eps_ikm eps_jln: sign of the permutations (i, k, m) and (j, l, n)
      const int si = ((k - i + 3) % 3 == 1) ? 1 : -1;
      const int sj = ((l - j + 3) % 3 == 1) ? 1 : -1;
      H[a + 9 * b] += T(si * sj) * c.B1 * F[m + 3 * n];
    }
}

// In-place lower Cholesky of a symmetric N x N (column-major) with every
// pivot required above floor_.
template <int N, typename T> MI bool cholesky_n(T* A, T floor_) {
  bool ok = true;
#pragma unroll
  for (int j = 0; j < N; ++j) {
    T d = A[j + N * j];
#pragma unroll
    for (int k = 0; k < j; ++k) d -= A[j + N * k] * A[j + N * k];
    ok = ok && (d > floor_);
    T ljj = Prec<T>::sqrt_(d > floor_ ? d : (floor_ > T(0) ? floor_ : T(1)));
    A[j + N * j] = ljj;
    T inv = T(1) / ljj;
#pragma unroll
    for (int i = j + 1; i < N; ++i) {
      T v = A[i + N * j];
#pragma unroll
      for (int k = 0; k < j; ++k) v -= A[i + N * k] * A[j + N * k];
      A[i + N * j] = v * inv;
    }
  }
  return ok;
}

// Cyclic Jacobi eigen-decomposition of a symmetric N x N: the diagonal of A
// holds the eigenvalues and V (column-major) the eigenvectors on return.
template <int N, typename T> MI void jacobi_eig_n(T* A, T* V) {
  for (int i = 0; i < N * N; ++i) V[i] = (i % (N + 1) == 0) ? T(1) : T(0);
  for (int sweep = 0; sweep < 15; ++sweep) {
    T off = 0, tot = 0;
    for (int j = 0; j < N; ++j)
      for (int i = 0; i < N; ++i) {
        const T a = A[i + N * j] * A[i + N * j];
        tot += a;
        if (i != j) off += a;
      }
    if (!(off > (Prec<T>::kFP64 ? T(1e-30) : T(1e-14)) * tot)) break;
    for (int p = 0; p < N - 1; ++p)
      for (int q = p + 1; q < N; ++q) {
        const T apq = A[p + N * q];
        if (apq == T(0)) continue;
        const T theta = (A[q + N * q] - A[p + N * p]) / (T(2) * apq);
        const T tt = (theta >= T(0) ? T(1) : T(-1)) / (fabs(theta) + Prec<T>::sqrt_(theta * theta + T(1)));
        const T c = Prec<T>::rsqrt_(tt * tt + T(1)), sn = tt * c;
        for (int k = 0; k < N; ++k) {
          const T akp = A[k + N * p], akq = A[k + N * q];
          A[k + N * p] = c * akp - sn * akq;
          A[k + N * q] = sn * akp + c * akq;
        }
        for (int k = 0; k < N; ++k) {
          const T apk = A[p + N * k], aqk = A[q + N * k];
          A[p + N * k] = c * apk - sn * aqk;
          A[q + N * k] = sn * apk + c * aqk;
        }
        for (int k = 0; k < N; ++k) {
          const T vkp = V[k + N * p], vkq = V[k + N * q];
          V[k + N * p] = c * vkp - sn * vkq;
          V[k + N * q] = sn * vkp + c * vkq;
        }
      }
  }
}

// sim::simple_psd_fix on an N x N: eigenvalues below tol raised to tol and H
// rebuilt; unchanged when the Cholesky test (pivots above tol) passes.
template <int N, typename T> MI bool psd_fix_n(T* H, T tol) {
  T L[N * N];
#pragma unroll
  for (int i = 0; i < N * N; ++i) L[i] = H[i];
  if (cholesky_n<N>(L, tol)) return false;
  T V[N * N];
  for (int i = 0; i < N * N; ++i) L[i] = H[i];
  jacobi_eig_n<N>(L, V);
  T lam[N];
  for (int k = 0; k < N; ++k) lam[k] = L[k + N * k] < tol ? tol : L[k + N * k];
  for (int j = 0; j < N; ++j)
    for (int i = 0; i < N; ++i) {
      T v = 0;
      for (int k = 0; k < N; ++k) v += V[i + N * k] * lam[k] * V[j + N * k];
      H[i + N * j] = v;
    }
  return true;
}

// The psd-fixed d2psi/dF2 of a psi = A(|F|^2) + B(det F) material from its
// eigensystem in closed form (the structure used by Smith, de Goes and Kim,
// "Stable Neo-Hookean Flesh Simulation", 2018), instead of a 9x9 Jacobi
// eigen-decomposition.  With the signed SVD F = U diag(s) V^T (U, V
// rotations), in the basis vec(U E V^T):
//   twist (u_i v_j^T - u_j v_i^T)/sqrt2:  2 A1 + B1 s_m   (m the third index)
//   flip  (u_i v_j^T + u_j v_i^T)/sqrt2:  2 A1 - B1 s_m
//   scaling sum_i z_i u_i v_i^T, z an eigenvector of the 3x3
//     2 A1 I + 4 A2 s s^T + B2 c c^T + B1 [[0 s2 s1] [s2 0 s0] [s1 s0 0]],
//     c = (s1 s2, s0 s2, s0 s1)
// Eigenvalues below tol are raised to tol and H rebuilt from the nine modes.
// Returns false (H untouched) when the SVD is ill-conditioned (the two
// largest singular values not well separated from zero); the caller then
// takes the Jacobi route.
template <typename T> MI bool fem_hess_projected(int type, T mu, T la, const T* F, T tol, T H[81]) {
  T C[9], V[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      C[i + 3 * j] = F[3 * i] * F[3 * j] + F[3 * i + 1] * F[3 * j + 1] + F[3 * i + 2] * F[3 * j + 2];
  jacobi_eig_n<3>(C, V);
  // order the eigenpairs by decreasing eigenvalue
  int o[3] = {0, 1, 2};
  if (C[4 * o[1]] > C[4 * o[0]]) { const int t = o[0]; o[0] = o[1]; o[1] = t; }
  if (C[4 * o[2]] > C[4 * o[1]]) { const int t = o[1]; o[1] = o[2]; o[2] = t; }
  if (C[4 * o[1]] > C[4 * o[0]]) { const int t = o[0]; o[0] = o[1]; o[1] = t; }
  T Vs[9];
#pragma unroll
  for (int k = 0; k < 3; ++k)
#pragma unroll
    for (int r = 0; r < 3; ++r) Vs[r + 3 * k] = V[r + 3 * o[k]];
  const T detV = Vs[0] * (Vs[4] * Vs[8] - Vs[7] * Vs[5]) - Vs[3] * (Vs[1] * Vs[8] - Vs[7] * Vs[2]) +
                 Vs[6] * (Vs[1] * Vs[5] - Vs[4] * Vs[2]);
  if (detV < T(0)) {
#pragma unroll
    for (int r = 0; r < 3; ++r) Vs[r + 6] = -Vs[r + 6];
  }
  T B[9];  // F V
#pragma unroll
  for (int k = 0; k < 3; ++k)
#pragma unroll
    for (int r = 0; r < 3; ++r) B[r + 3 * k] = F[r] * Vs[3 * k] + F[r + 3] * Vs[3 * k + 1] + F[r + 6] * Vs[3 * k + 2];
  const T s0 = Prec<T>::sqrt_(B[0] * B[0] + B[1] * B[1] + B[2] * B[2]);
  if (!(s0 > T(0)) || !isfinite(s0)) return false;
  T U[9];
#pragma unroll
  for (int r = 0; r < 3; ++r) U[r] = B[r] / s0;
  const T d01 = U[0] * B[3] + U[1] * B[4] + U[2] * B[5];
  T b1[3] = {B[3] - d01 * U[0], B[4] - d01 * U[1], B[5] - d01 * U[2]};
  const T s1 = Prec<T>::sqrt_(b1[0] * b1[0] + b1[1] * b1[1] + b1[2] * b1[2]);
  if (!(s1 > T(Prec<T>::kFP64 ? 1e-10 : 1e-4) * s0)) return false;
#pragma unroll
  for (int r = 0; r < 3; ++r) U[3 + r] = b1[r] / s1;
  U[6] = U[1] * U[5] - U[2] * U[4];
  U[7] = U[2] * U[3] - U[0] * U[5];
  U[8] = U[0] * U[4] - U[1] * U[3];
  const T s2 = U[6] * B[6] + U[7] * B[7] + U[8] * B[8];  // signed: < 0 when inverted
  const T sg[3] = {s0, s1, s2};
  T Q = T(0);
#pragma unroll
  for (int i = 0; i < 9; ++i) Q += F[i] * F[i];
  const MatCoef<T> c = material_coef<T>(type, mu, la, Q, s0 * s1 * s2, T(0), false);
  const T cf[3] = {s1 * s2, s0 * s2, s0 * s1};
  T M3[9], Z[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      T v = T(4) * c.A2 * sg[i] * sg[j] + c.B2 * cf[i] * cf[j];
      if (i == j) v += T(2) * c.A1;
      else v += c.B1 * sg[3 - i - j];
      M3[i + 3 * j] = v;
    }
  jacobi_eig_n<3>(M3, Z);
#pragma unroll
  for (int i = 0; i < 81; ++i) H[i] = T(0);
  // scaling modes
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const T lam = M3[4 * k] < tol ? tol : M3[4 * k];
    T q[9];
#pragma unroll
    for (int cc = 0; cc < 3; ++cc)
#pragma unroll
      for (int r = 0; r < 3; ++r)
        q[r + 3 * cc] = Z[3 * k] * U[r] * Vs[cc] + Z[3 * k + 1] * U[3 + r] * Vs[3 + cc] +
                        Z[3 * k + 2] * U[6 + r] * Vs[6 + cc];
#pragma unroll
    for (int a = 0; a < 9; ++a)
#pragma unroll
      for (int b = 0; b < 9; ++b) H[a + 9 * b] += lam * q[a] * q[b];
  }
  // twist and flip modes of each pair (i, j), m the third index
  const T rs2 = T(0.70710678118654752440);
#pragma unroll
  for (int p = 0; p < 3; ++p) {
    const int i = p == 2 ? 1 : 0, j = p == 0 ? 1 : 2, m = 3 - i - j;
#pragma unroll
    for (int sgn = 0; sgn < 2; ++sgn) {
      const T e = sgn == 0 ? T(2) * c.A1 + c.B1 * sg[m] : T(2) * c.A1 - c.B1 * sg[m];
      const T lam = e < tol ? tol : e;
      const T pm = sgn == 0 ? T(-1) : T(1);
      T q[9];
#pragma unroll
      for (int cc = 0; cc < 3; ++cc)
#pragma unroll
        for (int r = 0; r < 3; ++r)
          q[r + 3 * cc] = rs2 * (U[3 * i + r] * Vs[3 * j + cc] + pm * U[3 * j + r] * Vs[3 * i + cc]);
#pragma unroll
      for (int a = 0; a < 9; ++a)
#pragma unroll
        for (int b = 0; b < 9; ++b) H[a + 9 * b] += lam * q[a] * q[b];
    }
  }
  return true;
}

// Element force of the mixed residual, in the precision of T:
//   f_a = -vol * P dphi_a,  P = sum_i q_i ds_i/dF = R (Q - [w]x),
// Q = sum_i q_i E_i (symmetric), w = W sum_i q_i c_i (the u_i of
// stretch_derivative_u contracted with q).  This is -PJW (dSdF gl) of
// MixedStretch::rhs (mixed_stretch.cpp:206-226) for one element, with
// q = Sym gl = H (S - s) + g.  Returns false if tr(S) I - S is singular.
template <typename T>
MI bool element_force(const T* R, const T s6[6], const T q[6], const T dph[12], T vol, T f[12]) {
  T t = s6[0] + s6[1] + s6[2];
  T m[6] = {t - s6[0], t - s6[1], t - s6[2], -s6[3], -s6[4], -s6[5]};
  // sum_i q_i c_i with the c_i of stretch_derivative_u
  T cq[3];
  cq[0] = -q[1] * s6[5] + q[2] * s6[5] - T(0.5) * q[3] * s6[4] + T(0.5) * q[4] * s6[3] +
          T(0.5) * q[5] * (s6[1] - s6[2]);
  cq[1] = q[0] * s6[4] - q[2] * s6[4] + T(0.5) * q[3] * s6[5] + T(0.5) * q[4] * (s6[2] - s6[0]) -
          T(0.5) * q[5] * s6[3];
  cq[2] = -q[0] * s6[3] + q[1] * s6[3] + T(0.5) * q[3] * (s6[0] - s6[1]) - T(0.5) * q[4] * s6[5] +
          T(0.5) * q[5] * s6[4];
  T w[3];
  bool ok = solve_sym3(m, cq, w);
  if (!ok) w[0] = w[1] = w[2] = T(0);
  // D = Q - [w]x (column-major)
  T D[9];
  D[0] = q[0];
  D[4] = q[1];
  D[8] = q[2];
  D[3] = T(0.5) * q[3] + w[2];   // (0,1)
  D[1] = T(0.5) * q[3] - w[2];   // (1,0)
  D[6] = T(0.5) * q[4] - w[1];   // (0,2)
  D[2] = T(0.5) * q[4] + w[1];   // (2,0)
  D[7] = T(0.5) * q[5] + w[0];   // (1,2)
  D[5] = T(0.5) * q[5] - w[0];   // (2,1)
  T P[9];
  mul33(R, D, P);
#pragma unroll
  for (int a = 1; a < 4; ++a)
#pragma unroll
    for (int r = 0; r < 3; ++r)
      f[3 * a + r] = -vol * madd(madd(P[r] * dph[3 * a], P[r + 3], dph[3 * a + 1]), P[r + 6], dph[3 * a + 2]);
  // dphi_0 = -(dphi_1 + dphi_2 + dphi_3)
#pragma unroll
  for (int r = 0; r < 3; ++r) f[r] = -(f[3 + r] + f[6 + r] + f[9 + r]);
  return ok;
}

// One Newton step of the Procrustes problem in the precision of T, with the
// rotation update expanded to second order (|omega| is at rounding level
// after a converged lower-precision solve).
template <typename T> MI void polish_rotation(T* R, const T* F) {
  T Y[9], g[3], h[6], om[3];
  mulABt(R, F, Y);
  procrustes_gH(Y, g, h);
  if (!solve_sym3(h, g, om)) return;
  om[0] = -om[0];
  om[1] = -om[1];
  om[2] = -om[2];
  // dR = I + [om]x + 1/2 [om]x^2
  T K[9] = {T(0), om[2], -om[1], -om[2], T(0), om[0], om[1], -om[0], T(0)};
  T K2[9];
  mul33(K, K, K2);
  T dR[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) dR[i] = ((i % 4 == 0) ? T(1) : T(0)) + K[i] + T(0.5) * K2[i];
  T tmp[9];
  mul33(dR, R, tmp);
#pragma unroll
  for (int i = 0; i < 9; ++i) R[i] = tmp[i];
}

// The same polish for the mixed path's float-float rotation.  Only the
// gradient g (the axial part of Y = R F^T, |g| ~ 1e-7 after the FP32
// Procrustes solve: a difference of O(1) entries) needs float-float.  The
// Hessian (O(1)), the 3x3 solve for omega and the increment
// dR R - R = (K + K^2/2) R, whose entries are ~|omega|, are taken in FP32:
// their rounding, about 6e-8 of ~1e-7, sits at the float-float resolution of
// R.  The increment is then added to R in float-float.
MI void polish_rotation(df64* R, const df64* F) {
  // Y(i, j) = sum_k R(i, k) F(j, k); off-diagonal entries in float-float
  auto y = [&](int i, int j) { return madd(madd(R[i] * F[j], R[i + 3], F[j + 3]), R[i + 6], F[j + 6]); };
  const df64 g0 = y(2, 1) - y(1, 2), g1 = y(0, 2) - y(2, 0), g2 = y(1, 0) - y(0, 1);
  float Rh[9], Fh[9], Yf[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    Rh[i] = R[i].hi;
    Fh[i] = F[i].hi;
  }
  mulABt(Rh, Fh, Yf);
  float g[3] = {g0.hi, g1.hi, g2.hi}, h[6], gy[3], om[3];
  procrustes_gH(Yf, gy, h);
  if (!solve_sym3(h, g, om)) return;
  // K = [omega]x with omega = -H^-1 g; M = K + K^2 / 2
  const float K[9] = {0.f, -om[2], om[1], om[2], 0.f, -om[0], -om[1], om[0], 0.f};
  float M[9], D[9];
  mul33(K, K, M);
#pragma unroll
  for (int i = 0; i < 9; ++i) M[i] = K[i] + 0.5f * M[i];
  mul33(M, Rh, D);
#pragma unroll
  for (int i = 0; i < 9; ++i) R[i] = R[i] + df64(D[i]);
}

// ---------------------------------------------------- compensated sums ---
struct KSum {
  double s, c;
  MI void add(double x) {  // Neumaier
    double t = s + x;
    c += (fabs(s) >= fabs(x)) ? (s - t) + x : (x - t) + s;
    s = t;
  }
  MI void merge(const KSum& o) {
    add(o.s);
    c += o.c;
  }
  MI double value() const { return s + c; }
};

}  // namespace mfem_gpu
