// The 2-D path on the GPU: triangle meshes in the plane (Tri2DMesh +
// MixedStretch<2> + NewtonOptimizer<2> of tytrusty/mfem), FP64 throughout,
// and its C ABI (mfem_gpu_tri2d_*, include/mfem_gb300.h).
//
// Reference correspondence:
//   set-up          src/mesh/tri2d_mesh.cpp:11-83, src/mesh/mesh.cpp:44-75,
//                   src/variables/displacement.cpp:75-98, mixed_stretch.cpp:261-304
//   element update  MixedStretch<2>::update_rotations + update_derivatives
//                   (polar_svd<2>, mixed_stretch.cpp:43-78; :133-204)
//   assembly        Assembler<double,2,-1>, src/utils/sparse_utils.cpp:19-203,
//                   plus PMP (linear_system.h:18-31)
//   PCG             Eigen ConjugateGradient + DiagonalPreconditioner
//                   ("eigen-pcg-diag", linear_solver_factory.cpp:74-84)
//   local solve     MixedStretch::solve, mixed_stretch.cpp:243-259
//   energy          energy_func, newton_optimizer.cpp:34-49
//   Newton loop     newton_optimizer.cpp:11-89 with linesearch.h:80-129
//   BC scripts      src/boundary_conditions/*.h (Rotation2D for bend/twist)
//
// Layout and launches.  The reference's 2-D scenes are meshes of a few
// hundred to a few thousand triangles, far below one wave of the GPU, so
// the design keeps the launch count per Newton iteration small and fixed:
//   t2_elem     one thread per triangle: polar, ds/dF, material, H^-1,
//               the 6x6 Aloc and the triangle's 6 RHS terms (94 doubles out)
//   t2_rows     one thread per free vertex: its 2x2 blocks gathered from
//               the Aloc of the incident triangles in the assembler's
//               sorted order, + mass, Jacobi inverse, and its RHS
//   t2_norm     one block: |rhs|^2
//   t2_pcg      ONE thread block for the whole PCG solve: every reduction a
//               fixed-order tree in shared memory, __syncthreads between the
//               phases, no grid-wide waits; one launch per solve.  Sheets
//               with more free rows than the block has threads run
//               t2_pcg_grid instead: the single-reduction form of the same
//               iteration over co-resident blocks, one bounded grid barrier
//               an iteration, also one launch per solve
//   t2_local    one thread per triangle: lambda and ds
//   t2_energy   one thread per triangle and vertex: the three energy parts
//   t2_esum     one block: the fixed-order sums (and max|dx|, max|ds|)
//   t2_apply, t2_history: the step along the line search, the BDF history
// All reductions are in a fixed order, so a scene's results are bitwise
// reproducible run to run.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <new>
#include <vector>

#include "../../include/mfem_gb300.h"
#include "device_math.cuh"

namespace {

using mfem_gpu::psd_fix_n;

constexpr int kThreads = 128;
constexpr int kBlock = 1024;  // the single-block kernels (PCG, sums)
constexpr double kPsdTol = 1e-6;
constexpr double kDsvdTol = 1e-4;  // dsvd.cpp:153

__constant__ double kSym2[3] = {1, 1, 2};
__constant__ double kSymInv2[3] = {1, 1, 0.5};

enum { SC_RN2 = 0, SC_E = 1, SC_DEC = 2, SC_CG_IT = 3, SC_CG_RN2 = 4, SC_CG_B2 = 5, SC_COUNT = 8 };

// Device pointers of one 2-D scene (kernel argument, by value).
struct T2 {
  int nv, nt, nf, nnzb;
  const int* tri;       // 3 nt
  const double* dX;     // 6 nt: dphi_k/dX_c at [6e + 2k + c]
  const double* vol;    // nt (doublearea)
  const double* mu;
  const double* la;
  const int* mat;
  const int* free_map;    // nv: free index or -1
  const int* row_vertex;  // nf
  double* x;    // 2 nf free positions
  double* dx;   // 2 nf
  double* b;    // 2 nv pinned positions (0 at free vertices)
  double* xt;   // 2 nv x~ of the BDF integrator
  double* s;    // 3 nt
  double* ds;
  double* lam;
  double* R;     // 4 nt
  double* S;     // 3 nt
  double* dSdF;  // 12 nt (4x3 column-major, Js^T Sym)
  double* g;     // 3 nt
  double* H;     // 9 nt
  double* Hinv;  // 9 nt
  double* Htil;  // 9 nt
  double* gl;    // 3 nt
  double* Aloc;  // 36 nt
  double* fel;   // 6 nt: vol Jloc^T (dSdF gl) per triangle vertex
  const int* m_ptr;  // mass CSR over all vertices
  const int* m_col;
  const double* m_val;
  const int* b_ptr;  // BCSR over free vertices
  const int* b_col;
  const double* b_mass;
  const int* c_ptr;  // nnzb+1: each block's contributions ...
  const int* c_ent;  // ... as 9 e + 3 j + k (sorted order of the assembler)
  const int* i_ptr;  // nf+1: each free row's incident (triangle, corner) ...
  const int* i_ent;  // ... as 3 e + k, in triangle order
  double* A;     // 4 nnzb row-major blocks
  double* rhs;   // 2 nf
  double* dinv;  // 2 nf
  double* r;     // PCG vectors, 2 nf
  double* p;
  double* q;
  double* sr;     // the grid PCG's r, w, s by iteration parity: 6 x 2 nf (r0 r1 w0 w1 s0 s1)
  double* part;   // the grid PCG's block partials: 3 x kT2MaxGrid
  unsigned int* bar;  // the grid PCG's barrier: arrivals, generation, error flag
  double* epart;  // 2 nt + nv energy parts
  double* scal;   // SC_COUNT device scalars
  int* status;    // worst status the kernels saw
  double h2f0, h2f1;  // dt^2 * body force
};

__device__ __forceinline__ void pos2(const T2& d, int v, double alpha, const double* xfull,
                                     double out[2]) {
  if (xfull) {
    out[0] = xfull[2 * v];
    out[1] = xfull[2 * v + 1];
    return;
  }
  const int f = d.free_map[v];
  if (f >= 0) {
    out[0] = d.x[2 * f] + alpha * d.dx[2 * f];
    out[1] = d.x[2 * f + 1] + alpha * d.dx[2 * f + 1];
  } else {
    out[0] = d.b[2 * v];
    out[1] = d.b[2 * v + 1];
  }
}

__device__ __forceinline__ void defgrad(const T2& d, int e, double alpha, const double* xfull,
                                        double F[4]) {
  F[0] = F[1] = F[2] = F[3] = 0.0;
  const double* dx = d.dX + 6 * size_t(e);
  for (int k = 0; k < 3; ++k) {
    double p[2];
    pos2(d, d.tri[3 * e + k], alpha, xfull, p);
    for (int c = 0; c < 2; ++c)
      for (int r = 0; r < 2; ++r) F[r + 2 * c] += p[r] * dx[2 * k + c];
  }
}

// polar_svd<2> (mixed_stretch.cpp:43-78) in closed form.  With
// e = (F00+F11)/2, f = (F00-F11)/2, g = (F10+F01)/2, h = (F10-F01)/2 the
// sign-fixed singular values are q +- r, q = |(e, h)|, r = |(f, g)|, and the
// nearest rotation is R = [[e, -h], [h, e]] / q.  The 2-D dsvd
// (dsvd.cpp:140-189) gives dR/dF_rc = a K R with K = [[0, 1], [-1, 0]],
// a = ((R^T E_rc)01 - (R^T E_rc)10) / (s0 + s1), and a = 0 where
// |s0^2 - s1^2| = 4 q r < 1e-4; so dS/dF_rc = R^T E_rc - a K S.
// dsdF (3x4 column-major, NULL: none) holds ds/dF for s = [S00, S11,
// (S01+S10)/2].  Returns false when q = 0 (no unique nearest rotation).
__device__ bool polar2(const double F[4], double R[4], double s[3], double* dsdF) {
  const double e = 0.5 * (F[0] + F[3]), f = 0.5 * (F[0] - F[3]);
  const double g = 0.5 * (F[1] + F[2]), h = 0.5 * (F[1] - F[2]);
  const double q = sqrt(e * e + h * h), r = sqrt(f * f + g * g);
  const bool ok = q > 0.0;
  const double iq = ok ? 1.0 / q : 0.0;
  R[0] = ok ? e * iq : 1.0;
  R[1] = h * iq;
  R[2] = -h * iq;
  R[3] = ok ? e * iq : 1.0;
  const double S00 = R[0] * F[0] + R[1] * F[1];
  const double S10 = R[2] * F[0] + R[3] * F[1];
  const double S01 = R[0] * F[2] + R[1] * F[3];
  const double S11 = R[2] * F[2] + R[3] * F[3];
  s[0] = S00;
  s[1] = S11;
  s[2] = 0.5 * (S10 + S01);
  if (dsdF) {
    const bool small = !ok || fabs(4.0 * q * r) < kDsvdTol;
    for (int c = 0; c < 2; ++c)
      for (int rr = 0; rr < 2; ++rr) {
        const double Rr0 = R[rr], Rr1 = R[rr + 2];  // R(rr, 0), R(rr, 1)
        const double P00 = c == 0 ? Rr0 : 0.0, P11 = c == 1 ? Rr1 : 0.0;
        const double P01 = c == 1 ? Rr0 : 0.0, P10 = c == 0 ? Rr1 : 0.0;
        const double a = small ? 0.0 : (P01 - P10) * 0.5 * iq;
        const int col = rr + 2 * c;
        dsdF[0 + 3 * col] = P00 - a * S10;
        dsdF[1 + 3 * col] = P11 + a * S01;
        dsdF[2 + 3 * col] = 0.5 * (P01 + P10 + a * (S00 - S11));
      }
  }
  return ok;
}

// The 3-vector materials as psi = A(Q) + B(J) + C(t), Q = s0^2 + s1^2 +
// 2 s2^2, J = s0 s1 - s2^2, t = s0 + s1 (the Vector3d sections of
// stable_neohookean.cpp:236-277, corotational.cpp:62-97,
// fixed_corotational.cpp:93-130, arap.cpp:67-99).
struct Coef2 {
  double psi, A1, B1, B2, C1, C2;
  bool psd;
};

__device__ Coef2 coef2(int type, double mu, double la, const double* s) {
  const double Q = s[0] * s[0] + s[1] * s[1] + 2 * s[2] * s[2];
  const double J = s[0] * s[1] - s[2] * s[2];
  const double t = s[0] + s[1];
  Coef2 c{0, 0, 0, 0, 0, 0, false};
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
    default:  // MFEM_MATERIAL_ARAP (create refuses the others)
      c.psi = 0.5 * mu * (Q - 2 * t + 2);
      c.A1 = 0.5 * mu;
      c.C1 = -mu;
      break;
  }
  return c;
}

__device__ void material2(int type, double mu, double la, const double* s, double g[3],
                          double H[9]) {
  const Coef2 c = coef2(type, mu, la, s);
  const double dJ[3] = {s[1], s[0], -2 * s[2]};
  for (int i = 0; i < 3; ++i) g[i] = 2 * c.A1 * kSym2[i] * s[i] + c.B1 * dJ[i] + (i < 2 ? c.C1 : 0.0);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double v = c.B2 * dJ[i] * dJ[j];
      if (i == j) v += 2 * c.A1 * kSym2[i];
      if (i < 2 && j < 2) v += c.C2;
      H[i + 3 * j] = v;
    }
  H[1] += c.B1;  // d2J/ds0ds1 = 1
  H[3] += c.B1;
  H[8] += -2 * c.B1;  // d2J/ds2^2 = -2
  if (c.psd) psd_fix_n<3>(H, kPsdTol);
}

__device__ bool inverse3(const double* A, double* Ai) {
  const double c00 = A[4] * A[8] - A[7] * A[5], c01 = A[7] * A[2] - A[1] * A[8],
               c02 = A[1] * A[5] - A[4] * A[2];
  const double det = A[0] * c00 + A[3] * c01 + A[6] * c02;
  if (!(det != 0.0) || !isfinite(det)) return false;
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

// MixedStretch<2>::update_rotations + update_derivatives + the triangle's
// share of MixedStretch::rhs (mixed_stretch.cpp:133-226, N = 3, M = 4).
// xfull: full positions (2 nv) for the parity entry point, else NULL.
__global__ void __launch_bounds__(kThreads) t2_elem(T2 d, double h2, const double* xfull) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= d.nt) return;
  double F[4], R[4], sv[3], dsdF[12];
  defgrad(d, e, 0.0, xfull, F);
  if (!polar2(F, R, sv, dsdF)) atomicMax(d.status, int(MFEM_ERR_PROCRUSTES));
  for (int k = 0; k < 4; ++k) d.R[4 * size_t(e) + k] = R[k];
  for (int k = 0; k < 3; ++k) d.S[3 * size_t(e) + k] = sv[k];
  double D[12];
  for (int i = 0; i < 3; ++i)
    for (int r = 0; r < 4; ++r) D[r + 4 * i] = dsdF[i + 3 * r] * kSym2[i];
  for (int k = 0; k < 12; ++k) d.dSdF[12 * size_t(e) + k] = D[k];
  const double si[3] = {d.s[3 * e], d.s[3 * e + 1], d.s[3 * e + 2]};
  const double vol = d.vol[e];
  double g[3], H[9], Hi[9], Ht[9];
  material2(d.mat[e], d.mu[e], d.la[e], si, g, H);
  for (int k = 0; k < 9; ++k) H[k] *= h2;
  for (int k = 0; k < 3; ++k) g[k] *= h2;
  if (!inverse3(H, Hi)) {
    atomicMax(d.status, int(MFEM_ERR_NONFINITE));
    for (int k = 0; k < 9; ++k) Hi[k] = 0.0;
  }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) Ht[i + 3 * j] = (1.0 / vol) * kSymInv2[i] * H[i + 3 * j] * kSymInv2[j];
  for (int k = 0; k < 9; ++k) {
    d.H[9 * size_t(e) + k] = H[k];
    d.Hinv[9 * size_t(e) + k] = Hi[k];
    d.Htil[9 * size_t(e) + k] = Ht[k];
  }
  double gl[3];
  {
    double dd[3];
    for (int i = 0; i < 3; ++i) dd[i] = kSym2[i] * (sv[i] - si[i]);
    for (int i = 0; i < 3; ++i) {
      double v = 0;
      for (int j = 0; j < 3; ++j) v += Ht[i + 3 * j] * dd[j];
      gl[i] = vol * v + kSymInv2[i] * g[i];
    }
  }
  for (int k = 0; k < 3; ++k) {
    d.g[3 * size_t(e) + k] = g[k];
    d.gl[3 * size_t(e) + k] = gl[k];
  }
  // Aloc = vol^2 Jloc^T (dSdF Htil dSdF^T) Jloc  (6x6 column-major)
  double DH[12], K4[16];
  for (int r = 0; r < 4; ++r)
    for (int j = 0; j < 3; ++j) {
      double v = 0;
      for (int i = 0; i < 3; ++i) v += D[r + 4 * i] * Ht[i + 3 * j];
      DH[r + 4 * j] = v;
    }
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) {
      double v = 0;
      for (int j = 0; j < 3; ++j) v += DH[r + 4 * j] * D[c + 4 * j];
      K4[r + 4 * c] = v;
    }
  const double* dx = d.dX + 6 * size_t(e);
  double* Al = d.Aloc + 36 * size_t(e);
  const double v2 = vol * vol;
  for (int a = 0; a < 3; ++a)
    for (int l = 0; l < 2; ++l)
      for (int bq = 0; bq < 3; ++bq)
        for (int m = 0; m < 2; ++m) {
          double v = 0;
          for (int c = 0; c < 2; ++c)
            for (int cc = 0; cc < 2; ++cc)
              v += dx[2 * a + c] * dx[2 * bq + cc] * K4[(2 * c + l) + 4 * (2 * cc + m)];
          Al[(2 * a + l) + 6 * (2 * bq + m)] = v * v2;
        }
  // the triangle's RHS terms: vol Jloc^T (dSdF gl)
  double tmp[4];
  for (int r = 0; r < 4; ++r) tmp[r] = D[r] * gl[0] + D[r + 4] * gl[1] + D[r + 8] * gl[2];
  for (int k = 0; k < 3; ++k)
    for (int l = 0; l < 2; ++l)
      d.fel[6 * size_t(e) + 2 * k + l] = vol * (dx[2 * k] * tmp[l] + dx[2 * k + 1] * tmp[l + 2]);
}

// One free vertex row: its 2x2 blocks (Assembler::update_matrix order) +
// PMP, the Jacobi inverse, and RHS = -PM(x - x~ - h^2 f) - PJW (dSdF gl).
__global__ void __launch_bounds__(kThreads) t2_rows(T2 d) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= d.nf) return;
  d.dinv[2 * r] = 1.0;
  d.dinv[2 * r + 1] = 1.0;
  for (int q = d.b_ptr[r]; q < d.b_ptr[r + 1]; ++q) {
    double a00 = 0, a01 = 0, a10 = 0, a11 = 0;
    for (int c = d.c_ptr[q]; c < d.c_ptr[q + 1]; ++c) {
      const int ent = d.c_ent[c];
      const int e = ent / 9, l = ent - 9 * e, j = l / 3, k = l - 3 * j;
      const double* Al = d.Aloc + 36 * size_t(e);
      a00 += Al[(2 * j) + 6 * (2 * k)];
      a01 += Al[(2 * j) + 6 * (2 * k + 1)];
      a10 += Al[(2 * j + 1) + 6 * (2 * k)];
      a11 += Al[(2 * j + 1) + 6 * (2 * k + 1)];
    }
    a00 += d.b_mass[q];
    a11 += d.b_mass[q];
    double* blk = d.A + 4 * size_t(q);
    blk[0] = a00;
    blk[1] = a01;
    blk[2] = a10;
    blk[3] = a11;
    if (d.b_col[q] == r) {
      d.dinv[2 * r] = a00 != 0.0 ? 1.0 / a00 : 1.0;
      d.dinv[2 * r + 1] = a11 != 0.0 ? 1.0 / a11 : 1.0;
    }
  }
  const int v = d.row_vertex[r];
  double m0 = 0, m1 = 0;
  for (int q = d.m_ptr[v]; q < d.m_ptr[v + 1]; ++q) {
    const int u = d.m_col[q];
    double p[2];
    pos2(d, u, 0.0, nullptr, p);
    m0 += d.m_val[q] * (p[0] - d.xt[2 * u] - d.h2f0);
    m1 += d.m_val[q] * (p[1] - d.xt[2 * u + 1] - d.h2f1);
  }
  double r0 = -m0, r1 = -m1;
  for (int i = d.i_ptr[r]; i < d.i_ptr[r + 1]; ++i) {
    const int ent = d.i_ent[i];
    const int e = ent / 3, k = ent - 3 * e;
    r0 -= d.fel[6 * size_t(e) + 2 * k];
    r1 -= d.fel[6 * size_t(e) + 2 * k + 1];
  }
  d.rhs[2 * r] = r0;
  d.rhs[2 * r + 1] = r1;
}

// Fixed-order block sum over kBlock threads.  Every thread of the block
// calls it (uniform control flow) and gets the total.
__device__ double block_sum(double v, double* sh) {
  const int t = threadIdx.x;
  sh[t] = v;
  __syncthreads();
  for (int w = kBlock / 2; w > 0; w >>= 1) {
    if (t < w) sh[t] += sh[t + w];
    __syncthreads();
  }
  const double out = sh[0];
  __syncthreads();
  return out;
}

__device__ double block_max(double v, double* sh) {
  const int t = threadIdx.x;
  sh[t] = v;
  __syncthreads();
  for (int w = kBlock / 2; w > 0; w >>= 1) {
    if (t < w) sh[t] = fmax(sh[t], sh[t + w]);
    __syncthreads();
  }
  const double out = sh[0];
  __syncthreads();
  return out;
}

__global__ void __launch_bounds__(kBlock) t2_norm(T2 d) {
  __shared__ double sh[kBlock];
  double part = 0;
  for (int i = threadIdx.x; i < 2 * d.nf; i += kBlock) part += d.rhs[i] * d.rhs[i];
  const double s = block_sum(part, sh);
  if (threadIdx.x == 0) d.scal[SC_RN2] = s;
}

// The whole Jacobi-PCG solve LHS dx = rhs from dx = 0 in one thread block,
// Eigen's ConjugateGradient iteration: stop when |r|^2 < max(tol^2 |b|^2,
// DBL_MIN) or after max_iter iterations (the breaking iteration is not
// counted).  Every loop bound and break test is block-uniform: the
// scalars come out of block_sum, which all threads read after a barrier.
__global__ void __launch_bounds__(kBlock) t2_pcg(T2 d, int max_iter, double tol) {
  __shared__ double sh[kBlock];
  const int n = 2 * d.nf, t = threadIdx.x;
  double part = 0;
  for (int i = t; i < n; i += kBlock) {
    const double ri = d.rhs[i];
    d.dx[i] = 0.0;
    d.r[i] = ri;
    part += ri * ri;
  }
  const double b2 = block_sum(part, sh);
  if (b2 == 0.0) {
    if (t == 0) {
      d.scal[SC_CG_IT] = 0;
      d.scal[SC_CG_RN2] = 0;
      d.scal[SC_CG_B2] = 0;
    }
    return;
  }
  const double thr = fmax(tol * tol * b2, DBL_MIN);
  double rn2 = b2;
  if (b2 < thr) {  // Eigen's test before the first iteration: no iteration
    if (t == 0) {
      d.scal[SC_CG_IT] = 0;
      d.scal[SC_CG_RN2] = b2;
      d.scal[SC_CG_B2] = b2;
    }
    return;
  }
  part = 0;
  for (int i = t; i < n; i += kBlock) {
    const double pi = d.dinv[i] * d.r[i];
    d.p[i] = pi;
    part += d.r[i] * pi;
  }
  double absNew = block_sum(part, sh);
  int it = 0;
  while (it < max_iter) {
    part = 0;
    for (int rr = t; rr < d.nf; rr += kBlock) {
      double y0 = 0, y1 = 0;
      for (int qq = d.b_ptr[rr]; qq < d.b_ptr[rr + 1]; ++qq) {
        const double* a = d.A + 4 * size_t(qq);
        const int c = d.b_col[qq];
        const double p0 = d.p[2 * c], p1 = d.p[2 * c + 1];
        y0 += a[0] * p0 + a[1] * p1;
        y1 += a[2] * p0 + a[3] * p1;
      }
      d.q[2 * rr] = y0;
      d.q[2 * rr + 1] = y1;
      part += d.p[2 * rr] * y0 + d.p[2 * rr + 1] * y1;
    }
    const double alpha = absNew / block_sum(part, sh);
    part = 0;
    for (int i = t; i < n; i += kBlock) {
      d.dx[i] += alpha * d.p[i];
      const double ri = d.r[i] - alpha * d.q[i];
      d.r[i] = ri;
      part += ri * ri;
    }
    rn2 = block_sum(part, sh);
    if (rn2 < thr) break;
    part = 0;
    for (int i = t; i < n; i += kBlock) part += d.r[i] * (d.dinv[i] * d.r[i]);
    const double absOld = absNew;
    absNew = block_sum(part, sh);
    const double beta = absNew / absOld;
    for (int i = t; i < n; i += kBlock) d.p[i] = d.dinv[i] * d.r[i] + beta * d.p[i];
    __syncthreads();  // p complete before the next product gathers it
    ++it;
  }
  if (t == 0) {
    d.scal[SC_CG_IT] = it;
    d.scal[SC_CG_RN2] = rn2;
    d.scal[SC_CG_B2] = b2;
  }
}

// ----------------------------------------------------- grid PCG ---
// The Jacobi-PCG over many blocks for sheets too large for one (the FP64
// work of a 10^4-triangle sheet on one SM at GB300's FP64 rate sets ~40 us
// per iteration).  One cooperative launch of G blocks of kGridThreads, each
// owning a contiguous range of free rows; a reduction is each block's
// fixed-order partial, a bounded grid barrier, and the G partials summed in
// the same fixed order by every block (so every block takes the same
// branches).  The iteration is the single-reduction form of the same PCG
// (Chronopoulos & Gear 1989; equal to Eigen's iteration in exact
// arithmetic): with u = D^-1 r, w = A u, s = A p, each iteration needs one
// reduction of (r, u), (w, u) and |r|^2 -- one grid barrier.  A
// neighbouring row's u_{k+1} = D^-1 (r_k - a_k (w_k + b_k s_{k-1})) is
// formed where the product gathers it, with the expression its owner
// evaluates (t2_next), so r, w, s alternate between two buffers by the
// iteration's parity and no barrier separates the updates from the product.
// Eigen's stop: |r|^2 < max(tol^2 |b|^2, DBL_MIN), the iteration that meets
// it not counted.  Every wait is bounded (kT2BarrierNs or kT2BarrierPolls):
// when one runs out the kernel flags MFEM_ERR_TIMEOUT in the scene's status
// and every block leaves at its next barrier.
constexpr int kGridThreads = 256;
constexpr int kT2MaxGrid = 1024;
constexpr unsigned long long kT2BarrierNs = 2000000000ull;
constexpr unsigned int kT2BarrierPolls = 1u << 26;

__device__ __forceinline__ unsigned long long t2_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// bar[0] arrivals, bar[1] generation, bar[2] error.  False: leave the kernel.
__device__ bool t2_grid_sync(const T2& d) {
  __shared__ int ok_s;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned int* gen = d.bar + 1;
    volatile unsigned int* err = d.bar + 2;
    int ok = *err == 0u;
    if (ok) {
      const unsigned int g = *gen;
      __threadfence();
      if (atomicAdd(d.bar, 1u) + 1u == gridDim.x) {
        d.bar[0] = 0u;
        __threadfence();
        atomicAdd(d.bar + 1, 1u);
      } else {
        const unsigned long long t0 = t2_ns();
        unsigned int polls = 0;
        while (*gen == g) {
          if (*err) {
            ok = 0;
            break;
          }
          if (++polls >= kT2BarrierPolls || ((polls & 255u) == 0 && t2_ns() - t0 > kT2BarrierNs)) {
            atomicExch(d.bar + 2, 1u);
            atomicExch(d.status, MFEM_ERR_TIMEOUT);
            ok = 0;
            break;
          }
          __nanosleep(32);
        }
      }
      __threadfence();
    }
    ok_s = ok;
  }
  __syncthreads();
  return ok_s != 0;
}

// The NQ block partials of this block into part[q * kT2MaxGrid + block]:
// a shuffle tree in each warp, then warp 0 combines the warps' sums, in a
// fixed order (one barrier).
template <int NQ> __device__ void t2_put_partials(const T2& d, const double (&v)[NQ], double* sh) {
  constexpr int kWarps = kGridThreads / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double x[NQ];
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    x[q] = v[q];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) x[q] += __shfl_down_sync(0xffffffffu, x[q], off);
  }
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < NQ; ++q) sh[q * kWarps + warp] = x[q];
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      double y = lane < kWarps ? sh[q * kWarps + lane] : 0.0;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) y += __shfl_down_sync(0xffffffffu, y, off);
      if (lane == 0) d.part[q * kT2MaxGrid + blockIdx.x] = y;
    }
  }
  __syncthreads();  // sh is free again
}

// The sums of the G partials of quantities 0..NQ-1, in the same order in
// every block (lane l sums entries l, l + 32, ... ; then a shuffle tree).
template <int NQ> __device__ void t2_totals(const T2& d, double (&out)[NQ], double* sh) {
  if (threadIdx.x < 32) {
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      double a = 0.0;
      for (int i = threadIdx.x; i < (int)gridDim.x; i += 32) a += __ldcg(d.part + q * kT2MaxGrid + i);
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) a += __shfl_down_sync(0xffffffffu, a, off);
      if (threadIdx.x == 0) sh[q] = a;
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < NQ; ++q) out[q] = sh[q];
  __syncthreads();
}

// s_k, r_{k+1} and u_{k+1} of one dof from r_k, w_k, s_{k-1} (wherever a
// row's values are formed: the same operations in the same order).
__device__ __forceinline__ void t2_next(double r, double w, double sp, double di, double a, double b,
                                        double& s, double& rn, double& u) {
  s = fma(b, sp, w);
  rn = fma(-a, s, r);
  u = di * rn;
}

__global__ void __launch_bounds__(kGridThreads) t2_pcg_grid(T2 d, int max_iter, double tol) {
  __shared__ double sh[kGridThreads];
  const int G = gridDim.x;
  const int per = (d.nf + G - 1) / G;
  const int r0 = min(d.nf, (int)blockIdx.x * per), r1 = min(d.nf, r0 + per);
  const int t = threadIdx.x;
  const size_t n2 = 2 * (size_t)d.nf;
  double* R[2] = {d.sr, d.sr + n2};
  double* W[2] = {d.sr + 2 * n2, d.sr + 3 * n2};
  double* S[2] = {d.sr + 4 * n2, d.sr + 5 * n2};
  // iteration -1: r_0 = b, s_{-1} = 0, p_{-1} = 0, dx = 0; w_0 = A u_0 with
  // u_0 = D^-1 b (formed where gathered); (r_0, u_0), (w_0, u_0), |b|^2
  double v3[3] = {0.0, 0.0, 0.0};
  for (int rr = r0 + t; rr < r1; rr += kGridThreads) {
    double y0 = 0, y1 = 0;
    for (int qq = d.b_ptr[rr]; qq < d.b_ptr[rr + 1]; ++qq) {
      const double* a = d.A + 4 * size_t(qq);
      const int c = d.b_col[qq];
      const double u0 = d.dinv[2 * c] * d.rhs[2 * c], u1 = d.dinv[2 * c + 1] * d.rhs[2 * c + 1];
      y0 += a[0] * u0 + a[1] * u1;
      y1 += a[2] * u0 + a[3] * u1;
    }
    const double y[2] = {y0, y1};
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const size_t i = 2 * (size_t)rr + k;
      const double b = d.rhs[i], u = d.dinv[i] * b;
      R[0][i] = b;
      W[0][i] = y[k];
      S[1][i] = 0.0;  // s_{-1}
      d.p[i] = 0.0;
      d.dx[i] = 0.0;
      v3[0] += b * u;
      v3[1] += y[k] * u;
      v3[2] += b * b;
    }
  }
  t2_put_partials<3>(d, v3, sh);
  if (!t2_grid_sync(d)) return;
  double tot[3];
  t2_totals<3>(d, tot, sh);
  double g = tot[0];
  const double dl = tot[1], b2 = tot[2];
  const double thr = fmax(tol * tol * b2, DBL_MIN);
  if (b2 == 0.0 || b2 < thr) {  // Eigen's test before the first iteration: no iteration
    if (blockIdx.x == 0 && t == 0) {
      d.scal[SC_CG_IT] = 0;
      d.scal[SC_CG_RN2] = b2;
      d.scal[SC_CG_B2] = b2;
    }
    return;
  }
  double a = g / dl, bt = 0.0, rn2 = b2;
  int it = 0;
  while (it < max_iter) {
    const int c0 = it & 1, c1 = c0 ^ 1;
    const double* r_o = R[c0];
    const double* w_o = W[c0];
    const double* s_p = S[c1];  // s_{k-1}
    double* r_n = R[c1];
    double* w_n = W[c1];
    double* s_n = S[c0];  // s_k
    v3[0] = v3[1] = v3[2] = 0.0;
    for (int rr = r0 + t; rr < r1; rr += kGridThreads) {
      // w_{k+1} = A u_{k+1}, each column's u_{k+1} formed from its r, w, s
      double y0 = 0, y1 = 0;
#pragma unroll 4
      for (int qq = d.b_ptr[rr]; qq < d.b_ptr[rr + 1]; ++qq) {
        const double* am = d.A + 4 * size_t(qq);
        const int c = d.b_col[qq];
        double sc0, rc0, u0, sc1, rc1, u1;
        t2_next(__ldcg(r_o + 2 * c), __ldcg(w_o + 2 * c), __ldcg(s_p + 2 * c), d.dinv[2 * c], a, bt, sc0, rc0, u0);
        t2_next(__ldcg(r_o + 2 * c + 1), __ldcg(w_o + 2 * c + 1), __ldcg(s_p + 2 * c + 1), d.dinv[2 * c + 1], a,
                bt, sc1, rc1, u1);
        y0 += am[0] * u0 + am[1] * u1;
        y1 += am[2] * u0 + am[3] * u1;
      }
      const double y[2] = {y0, y1};
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        const size_t i = 2 * (size_t)rr + k;
        const double r = __ldcg(r_o + i), w = __ldcg(w_o + i), sp = __ldcg(s_p + i);
        double sv, rn, un;
        t2_next(r, w, sp, d.dinv[i], a, bt, sv, rn, un);
        // p_k = u_k + b p_{k-1} with u_k = D^-1 r_k; x += a p_k
        const double pk = fma(bt, d.p[i], d.dinv[i] * r);
        d.p[i] = pk;
        d.dx[i] = fma(a, pk, d.dx[i]);
        s_n[i] = sv;
        r_n[i] = rn;
        w_n[i] = y[k];
        v3[0] += rn * un;
        v3[1] += y[k] * un;
        v3[2] += rn * rn;
      }
    }
    t2_put_partials<3>(d, v3, sh);
    if (!t2_grid_sync(d)) return;
    t2_totals<3>(d, tot, sh);
    const double gn = tot[0], dn = tot[1];
    rn2 = tot[2];
    if (rn2 < thr) break;
    const double bn = gn / g;
    a = gn / (dn - bn * gn / a);
    bt = bn;
    g = gn;
    ++it;
  }
  if (blockIdx.x == 0 && t == 0) {
    d.scal[SC_CG_IT] = it;
    d.scal[SC_CG_RN2] = rn2;
    d.scal[SC_CG_B2] = b2;
  }
}

// MixedStretch::solve (mixed_stretch.cpp:243-259): Jdx = -vol Jloc dx,
// lambda = -gl + Htil dSdF^T Jdx, ds = -H^-1 (Sym lambda + g).
__global__ void __launch_bounds__(kThreads) t2_local(T2 d) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= d.nt) return;
  const double vol = d.vol[e];
  const double* dX = d.dX + 6 * size_t(e);
  double Jdx[4] = {0, 0, 0, 0};
  for (int k = 0; k < 3; ++k) {
    const int f = d.free_map[d.tri[3 * e + k]];
    const double u[2] = {f >= 0 ? d.dx[2 * f] : 0.0, f >= 0 ? d.dx[2 * f + 1] : 0.0};
    for (int c = 0; c < 2; ++c)
      for (int r = 0; r < 2; ++r) Jdx[2 * c + r] -= vol * dX[2 * k + c] * u[r];
  }
  const double* D = d.dSdF + 12 * size_t(e);
  double DtJ[3];
  for (int i = 0; i < 3; ++i)
    DtJ[i] = D[4 * i] * Jdx[0] + D[4 * i + 1] * Jdx[1] + D[4 * i + 2] * Jdx[2] + D[4 * i + 3] * Jdx[3];
  const double* Ht = d.Htil + 9 * size_t(e);
  double w[3];
  for (int i = 0; i < 3; ++i) {
    const double la = -d.gl[3 * size_t(e) + i] + (Ht[i] * DtJ[0] + Ht[i + 3] * DtJ[1] + Ht[i + 6] * DtJ[2]);
    d.lam[3 * size_t(e) + i] = la;
    w[i] = kSym2[i] * la + d.g[3 * size_t(e) + i];
  }
  const double* Hi = d.Hinv + 9 * size_t(e);
  for (int i = 0; i < 3; ++i)
    d.ds[3 * size_t(e) + i] = -(Hi[i] * w[0] + Hi[i + 3] * w[1] + Hi[i + 6] * w[2]);
}

// The parts of energy_func(alpha) (newton_optimizer.cpp:34-49): per
// triangle vol psi(s + alpha ds) and vol lambda^T Sym (S(x + alpha dx) -
// s - alpha ds); per vertex d^T (M d) with d = x + alpha dx - x~ - h^2 f.
__global__ void __launch_bounds__(kThreads) t2_energy(T2 d, double alpha) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < d.nt) {
    double F[4], R[4], st[3], si[3];
    defgrad(d, i, alpha, nullptr, F);
    polar2(F, R, st, nullptr);
    for (int k = 0; k < 3; ++k) si[k] = d.s[3 * size_t(i) + k] + alpha * d.ds[3 * size_t(i) + k];
    const double vol = d.vol[i];
    d.epart[i] = coef2(d.mat[i], d.mu[i], d.la[i], si).psi * vol;
    double c = 0;
    for (int k = 0; k < 3; ++k) c += d.lam[3 * size_t(i) + k] * kSym2[k] * (st[k] - si[k]);
    d.epart[d.nt + i] = c * vol;
  }
  if (i < d.nv) {
    double p[2];
    pos2(d, i, alpha, nullptr, p);
    const double d0 = p[0] - d.xt[2 * i] - d.h2f0, d1 = p[1] - d.xt[2 * i + 1] - d.h2f1;
    double m0 = 0, m1 = 0;
    for (int q = d.m_ptr[i]; q < d.m_ptr[i + 1]; ++q) {
      const int u = d.m_col[q];
      double pu[2];
      pos2(d, u, alpha, nullptr, pu);
      m0 += d.m_val[q] * (pu[0] - d.xt[2 * u] - d.h2f0);
      m1 += d.m_val[q] * (pu[1] - d.xt[2 * u + 1] - d.h2f1);
    }
    d.epart[2 * d.nt + i] = d0 * m0 + d1 * m1;
  }
}

// E = 1/2 sum d^T M d + h^2 sum vol psi - sum vol lambda^T Sym (S - s),
// each sum in a fixed order, into scal[slot]; with_dec also writes
// max(|dx|_inf, |ds|_inf) (the Newton decrement).
__global__ void __launch_bounds__(kBlock) t2_esum(T2 d, double h2, int slot, int with_dec) {
  __shared__ double sh[kBlock];
  const int t = threadIdx.x;
  double a = 0, b = 0, c = 0;
  for (int i = t; i < d.nt; i += kBlock) a += d.epart[i];
  for (int i = t; i < d.nt; i += kBlock) b += d.epart[d.nt + i];
  for (int i = t; i < d.nv; i += kBlock) c += d.epart[2 * d.nt + i];
  const double sp = block_sum(a, sh);
  const double sq = block_sum(b, sh);
  const double sm = block_sum(c, sh);
  if (t == 0) d.scal[slot] = 0.5 * sm + h2 * sp - sq;
  if (with_dec) {
    double m = 0;
    for (int i = t; i < 2 * d.nf; i += kBlock) m = fmax(m, fabs(d.dx[i]));
    for (int i = t; i < 3 * d.nt; i += kBlock) m = fmax(m, fabs(d.ds[i]));
    const double mx = block_max(m, sh);
    if (t == 0) d.scal[SC_DEC] = mx;
  }
}

__global__ void __launch_bounds__(kThreads) t2_apply(T2 d, double alpha) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < 2 * d.nf) d.x[i] += alpha * d.dx[i];
  if (i < 3 * d.nt) d.s[i] += alpha * d.ds[i];
}

struct Bdf {
  double a[6];
  int order;
  int slot[6];  // slot of the i-th most recent entry
  double dt;    // beta h
};

// BDF<I> (BDF.cpp:6-93): with push, the new positions (free x, pinned b)
// and velocity (x - sum a_i x_i) / dt enter the history at slot `head`;
// then x~ = sum a_i x_i + dt sum a_i v_i over the (new) history.  One
// thread per vertex; flags a non-finite position.
__global__ void __launch_bounds__(kThreads) t2_history(T2 d, double* xh, double* vh, Bdf old_h,
                                                       Bdf new_h, int push) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= d.nv) return;
  const size_t n2 = 2 * size_t(d.nv);
  if (push) {
    double p[2];
    pos2(d, v, 0.0, nullptr, p);
    for (int k = 0; k < 2; ++k) {
      double w = 0;
      for (int i = 0; i < old_h.order; ++i) w += old_h.a[i] * xh[old_h.slot[i] * n2 + 2 * v + k];
      const double vn = (p[k] - w) / old_h.dt;
      xh[new_h.slot[0] * n2 + 2 * v + k] = p[k];
      vh[new_h.slot[0] * n2 + 2 * v + k] = vn;
      if (!isfinite(p[k])) atomicMax(d.status, int(MFEM_ERR_NONFINITE));
    }
  }
  for (int k = 0; k < 2; ++k) {
    double wx = 0, wv = 0;
    for (int i = 0; i < new_h.order; ++i) wx += new_h.a[i] * xh[new_h.slot[i] * n2 + 2 * v + k];
    for (int i = 0; i < new_h.order; ++i) wv += new_h.a[i] * vh[new_h.slot[i] * n2 + 2 * v + k];
    d.xt[2 * v + k] = wx + new_h.dt * wv;
  }
}

// Initial rotations and stretches (MixedStretch::reset, mixed_stretch.cpp:
// 261-304): s = S = polar(F(x0)), H = H^-1 = I.
__global__ void __launch_bounds__(kThreads) t2_init(T2 d) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= d.nt) return;
  double F[4], R[4], sv[3];
  defgrad(d, e, 0.0, nullptr, F);
  if (!polar2(F, R, sv, nullptr)) atomicMax(d.status, int(MFEM_ERR_PROCRUSTES));
  for (int k = 0; k < 4; ++k) d.R[4 * size_t(e) + k] = R[k];
  for (int k = 0; k < 3; ++k) d.s[3 * size_t(e) + k] = d.S[3 * size_t(e) + k] = sv[k];
  for (int k = 0; k < 9; ++k) d.H[9 * size_t(e) + k] = d.Hinv[9 * size_t(e) + k] = (k % 4 == 0) ? 1.0 : 0.0;
}

int grid_of(long n) { return int(std::max(1L, (n + kThreads - 1) / kThreads)); }

size_t align256(size_t v) { return (v + 255) / 256 * 256; }

}  // namespace

// ---------------------------------------------------------------------------
struct mfem_tri2d {
  int nv = 0, nt = 0, nf = 0, nnzb = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  char* dev = nullptr;
  T2 d{};
  double* xh = nullptr;  // bdf slots of 2 nv positions
  double* vh = nullptr;
  double* xscratch = nullptr;  // 2 nv (parity entry point)
  int head = 0;
  // launch counts (always) and CUDA-event times (profiling on) per kernel
  int64_t launches[MFEM_T2_K_COUNT] = {};
  double kernel_ms[MFEM_T2_K_COUNT] = {};
  bool profiling = false;
  std::vector<cudaEvent_t> ev_pool;
  struct Pending { int kernel, a, b; };
  std::vector<Pending> ev_pending;
  size_t ev_used = 0;
  // blocks of the grid PCG (t2_pcg_grid), 0: the one-block t2_pcg
  int pcg_grid = 0;
  // configuration
  int bdf = 1, max_newton = 5, ls_iters = 20, cg_iters = 500;
  double h = 0.0333, cg_tol = 1e-4, newton_tol = 1e-10, res_tol = 0, load_norm = 0;
  // host copies: the BC scripts move pinned vertices on the host
  std::vector<double> Vref, V, bhost;
  std::vector<int> is_fixed, free_map, b_ptr, b_col;
  int bc_type = 0, bc_axis = 0;
  double bc_ratio = 0.1, bc_vel = 0.1;
  std::vector<std::vector<int>> groups;
  double twist_center[2] = {0, 0};
  double group_center[2][2] = {{0, 0}, {0, 0}};

  ~mfem_tri2d() {
    for (cudaEvent_t e : ev_pool) cudaEventDestroy(e);
    if (dev) cudaFree(dev);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (stream) cudaStreamDestroy(stream);
  }
  double dt_bdf() const {
    static const double beta[7] = {0, 1.0, 2.0 / 3, 6.0 / 11, 12.0 / 25, 60.0 / 137, 60.0 / 147};
    return beta[bdf] * h;
  }
  Bdf bdf_at(int hd) const {
    static const double a[7][6] = {
        {0},
        {1.0},
        {4.0 / 3, -1.0 / 3},
        {18.0 / 11, -9.0 / 11, 2.0 / 11},
        {48.0 / 25, -36.0 / 25, 16.0 / 25, -3.0 / 25},
        {300.0 / 137, -300.0 / 137, 200.0 / 137, -75.0 / 137, 12.0 / 137},
        {360.0 / 147, -450.0 / 147, 400.0 / 147, -225.0 / 147, 72.0 / 147, -10.0 / 147}};
    Bdf b{};
    b.order = bdf;
    b.dt = dt_bdf();
    for (int i = 0; i < 6; ++i) {
      b.a[i] = a[bdf][i];
      b.slot[i] = (hd + i) % bdf;
    }
    return b;
  }
};

namespace {

void bbox2(const std::vector<double>& V, int nv, double lo[2], double hi[2]) {
  for (int k = 0; k < 2; ++k) {
    lo[k] = INFINITY;
    hi[k] = -INFINITY;
  }
  for (int v = 0; v < nv; ++v)
    for (int k = 0; k < 2; ++k) {
      lo[k] = std::min(lo[k], V[2 * v + k]);
      hi[k] = std::max(hi[k], V[2 * v + k]);
    }
}

// BoundaryCondition::init_boundary_groups (boundary_condition.cpp:5-21) and
// the scripts' init (fixed_boundary_conditions.h, stretch/twist/bend_*.h).
void bc_init(mfem_tri2d& sc, const int32_t* override_fixed) {
  double lo[2], hi[2];
  bbox2(sc.Vref, sc.nv, lo, hi);
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
  bbox2(sc.V, sc.nv, lo, hi);
  double ctr[2] = {0.5 * (lo[0] + hi[0]), 0.5 * (lo[1] + hi[1])};
  switch (sc.bc_type) {
    case MFEM_BC_SCALEF:
      for (int v = 0; v < sc.nv; ++v)
        for (int k = 0; k < 2; ++k) sc.V[2 * v + k] = (sc.V[2 * v + k] - ctr[k]) * 1.5 + ctr[k];
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
        for (int k = 0; k < 2; ++k) sc.V[2 * v + k] += ctr[k] - r0[k];
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
      sc.twist_center[0] = ctr[0];
      sc.twist_center[1] = ctr[1];
      for (int i = 0; i < 2; ++i) {
        const int v = sc.groups[i].empty() ? 0 : sc.groups[i].back();
        sc.group_center[i][0] = sc.V[2 * v];
        sc.group_center[i][1] = sc.V[2 * v + 1];
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

// BoundaryCondition::step of the scripted BCs (Meshes::update_bcs).
void bc_step(mfem_tri2d& sc, double dt) {
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
        for (int v : sc.groups[i]) rotate2(&sc.V[2 * v], sc.twist_center, a);
      }
      break;
    case MFEM_BC_BEND:
      for (int i = 0; i < 2; ++i) {
        const double a = (i == 0 ? 1 : -1) * sc.bc_vel * M_PI * dt;
        for (int v : sc.groups[i]) rotate2(&sc.V[2 * v], sc.group_center[i], a);
      }
      break;
    default:
      break;
  }
}

#define T2_CUDA(expr)                          \
  do {                                         \
    if ((expr) != cudaSuccess) return MFEM_ERR_CUDA; \
  } while (0)

int launch_status() { return cudaGetLastError() == cudaSuccess ? MFEM_OK : MFEM_ERR_CUDA; }

// An event of the scene's pool (created on first use, reused after each
// collection); -1 when none can be created.
int take_event(mfem_tri2d& sc) {
  if (sc.ev_used == sc.ev_pool.size()) {
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) {
      cudaGetLastError();
      return -1;
    }
    sc.ev_pool.push_back(e);
  }
  return int(sc.ev_used++);
}

// Counts a launch of kernel k and, with profiling on, brackets it by events.
template <typename F> void launch(mfem_tri2d& sc, int k, F&& f) {
  ++sc.launches[k];
  if (!sc.profiling) {
    f();
    return;
  }
  const int a = take_event(sc), b = take_event(sc);
  if (a >= 0 && b >= 0) cudaEventRecord(sc.ev_pool[a], sc.stream);
  f();
  if (a >= 0 && b >= 0) {
    cudaEventRecord(sc.ev_pool[b], sc.stream);
    sc.ev_pending.push_back({k, a, b});
  }
}

// Adds the bracketed launches' times (the stream has been synchronised).
void collect_events(mfem_tri2d& sc) {
  for (const auto& p : sc.ev_pending) {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, sc.ev_pool[p.a], sc.ev_pool[p.b]) == cudaSuccess)
      sc.kernel_ms[p.kernel] += ms;
  }
  sc.ev_pending.clear();
  sc.ev_used = 0;
}

// elem + rows at the current state (update_system of the Newton loop).
int t2_update(mfem_tri2d& sc, const double* xfull) {
  const double dt = sc.dt_bdf();
  launch(sc, MFEM_T2_K_ELEM,
         [&] { t2_elem<<<grid_of(sc.nt), kThreads, 0, sc.stream>>>(sc.d, dt * dt, xfull); });
  if (!xfull && sc.nf > 0)
    launch(sc, MFEM_T2_K_ROWS, [&] { t2_rows<<<grid_of(sc.nf), kThreads, 0, sc.stream>>>(sc.d); });
  return launch_status();
}

int t2_energy_at(mfem_tri2d& sc, double alpha, int with_dec, double* scal_host) {
  const double dt = sc.dt_bdf();
  launch(sc, MFEM_T2_K_ENERGY, [&] {
    t2_energy<<<grid_of(std::max(sc.nt, sc.nv)), kThreads, 0, sc.stream>>>(sc.d, alpha);
  });
  launch(sc, MFEM_T2_K_ESUM,
         [&] { t2_esum<<<1, kBlock, 0, sc.stream>>>(sc.d, dt * dt, SC_E, with_dec); });
  if (launch_status() != MFEM_OK) return MFEM_ERR_CUDA;
  T2_CUDA(cudaMemcpyAsync(scal_host, sc.d.scal, sizeof(double) * SC_COUNT, cudaMemcpyDeviceToHost,
                          sc.stream));
  T2_CUDA(cudaStreamSynchronize(sc.stream));
  return MFEM_OK;
}

int read_status(mfem_tri2d& sc, int* st) {
  T2_CUDA(cudaMemcpyAsync(st, sc.d.status, sizeof(int), cudaMemcpyDeviceToHost, sc.stream));
  T2_CUDA(cudaStreamSynchronize(sc.stream));
  return MFEM_OK;
}

// NewtonOptimizer<2>::step (newton_optimizer.cpp:11-89).
int t2_step(mfem_tri2d& sc, mfem_step_stats* out) {
  mfem_step_stats st{};
  int status = MFEM_OK;
  int i = 0;
  double E = 0, E_prev = 0, res = 0, dec = 0;
  double scal[SC_COUNT];
  T2_CUDA(cudaEventRecord(sc.ev0, sc.stream));
  do {
    T2_CUDA(cudaMemsetAsync(sc.d.status, 0, sizeof(int), sc.stream));
    if (t2_update(sc, nullptr) != MFEM_OK) return MFEM_ERR_CUDA;
    launch(sc, MFEM_T2_K_NORM, [&] { t2_norm<<<1, kBlock, 0, sc.stream>>>(sc.d); });
    if (launch_status() != MFEM_OK) return MFEM_ERR_CUDA;
    int kst = 0;
    T2_CUDA(cudaMemcpyAsync(scal, sc.d.scal, sizeof(scal), cudaMemcpyDeviceToHost, sc.stream));
    if (read_status(sc, &kst) != MFEM_OK) return MFEM_ERR_CUDA;
    if (kst != MFEM_OK) status = kst;
    const double rn = std::sqrt(scal[SC_RN2]);
    if (i == 0) st.residual0 = rn;
    st.residual = rn;
    if (sc.res_tol > 0 && ((i > 0 && rn <= sc.res_tol * st.residual0) || rn <= sc.res_tol * sc.load_norm))
      break;
    if (sc.nf > 0 && sc.pcg_grid > 0) {
      // a fresh barrier (arrivals, generation, error) for the cooperative launch
      T2_CUDA(cudaMemsetAsync(sc.d.bar, 0, 4 * sizeof(unsigned int), sc.stream));
      cudaError_t e = cudaSuccess;
      launch(sc, MFEM_T2_K_PCG, [&] {
        T2 dd = sc.d;
        int mi = sc.cg_iters;
        double tl = sc.cg_tol;
        void* args[] = {&dd, &mi, &tl};
        e = cudaLaunchCooperativeKernel((const void*)t2_pcg_grid, dim3(sc.pcg_grid), dim3(kGridThreads), args, 0,
                                        sc.stream);
      });
      T2_CUDA(e);
    } else if (sc.nf > 0) {
      launch(sc, MFEM_T2_K_PCG,
             [&] { t2_pcg<<<1, kBlock, 0, sc.stream>>>(sc.d, sc.cg_iters, sc.cg_tol); });
    }
    launch(sc, MFEM_T2_K_LOCAL, [&] { t2_local<<<grid_of(sc.nt), kThreads, 0, sc.stream>>>(sc.d); });
    if (launch_status() != MFEM_OK) return MFEM_ERR_CUDA;
    if (t2_energy_at(sc, 0.0, 1, scal) != MFEM_OK) return MFEM_ERR_CUDA;
    const int iters = sc.nf > 0 ? int(scal[SC_CG_IT]) : 0;
    const double b2 = sc.nf > 0 ? scal[SC_CG_B2] : 0.0;
    if (sc.nf > 0 && iters >= sc.cg_iters && status == MFEM_OK) status = MFEM_ERR_CG_MAXITER;
    st.cg_iterations += iters;
    st.cg_error = b2 > 0 ? std::sqrt(scal[SC_CG_RN2] / b2) : 0.0;
    dec = scal[SC_DEC];
    E = scal[SC_E];
    res = std::fabs((E - E_prev) / (E + 1e-6));
    E_prev = E;
    double alpha = 1.0;
    const double fx0 = E;
    int it = 0;
    while (it < sc.ls_iters) {
      if (t2_energy_at(sc, alpha, 0, scal) != MFEM_OK) return MFEM_ERR_CUDA;
      if (scal[SC_E] < fx0) break;
      alpha *= 0.5;
      ++it;
    }
    st.ls_iterations += it;
    if (it < sc.ls_iters) {
      launch(sc, MFEM_T2_K_APPLY, [&] {
        t2_apply<<<grid_of(std::max(2L * sc.nf, 3L * sc.nt)), kThreads, 0, sc.stream>>>(sc.d, alpha);
      });
      if (launch_status() != MFEM_OK) return MFEM_ERR_CUDA;
    } else if (status == MFEM_OK) {
      status = MFEM_ERR_LS_FAILED;
    }
    st.alpha = alpha;
    ++i;
  } while (i < sc.max_newton && dec > sc.newton_tol && res > 1e-12);
  st.newton_iterations = i;
  st.energy = E;
  st.energy_residual = res;
  st.decrement = dec;
  // update_bcs, Displacement::post_solve (BDF update), MixedStretch::post_solve (lambda = 0)
  bc_step(sc, sc.h);
  for (int v = 0; v < sc.nv; ++v)
    if (sc.is_fixed[v])
      for (int k = 0; k < 2; ++k) sc.bhost[2 * v + k] = sc.V[2 * v + k];
  T2_CUDA(cudaMemcpyAsync(sc.d.b, sc.bhost.data(), sizeof(double) * 2 * sc.nv, cudaMemcpyHostToDevice,
                          sc.stream));
  T2_CUDA(cudaMemsetAsync(sc.d.status, 0, sizeof(int), sc.stream));
  const Bdf old_h = sc.bdf_at(sc.head);
  const int new_head = (sc.head + sc.bdf - 1) % sc.bdf;
  const Bdf new_h = sc.bdf_at(new_head);
  launch(sc, MFEM_T2_K_HISTORY, [&] {
    t2_history<<<grid_of(sc.nv), kThreads, 0, sc.stream>>>(sc.d, sc.xh, sc.vh, old_h, new_h, 1);
  });
  if (launch_status() != MFEM_OK) return MFEM_ERR_CUDA;
  sc.head = new_head;
  T2_CUDA(cudaMemsetAsync(sc.d.lam, 0, sizeof(double) * 3 * sc.nt, sc.stream));
  T2_CUDA(cudaEventRecord(sc.ev1, sc.stream));
  int kst = 0;
  if (read_status(sc, &kst) != MFEM_OK) return MFEM_ERR_CUDA;
  if (kst != MFEM_OK) status = kst;
  float ms = 0;
  T2_CUDA(cudaEventElapsedTime(&ms, sc.ev0, sc.ev1));
  st.device_ms = ms;
  collect_events(sc);
  st.status = status;
  if (out) *out = st;
  return status;
}

struct Layout {
  size_t off = 0;
  template <typename T> size_t take(size_t n) {
    const size_t o = align256(off);
    off = o + n * sizeof(T);
    return o;
  }
};

}  // namespace

extern "C" {

int mfem_gpu_tri2d_create(const mfem_tri2d_desc* dsc, mfem_tri2d** out) {
  if (!out) return MFEM_ERR_INVALID;
  *out = nullptr;
  if (!dsc || dsc->n_vertices <= 0 || dsc->n_tris <= 0 || !dsc->V_rest || !dsc->tris || !dsc->mu ||
      !dsc->lambda || dsc->bdf_order < 1 || dsc->bdf_order > 6 || dsc->bc_axis < 0 || dsc->bc_axis > 1 ||
      !(dsc->dt > 0) || dsc->max_newton_iterations < 1 || dsc->max_linesearch_iterations < 0 ||
      dsc->max_iterative_solver_iters < 0)
    return MFEM_ERR_INVALID;
  if (dsc->linear_solver != MFEM_SOLVER_EIGEN_CG_DIAG) return MFEM_ERR_UNSUPPORTED;
  const int nv = dsc->n_vertices, nt = dsc->n_tris;
  std::vector<int> mat(nt, MFEM_MATERIAL_SNH);
  if (dsc->material)
    for (int e = 0; e < nt; ++e) {
      mat[e] = dsc->material[e];
      if (mat[e] != MFEM_MATERIAL_SNH && mat[e] != MFEM_MATERIAL_COROT && mat[e] != MFEM_MATERIAL_FCR &&
          mat[e] != MFEM_MATERIAL_ARAP)
        return MFEM_ERR_UNSUPPORTED;
    }
  for (int k = 0; k < 3 * nt; ++k)
    if (dsc->tris[k] < 0 || dsc->tris[k] >= nv) return MFEM_ERR_INVALID;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return MFEM_ERR_NO_DEVICE;

  auto sc = std::unique_ptr<mfem_tri2d>(new (std::nothrow) mfem_tri2d());
  if (!sc) return MFEM_ERR_OOM;
  sc->nv = nv;
  sc->nt = nt;
  sc->bdf = dsc->bdf_order;
  sc->max_newton = dsc->max_newton_iterations;
  sc->ls_iters = dsc->max_linesearch_iterations;
  sc->cg_iters = dsc->max_iterative_solver_iters;
  sc->h = dsc->dt;
  sc->cg_tol = dsc->iterative_solver_tolerance;
  sc->newton_tol = dsc->newton_tol;
  sc->res_tol = dsc->newton_residual_tolerance;
  sc->bc_type = dsc->bc_type;
  sc->bc_axis = dsc->bc_axis;
  sc->bc_ratio = dsc->bc_ratio;
  sc->bc_vel = dsc->bc_velocity;
  sc->Vref.assign(dsc->V_rest, dsc->V_rest + 2 * size_t(nv));
  sc->V = dsc->V_init ? std::vector<double>(dsc->V_init, dsc->V_init + 2 * size_t(nv)) : sc->Vref;
  bc_init(*sc, dsc->is_fixed);
  sc->free_map.assign(nv, -1);
  std::vector<int> row_vertex;
  for (int v = 0; v < nv; ++v)
    if (!sc->is_fixed[v]) {
      sc->free_map[v] = sc->nf++;
      row_vertex.push_back(v);
    }
  const int nf = sc->nf;
  const int* T = dsc->tris;
  // doublearea volumes and dphi/dX (rows of Dm^-1)
  std::vector<double> vol(nt), dX(6 * size_t(nt)), mu(nt), la(nt), rho(nt);
  for (int e = 0; e < nt; ++e) {
    const double* X0 = &sc->Vref[2 * T[3 * e]];
    const double* X1 = &sc->Vref[2 * T[3 * e + 1]];
    const double* X2 = &sc->Vref[2 * T[3 * e + 2]];
    const double m00 = X1[0] - X0[0], m10 = X1[1] - X0[1];
    const double m01 = X2[0] - X0[0], m11 = X2[1] - X0[1];
    const double det = m00 * m11 - m01 * m10;
    if (!(det > 0) || !std::isfinite(det)) return MFEM_ERR_INVALID;  // clockwise or degenerate
    vol[e] = det;
    const double i00 = m11 / det, i01 = -m01 / det, i10 = -m10 / det, i11 = m00 / det;
    double* dx = &dX[6 * size_t(e)];
    dx[2] = i00;
    dx[3] = i01;
    dx[4] = i10;
    dx[5] = i11;
    dx[0] = -(i00 + i10);
    dx[1] = -(i01 + i11);
    mu[e] = dsc->mu[e];
    la[e] = dsc->lambda[e];
    rho[e] = dsc->density ? dsc->density[e] : dsc->density_const;
  }
  // consistent P1 mass rho vol/12 (1 + delta_ab) as a scalar vertex CSR
  std::vector<int> m_ptr(nv + 1, 0), m_col;
  std::vector<double> m_val;
  {
    std::vector<std::vector<std::pair<int, double>>> rows(nv);
    for (int e = 0; e < nt; ++e) {
      const double m = rho[e] * vol[e] / 12.0;
      for (int a = 0; a < 3; ++a)
        for (int bq = 0; bq < 3; ++bq) rows[T[3 * e + a]].push_back({T[3 * e + bq], a == bq ? 2 * m : m});
    }
    for (int v = 0; v < nv; ++v) {
      auto& r = rows[v];
      std::stable_sort(r.begin(), r.end(), [](auto& u, auto& w) { return u.first < w.first; });
      for (size_t i = 0; i < r.size(); ++i) {
        if (i > 0 && r[i].first == r[i - 1].first) {
          m_val.back() += r[i].second;
        } else {
          m_col.push_back(r[i].first);
          m_val.push_back(r[i].second);
        }
      }
      m_ptr[v + 1] = int(m_col.size());
    }
  }
  // Assembler<double,2,-1>: free (row, col) pairs sorted row-major; each
  // block's contributions in triangle order
  struct P { int r, c, ent; };
  std::vector<P> pairs;
  pairs.reserve(9 * size_t(nt));
  for (int e = 0; e < nt; ++e)
    for (int j = 0; j < 3; ++j) {
      const int a = sc->free_map[T[3 * e + j]];
      if (a < 0) continue;
      for (int k = 0; k < 3; ++k) {
        const int bq = sc->free_map[T[3 * e + k]];
        if (bq < 0) continue;
        pairs.push_back({a, bq, 9 * e + 3 * j + k});
      }
    }
  std::stable_sort(pairs.begin(), pairs.end(),
                   [](const P& u, const P& w) { return u.r < w.r || (u.r == w.r && u.c < w.c); });
  sc->b_ptr.assign(nf + 1, 0);
  std::vector<int> c_ptr(1, 0), c_ent(pairs.size());
  for (size_t i = 0; i < pairs.size(); ++i) {
    if (i == 0 || pairs[i].r != pairs[i - 1].r || pairs[i].c != pairs[i - 1].c) {
      if (i > 0) c_ptr.push_back(int(i));
      sc->b_col.push_back(pairs[i].c);
      sc->b_ptr[pairs[i].r + 1]++;
    }
    c_ent[i] = pairs[i].ent;
  }
  c_ptr.push_back(int(pairs.size()));
  if (pairs.empty()) c_ptr.assign(1, 0);
  for (int r = 0; r < nf; ++r) sc->b_ptr[r + 1] += sc->b_ptr[r];
  const int nnzb = int(sc->b_col.size());
  sc->nnzb = nnzb;
  std::vector<double> b_mass(nnzb, 0.0);
  for (int a = 0; a < nv; ++a) {
    const int fa = sc->free_map[a];
    if (fa < 0) continue;
    for (int q = m_ptr[a]; q < m_ptr[a + 1]; ++q) {
      const int fb = sc->free_map[m_col[q]];
      if (fb < 0) continue;
      const int* beg = sc->b_col.data() + sc->b_ptr[fa];
      const int* end = sc->b_col.data() + sc->b_ptr[fa + 1];
      const int* it = std::lower_bound(beg, end, fb);
      if (it != end && *it == fb) b_mass[it - sc->b_col.data()] += m_val[q];
    }
  }
  // each free row's incident (triangle, corner) in triangle order
  std::vector<int> i_ptr(nf + 1, 0), i_ent;
  {
    std::vector<std::vector<int>> inc(nf);
    for (int e = 0; e < nt; ++e)
      for (int k = 0; k < 3; ++k) {
        const int f = sc->free_map[T[3 * e + k]];
        if (f >= 0) inc[f].push_back(3 * e + k);
      }
    for (int r = 0; r < nf; ++r) {
      i_ent.insert(i_ent.end(), inc[r].begin(), inc[r].end());
      i_ptr[r + 1] = int(i_ent.size());
    }
  }
  // Displacement::reset: positions, pins, gravity load scale
  const double dtb = sc->dt_bdf();
  sc->bhost.assign(2 * size_t(nv), 0.0);
  std::vector<double> xfree(2 * size_t(nf));
  for (int v = 0; v < nv; ++v)
    for (int k = 0; k < 2; ++k) {
      if (sc->is_fixed[v])
        sc->bhost[2 * v + k] = sc->V[2 * v + k];
      else
        xfree[2 * sc->free_map[v] + k] = sc->V[2 * v + k];
    }
  const double fext[2] = {double(float(dsc->body_force[0])), double(float(dsc->body_force[1]))};
  {
    double acc = 0;
    const double dt2 = dtb * dtb;
    for (int v = 0; v < nv; ++v) {
      if (sc->free_map[v] < 0) continue;
      double m = 0;
      for (int q = m_ptr[v]; q < m_ptr[v + 1]; ++q) m += m_val[q];
      for (int k = 0; k < 2; ++k) acc += (dt2 * m * fext[k]) * (dt2 * m * fext[k]);
    }
    sc->load_norm = std::sqrt(acc);
  }
  std::vector<double> v0 = dsc->v_init ? std::vector<double>(dsc->v_init, dsc->v_init + 2 * size_t(nv))
                                       : std::vector<double>(2 * size_t(nv), 0.0);

  // one device allocation
  Layout L;
  const size_t o_tri = L.take<int>(3 * size_t(nt)), o_dX = L.take<double>(6 * size_t(nt)),
               o_vol = L.take<double>(nt), o_mu = L.take<double>(nt), o_la = L.take<double>(nt),
               o_mat = L.take<int>(nt), o_fm = L.take<int>(nv), o_rv = L.take<int>(std::max(nf, 1)),
               o_x = L.take<double>(2 * size_t(std::max(nf, 1))), o_dx = L.take<double>(2 * size_t(std::max(nf, 1))),
               o_b = L.take<double>(2 * size_t(nv)), o_xt = L.take<double>(2 * size_t(nv)),
               o_s = L.take<double>(3 * size_t(nt)), o_ds = L.take<double>(3 * size_t(nt)),
               o_lam = L.take<double>(3 * size_t(nt)), o_R = L.take<double>(4 * size_t(nt)),
               o_S = L.take<double>(3 * size_t(nt)), o_dSdF = L.take<double>(12 * size_t(nt)),
               o_g = L.take<double>(3 * size_t(nt)), o_H = L.take<double>(9 * size_t(nt)),
               o_Hinv = L.take<double>(9 * size_t(nt)), o_Htil = L.take<double>(9 * size_t(nt)),
               o_gl = L.take<double>(3 * size_t(nt)), o_Aloc = L.take<double>(36 * size_t(nt)),
               o_fel = L.take<double>(6 * size_t(nt)), o_mptr = L.take<int>(nv + 1),
               o_mcol = L.take<int>(m_col.size()), o_mval = L.take<double>(m_val.size()),
               o_bptr = L.take<int>(nf + 1), o_bcol = L.take<int>(std::max(nnzb, 1)),
               o_bmass = L.take<double>(std::max(nnzb, 1)), o_cptr = L.take<int>(c_ptr.size()),
               o_cent = L.take<int>(std::max<size_t>(c_ent.size(), 1)), o_iptr = L.take<int>(nf + 1),
               o_ient = L.take<int>(std::max<size_t>(i_ent.size(), 1)),
               o_A = L.take<double>(4 * size_t(std::max(nnzb, 1))),
               o_rhs = L.take<double>(2 * size_t(std::max(nf, 1))),
               o_dinv = L.take<double>(2 * size_t(std::max(nf, 1))),
               o_r = L.take<double>(2 * size_t(std::max(nf, 1))), o_p = L.take<double>(2 * size_t(std::max(nf, 1))),
               o_q = L.take<double>(2 * size_t(std::max(nf, 1))),
               o_sr = L.take<double>(12 * size_t(std::max(nf, 1))), o_part = L.take<double>(3 * kT2MaxGrid),
               o_bar = L.take<unsigned int>(4),
               o_ep = L.take<double>(2 * size_t(nt) + nv), o_scal = L.take<double>(SC_COUNT),
               o_st = L.take<int>(4), o_xh = L.take<double>(2 * size_t(nv) * sc->bdf),
               o_vh = L.take<double>(2 * size_t(nv) * sc->bdf), o_xs = L.take<double>(2 * size_t(nv));
  const size_t total = align256(L.off);
  if (cudaStreamCreateWithFlags(&sc->stream, cudaStreamNonBlocking) != cudaSuccess) return MFEM_ERR_CUDA;
  if (cudaEventCreate(&sc->ev0) != cudaSuccess || cudaEventCreate(&sc->ev1) != cudaSuccess)
    return MFEM_ERR_CUDA;
  if (cudaMalloc(&sc->dev, total) != cudaSuccess) {
    sc->dev = nullptr;
    cudaGetLastError();
    return MFEM_ERR_OOM;
  }
  char* base = sc->dev;
  if (cudaMemsetAsync(base, 0, total, sc->stream) != cudaSuccess) return MFEM_ERR_CUDA;
  // sheets with more free rows than the one-block PCG can carry (one row a
  // thread) iterate over co-resident blocks of at least 64 rows each
  if (nf > kBlock) {
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, t2_pcg_grid, kGridThreads, 0) != cudaSuccess)
      return MFEM_ERR_CUDA;
    sc->pcg_grid = std::max(1, std::min({per_sm * sms, (nf + 63) / 64, kT2MaxGrid}));
  }
  T2& d = sc->d;
  d.nv = nv;
  d.nt = nt;
  d.nf = nf;
  d.nnzb = nnzb;
  auto dp = [&](size_t o) { return reinterpret_cast<double*>(base + o); };
  auto ip = [&](size_t o) { return reinterpret_cast<int*>(base + o); };
  d.tri = ip(o_tri);
  d.dX = dp(o_dX);
  d.vol = dp(o_vol);
  d.mu = dp(o_mu);
  d.la = dp(o_la);
  d.mat = ip(o_mat);
  d.free_map = ip(o_fm);
  d.row_vertex = ip(o_rv);
  d.x = dp(o_x);
  d.dx = dp(o_dx);
  d.b = dp(o_b);
  d.xt = dp(o_xt);
  d.s = dp(o_s);
  d.ds = dp(o_ds);
  d.lam = dp(o_lam);
  d.R = dp(o_R);
  d.S = dp(o_S);
  d.dSdF = dp(o_dSdF);
  d.g = dp(o_g);
  d.H = dp(o_H);
  d.Hinv = dp(o_Hinv);
  d.Htil = dp(o_Htil);
  d.gl = dp(o_gl);
  d.Aloc = dp(o_Aloc);
  d.fel = dp(o_fel);
  d.m_ptr = ip(o_mptr);
  d.m_col = ip(o_mcol);
  d.m_val = dp(o_mval);
  d.b_ptr = ip(o_bptr);
  d.b_col = ip(o_bcol);
  d.b_mass = dp(o_bmass);
  d.c_ptr = ip(o_cptr);
  d.c_ent = ip(o_cent);
  d.i_ptr = ip(o_iptr);
  d.i_ent = ip(o_ient);
  d.A = dp(o_A);
  d.rhs = dp(o_rhs);
  d.dinv = dp(o_dinv);
  d.r = dp(o_r);
  d.p = dp(o_p);
  d.q = dp(o_q);
  d.sr = dp(o_sr);
  d.part = dp(o_part);
  d.bar = reinterpret_cast<unsigned int*>(base + o_bar);
  d.epart = dp(o_ep);
  d.scal = dp(o_scal);
  d.status = ip(o_st);
  d.h2f0 = (dtb * dtb) * fext[0];
  d.h2f1 = (dtb * dtb) * fext[1];
  sc->xh = dp(o_xh);
  sc->vh = dp(o_vh);
  sc->xscratch = dp(o_xs);
  auto up = [&](size_t o, const void* src, size_t bytes) {
    return bytes == 0 || cudaMemcpyAsync(base + o, src, bytes, cudaMemcpyHostToDevice, sc->stream) == cudaSuccess;
  };
  bool ok = up(o_tri, T, 12 * size_t(nt)) && up(o_dX, dX.data(), 8 * dX.size()) &&
            up(o_vol, vol.data(), 8 * size_t(nt)) && up(o_mu, mu.data(), 8 * size_t(nt)) &&
            up(o_la, la.data(), 8 * size_t(nt)) && up(o_mat, mat.data(), 4 * size_t(nt)) &&
            up(o_fm, sc->free_map.data(), 4 * size_t(nv)) && up(o_rv, row_vertex.data(), 4 * row_vertex.size()) &&
            up(o_x, xfree.data(), 8 * xfree.size()) && up(o_b, sc->bhost.data(), 8 * sc->bhost.size()) &&
            up(o_mptr, m_ptr.data(), 4 * m_ptr.size()) && up(o_mcol, m_col.data(), 4 * m_col.size()) &&
            up(o_mval, m_val.data(), 8 * m_val.size()) && up(o_bptr, sc->b_ptr.data(), 4 * sc->b_ptr.size()) &&
            up(o_bcol, sc->b_col.data(), 4 * sc->b_col.size()) && up(o_bmass, b_mass.data(), 8 * b_mass.size()) &&
            up(o_cptr, c_ptr.data(), 4 * c_ptr.size()) && up(o_cent, c_ent.data(), 4 * c_ent.size()) &&
            up(o_iptr, i_ptr.data(), 4 * i_ptr.size()) && up(o_ient, i_ent.data(), 4 * i_ent.size());
  // the BDF history: every slot holds (x0, v0)
  for (int i = 0; i < sc->bdf && ok; ++i)
    ok = up(o_xh + 8 * 2 * size_t(nv) * i, sc->V.data(), 8 * 2 * size_t(nv)) &&
         up(o_vh + 8 * 2 * size_t(nv) * i, v0.data(), 8 * 2 * size_t(nv));
  if (!ok) return MFEM_ERR_CUDA;
  sc->head = 0;
  const Bdf hb = sc->bdf_at(0);
  t2_history<<<grid_of(nv), kThreads, 0, sc->stream>>>(d, sc->xh, sc->vh, hb, hb, 0);
  t2_init<<<grid_of(nt), kThreads, 0, sc->stream>>>(d);
  if (launch_status() != MFEM_OK) return MFEM_ERR_CUDA;
  int kst = 0;
  if (read_status(*sc, &kst) != MFEM_OK) return MFEM_ERR_CUDA;
  if (kst != MFEM_OK) return kst;
  *out = sc.release();
  return MFEM_OK;
}

int mfem_gpu_tri2d_destroy(mfem_tri2d* scene) {
  if (!scene) return MFEM_ERR_INVALID;
  if (scene->stream) cudaStreamSynchronize(scene->stream);
  delete scene;
  return MFEM_OK;
}

int mfem_gpu_tri2d_step(mfem_tri2d* scene, mfem_step_stats* stats) {
  if (!scene) return MFEM_ERR_INVALID;
  return t2_step(*scene, stats);
}

int mfem_gpu_tri2d_sizes(const mfem_tri2d* scene, int32_t* n_vertices, int32_t* n_tris, int32_t* n_free,
                         int32_t* nnzb) {
  if (!scene) return MFEM_ERR_INVALID;
  if (n_vertices) *n_vertices = scene->nv;
  if (n_tris) *n_tris = scene->nt;
  if (n_free) *n_free = scene->nf;
  if (nnzb) *nnzb = scene->nnzb;
  return MFEM_OK;
}

int mfem_gpu_tri2d_get_state(mfem_tri2d* sc, double* x, double* v, double* s, double* R, double* la) {
  if (!sc) return MFEM_ERR_INVALID;
  const size_t nv = sc->nv, nt = sc->nt;
  if (x) {
    std::vector<double> xf(2 * size_t(std::max(sc->nf, 1)));
    if (sc->nf > 0)
      T2_CUDA(cudaMemcpyAsync(xf.data(), sc->d.x, 8 * 2 * size_t(sc->nf), cudaMemcpyDeviceToHost, sc->stream));
    T2_CUDA(cudaStreamSynchronize(sc->stream));
    for (size_t u = 0; u < nv; ++u) {
      const int f = sc->free_map[u];
      for (int k = 0; k < 2; ++k) x[2 * u + k] = f >= 0 ? xf[2 * size_t(f) + k] : sc->bhost[2 * u + k];
    }
  }
  if (v)
    T2_CUDA(cudaMemcpyAsync(v, sc->vh + 2 * nv * size_t(sc->head), 8 * 2 * nv, cudaMemcpyDeviceToHost,
                            sc->stream));
  if (s) T2_CUDA(cudaMemcpyAsync(s, sc->d.s, 8 * 3 * nt, cudaMemcpyDeviceToHost, sc->stream));
  if (R) T2_CUDA(cudaMemcpyAsync(R, sc->d.R, 8 * 4 * nt, cudaMemcpyDeviceToHost, sc->stream));
  if (la) T2_CUDA(cudaMemcpyAsync(la, sc->d.lam, 8 * 3 * nt, cudaMemcpyDeviceToHost, sc->stream));
  T2_CUDA(cudaStreamSynchronize(sc->stream));
  return MFEM_OK;
}

int mfem_gpu_tri2d_elem_update(mfem_tri2d* sc, const double* x, double h, double* R, double* S,
                               double* dSdF, double* g, double* H, double* Hinv, double* Aloc,
                               double* gl) {
  if (!sc || !x || !(h > 0)) return MFEM_ERR_INVALID;
  const size_t nv = sc->nv, nt = sc->nt;
  T2_CUDA(cudaMemcpyAsync(sc->xscratch, x, 8 * 2 * nv, cudaMemcpyHostToDevice, sc->stream));
  T2_CUDA(cudaMemsetAsync(sc->d.status, 0, sizeof(int), sc->stream));
  t2_elem<<<grid_of(sc->nt), kThreads, 0, sc->stream>>>(sc->d, h * h, sc->xscratch);
  if (launch_status() != MFEM_OK) return MFEM_ERR_CUDA;
  auto down = [&](double* dst, const double* src, size_t n) {
    return !dst || cudaMemcpyAsync(dst, src, 8 * n, cudaMemcpyDeviceToHost, sc->stream) == cudaSuccess;
  };
  if (!(down(R, sc->d.R, 4 * nt) && down(S, sc->d.S, 3 * nt) && down(dSdF, sc->d.dSdF, 12 * nt) &&
        down(g, sc->d.g, 3 * nt) && down(H, sc->d.H, 9 * nt) && down(Hinv, sc->d.Hinv, 9 * nt) &&
        down(Aloc, sc->d.Aloc, 36 * nt) && down(gl, sc->d.gl, 3 * nt)))
    return MFEM_ERR_CUDA;
  int kst = 0;
  if (read_status(*sc, &kst) != MFEM_OK) return MFEM_ERR_CUDA;
  return kst;
}

int mfem_gpu_tri2d_get_system(mfem_tri2d* sc, int32_t* row_ptr, int32_t* col, double* val, double* rhs) {
  if (!sc) return MFEM_ERR_INVALID;
  T2_CUDA(cudaMemsetAsync(sc->d.status, 0, sizeof(int), sc->stream));
  if (t2_update(*sc, nullptr) != MFEM_OK) return MFEM_ERR_CUDA;
  if (val && sc->nnzb > 0)
    T2_CUDA(cudaMemcpyAsync(val, sc->d.A, 8 * 4 * size_t(sc->nnzb), cudaMemcpyDeviceToHost, sc->stream));
  if (rhs && sc->nf > 0)
    T2_CUDA(cudaMemcpyAsync(rhs, sc->d.rhs, 8 * 2 * size_t(sc->nf), cudaMemcpyDeviceToHost, sc->stream));
  int kst = 0;
  if (read_status(*sc, &kst) != MFEM_OK) return MFEM_ERR_CUDA;
  collect_events(*sc);
  if (row_ptr) std::memcpy(row_ptr, sc->b_ptr.data(), 4 * sc->b_ptr.size());
  if (col) std::memcpy(col, sc->b_col.data(), 4 * sc->b_col.size());
  return kst;
}

int mfem_gpu_tri2d_set_profiling(mfem_tri2d* sc, int enable) {
  if (!sc) return MFEM_ERR_INVALID;
  if (enable && !sc->profiling)
    for (int k = 0; k < MFEM_T2_K_COUNT; ++k) sc->kernel_ms[k] = 0.0;
  sc->profiling = enable != 0;
  return MFEM_OK;
}

int mfem_gpu_tri2d_kernel_stats(mfem_tri2d* sc, int kernel, double* total_ms, int64_t* launches) {
  if (!sc || kernel < 0 || kernel >= MFEM_T2_K_COUNT) return MFEM_ERR_INVALID;
  if (total_ms) *total_ms = sc->kernel_ms[kernel];
  if (launches) *launches = sc->launches[kernel];
  return MFEM_OK;
}

}  // extern "C"
