// Block-Jacobi PCG on a caller-owned, device-resident 3x3 block-CSR matrix
// that allocates nothing: every scratch vector, the tile partials, the
// tickets and the scalars live in one file-scope __device__ array of fixed
// size (MFEM_NOALLOC_PCG_MAX_ROWS block rows).
//
// The iteration is the one of the scene PCG (Eigen's ConjugateGradient with
// a block-diagonal preconditioner, src/linear_solvers/eigen_iterative_solver.h:20-29):
// x0 = 0, stop when |r|^2 < tol^2 |b|^2 or after max_iters iterations.  The
// p update is folded into the SpMV (p = z + beta p_prev formed per column),
// and the dot products are reduced deterministically: fixed-order block
// sums per tile, then the last tile (atomic ticket, no thread waits) sums
// the tile partials in tile order.
//
// Scratch state and what must start at zero: the ticket counter.  It is zero
// when the module loads, the last tile of every kernel returns it to zero,
// and each call clears the scalar block (ticket included) with
// cudaMemsetAsync before its first kernel.  Everything else in the scratch
// is written before it is read within a call.
//
// Calls on one device share that scratch, so two calls that overlapped on
// one device would race.  The entry point therefore holds that device's
// lock from its first launch until its stream has drained; calls on
// different devices use different scratch copies and different locks.
#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>
#include <cstdint>
#include <mutex>

#include "../../include/mfem_gb300.h"

namespace {

constexpr int kNaThreads = 256;
constexpr int kNaMaxRows = MFEM_NOALLOC_PCG_MAX_ROWS;
constexpr int kNaMaxTiles = (kNaMaxRows + kNaThreads - 1) / kNaThreads;
constexpr int kNaChunk = 16;  // iterations launched between two host checks
constexpr int kNaMaxDevices = 64;

struct NaScalars {
  double rr0, thr, rz, alpha, beta, err;
  int iter, active, status, max_iters;
  unsigned int ticket;
};

constexpr size_t na_align(size_t v) { return (v + 255) / 256 * 256; }
constexpr size_t kNaVecBytes = 3 * sizeof(double) * (size_t)kNaMaxRows;
constexpr size_t kNaOffPartials = na_align(sizeof(NaScalars));
constexpr size_t kNaOffDinv = na_align(kNaOffPartials + 2 * sizeof(double) * kNaMaxTiles);
constexpr size_t kNaOffVecs = na_align(kNaOffDinv + 9 * sizeof(double) * (size_t)kNaMaxRows);
constexpr size_t kNaScratchBytes = kNaOffVecs + 5 * kNaVecBytes;  // r, z, p0, p1, Ap
static_assert(kNaScratchBytes < (size_t(8) << 20), "scratch stays a few MiB");

static __device__ __align__(256) unsigned char g_na_scratch[kNaScratchBytes];

struct NaView {
  NaScalars* sc;
  double* partials;  // [2][kNaMaxTiles]
  double* dinv;      // 9 per row, row-major 3x3
  double* r;
  double* z;
  double* p[2];
  double* Ap;
};

NaView na_view(unsigned char* base) {
  NaView v;
  v.sc = reinterpret_cast<NaScalars*>(base);
  v.partials = reinterpret_cast<double*>(base + kNaOffPartials);
  v.dinv = reinterpret_cast<double*>(base + kNaOffDinv);
  double* vec = reinterpret_cast<double*>(base + kNaOffVecs);
  const size_t n3 = 3 * (size_t)kNaMaxRows;
  v.r = vec;
  v.z = vec + n3;
  v.p[0] = vec + 2 * n3;
  v.p[1] = vec + 3 * n3;
  v.Ap = vec + 4 * n3;
  return v;
}

struct NaMatrix {
  int n, nnzb;
  const int32_t* row_ptr;
  const int32_t* col;
  const double* val;
};

// Fixed-order block sums of NQ values; written as tile partials by thread 0.
template <int NQ>
__device__ __forceinline__ void na_tile_partials(double (&v)[NQ], double* partials) {
  __shared__ double red[kNaThreads / 32][NQ];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < NQ; ++q)
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v[q] += __shfl_down_sync(0xffffffffu, v[q], off);
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < NQ; ++q) red[warp][q] = v[q];
  __syncthreads();
  if (threadIdx.x == 0)
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      double a = red[0][q];
      for (int w = 1; w < kNaThreads / 32; ++w) a += red[w][q];
      partials[q * kNaMaxTiles + blockIdx.x] = a;
    }
}

// True in thread 0 of the tile that arrived last; that thread then sees
// every other tile's partials.
__device__ __forceinline__ bool na_last_tile(NaScalars* sc) {
  if (threadIdx.x != 0) return false;
  __threadfence();
  if (atomicAdd(&sc->ticket, 1u) + 1u != gridDim.x) return false;
  sc->ticket = 0u;
  __threadfence();
  return true;
}

// Status flags raised by atomics of other tiles in the same launch.
__device__ __forceinline__ int na_status(NaScalars* sc) { return *(volatile int*)&sc->status; }

__device__ __forceinline__ double na_sum(const double* partials, int q) {
  double a = 0.0;
  for (int t = 0; t < (int)gridDim.x; ++t) a += __ldcg(partials + q * kNaMaxTiles + t);
  return a;
}

__device__ __forceinline__ void na_prec(const double* D, const double r[3], double z[3]) {
#pragma unroll
  for (int c = 0; c < 3; ++c) z[c] = D[3 * c] * r[0] + D[3 * c + 1] * r[1] + D[3 * c + 2] * r[2];
}

// True if the row's entries lie inside the matrix; records MFEM_ERR_INVALID
// otherwise, so that a malformed pattern is skipped instead of read.
__device__ __forceinline__ bool na_row_ok(const NaMatrix& A, int row, int& k0, int& k1, NaScalars* sc) {
  k0 = A.row_ptr[row];
  k1 = A.row_ptr[row + 1];
  if (k0 < 0 || k1 < k0 || k1 > A.nnzb) {
    atomicMax(&sc->status, MFEM_ERR_INVALID);
    return false;
  }
  return true;
}

// D^{-1} of the diagonal blocks, r = b, z = D^{-1} b, x = 0, |b|^2, r.z.
__global__ void __launch_bounds__(kNaThreads) k_na_init(NaMatrix A, const double* b, double* x,
                                                        NaView v, int max_iters, double tol) {
  NaScalars* sc = v.sc;
  double dots[2] = {0.0, 0.0};
  const int row = blockIdx.x * kNaThreads + threadIdx.x;
  if (row < A.n) {
    int k0, k1;
    const double* D = nullptr;
    if (na_row_ok(A, row, k0, k1, sc))
      for (int k = k0; k < k1; ++k)
        if (A.col[k] == row) D = A.val + 9 * (size_t)k;
    double* Di = v.dinv + 9 * (size_t)row;
    const double c00 = D ? D[4] * D[8] - D[5] * D[7] : 0.0;
    const double c01 = D ? D[5] * D[6] - D[3] * D[8] : 0.0;
    const double c02 = D ? D[3] * D[7] - D[4] * D[6] : 0.0;
    const double det = D ? D[0] * c00 + D[1] * c01 + D[2] * c02 : 0.0;
    if (det != 0.0 && std::isfinite(det)) {
      const double id = 1.0 / det;
      Di[0] = c00 * id;
      Di[1] = (D[2] * D[7] - D[1] * D[8]) * id;
      Di[2] = (D[1] * D[5] - D[2] * D[4]) * id;
      Di[3] = c01 * id;
      Di[4] = (D[0] * D[8] - D[2] * D[6]) * id;
      Di[5] = (D[2] * D[3] - D[0] * D[5]) * id;
      Di[6] = c02 * id;
      Di[7] = (D[1] * D[6] - D[0] * D[7]) * id;
      Di[8] = (D[0] * D[4] - D[1] * D[3]) * id;
    } else {
      atomicMax(&sc->status, MFEM_ERR_INVALID);  // missing or singular diagonal block
#pragma unroll
      for (int e = 0; e < 9; ++e) Di[e] = (e % 4 == 0) ? 1.0 : 0.0;
    }
    double r[3] = {b[3 * row], b[3 * row + 1], b[3 * row + 2]}, z[3];
    na_prec(Di, r, z);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      v.r[3 * row + c] = r[c];
      v.z[3 * row + c] = z[c];
      x[3 * row + c] = 0.0;
      dots[0] += r[c] * r[c];
      dots[1] += r[c] * z[c];
    }
  }
  na_tile_partials<2>(dots, v.partials);
  if (na_last_tile(sc)) {
    const double rr = na_sum(v.partials, 0), rz = na_sum(v.partials, 1);
    sc->rr0 = rr;
    sc->rz = rz;
    sc->beta = 0.0;
    sc->iter = 0;
    sc->max_iters = max_iters;
    sc->thr = fmax(tol * tol * rr, DBL_MIN);
    sc->err = rr == 0.0 ? 0.0 : 1.0;
    sc->active = (na_status(sc) == 0 && rr != 0.0 && rr >= sc->thr && max_iters > 0) ? 1 : 0;
    // No iteration allowed while the residual is above the threshold: the
    // solve stops on max_iters, as Eigen's NoConvergence.
    if (na_status(sc) == 0 && rr != 0.0 && rr >= sc->thr && max_iters == 0) sc->status = MFEM_ERR_CG_MAXITER;
    if (!(rr == rr) || !(rz == rz)) sc->status = MFEM_ERR_NONFINITE;
  }
}

// Ap = A p, p = z + beta p_prev (formed per column), p.Ap; alpha = rz / p.Ap.
__global__ void __launch_bounds__(kNaThreads) k_na_spmv(NaMatrix A, NaView v) {
  NaScalars* sc = v.sc;
  if (!sc->active) return;
  const int it = sc->iter;
  const double beta = sc->beta;
  const bool first = it == 0;
  const double* pin = (it & 1) ? v.p[0] : v.p[1];
  double* pout = (it & 1) ? v.p[1] : v.p[0];
  double dots[1] = {0.0};
  const int row = blockIdx.x * kNaThreads + threadIdx.x;
  if (row < A.n) {
    int k0, k1;
    double acc[3] = {0.0, 0.0, 0.0};
    if (na_row_ok(A, row, k0, k1, sc))
      for (int k = k0; k < k1; ++k) {
        const int c = A.col[k];
        if (c < 0 || c >= A.n) {
          atomicMax(&sc->status, MFEM_ERR_INVALID);
          continue;
        }
        const double* B = A.val + 9 * (size_t)k;
        double p[3];
#pragma unroll
        for (int j = 0; j < 3; ++j) p[j] = first ? v.z[3 * c + j] : v.z[3 * c + j] + beta * pin[3 * c + j];
#pragma unroll
        for (int i = 0; i < 3; ++i) acc[i] += B[3 * i] * p[0] + B[3 * i + 1] * p[1] + B[3 * i + 2] * p[2];
      }
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const double p = first ? v.z[3 * row + i] : v.z[3 * row + i] + beta * pin[3 * row + i];
      pout[3 * row + i] = p;
      v.Ap[3 * row + i] = acc[i];
      dots[0] += p * acc[i];
    }
  }
  na_tile_partials<1>(dots, v.partials);
  if (na_last_tile(sc)) sc->alpha = sc->rz / na_sum(v.partials, 0);
}

// x += alpha p, r -= alpha Ap, z = D^{-1} r; then the stopping test and beta.
__global__ void __launch_bounds__(kNaThreads) k_na_update(int n, double* x, NaView v) {
  NaScalars* sc = v.sc;
  if (!sc->active) return;
  const int it = sc->iter;
  const double alpha = sc->alpha;
  const double* p = (it & 1) ? v.p[1] : v.p[0];
  double dots[2] = {0.0, 0.0};
  const int row = blockIdx.x * kNaThreads + threadIdx.x;
  if (row < n) {
    double r[3], z[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      x[3 * row + c] += alpha * p[3 * row + c];
      r[c] = v.r[3 * row + c] - alpha * v.Ap[3 * row + c];
      v.r[3 * row + c] = r[c];
      dots[0] += r[c] * r[c];
    }
    na_prec(v.dinv + 9 * (size_t)row, r, z);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      v.z[3 * row + c] = z[c];
      dots[1] += r[c] * z[c];
    }
  }
  na_tile_partials<2>(dots, v.partials);
  if (na_last_tile(sc)) {
    const double rr = na_sum(v.partials, 0), rz = na_sum(v.partials, 1);
    // As in Eigen's loop, the iteration that meets the threshold is not
    // counted.
    sc->err = sqrt(rr / sc->rr0);
    if (!(rr == rr) || !(rz == rz)) {
      sc->status = MFEM_ERR_NONFINITE;
      sc->active = 0;
    } else if (na_status(sc) != 0 || rr < sc->thr) {
      sc->active = 0;
    } else {
      sc->beta = rz / sc->rz;
      sc->rz = rz;
      sc->iter = it + 1;
      if (it + 1 >= sc->max_iters) {
        sc->status = MFEM_ERR_CG_MAXITER;
        sc->active = 0;
      }
    }
  }
}

std::mutex g_na_mu[kNaMaxDevices];  // one per device: its scratch copy
unsigned char* g_na_base[kNaMaxDevices] = {};

bool na_device_pointer(const void* p, int dev) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) && a.device == dev;
}

}  // namespace

extern "C" int mfem_gpu_bsr_pcg_noalloc(int32_t n_block_rows, int32_t nnzb, const int32_t* row_ptr,
                                        const int32_t* col, const double* val, const double* b,
                                        double* x, int32_t max_iters, double tol, void* stream,
                                        int32_t* iterations, double* rel_residual) {
  if (iterations) *iterations = 0;
  if (rel_residual) *rel_residual = 0.0;
  if (n_block_rows < 0 || nnzb < 0 || max_iters < 0 || !(tol >= 0.0)) return MFEM_ERR_INVALID;
  if (n_block_rows > kNaMaxRows) return MFEM_ERR_CAPACITY;
  if (n_block_rows == 0) return MFEM_OK;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return MFEM_ERR_NO_DEVICE;
  }
  if (dev < 0 || dev >= kNaMaxDevices) return MFEM_ERR_CAPACITY;
  if (!na_device_pointer(row_ptr, dev) || !na_device_pointer(b, dev) || !na_device_pointer(x, dev) ||
      (nnzb > 0 && (!na_device_pointer(col, dev) || !na_device_pointer(val, dev))))
    return MFEM_ERR_INVALID;

  std::lock_guard<std::mutex> lock(g_na_mu[dev]);
  if (!g_na_base[dev]) {  // once per device: the address of the static scratch
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_na_scratch) != cudaSuccess || !p) {
      cudaGetLastError();
      return MFEM_ERR_CUDA;
    }
    g_na_base[dev] = static_cast<unsigned char*>(p);
  }
  const NaView v = na_view(g_na_base[dev]);
  const NaMatrix A{n_block_rows, nnzb, row_ptr, col, val};
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int ntiles = (n_block_rows + kNaThreads - 1) / kNaThreads;
  // Launch errors are read with cudaPeekAtLastError right after this call's
  // own launches (it leaves any pending error of the caller's in place);
  // faults while the kernels run come back from cudaStreamSynchronize.
  if (cudaMemsetAsync(v.sc, 0, sizeof(NaScalars), st) != cudaSuccess) return MFEM_ERR_CUDA;
  k_na_init<<<ntiles, kNaThreads, 0, st>>>(A, b, x, v, max_iters, tol);
  if (cudaPeekAtLastError() != cudaSuccess) return MFEM_ERR_CUDA;
  NaScalars h{};
  int launched = 0;
  for (;;) {
    if (cudaMemcpyAsync(&h, v.sc, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return MFEM_ERR_CUDA;
    if (!h.active || launched >= max_iters) break;
    const int c = max_iters - launched < kNaChunk ? max_iters - launched : kNaChunk;
    for (int k = 0; k < c; ++k) {
      k_na_spmv<<<ntiles, kNaThreads, 0, st>>>(A, v);
      k_na_update<<<ntiles, kNaThreads, 0, st>>>(n_block_rows, x, v);
    }
    if (cudaPeekAtLastError() != cudaSuccess) return MFEM_ERR_CUDA;
    launched += c;
  }
  if (iterations) *iterations = h.iter;
  if (rel_residual) *rel_residual = h.err;
  return h.status;
}
