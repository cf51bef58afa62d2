// Host side of the GB300 mixed-FEM Newton timestep: scene set-up (what
// SimState::load + Mesh::init + the variables' reset() build in the
// reference), batches of scenes, the Newton loop that launches the kernels,
// and the C ABI of include/mfem_gb300.h.
//
// Reference correspondence (tytrusty/mfem):
//   scene set-up      src/mesh/mesh.cpp:124-175, src/mesh/tet_mesh.cpp:31-75,
//                     src/variables/displacement.cpp:75-98, mixed_stretch.cpp:261-304
//   assembly pattern  src/utils/sparse_utils.cpp:19-138 (sorted free pairs)
//   boundary scripts  src/boundary_conditions/*.h, boundary_condition.cpp:5-21
//   Newton loop       src/optimizers/newton_optimizer.cpp:11-89
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstddef>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <sys/stat.h>
#include <new>
#include <string>
#include <vector>

#include "../../include/mfem_gb300.h"
#include "kernels.cuh"

using namespace mfem_gpu;

namespace {

thread_local char g_last_error[256] = {0};

void set_error(const char* what, cudaError_t e) {
  snprintf(g_last_error, sizeof(g_last_error), "%s: %s", what, cudaGetErrorString(e));
}

#define CUDA_OR(expr, code)                 \
  do {                                      \
    cudaError_t e_ = (expr);                \
    if (e_ != cudaSuccess) {                \
      set_error(#expr, e_);                 \
      return (code);                        \
    }                                       \
  } while (0)

std::once_flag g_configured;
constexpr int kMaxCallSteps = MFEM_BATCH_MAX_STEPS;  // timesteps of one mfem_gpu_batch_step_n call

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// The column of a packed ELL slot, stored as the integer's bits in a Real word.
template <typename T> T col_word(int c);
template <> float col_word<float>(int c) {
  float f;
  std::memcpy(&f, &c, 4);
  return f;
}
template <> double col_word<double>(int c) {
  const long long l = c;
  double d;
  std::memcpy(&d, &l, 8);
  return d;
}

// A double as a float pair hi + lo (df64) for the mixed path's constants.
float2 split_df(double d) {
  const float hi = float(d);
  return make_float2(hi, float(d - double(hi)));
}

// Sub-allocations of one device allocation.
struct Arena {
  char* base = nullptr;
  size_t used = 0;
  template <typename T> T* take(size_t n) {
    size_t off = align_up(used, 256);
    used = off + n * sizeof(T);
    return base ? reinterpret_cast<T*>(base + off) : nullptr;
  }
  void* take_bytes(size_t n) {
    size_t off = align_up(used, 256);
    used = off + n;
    return base ? static_cast<void*>(base + off) : nullptr;
  }
};

// Host-side structures of one scene, built once.
struct HostMesh {
  int nv = 0, nt = 0, nf = 0, npin = 0, nnzb = 0;
  std::vector<double> V0;      // initial positions after BC init
  std::vector<double> v0;      // initial velocities
  std::vector<int> T;          // 4 nt
  std::vector<double> dphi;    // 9 nt  (rows k = 1..3 of Dm^{-1}), element-major
  std::vector<double> vol;
  std::vector<double> mu, lam;
  std::vector<int8_t> mat;
  int material_uniform = 0;
  std::vector<int> is_fixed, free_map, free_vert, pin_vert;
  std::vector<int> m_ptr, m_col;
  std::vector<double> m_val;
  std::vector<int> b_ptr, b_col;
  std::vector<double> b_mass;
  std::vector<int> slice_off, ell_col;  // sliced-ELL layout of the block values
  std::vector<int> ref_of_row, row_of_ref;  // device free row <-> reference free index
  std::vector<int> inc_ptr;
  std::vector<int2> inc;
  // boundary script
  int bc_type = 0, bc_axis = 0;
  double bc_vel = 0.0;
  std::vector<int> pin_group;    // per pinned vertex: 0/1 BC group, -1 none
  double twist_center[3] = {0, 0, 0};
  double bend_center[2][3] = {{0, 0, 0}, {0, 0, 0}};
};

// Boundary groups (BoundaryCondition::init_boundary_groups): vertices within
// ratio*range of the min / max of the axis, computed on the rest shape.
void boundary_groups(const std::vector<double>& V, int nv, int axis, double ratio,
                     std::vector<int>& group) {
  double lo = std::numeric_limits<double>::infinity(), hi = -lo;
  for (int v = 0; v < nv; ++v) {
    lo = std::min(lo, V[3 * v + axis]);
    hi = std::max(hi, V[3 * v + axis]);
  }
  const double range = hi - lo;
  group.assign(nv, -1);
  for (int v = 0; v < nv; ++v) {
    const double c = V[3 * v + axis];
    if (c < lo + range * ratio)
      group[v] = 0;
    else if (c > hi - range * ratio)
      group[v] = 1;
  }
}

void bbox_center(const std::vector<double>& V, int nv, double c[3]) {
  for (int d = 0; d < 3; ++d) {
    double lo = std::numeric_limits<double>::infinity(), hi = -lo;
    for (int v = 0; v < nv; ++v) {
      lo = std::min(lo, V[3 * v + d]);
      hi = std::max(hi, V[3 * v + d]);
    }
    c[d] = 0.5 * (lo + hi);
  }
}

void rotate_about(double* p, const double* o, int axis, double ang) {
  double q[3] = {p[0] - o[0], p[1] - o[1], p[2] - o[2]};
  const double c = std::cos(ang), s = std::sin(ang);
  const int i = (axis + 1) % 3, j = (axis + 2) % 3;
  const double qi = c * q[i] - s * q[j], qj = s * q[i] + c * q[j];
  q[i] = qi;
  q[j] = qj;
  for (int d = 0; d < 3; ++d) p[d] = q[d] + o[d];
}

bool invert3(const double* A, double* Ai, double* det_out) {
  // A column-major
  const double c00 = A[4] * A[8] - A[7] * A[5];
  const double c01 = A[7] * A[2] - A[1] * A[8];
  const double c02 = A[1] * A[5] - A[4] * A[2];
  const double det = A[0] * c00 + A[3] * c01 + A[6] * c02;
  *det_out = det;
  if (det == 0.0 || !std::isfinite(det)) return false;
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

int build_host_mesh(const mfem_scene_desc* d, HostMesh& M) {
  if (!d || d->n_vertices <= 0 || d->n_tets <= 0 || !d->V_rest || !d->tets || !d->mu ||
      !d->lambda)
    return MFEM_ERR_INVALID;
  if (d->bdf_order < 1 || d->bdf_order > 6 || !(d->dt > 0)) return MFEM_ERR_INVALID;
  if (d->bc_axis < 0 || d->bc_axis > 2) return MFEM_ERR_INVALID;
  M.nv = d->n_vertices;
  M.nt = d->n_tets;
  const int nv = M.nv, nt = M.nt;
  std::vector<double> Vref(d->V_rest, d->V_rest + 3 * (size_t)nv);
  M.V0 = d->V_init ? std::vector<double>(d->V_init, d->V_init + 3 * (size_t)nv) : Vref;
  M.v0 = d->v_init ? std::vector<double>(d->v_init, d->v_init + 3 * (size_t)nv)
                   : std::vector<double>(3 * (size_t)nv, 0.0);
  M.T.assign(d->tets, d->tets + 4 * (size_t)nt);
  for (int v : M.T)
    if (v < 0 || v >= nv) return MFEM_ERR_INVALID;
  M.mu.assign(d->mu, d->mu + nt);
  M.lam.assign(d->lambda, d->lambda + nt);
  M.material_uniform = d->material ? d->material[0] : MFEM_MATERIAL_SNH;
  if (d->material) {
    M.mat.resize(nt);
    for (int e = 0; e < nt; ++e) {
      if (d->material[e] < 0 || d->material[e] > MFEM_MATERIAL_FUNG) return MFEM_ERR_INVALID;
      M.mat[e] = (int8_t)d->material[e];
      if (d->material[e] != M.material_uniform) M.material_uniform = -1;
    }
  }
  // ---- boundary script (Mesh::init_bcs, mesh.cpp:161-175)
  M.bc_type = d->bc_type;
  M.bc_axis = d->bc_axis;
  M.bc_vel = d->bc_velocity;
  std::vector<int> group;
  boundary_groups(Vref, nv, d->bc_axis, d->bc_ratio, group);
  M.is_fixed.assign(nv, 0);
  std::vector<int> g0, g1;
  for (int v = 0; v < nv; ++v) {
    if (group[v] == 0) g0.push_back(v);
    if (group[v] == 1) g1.push_back(v);
  }
  switch (d->bc_type) {
    case MFEM_BC_NULL:
      break;
    case MFEM_BC_SCALEF: {  // ScaleBC::init
      double c[3];
      bbox_center(M.V0, nv, c);
      for (int v = 0; v < nv; ++v)
        for (int k = 0; k < 3; ++k) M.V0[3 * v + k] = (M.V0[3 * v + k] - c[k]) * 1.5 + c[k];
      break;
    }
    case MFEM_BC_RANDOM: {  // RandomizeBC::init with a seeded generator
      double c[3], lo = 1e300, hi = -1e300;
      bbox_center(M.V0, nv, c);
      for (int v = 0; v < nv; ++v) {
        lo = std::min(lo, M.V0[3 * v + 1]);
        hi = std::max(hi, M.V0[3 * v + 1]);
      }
      uint64_t st = 0x9E3779B97F4A7C15ull;
      for (auto& x : M.V0) {
        st = st * 6364136223846793005ull + 1442695040888963407ull;
        x = (double((st >> 11) & ((1ull << 53) - 1)) / double(1ull << 53) * 2 - 1) / 2.0;
      }
      c[1] += (hi - lo) * 0.5;
      const double r0[3] = {M.V0[0], M.V0[1], M.V0[2]};
      for (int v = 0; v < nv; ++v)
        for (int k = 0; k < 3; ++k) M.V0[3 * v + k] += c[k] - r0[k];
      break;
    }
    case MFEM_BC_ONEPOINT:
      M.is_fixed[0] = 1;
      break;
    case MFEM_BC_HANG:
      if (!g0.empty()) M.is_fixed[g0.back()] = 1;
      if (!g1.empty()) M.is_fixed[g1.back()] = 1;
      break;
    case MFEM_BC_HANGENDS:
      for (int v : g1) M.is_fixed[v] = 1;
      break;
    case MFEM_BC_PINMIN:
      for (int v : g0) M.is_fixed[v] = 1;
      break;
    case MFEM_BC_STRETCH:
    case MFEM_BC_COMPRESS:
    case MFEM_BC_TWIST:
    case MFEM_BC_BEND:
      for (int v : g0) M.is_fixed[v] = 1;
      for (int v : g1) M.is_fixed[v] = 1;
      if (d->bc_type == MFEM_BC_TWIST) bbox_center(M.V0, nv, M.twist_center);
      if (d->bc_type == MFEM_BC_BEND) {
        const int a = g0.empty() ? 0 : g0.back(), b = g1.empty() ? 0 : g1.back();
        for (int k = 0; k < 3; ++k) {
          M.bend_center[0][k] = M.V0[3 * a + k];
          M.bend_center[1][k] = M.V0[3 * b + k];
        }
      }
      break;
    default:
      return MFEM_ERR_UNSUPPORTED;
  }
  if (d->is_fixed)
    for (int v = 0; v < nv; ++v) M.is_fixed[v] = d->is_fixed[v] ? 1 : 0;
  M.free_map.assign(nv, 0);
  M.free_vert.clear();
  M.pin_vert.clear();
  M.pin_group.clear();
  std::vector<int> ref_free;  // free vertices in vertex order (the reference's numbering)
  for (int v = 0; v < nv; ++v) {
    if (M.is_fixed[v]) {
      M.free_map[v] = -1 - (int)M.pin_vert.size();
      M.pin_vert.push_back(v);
      M.pin_group.push_back(group[v]);
    } else {
      ref_free.push_back(v);
    }
  }
  M.nf = (int)ref_free.size();
  M.npin = (int)M.pin_vert.size();
  // ---- geometry: |det Dm|/6 and dphi/dX = rows of Dm^{-1} (tet_mesh.cpp:31-75)
  M.vol.resize(nt);
  M.dphi.resize(9 * (size_t)nt);
  for (int e = 0; e < nt; ++e) {
    const double* X0 = &Vref[3 * M.T[4 * e]];
    double Dm[9], Di[9], det;
    for (int k = 1; k < 4; ++k) {
      const double* Xk = &Vref[3 * M.T[4 * e + k]];
      for (int r = 0; r < 3; ++r) Dm[r + 3 * (k - 1)] = Xk[r] - X0[r];
    }
    if (!invert3(Dm, Di, &det)) return MFEM_ERR_INVALID;
    M.vol[e] = std::fabs(det) / 6.0;
    for (int k = 1; k < 4; ++k)
      for (int c = 0; c < 3; ++c) M.dphi[9 * (size_t)e + 3 * (k - 1) + c] = Di[(k - 1) + 3 * c];
  }
  // ---- vertex -> tet incidence
  std::vector<int> vt_ptr(nv + 1, 0), vt(4 * (size_t)nt);
  for (int v : M.T) vt_ptr[v + 1]++;
  for (int v = 0; v < nv; ++v) vt_ptr[v + 1] += vt_ptr[v];
  {
    std::vector<int> fill(vt_ptr.begin(), vt_ptr.end() - 1);
    for (int e = 0; e < nt; ++e)
      for (int k = 0; k < 4; ++k) vt[fill[M.T[4 * e + k]]++] = 4 * e + k;  // sorted by e
  }
  // ---- device numbering of the free rows: within each window of kCgRows
  // rows (vertex order), by decreasing block count, so that the sliced-ELL
  // slices of 32 rows need almost no padding (SELL-C-sigma)
  {
    std::vector<int> cnt(M.nf, 0), mark(nv, -1);
    for (int i = 0; i < M.nf; ++i) {
      const int a = ref_free[i];
      for (int q = vt_ptr[a]; q < vt_ptr[a + 1]; ++q) {
        const int e = vt[q] / 4;
        for (int k = 0; k < 4; ++k) {
          const int b = M.T[4 * e + k];
          if (!M.is_fixed[b] && mark[b] != i) {
            mark[b] = i;
            cnt[i] += 1;
          }
        }
      }
    }
    std::vector<int> order(M.nf);
    for (int i = 0; i < M.nf; ++i) order[i] = i;
    for (int w = 0; w < M.nf; w += kCgRows) {
      const int we = std::min(M.nf, w + kCgRows);
      std::stable_sort(order.begin() + w, order.begin() + we,
                       [&](int x, int y) { return cnt[x] > cnt[y]; });
    }
    M.free_vert.resize(M.nf);
    M.ref_of_row.resize(M.nf);
    M.row_of_ref.resize(M.nf);
    for (int r = 0; r < M.nf; ++r) {
      const int i = order[r];
      M.free_vert[r] = ref_free[i];
      M.free_map[ref_free[i]] = r;
      M.ref_of_row[r] = i;
      M.row_of_ref[i] = r;
    }
  }
  // ---- consistent P1 mass over all vertices (linear_tetmesh_mass_matrix)
  const double* rho = d->density;
  M.m_ptr.assign(nv + 1, 0);
  M.m_col.clear();
  M.m_val.clear();
  {
    std::vector<std::pair<int, double>> row;
    for (int a = 0; a < nv; ++a) {
      row.clear();
      for (int q = vt_ptr[a]; q < vt_ptr[a + 1]; ++q) {
        const int e = vt[q] / 4, i = vt[q] % 4;
        const double m = (rho ? rho[e] : d->density_const) * M.vol[e] / 20.0;
        for (int k = 0; k < 4; ++k) row.push_back({M.T[4 * e + k], k == i ? 2 * m : m});
      }
      std::sort(row.begin(), row.end(),
                [](const std::pair<int, double>& x, const std::pair<int, double>& y) {
                  return x.first < y.first;
                });
      for (size_t k = 0; k < row.size(); ++k) {
        if (k > 0 && row[k].first == row[k - 1].first)
          M.m_val.back() += row[k].second;
        else {
          M.m_col.push_back(row[k].first);
          M.m_val.push_back(row[k].second);
        }
      }
      M.m_ptr[a + 1] = (int)M.m_col.size();
    }
  }
  // ---- block pattern over free vertices (the sorted free pairs of the Assembler)
  M.b_ptr.assign(M.nf + 1, 0);
  M.b_col.clear();
  M.b_mass.clear();
  M.inc_ptr.assign(M.nf + 1, 0);
  M.inc.clear();
  {
    std::vector<int> cols;
    for (int r = 0; r < M.nf; ++r) {
      const int a = M.free_vert[r];
      cols.clear();
      for (int q = vt_ptr[a]; q < vt_ptr[a + 1]; ++q) {
        const int e = vt[q] / 4;
        for (int k = 0; k < 4; ++k) {
          const int f = M.free_map[M.T[4 * e + k]];
          if (f >= 0) cols.push_back(f);
        }
      }
      std::sort(cols.begin(), cols.end());
      cols.erase(std::unique(cols.begin(), cols.end()), cols.end());
      if ((int)cols.size() > kMaxRowBlocks) return MFEM_ERR_CAPACITY;
      const int rb = (int)M.b_col.size();
      M.b_col.insert(M.b_col.end(), cols.begin(), cols.end());
      M.b_ptr[r + 1] = (int)M.b_col.size();
      // mass of each free-free block
      for (size_t k = 0; k < cols.size(); ++k) M.b_mass.push_back(0.0);
      for (int q = M.m_ptr[a]; q < M.m_ptr[a + 1]; ++q) {
        const int f = M.free_map[M.m_col[q]];
        if (f < 0) continue;
        const int pos = int(std::lower_bound(cols.begin(), cols.end(), f) - cols.begin());
        M.b_mass[rb + pos] += M.m_val[q];
      }
      // incidences (element, local vertex) in element order
      for (int q = vt_ptr[a]; q < vt_ptr[a + 1]; ++q) {
        const int e = vt[q] / 4, i = vt[q] % 4;
        int code = i;
        for (int k = 0; k < 4; ++k) {
          const int f = M.free_map[M.T[4 * e + k]];
          int slot = 127;
          if (f >= 0) slot = int(std::lower_bound(cols.begin(), cols.end(), f) - cols.begin());
          code |= slot << (2 + 7 * k);
        }
        M.inc.push_back(make_int2(e, code));
      }
      M.inc_ptr[r + 1] = (int)M.inc.size();
    }
  }
  M.nnzb = (int)M.b_col.size();
  // sliced-ELL layout: slices of 32 rows padded to their longest row;
  // padding blocks point at the row itself (their values are zero)
  {
    const int ns = (M.nf + 31) / 32;
    M.slice_off.assign(ns + 1, 0);
    for (int sl = 0; sl < ns; ++sl) {
      int len = 0;
      for (int r = 32 * sl; r < std::min(M.nf, 32 * sl + 32); ++r) len = std::max(len, M.b_ptr[r + 1] - M.b_ptr[r]);
      M.slice_off[sl + 1] = M.slice_off[sl] + 32 * len;
    }
    M.ell_col.assign(M.slice_off[ns], 0);
    for (int sl = 0; sl < ns; ++sl) {
      const int len = (M.slice_off[sl + 1] - M.slice_off[sl]) / 32;
      for (int rs = 0; rs < 32; ++rs) {
        const int r = 32 * sl + rs;
        for (int k = 0; k < len; ++k) {
          int c = (r < M.nf) ? r : 0;
          if (r < M.nf && k < M.b_ptr[r + 1] - M.b_ptr[r]) c = M.b_col[M.b_ptr[r] + k];
          M.ell_col[M.slice_off[sl] + 32 * k + rs] = c;
        }
      }
    }
  }
  return MFEM_OK;
}

}  // namespace

// ---------------------------------------------------------------- types ---
struct mfem_scene {
  HostMesh M;
  int fp64 = 0;
  size_t rsz = 4;
  int ntp = 0;
  double h = 0, dt = 0, h2 = 0;
  mfem_scene_desc cfg{};
  std::vector<double> pin_pos;  // current pinned positions (host BC state)
  char* dmem = nullptr;
  size_t dbytes = 0;
  SceneDev dev{};
  SceneScalars* d_sc = nullptr;
  double* d_pin_pos = nullptr;
  mfem_batch* solo = nullptr;
  int nnzb = 0;
  bool pins_driven = false;  // pins set by the caller for the next step
  // mfem_gpu_batch_step_n: the pins after each BC step of a call (grown on
  // demand; 3 npin doubles per step) and its pinned host staging
  double* d_pin_traj = nullptr;
  size_t pin_traj_cap = 0;  // steps it holds
  // device checkpoint (mfem_gpu_scene_checkpoint): raw copies of the state
  char* ckpt = nullptr;
  int ckpt_head = 0;
  std::vector<double> ckpt_pins;
};

struct mfem_batch {
  std::vector<mfem_scene*> scenes;
  int fp64 = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  char* dmem = nullptr;
  Tile* d_tiles[TB_COUNT] = {nullptr, nullptr, nullptr, nullptr};
  int ntiles[TB_COUNT] = {0, 0, 0, 0};
  // the tables the kernels are launched over: the full ones, or during a
  // multi-step call the tiles of the scenes still stepping (compacted into
  // d_tiles_c as scenes finish), with each scene's tile range
  Tile* cur_tiles[TB_COUNT] = {nullptr, nullptr, nullptr, nullptr};
  int cur_ntiles[TB_COUNT] = {0, 0, 0, 0};
  Tile* d_tiles_c[TB_COUNT] = {nullptr, nullptr, nullptr, nullptr};
  std::vector<Tile> h_tiles[TB_COUNT];
  std::vector<int> full_first, full_count;  // scene x TB_COUNT
  SceneDev* d_sds = nullptr;
  std::vector<SceneDev> h_sds;
  double* d_partials = nullptr;
  BatchCounters* d_ctr = nullptr;
  BatchCounters* h_ctr = nullptr;   // pinned
  BatchCounters* h_ctr_pipe = nullptr;  // pinned, 2 slots: PCG chunk checks in flight
  cudaGraphExec_t cg_graph = nullptr;   // one chunk of PCG iterations, captured once
  // the whole PCG loop as one graph: a WHILE node around a chunk of
  // iterations and the loop's condition kernel (the device decides when
  // the solve has ended; no host round trip per chunk); cg_loop_len
  // iterations a body; loop_pending: a solve whose bodies the host has not
  // yet counted (read with the next counter sync)
  cudaGraphExec_t cg_loop = nullptr;
  bool cg_loop_on = true;
  bool loop_pending = false;
  int cg_loop_len = 8;
  bool loop_fused = true;
  cudaEvent_t ev_pipe[2] = {nullptr, nullptr};
  SceneScalars* h_sc = nullptr;     // pinned, one per scene
  int max_newton = 0, max_ls = 0, max_cg = 0;
  // Iterations to launch before the first convergence check of a linear
  // solve, per Newton iteration index (3/4 of the previous step's count at
  // that index): the first Newton iteration of a step needs several times
  // the iterations of the last, so one shared hint made the early solves
  // check too often and the late ones launch dozens of finished iterations.
  std::vector<int> cg_hints;
  int newton_index = 0;
  int& cg_hint() {
    if (cg_hints.empty()) cg_hints.assign(64, 16);
    return cg_hints[std::min(newton_index, (int)cg_hints.size() - 1)];
  }
  int pcg_kernel = MFEM_PCG_KERNEL_PERSISTENT;
  CgfShape cgf_shape{0, 0, 1, 0};  // shape of the fused PCG iteration (same bits in every shape)
  // register-budget variants of K1, K5, K6 chosen by the autotuner
  int var_elem = 0, var_local = 0, var_ls = 0;
  std::string tune_report = "{\"source\": \"default\"}";
  // mfem_gpu_batch_step_n: per scene and step the device time it was done
  // (kMaxCallSteps per scene, then the call's start), and the ticked form's
  // graph of one tick (captured on first use, dropped when a kernel shape or
  // variant changes)
  unsigned long long* d_step_ns = nullptr;
  cudaGraphExec_t tick_graph = nullptr;
  cudaGraphExec_t tick_graph_c = nullptr;  // the same over compacted tables
  // PCG iterations in one tick: 16 measured best between the 64-scene mix's
  // total time (8 iterations: 8.6 s for 100 steps, 16: 8.0 s, 32: 7.7 s) and
  // the per-step latency of its light scenes
  int tick_pcg = 16;
  int minres = 0;  // every scene uses "minres-indefinite-block"
  int fem = 0;     // every scene uses the standard-FEM variable
  int jacobi = 1;  // no scene uses the 3x3 block-Jacobi preconditioner
  int coop_grid = 0;  // blocks of the persistent PCG (all co-resident)
  int pstride = 0;  // tiles per partials quantity
  // instrumentation
  bool profiling = false;
  std::vector<cudaEvent_t> ev_pool;
  std::vector<int> ev_kernel;   // kernel id of each recorded pair
  size_t ev_used = 0;           // pairs recorded since the last harvest
  double k_ms[MFEM_K_COUNT] = {0};
  int64_t k_launches[MFEM_K_COUNT] = {0};
};

namespace {

// Brackets one kernel launch with CUDA events when profiling is on.
struct KTimer {
  mfem_batch* b;
  int id;
  cudaEvent_t e1 = nullptr;
  KTimer(mfem_batch* batch, int kernel) : b(batch), id(kernel) {
    b->k_launches[id] += 1;
    if (!b->profiling) return;
    if (b->ev_used * 2 + 2 > b->ev_pool.size()) {
      for (int k = 0; k < 256; ++k) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        b->ev_pool.push_back(e);
      }
      b->ev_kernel.resize(b->ev_pool.size() / 2);
    }
    cudaEventRecord(b->ev_pool[2 * b->ev_used], b->stream);
    e1 = b->ev_pool[2 * b->ev_used + 1];
    b->ev_kernel[b->ev_used] = id;
  }
  ~KTimer() {
    if (!e1) return;
    cudaEventRecord(e1, b->stream);
    b->ev_used += 1;
  }
};

// Adds the recorded pairs to the per-kernel totals (after a stream sync).
void harvest_timers(mfem_batch* b) {
  for (size_t i = 0; i < b->ev_used; ++i) {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, b->ev_pool[2 * i], b->ev_pool[2 * i + 1]) == cudaSuccess)
      b->k_ms[b->ev_kernel[i]] += ms;
  }
  b->ev_used = 0;
}

Launch make_launch(mfem_batch* b, int table) {
  Launch L;
  L.stream = b->stream;
  L.tiles = b->cur_tiles[table];
  L.ntiles = b->cur_ntiles[table];
  L.sds = b->d_sds;
  L.partials = b->d_partials;
  L.pstride = b->pstride;
  L.counters = b->d_ctr;
  L.fp64 = b->fp64;
  L.fem = b->fem;
  L.jacobi = b->jacobi;
  return L;
}

// Device layout of a scene (dry run with base == nullptr to size it).
void layout_scene(mfem_scene* s, Arena& A) {
  const HostMesh& M = s->M;
  const size_t r = s->rsz, ntp = s->ntp;
  SceneDev& D = s->dev;
  const int I = s->cfg.bdf_order;
  D.tets = A.take<int4>(M.nt);
  D.dphi = A.take_bytes(9 * ntp * r);
  D.vol = A.take_bytes(ntp * r);
  D.mu = A.take_bytes(ntp * r);
  D.lam = A.take_bytes(ntp * r);
  D.mat = M.mat.empty() ? nullptr : A.take<int8_t>(ntp);
  D.quat = A.take_bytes(4 * ntp * r);
  D.s = A.take_bytes(6 * ntp * 8);
  D.la = A.take_bytes(6 * ntp * r);
  D.dS = A.take_bytes(6 * ntp * r);
  D.ds = A.take_bytes(6 * ntp * r);
  D.rec = A.take<unsigned char>((size_t)rec_bytes((int)r) * M.nt);
  D.x = A.take_bytes(3 * (size_t)M.nv * 8);
  D.xt = A.take_bytes(3 * (size_t)M.nv * 8);
  D.xhist = A.take_bytes(3 * (size_t)M.nv * I * 8);
  D.vhist = A.take_bytes(3 * (size_t)M.nv * I * 8);
  D.free_map = A.take<int>(M.nv);
  D.free_vert = A.take<int>(std::max(M.nf, 1));
  D.pin_vert = A.take<int>(std::max(M.npin, 1));
  s->d_pin_pos = A.take<double>(3 * (size_t)std::max(M.npin, 1));
  D.pin_pos = s->d_pin_pos;
  D.m_ptr = A.take<int>(M.nv + 1);
  D.m_col = A.take<int>(M.m_col.size());
  D.m_val = A.take_bytes(M.m_val.size() * r);
  D.b_ptr = A.take<int>(M.nf + 1);
  D.b_col = A.take<int>(std::max(M.nnzb, 1));
  D.b_mass = A.take_bytes(std::max(M.nnzb, 1) * r);
  D.slice_off = A.take<int>(M.slice_off.size());
  D.ell = A.take_bytes(10 * std::max<size_t>(M.ell_col.size(), 1) * r);
  D.dinv = A.take_bytes(9 * (size_t)std::max(M.nf, 1) * r);
  D.inc_ptr = A.take<int>(M.nf + 1);
  D.inc = A.take<int2>(std::max<size_t>(M.inc.size(), 1));
  const size_t n4 = 4 * (size_t)std::max(M.nf, 1);
  D.rhs = A.take_bytes(n4 * r);
  D.cg_x = A.take_bytes(n4 * r);
  D.cg_xe = s->fp64 ? nullptr : A.take_bytes(n4 * 8);
  D.cg_r = A.take_bytes(n4 * r);
  D.cg_z = A.take_bytes(n4 * r);
  D.cg_p[0] = A.take_bytes(n4 * r);
  D.cg_p[1] = A.take_bytes(n4 * r);
  D.cg_Ap = A.take_bytes(n4 * r);
  if (s->cfg.pcg_kernel == MFEM_PCG_KERNEL_FUSED || s->cfg.pcg_kernel == MFEM_PCG_KERNEL_AUTO) {
    for (int k = 0; k < 2; ++k) {
      D.cgf_r[k] = A.take_bytes(n4 * r);
      D.cgf_w[k] = A.take_bytes(n4 * r);
      D.cgf_s[k] = A.take_bytes(n4 * r);
    }
  }
  if (s->cfg.linear_solver == MFEM_SOLVER_MINRES_ID) {
    D.mr_len = 4 * (size_t)std::max(M.nf, 1) + 12 * ntp;
    D.mr_B = A.take_bytes(72 * ntp * r);
    D.mr_H = A.take_bytes(21 * ntp * r);
    D.mr_vec = A.take<double>(8 * D.mr_len);
    D.mr_y = A.take<double>(12 * ntp);
    D.mr_hinv = A.take<double>(21 * ntp);
    D.mr_sinv = A.take<double>(21 * ntp);
    D.mr_mlinv = A.take<double>(std::max(M.nf, 1));
  }
  s->d_sc = A.take<SceneScalars>(1);
  D.sc = s->d_sc;
  // first-level ticket counters: one per group of kTicketGroup tiles per table
  const int maxtiles = std::max({(M.nt + kElemTile - 1) / kElemTile + (M.nv + kVertTile - 1) / kVertTile,
                                 (M.nf + kRowTile - 1) / kRowTile, (M.nf + kCgRows - 1) / kCgRows, 1});
  D.gmax = (maxtiles + kTicketGroup - 1) / kTicketGroup;
  D.gctr = A.take<unsigned int>((size_t)TB_COUNT * D.gmax);
}

template <typename T>
std::vector<T> soa(const std::vector<double>& src, int n, int ncomp, int ntp) {
  // element-major (ncomp per element) -> component-major with stride ntp
  std::vector<T> out((size_t)ncomp * ntp, T(0));
  for (int e = 0; e < n; ++e)
    for (int k = 0; k < ncomp; ++k) out[(size_t)k * ntp + e] = T(src[(size_t)ncomp * e + k]);
  return out;
}

// Ext storage of doubles: doubles in the FP64 path, (hi, lo) float pairs
// with hi + lo == v to ~48 bits in the mixed path; 8 bytes per value either way.
std::vector<double> to_ext(const double* v, size_t n, int fp64) {
  std::vector<double> out(n);
  if (fp64) {
    std::memcpy(out.data(), v, n * 8);
  } else {
    float* f = reinterpret_cast<float*>(out.data());
    for (size_t i = 0; i < n; ++i) {
      const float hi = float(v[i]);
      f[2 * i] = hi;
      f[2 * i + 1] = float(v[i] - double(hi));
    }
  }
  return out;
}
void from_ext(const void* buf, size_t n, int fp64, double* out) {
  if (fp64) {
    std::memcpy(out, buf, n * 8);
  } else {
    const float* f = static_cast<const float*>(buf);
    for (size_t i = 0; i < n; ++i) out[i] = double(f[2 * i]) + double(f[2 * i + 1]);
  }
}
int put_ext(void* dst, const double* src, size_t n, int fp64) {
  std::vector<double> e = to_ext(src, n, fp64);
  CUDA_OR(cudaMemcpy(dst, e.data(), n * 8, cudaMemcpyHostToDevice), MFEM_ERR_CUDA);
  return MFEM_OK;
}
int get_ext(double* dst, const void* src, size_t n, int fp64) {
  std::vector<double> e(n);
  CUDA_OR(cudaMemcpy(e.data(), src, n * 8, cudaMemcpyDeviceToHost), MFEM_ERR_CUDA);
  from_ext(e.data(), n, fp64, dst);
  return MFEM_OK;
}
char* byte_ptr(void* p, size_t off) { return static_cast<char*>(p) + off; }

template <typename T>
int upload_reals(void* dst, const std::vector<double>& src, size_t count, cudaStream_t st) {
  std::vector<T> tmp(count, T(0));
  for (size_t i = 0; i < std::min(count, src.size()); ++i) tmp[i] = T(src[i]);
  CUDA_OR(cudaMemcpyAsync(dst, tmp.data(), count * sizeof(T), cudaMemcpyHostToDevice, st), MFEM_ERR_CUDA);
  CUDA_OR(cudaStreamSynchronize(st), MFEM_ERR_CUDA);
  return MFEM_OK;
}

template <typename T>
int upload_scene_reals(mfem_scene* s, cudaStream_t st) {
  static_assert(sizeof(T) == 4 || sizeof(T) == 8, "Real");
  const HostMesh& M = s->M;
  const int ntp = s->ntp;
  SceneDev& D = s->dev;
  auto put = [&](const void* dst, const std::vector<T>& v) -> int {
    CUDA_OR(cudaMemcpyAsync(const_cast<void*>(dst), v.data(), v.size() * sizeof(T),
                            cudaMemcpyHostToDevice, st),
            MFEM_ERR_CUDA);
    return MFEM_OK;
  };
  int rc;
  if ((rc = put(D.dphi, soa<T>(M.dphi, M.nt, 9, ntp)))) return rc;
  if ((rc = put(D.vol, soa<T>(M.vol, M.nt, 1, ntp)))) return rc;
  if ((rc = put(D.mu, soa<T>(M.mu, M.nt, 1, ntp)))) return rc;
  if ((rc = put(D.lam, soa<T>(M.lam, M.nt, 1, ntp)))) return rc;
  {
    std::vector<T> mv(M.m_val.size());
    for (size_t k = 0; k < mv.size(); ++k) mv[k] = T(M.m_val[k]);
    if ((rc = put(D.m_val, mv))) return rc;
  }
  std::vector<T> bm(std::max(M.nnzb, 1), T(0));
  for (int k = 0; k < M.nnzb; ++k) bm[k] = T(M.b_mass[k]);
  if ((rc = put(D.b_mass, bm))) return rc;
  // packed ELL slots: the column word of every slot (values start at zero
  // and are written by the assembly)
  {
    std::vector<T> ell(10 * std::max<size_t>(M.ell_col.size(), 1), T(0));
    const int ns = (int)M.slice_off.size() - 1;
    for (int sl = 0; sl < ns; ++sl) {
      const int soff = M.slice_off[sl], len = (M.slice_off[sl + 1] - soff) / 32;
      for (int k = 0; k < len; ++k)
        for (int rs = 0; rs < 32; ++rs)
          ell[2 * ell_pair(soff, k, rs, 0)] = col_word<T>(M.ell_col[soff + 32 * k + rs]);
    }
    if ((rc = put(D.ell, ell))) return rc;
  }
  CUDA_OR(cudaStreamSynchronize(st), MFEM_ERR_CUDA);
  return MFEM_OK;
}

int batch_build(mfem_scene* const* scenes, int n, mfem_batch** out);

int sync_counters(mfem_batch* b) {
  CUDA_OR(cudaMemcpyAsync(b->h_ctr, b->d_ctr, sizeof(BatchCounters), cudaMemcpyDeviceToHost, b->stream),
          MFEM_ERR_CUDA);
  CUDA_OR(cudaStreamSynchronize(b->stream), MFEM_ERR_CUDA);
  if (b->loop_pending) {
    // a device-driven PCG loop has finished: its launches into the counts
    const int64_t bodies = b->h_ctr->cg_bodies;
    b->k_launches[MFEM_K_CG_LOOP] += 1 + bodies;  // k_cg_enter and one k_cg_continue a body
    if (b->loop_fused) {
      b->k_launches[MFEM_K_CGF_ITER] += bodies * b->cg_loop_len;
    } else {
      b->k_launches[MFEM_K_CG_SPMV] += bodies * b->cg_loop_len;
      b->k_launches[MFEM_K_CG_UPDATE] += bodies * b->cg_loop_len;
      if (!b->fp64) b->k_launches[MFEM_K_CG_REPLACE] += bodies;
    }
    b->loop_pending = false;
  }
  return MFEM_OK;
}

// Moves the pinned vertices by one BC step on the host
// (Meshes::update_bcs, meshes.cpp:156-167); true if any moved.
bool bc_advance(mfem_scene* s) {
  HostMesh& M = s->M;
  bool moved = false;
  const double dt = s->h;
  for (int p = 0; p < M.npin; ++p) {
    const int grp = M.pin_group[p];
    double* x = &s->pin_pos[3 * p];
    switch (M.bc_type) {
      case MFEM_BC_STRETCH:
        if (grp >= 0) {
          x[M.bc_axis] += (grp == 0 ? 1.0 : -1.0) * M.bc_vel * dt;
          moved = true;
        }
        break;
      case MFEM_BC_COMPRESS:
        if (grp == 1) {
          x[M.bc_axis] += M.bc_vel * dt;
          moved = true;
        }
        break;
      case MFEM_BC_TWIST:
        if (grp >= 0) {
          rotate_about(x, M.twist_center, 0, (grp == 0 ? 1.0 : -1.0) * M.bc_vel * M_PI * dt);
          moved = true;
        }
        break;
      case MFEM_BC_BEND:
        if (grp >= 0) {
          rotate_about(x, M.bend_center[grp], 2, (grp == 0 ? 1.0 : -1.0) * M.bc_vel * M_PI * dt);
          moved = true;
        }
        break;
      default:
        break;
    }
  }
  return moved;
}

// One BC step of the pins, uploaded for the step's end.
int bc_step_upload(mfem_scene* s, cudaStream_t st) {
  if (s->pins_driven) {  // the caller already uploaded this step's pins
    s->pins_driven = false;
    return MFEM_OK;
  }
  if (bc_advance(s) && s->M.npin > 0)
    CUDA_OR(cudaMemcpyAsync(s->d_pin_pos, s->pin_pos.data(), 3 * sizeof(double) * s->M.npin,
                            cudaMemcpyHostToDevice, st),
            MFEM_ERR_CUDA);
  return MFEM_OK;
}

int worst_status(const SceneScalars& sc) {
  if (sc.status == MFEM_ERR_NONFINITE) return MFEM_ERR_NONFINITE;
  if (sc.procrustes_fail) return MFEM_ERR_PROCRUSTES;
  if (sc.status) return sc.status;
  if (sc.cg_status) return sc.cg_status;
  return MFEM_OK;
}

// PCG iterations after k_cg_init: one cooperative launch for the whole solve,
// or SpMV/update launch pairs in chunks with a host check of the active
// count after each chunk.
// The same chunked loop with each chunk a CUDA graph captured once per batch
// (the kernels' arguments are fixed for the batch's lifetime): one graph
// launch replaces 8 (single-reduction) or 50-75 (two-reduction) kernel
// launches.  A two-reduction chunk is kCgReplace iterations long, so that the
// residual replacement keeps its period.
// One chunk of PCG iterations of the batch as an instantiated CUDA graph.
int capture_cg_graph(mfem_batch* b, const Launch& Lcg, bool fused, cudaGraphExec_t* out) {
  const int len = fused ? 8 : kCgReplace;
  cudaGraph_t g = nullptr;
  CUDA_OR(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), MFEM_ERR_CUDA);
  for (int k = 0; k < len; ++k) {
    if (fused) {
      launch_cgf_iter(Lcg, b->cgf_shape);
    } else {
      launch_cg_spmv(Lcg);
      launch_cg_update(Lcg);
      if (!b->fp64 && k + 1 == kCgReplace) launch_cg_replace(Lcg);
    }
  }
  const cudaError_t ec = cudaStreamEndCapture(b->stream, &g);
  if (ec != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    CUDA_OR(ec, MFEM_ERR_CUDA);
  }
  const cudaError_t ei = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  CUDA_OR(ei, MFEM_ERR_CUDA);
  return MFEM_OK;
}

// The whole PCG loop of a batch as one CUDA graph: k_cg_enter sets the
// condition of a WHILE node whose body is one chunk of iterations (as
// capture_cg_graph) followed by k_cg_continue, which sets it again from the
// batch's counters.  A solve ends within one chunk of its last iteration,
// with no host round trip.
int capture_cg_loop(mfem_batch* b, const Launch& Lcg, bool fused, cudaGraphExec_t* out) {
  const int len = fused ? 8 : kCgReplace;
  const int max_launch = b->max_cg + (fused && !b->fp64 ? 9 : 0);
  const int max_bodies = (max_launch + len - 1) / len + 1;
  cudaGraph_t g = nullptr;
  CUDA_OR(cudaGraphCreate(&g, 0), MFEM_ERR_CUDA);
  auto fail = [&](cudaError_t e) {
    cudaGraphDestroy(g);
    set_error("PCG loop graph", e);
    return MFEM_ERR_CUDA;
  };
  cudaGraphConditionalHandle h;
  cudaError_t e = cudaGraphConditionalHandleCreate(&h, g, 0u, cudaGraphCondAssignDefault);
  if (e != cudaSuccess) return fail(e);
  // the loop is entered only if a scene's solve is active (a Newton pass
  // that met the residual test at assembly runs no body)
  if ((e = cudaStreamBeginCaptureToGraph(b->stream, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal)) !=
      cudaSuccess)
    return fail(e);
  launch_cg_enter(Lcg, h);
  {
    cudaGraph_t cap = g;
    if ((e = cudaStreamEndCapture(b->stream, &cap)) != cudaSuccess) return fail(e);
  }
  cudaGraphNode_t enter = nullptr;
  size_t nn = 1;
  if ((e = cudaGraphGetNodes(g, &enter, &nn)) != cudaSuccess || nn != 1) return fail(e);
  cudaGraphNodeParams np = {};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = h;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t node = nullptr;
  if ((e = cudaGraphAddNode(&node, g, &enter, nullptr, 1, &np)) != cudaSuccess) return fail(e);
  cudaGraph_t body = np.conditional.phGraph_out[0];
  if ((e = cudaStreamBeginCaptureToGraph(b->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal)) !=
      cudaSuccess)
    return fail(e);
  for (int k = 0; k < len; ++k) {
    if (fused) {
      launch_cgf_iter(Lcg, b->cgf_shape);
    } else {
      launch_cg_spmv(Lcg);
      launch_cg_update(Lcg);
      if (!b->fp64 && k + 1 == kCgReplace) launch_cg_replace(Lcg);
    }
  }
  launch_cg_continue(Lcg, h, max_bodies);
  cudaGraph_t cap = body;
  e = cudaStreamEndCapture(b->stream, &cap);
  if (e != cudaSuccess) return fail(e);
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  CUDA_OR(e, MFEM_ERR_CUDA);
  b->cg_loop_len = len;
  b->loop_fused = fused;
  return MFEM_OK;
}

int run_pcg_graph(mfem_batch* b, const Launch& Lcg, bool fused) {
  const int len = fused ? 8 : kCgReplace;
  if (b->cg_loop_on && !b->cg_loop) {
    if (capture_cg_loop(b, Lcg, fused, &b->cg_loop) != MFEM_OK) {
      // conditional nodes unavailable: chunks with host checks instead
      cudaGetLastError();
      b->cg_loop = nullptr;
      b->cg_loop_on = false;
    }
  }
  if (b->cg_loop) {
    CUDA_OR(cudaMemsetAsync(&b->d_ctr->cg_bodies, 0, sizeof(int), b->stream), MFEM_ERR_CUDA);
    CUDA_OR(cudaGraphLaunch(b->cg_loop, b->stream), MFEM_ERR_CUDA);
    b->loop_pending = true;
    return MFEM_OK;
  }
  if (!b->cg_graph) {
    const int rc = capture_cg_graph(b, Lcg, fused, &b->cg_graph);
    if (rc) return rc;
  }
  // the mixed single-reduction form verifies its stop in launches of its
  // own (at most 4 rounds of two, and one to write the solution)
  const int max_launch = b->max_cg + (fused && !b->fp64 ? 9 : 0);
  int it = 0, nchunk = 0;
  int reps = std::max(1, (b->cg_hint() + len - 1) / len);
  while (it < max_launch) {
    for (int r = 0; r < reps && it < max_launch; ++r, it += len) {
      CUDA_OR(cudaGraphLaunch(b->cg_graph, b->stream), MFEM_ERR_CUDA);
      if (fused) {
        b->k_launches[MFEM_K_CGF_ITER] += len;
      } else {
        b->k_launches[MFEM_K_CG_SPMV] += len;
        b->k_launches[MFEM_K_CG_UPDATE] += len;
        if (!b->fp64) b->k_launches[MFEM_K_CG_REPLACE] += 1;
      }
    }
    const int slot = nchunk & 1;
    CUDA_OR(cudaMemcpyAsync(&b->h_ctr_pipe[slot], b->d_ctr, sizeof(BatchCounters), cudaMemcpyDeviceToHost,
                            b->stream),
            MFEM_ERR_CUDA);
    CUDA_OR(cudaEventRecord(b->ev_pipe[slot], b->stream), MFEM_ERR_CUDA);
    if (nchunk > 0) {
      CUDA_OR(cudaEventSynchronize(b->ev_pipe[slot ^ 1]), MFEM_ERR_CUDA);
      if (b->h_ctr_pipe[slot ^ 1].cg_active == 0) break;
    }
    ++nchunk;
    reps = 1;
  }
  b->cg_hint() = std::max(4, (it * 3) / 4);
  return MFEM_OK;
}

int run_pcg(mfem_batch* b, const Launch& Lcg) {
  const bool fused = b->pcg_kernel == MFEM_PCG_KERNEL_FUSED;
  {
    KTimer t(b, MFEM_K_CG_INIT);
    if (fused) {
      launch_cgf_scale(Lcg);  // mixed path only
      launch_cgf_init(Lcg);
    } else {
      launch_cg_init(Lcg);
    }
  }
  if (b->pcg_kernel == MFEM_PCG_KERNEL_PERSISTENT) {
    cudaError_t e;
    { KTimer t(b, MFEM_K_CG_SOLVE); e = launch_cg_solve(Lcg, b->coop_grid, b->max_cg + 1); }
    CUDA_OR(e, MFEM_ERR_CUDA);
    return MFEM_OK;
  }
  // Chunks of iterations with the convergence check one chunk behind: after
  // each chunk the counters are copied to a pinned slot and an event is
  // recorded; the host waits for the PREVIOUS chunk's copy, so the GPU
  // always has the current chunk queued while the host reads.  Iterations
  // launched after convergence return at once.
  if (!b->profiling) return run_pcg_graph(b, Lcg, fused);
  const int max_launch = b->max_cg + (fused && !b->fp64 ? 9 : 0);
  int it = 0, nchunk = 0;
  int chunk = std::max(4, b->cg_hint());
  while (it < max_launch) {
    const int c = std::min(chunk, max_launch - it);
    for (int k = 0; k < c; ++k, ++it) {
      if (fused) {
        KTimer t(b, MFEM_K_CGF_ITER);
        launch_cgf_iter(Lcg, b->cgf_shape);
      } else {
        { KTimer t(b, MFEM_K_CG_SPMV); launch_cg_spmv(Lcg); }
        { KTimer t(b, MFEM_K_CG_UPDATE); launch_cg_update(Lcg); }
        if (!b->fp64 && (it + 1) % kCgReplace == 0) {
          KTimer t(b, MFEM_K_CG_REPLACE);
          launch_cg_replace(Lcg);
        }
      }
    }
    const int slot = nchunk & 1;
    CUDA_OR(cudaMemcpyAsync(&b->h_ctr_pipe[slot], b->d_ctr, sizeof(BatchCounters), cudaMemcpyDeviceToHost,
                            b->stream),
            MFEM_ERR_CUDA);
    CUDA_OR(cudaEventRecord(b->ev_pipe[slot], b->stream), MFEM_ERR_CUDA);
    if (nchunk > 0) {
      CUDA_OR(cudaEventSynchronize(b->ev_pipe[slot ^ 1]), MFEM_ERR_CUDA);
      if (b->h_ctr_pipe[slot ^ 1].cg_active == 0) break;
    }
    ++nchunk;
    chunk = 8;
  }
  b->cg_hint() = std::max(4, (it * 3) / 4);
  return MFEM_OK;
}

// MINRES on the (x, s, lambda) system: init, then chunks of iterations
// (three launches each) with the convergence check one chunk behind as in
// run_pcg, then one more A1/A2 pair that applies the last pending update,
// and the export of dx.
int run_minres(mfem_batch* b, const Launch& Lev) {
  { KTimer t(b, MFEM_K_MR_INIT); launch_mr_init(Lev); }
  int it = 0, nchunk = 0;
  int chunk = std::max(4, b->cg_hint());
  while (it < b->max_cg) {
    const int c = std::min(chunk, b->max_cg - it);
    for (int k = 0; k < c; ++k, ++it) {
      { KTimer t(b, MFEM_K_MR_ELEM); launch_mr_elem(Lev); }
      { KTimer t(b, MFEM_K_MR_VERT); launch_mr_vert(Lev); }
      { KTimer t(b, MFEM_K_MR_UPDATE); launch_mr_update(Lev); }
    }
    const int slot = nchunk & 1;
    CUDA_OR(cudaMemcpyAsync(&b->h_ctr_pipe[slot], b->d_ctr, sizeof(BatchCounters), cudaMemcpyDeviceToHost,
                            b->stream),
            MFEM_ERR_CUDA);
    CUDA_OR(cudaEventRecord(b->ev_pipe[slot], b->stream), MFEM_ERR_CUDA);
    if (nchunk > 0) {
      CUDA_OR(cudaEventSynchronize(b->ev_pipe[slot ^ 1]), MFEM_ERR_CUDA);
      if (b->h_ctr_pipe[slot ^ 1].cg_active == 0) break;
    }
    ++nchunk;
    chunk = 8;
  }
  { KTimer t(b, MFEM_K_MR_ELEM); launch_mr_elem(Lev); }
  { KTimer t(b, MFEM_K_MR_VERT); launch_mr_vert(Lev); }
  { KTimer t(b, MFEM_K_MR_EXPORT); launch_mr_export(Lev); }
  b->cg_hint() = std::max(4, (it * 3) / 4);
  return MFEM_OK;
}

// The Newton loop of NewtonOptimizer::step for every scene of the batch.
int batch_newton(mfem_batch* b) {
  const int n = (int)b->scenes.size();
  Launch Lev = make_launch(b, TB_EV);
  { KTimer t(b, MFEM_K_SCALARS); launch_scalars_begin(Lev, n); }
  { KTimer t(b, MFEM_K_STEP_BEGIN); launch_step_begin(Lev); }
  int rc;
  for (int newton = 0; newton <= b->max_newton + 1; ++newton) {
    b->newton_index = newton;
    {
      KTimer t(b, MFEM_K_ELEM_UPDATE);
      Launch l = make_launch(b, TB_ELEM);
      l.variant = b->var_elem;
      launch_elem_update(l, nullptr);
    }
    { KTimer t(b, MFEM_K_ASSEMBLE); launch_assemble(make_launch(b, TB_ROW)); }
    if (b->minres) {
      if ((rc = run_minres(b, Lev))) return rc;
    } else if ((rc = run_pcg(b, make_launch(b, TB_CG)))) {
      return rc;
    }
    {
      KTimer t(b, MFEM_K_LOCAL_SOLVE);
      Launch l = Lev;
      l.variant = b->var_local;
      launch_local_solve(l);
    }
    for (int l = 0; l < b->max_ls; ++l) {
      {
        KTimer t(b, MFEM_K_LS_ENERGY);
        Launch le = Lev;
        le.variant = b->var_ls;
        launch_ls_energy(le);
      }
      if ((rc = sync_counters(b))) return rc;
      if (b->h_ctr->ls_active == 0) break;
    }
    { KTimer t(b, MFEM_K_APPLY); launch_apply(Lev); }
    if ((rc = sync_counters(b))) return rc;
    if (b->h_ctr->error) return MFEM_ERR_TIMEOUT;
    if (b->h_ctr->newton_active == 0) break;
  }
  return MFEM_OK;
}

int batch_step_impl(mfem_batch* b, mfem_step_stats* stats) {
  std::call_once(g_configured, configure_kernels);
  const int n = (int)b->scenes.size();
  CUDA_OR(cudaEventRecord(b->ev0, b->stream), MFEM_ERR_CUDA);
  int rc = batch_newton(b);
  if (rc) return rc;
  for (int i = 0; i < n; ++i)
    if ((rc = bc_step_upload(b->scenes[i], b->stream))) return rc;
  { KTimer t(b, MFEM_K_STEP_END); launch_step_end(make_launch(b, TB_EV)); }
  CUDA_OR(cudaEventRecord(b->ev1, b->stream), MFEM_ERR_CUDA);
  for (int i = 0; i < n; ++i)
    CUDA_OR(cudaMemcpyAsync(&b->h_sc[i], b->scenes[i]->d_sc, sizeof(SceneScalars),
                            cudaMemcpyDeviceToHost, b->stream),
            MFEM_ERR_CUDA);
  CUDA_OR(cudaStreamSynchronize(b->stream), MFEM_ERR_CUDA);
  CUDA_OR(cudaGetLastError(), MFEM_ERR_CUDA);
  harvest_timers(b);
  float ms = 0;
  cudaEventElapsedTime(&ms, b->ev0, b->ev1);
  int worst = MFEM_OK;
  for (int i = 0; i < n; ++i) {
    const SceneScalars& sc = b->h_sc[i];
    if (stats) {
      mfem_step_stats& st = stats[i];
      st.status = worst_status(sc);
      st.newton_iterations = sc.newton_iter;
      st.cg_iterations = sc.cg_total;
      st.ls_iterations = sc.ls_total;
      st.energy = sc.E;
      st.energy_residual = sc.eres;
      st.decrement = sc.decrement;
      st.alpha = sc.alpha_ls;
      st.residual0 = sc.rhs_norm0;
      st.residual = sc.rhs_norm;
      st.cg_error = sc.cg_err;
      st.device_ms = ms;
    }
    if (sc.status == MFEM_ERR_NONFINITE) worst = MFEM_ERR_NONFINITE;
  }
  return worst;
}

int upload_sds(mfem_batch* b);

// One tick of the ticked multi-step form as a CUDA graph over the current
// tables: every kernel of a Newton iteration once, each acting on the
// scenes in its phase, with tick_pcg PCG iterations and one line-search
// trial.
int capture_tick_graph(mfem_batch* b, cudaGraphExec_t* out) {
  Launch Lel = make_launch(b, TB_ELEM);
  Lel.variant = b->var_elem;
  const Launch Lev = make_launch(b, TB_EV);
  Launch Llo = Lev, Lls = Lev;
  Llo.variant = b->var_local;
  Lls.variant = b->var_ls;
  const Launch Lcg = make_launch(b, TB_CG);
  cudaGraph_t g = nullptr;
  CUDA_OR(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), MFEM_ERR_CUDA);
  launch_elem_update(Lel, nullptr);
  launch_assemble(make_launch(b, TB_ROW));
  launch_cgf_scale(Lcg);
  launch_cgf_init(Lcg);
  for (int k = 0; k < b->tick_pcg; ++k) launch_cgf_iter(Lcg, b->cgf_shape);
  launch_local_solve(Llo);
  launch_ls_energy(Lls);
  launch_apply(Lev);
  launch_step_turn(Lev);
  const cudaError_t ec = cudaStreamEndCapture(b->stream, &g);
  if (ec != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    CUDA_OR(ec, MFEM_ERR_CUDA);
  }
  const cudaError_t ei = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  CUDA_OR(ei, MFEM_ERR_CUDA);
  return MFEM_OK;
}

// The kernels' tables become the tiles of the scenes with active[i] set
// (each scene's tiles stay contiguous, so its ticket groups and partials are
// unchanged); the others get no tiles.  The stream must be idle.
int compact_tables(mfem_batch* b, const std::vector<char>& active) {
  const int n = (int)b->scenes.size();
  for (int tb = 0; tb < TB_COUNT; ++tb) {
    std::vector<Tile> t;
    for (int i = 0; i < n; ++i) {
      const int f = b->full_first[(size_t)i * TB_COUNT + tb], c = b->full_count[(size_t)i * TB_COUNT + tb];
      b->h_sds[i].tile_first[tb] = (int)t.size();
      b->h_sds[i].tile_count[tb] = active[i] ? c : 0;
      if (active[i]) t.insert(t.end(), b->h_tiles[tb].begin() + f, b->h_tiles[tb].begin() + f + c);
    }
    if (!t.empty())
      CUDA_OR(cudaMemcpyAsync(b->d_tiles_c[tb], t.data(), sizeof(Tile) * t.size(), cudaMemcpyHostToDevice,
                              b->stream),
              MFEM_ERR_CUDA);
    b->cur_tiles[tb] = b->d_tiles_c[tb];
    b->cur_ntiles[tb] = (int)t.size();
  }
  int rc = upload_sds(b);
  if (rc) return rc;
  if (b->tick_graph_c) cudaGraphExecDestroy(b->tick_graph_c);
  b->tick_graph_c = nullptr;
  return capture_tick_graph(b, &b->tick_graph_c);
}

// The full tables again.
int restore_tables(mfem_batch* b) {
  const int n = (int)b->scenes.size();
  for (int tb = 0; tb < TB_COUNT; ++tb) {
    b->cur_tiles[tb] = b->d_tiles[tb];
    b->cur_ntiles[tb] = b->ntiles[tb];
    for (int i = 0; i < n; ++i) {
      b->h_sds[i].tile_first[tb] = b->full_first[(size_t)i * TB_COUNT + tb];
      b->h_sds[i].tile_count[tb] = b->full_count[(size_t)i * TB_COUNT + tb];
    }
  }
  if (b->tick_graph_c) cudaGraphExecDestroy(b->tick_graph_c);
  b->tick_graph_c = nullptr;
  return upload_sds(b);
}

// Several timesteps per scene in one call, each scene at its own pace
// (mfem_gpu_batch_step_n).  A round is one Newton iteration of every scene
// that still has steps to take: K1, assembly, the linear solve, the local
// solve, the line search, the update; then k_step_turn turns over every
// scene whose Newton loop ended in the round, so that it starts its next
// timestep in the next round instead of waiting for the batch's slowest
// scene.  The arithmetic of each scene is that of n calls of
// mfem_gpu_batch_step (the same kernels and device functions).
int batch_step_n_impl(mfem_batch* b, int steps, mfem_step_stats* stats, double* step_done_ms) {
  std::call_once(g_configured, configure_kernels);
  const int n = (int)b->scenes.size();
  int rc;
  // pins after each BC step of the call, for scenes whose pins move
  for (int i = 0; i < n; ++i) {
    mfem_scene* s = b->scenes[i];
    const int np = s->M.npin;
    const bool scripted = np > 0 && (s->pins_driven || s->M.bc_type == MFEM_BC_STRETCH ||
                                     s->M.bc_type == MFEM_BC_COMPRESS || s->M.bc_type == MFEM_BC_TWIST ||
                                     s->M.bc_type == MFEM_BC_BEND);
    b->h_sds[i].pin_traj = nullptr;
    if (!scripted) continue;
    if (s->pin_traj_cap < (size_t)steps) {
      if (s->d_pin_traj) cudaFree(s->d_pin_traj);
      s->d_pin_traj = nullptr;
      s->pin_traj_cap = 0;
      CUDA_OR(cudaMalloc(&s->d_pin_traj, sizeof(double) * 3 * (size_t)np * steps), MFEM_ERR_OOM);
      s->pin_traj_cap = (size_t)steps;
    }
    std::vector<double> traj(3 * (size_t)np * steps);
    for (int j = 0; j < steps; ++j) {
      if (j == 0 && s->pins_driven) s->pins_driven = false;  // the caller's pins for the first step
      else bc_advance(s);
      std::memcpy(&traj[3 * (size_t)np * j], s->pin_pos.data(), sizeof(double) * 3 * np);
    }
    CUDA_OR(cudaMemcpyAsync(s->d_pin_traj, traj.data(), sizeof(double) * traj.size(), cudaMemcpyHostToDevice,
                            b->stream),
            MFEM_ERR_CUDA);
    // the pins after the call, as the plain form leaves them for later steps
    CUDA_OR(cudaMemcpyAsync(s->d_pin_pos, s->pin_pos.data(), sizeof(double) * 3 * np, cudaMemcpyHostToDevice,
                            b->stream),
            MFEM_ERR_CUDA);
    b->h_sds[i].pin_traj = s->d_pin_traj;
  }
  if ((rc = upload_sds(b))) return rc;  // synchronises: the host trajectories may go
  // the ticked form needs every kernel of a Newton iteration to be gated by
  // the scene's phase (the single-reduction PCG and the reduced system) and
  // every scene to have rows to assemble and solve
  bool ticked = b->pcg_kernel == MFEM_PCG_KERNEL_FUSED && !b->minres;
  for (mfem_scene* s : b->scenes)
    if (s->M.nf == 0) ticked = false;
  unsigned long long* t_start = b->d_step_ns + (size_t)n * kMaxCallSteps;
  CUDA_OR(cudaEventRecord(b->ev0, b->stream), MFEM_ERR_CUDA);
  launch_stamp(t_start, b->stream);
  Launch Lev = make_launch(b, TB_EV);
  { KTimer t(b, MFEM_K_SCALARS); launch_scalars_begin_n(Lev, n, steps, ticked ? 1 : 0); }
  { KTimer t(b, MFEM_K_STEP_BEGIN); launch_step_begin(Lev); }
  if (ticked) {
    // One tick: every kernel of a Newton iteration once, each acting on the
    // scenes in its phase, with tick_pcg PCG iterations and one line-search
    // trial; a scene goes as far through its iteration as the tick takes it
    // and never waits for another scene.  The host reads the batch's
    // counters after every few ticks, one check behind.
    if (!b->tick_graph && (rc = capture_tick_graph(b, &b->tick_graph))) return rc;
    constexpr int kTicksPerCheck = 4;
    const long max_ticks = (long)steps * (b->max_newton + 2) * ((b->max_cg + 17) / b->tick_pcg + b->max_ls + 4);
    long ticks = 0;
    int nchunk = 0;
    bool finished = false;
    int table_scenes = n;  // scenes in the tables the ticks run over
    cudaGraphExec_t tick = b->tick_graph;
    while (ticks < max_ticks) {
      for (int r = 0; r < kTicksPerCheck; ++r, ++ticks) {
        const cudaError_t e = cudaGraphLaunch(tick, b->stream);
        if (e != cudaSuccess) {
          if (tick != b->tick_graph) restore_tables(b);
          CUDA_OR(e, MFEM_ERR_CUDA);
        }
      }
      const int slot = nchunk & 1;
      CUDA_OR(cudaMemcpyAsync(&b->h_ctr_pipe[slot], b->d_ctr, sizeof(BatchCounters), cudaMemcpyDeviceToHost,
                              b->stream),
              MFEM_ERR_CUDA);
      CUDA_OR(cudaEventRecord(b->ev_pipe[slot], b->stream), MFEM_ERR_CUDA);
      if (nchunk > 0) {
        CUDA_OR(cudaEventSynchronize(b->ev_pipe[slot ^ 1]), MFEM_ERR_CUDA);
        const BatchCounters& c = b->h_ctr_pipe[slot ^ 1];
        if (c.error) {
          if (tick != b->tick_graph) restore_tables(b);
          return MFEM_ERR_TIMEOUT;
        }
        if (c.newton_active == 0) {
          finished = true;
          break;
        }
        // half the scenes in the tables have finished: launch over the
        // tiles of those still stepping from now on
        if (table_scenes >= 4 && c.newton_active <= table_scenes / 2) {
          CUDA_OR(cudaStreamSynchronize(b->stream), MFEM_ERR_CUDA);
          for (int i = 0; i < n; ++i)
            CUDA_OR(cudaMemcpyAsync(&b->h_sc[i], b->scenes[i]->d_sc, sizeof(SceneScalars),
                                    cudaMemcpyDeviceToHost, b->stream),
                    MFEM_ERR_CUDA);
          CUDA_OR(cudaStreamSynchronize(b->stream), MFEM_ERR_CUDA);
          std::vector<char> active(n);
          int na = 0;
          for (int i = 0; i < n; ++i) na += (active[i] = b->h_sc[i].newton_active ? 1 : 0);
          if (na == 0) {
            finished = true;
            break;
          }
          if ((rc = compact_tables(b, active))) {
            restore_tables(b);
            return rc;
          }
          tick = b->tick_graph_c;
          table_scenes = na;
          nchunk = 0;
          continue;
        }
      }
      ++nchunk;
    }
    if (tick != b->tick_graph && (rc = restore_tables(b))) return rc;
    if (!finished) {
      if ((rc = sync_counters(b))) return rc;
      if (b->h_ctr->error) return MFEM_ERR_TIMEOUT;
    }
  } else {
    // rounds: one Newton iteration of every scene that still has steps to
    // take; every step of a scene ends within max_newton + 2 rounds
    const long max_rounds = (long)steps * (b->max_newton + 2);
    for (long round = 0; round < max_rounds; ++round) {
      b->newton_index = 0;  // scenes sit at different Newton iterations: one shared PCG hint
      {
        KTimer t(b, MFEM_K_ELEM_UPDATE);
        Launch l = make_launch(b, TB_ELEM);
        l.variant = b->var_elem;
        launch_elem_update(l, nullptr);
      }
      { KTimer t(b, MFEM_K_ASSEMBLE); launch_assemble(make_launch(b, TB_ROW)); }
      if (b->minres) {
        if ((rc = run_minres(b, Lev))) return rc;
      } else if ((rc = run_pcg(b, make_launch(b, TB_CG)))) {
        return rc;
      }
      {
        KTimer t(b, MFEM_K_LOCAL_SOLVE);
        Launch l = Lev;
        l.variant = b->var_local;
        launch_local_solve(l);
      }
      for (int l = 0; l < b->max_ls; ++l) {
        {
          KTimer t(b, MFEM_K_LS_ENERGY);
          Launch le = Lev;
          le.variant = b->var_ls;
          launch_ls_energy(le);
        }
        if ((rc = sync_counters(b))) return rc;
        if (b->h_ctr->ls_active == 0) break;
      }
      { KTimer t(b, MFEM_K_APPLY); launch_apply(Lev); }
      { KTimer t(b, MFEM_K_STEP_END); launch_step_turn(Lev); }
      if ((rc = sync_counters(b))) return rc;
      if (b->h_ctr->error) return MFEM_ERR_TIMEOUT;
      if (b->h_ctr->newton_active == 0) break;
    }
  }
  CUDA_OR(cudaEventRecord(b->ev1, b->stream), MFEM_ERR_CUDA);
  for (int i = 0; i < n; ++i)
    CUDA_OR(cudaMemcpyAsync(&b->h_sc[i], b->scenes[i]->d_sc, sizeof(SceneScalars), cudaMemcpyDeviceToHost,
                            b->stream),
            MFEM_ERR_CUDA);
  std::vector<unsigned long long> sns((size_t)n * kMaxCallSteps + 1);
  CUDA_OR(cudaMemcpyAsync(sns.data(), b->d_step_ns, sizeof(unsigned long long) * sns.size(),
                          cudaMemcpyDeviceToHost, b->stream),
          MFEM_ERR_CUDA);
  CUDA_OR(cudaStreamSynchronize(b->stream), MFEM_ERR_CUDA);
  CUDA_OR(cudaGetLastError(), MFEM_ERR_CUDA);
  harvest_timers(b);
  float ms = 0;
  cudaEventElapsedTime(&ms, b->ev0, b->ev1);
  const unsigned long long t0 = sns[(size_t)n * kMaxCallSteps];
  int worst = MFEM_OK;
  for (int i = 0; i < n; ++i) {
    const SceneScalars& sc = b->h_sc[i];
    const int done = sc.steps_done;
    if (stats) {
      mfem_step_stats& st = stats[i];
      // a scene retired by a failed step reports that step's status; one
      // cut off by the call's bound reports what it finished plus the step
      // in progress
      const bool retired = done < steps && (sc.acc_status == MFEM_ERR_NONFINITE ||
                                            sc.acc_status == MFEM_ERR_PROCRUSTES);
      const bool cut = done < steps && !retired;
      st.status = cut ? MFEM_ERR_TIMEOUT : sc.acc_status;
      st.newton_iterations = sc.acc_newton + (cut ? sc.newton_iter : 0);
      st.cg_iterations = sc.acc_cg + (cut ? sc.cg_total : 0);
      st.ls_iterations = sc.acc_ls + (cut ? sc.ls_total : 0);
      st.energy = sc.E;
      st.energy_residual = sc.eres;
      st.decrement = sc.decrement;
      st.alpha = sc.alpha_ls;
      st.residual0 = sc.rhs_norm0;
      st.residual = sc.rhs_norm;
      st.cg_error = sc.cg_err;
      st.device_ms = ms;
    }
    if (step_done_ms)
      for (int j = 0; j < steps; ++j) {
        const unsigned long long t = sns[(size_t)i * kMaxCallSteps + j];
        step_done_ms[(size_t)i * steps + j] = (j < done && t >= t0) ? double(t - t0) * 1e-6 : -1.0;
      }
    if (sc.acc_status == MFEM_ERR_NONFINITE) worst = MFEM_ERR_NONFINITE;
    if (done < steps && sc.acc_status != MFEM_ERR_NONFINITE && sc.acc_status != MFEM_ERR_PROCRUSTES)
      worst = MFEM_ERR_TIMEOUT;
  }
  return worst;
}

int upload_sds(mfem_batch* b) {
  CUDA_OR(cudaMemcpyAsync(b->d_sds, b->h_sds.data(), sizeof(SceneDev) * b->h_sds.size(),
                          cudaMemcpyHostToDevice, b->stream),
          MFEM_ERR_CUDA);
  CUDA_OR(cudaStreamSynchronize(b->stream), MFEM_ERR_CUDA);
  return MFEM_OK;
}

// ------------------------------------------------------------ autotuner ---
// A batch picks, per kernel, the fastest of variants that compute the same
// bits: the fused PCG iteration's shape (matrix through registers or
// staged through 2-4 shared-memory buffers, L2 keep policy, two slots in
// flight, programmatic dependent launch) and the register budgets of K1,
// K5 and K6.  At batch creation every candidate is timed on the batch's
// own system with CUDA events (a few launches each); the choice is cached
// in memory and on disk, keyed by GPU, precision, solver and the size
// class of the batch (half-octaves of its element and PCG tile counts), so
// that later batches of that class skip the timing.
//   MFEM_GB300_TUNE        "0": built-in defaults, no timing; "force":
//                          always time; otherwise time on a cache miss
//   MFEM_GB300_TUNE_CACHE  cache file (default
//                          $XDG_CACHE_HOME or ~/.cache, mfem_gb300/tune-v1.txt)
// Nothing the timing runs leaves a trace: the rotation warm starts K1
// overwrites are saved and restored, and every other buffer it writes is
// recomputed before it is read in a step.
namespace {

std::mutex g_tune_mu;
std::map<std::string, std::string> g_tune_mem;
bool g_tune_loaded = false;

std::atomic<int> g_tune_override{-1};  // mfem_gpu_set_tuning; -1: the environment decides

int tune_mode() {
  const int o = g_tune_override.load();
  if (o >= 0) return o;
  const char* v = std::getenv("MFEM_GB300_TUNE");
  if (!v) return 1;
  if (!std::strcmp(v, "0") || !std::strcmp(v, "off")) return 0;
  if (!std::strcmp(v, "force")) return 2;
  return 1;
}

std::string tune_cache_path() {
  if (const char* p = std::getenv("MFEM_GB300_TUNE_CACHE")) return p;
  std::string base;
  if (const char* x = std::getenv("XDG_CACHE_HOME")) base = x;
  else if (const char* h = std::getenv("HOME")) base = std::string(h) + "/.cache";
  else return std::string();
  return base + "/mfem_gb300/tune-v1.txt";
}

void tune_load_locked() {
  if (g_tune_loaded) return;
  g_tune_loaded = true;
  const std::string path = tune_cache_path();
  if (path.empty()) return;
  FILE* f = std::fopen(path.c_str(), "r");
  if (!f) return;
  char line[1024];
  while (std::fgets(line, sizeof line, f)) {
    char* tab = std::strchr(line, '\t');
    if (!tab) continue;
    *tab = 0;
    std::string val(tab + 1);
    while (!val.empty() && (val.back() == '\n' || val.back() == '\r')) val.pop_back();
    g_tune_mem[line] = val;
  }
  std::fclose(f);
}

void tune_store_locked(const std::string& key, const std::string& val) {
  g_tune_mem[key] = val;
  const std::string path = tune_cache_path();
  if (path.empty()) return;
  const size_t slash = path.rfind('/');
  if (slash != std::string::npos && slash > 0) {
    const std::string dir = path.substr(0, slash);
    const size_t up = dir.rfind('/');
    if (up != std::string::npos && up > 0) mkdir(dir.substr(0, up).c_str(), 0755);
    mkdir(dir.c_str(), 0755);
  }
  if (FILE* f = std::fopen(path.c_str(), "a")) {
    std::fprintf(f, "%s\t%s\n", key.c_str(), val.c_str());
    std::fclose(f);
  }
}

int size_class(int n) {  // half-octaves of a tile count
  return n <= 1 ? 0 : (int)std::lround(2.0 * std::log2((double)n));
}

std::string tune_key(const mfem_batch* b) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceProp prop;
  std::string name = "gpu";
  if (cudaGetDeviceProperties(&prop, dev) == cudaSuccess) name = prop.name;
  for (char& c : name)
    if (c == ' ' || c == '\t' || c == '|' || c == '"' || c == '\\') c = '_';
  char buf[512];
  std::snprintf(buf, sizeof buf, "%s|%d|fp64=%d|jacobi=%d|fem=%d|minres=%d|pcg=%d|elem=%d|cg=%d", name.c_str(),
                sms, b->fp64, b->jacobi, b->fem, b->minres, b->pcg_kernel, size_class(b->ntiles[TB_ELEM]),
                size_class(b->ntiles[TB_CG]));
  return buf;
}

// Mean device time of one call of `launch` (after one untimed call).
template <typename F>
int time_calls(mfem_batch* b, int reps, F&& launch, float* ms) {
  launch();
  CUDA_OR(cudaEventRecord(b->ev0, b->stream), MFEM_ERR_CUDA);
  for (int r = 0; r < reps; ++r) launch();
  CUDA_OR(cudaEventRecord(b->ev1, b->stream), MFEM_ERR_CUDA);
  CUDA_OR(cudaEventSynchronize(b->ev1), MFEM_ERR_CUDA);
  CUDA_OR(cudaGetLastError(), MFEM_ERR_CUDA);
  float t = 0;
  CUDA_OR(cudaEventElapsedTime(&t, b->ev0, b->ev1), MFEM_ERR_CUDA);
  *ms = t / reps;
  return MFEM_OK;
}

// Mean device time of `launch` alone, each call preceded by an untimed
// `prep` that puts its input state back (the line search's energy runs
// only while the local solve has opened a line search).
template <typename P, typename F>
int time_prepped(mfem_batch* b, int reps, P&& prep, F&& launch, float* ms) {
  float total = 0;
  for (int r = 0; r <= reps; ++r) {
    prep();
    CUDA_OR(cudaEventRecord(b->ev0, b->stream), MFEM_ERR_CUDA);
    launch();
    CUDA_OR(cudaEventRecord(b->ev1, b->stream), MFEM_ERR_CUDA);
    CUDA_OR(cudaEventSynchronize(b->ev1), MFEM_ERR_CUDA);
    CUDA_OR(cudaGetLastError(), MFEM_ERR_CUDA);
    float t = 0;
    CUDA_OR(cudaEventElapsedTime(&t, b->ev0, b->ev1), MFEM_ERR_CUDA);
    if (r > 0) total += t;  // the first pair warms up
  }
  *ms = total / reps;
  return MFEM_OK;
}

// Index of the fastest candidate; a variant replaces the default (index 0)
// only if it is at least 2% faster.
int pick(const std::vector<float>& t) {
  int best = 0;
  for (int i = 1; i < (int)t.size(); ++i)
    if (t[i] < t[best]) best = i;
  return (best != 0 && t[best] < 0.98f * t[0]) ? best : 0;
}

std::vector<CgfShape> cgf_candidates(int fp64) {
  if (fp64) return {CgfShape{0, 0, 1, 0}, CgfShape{2, 0, 1, 0}, CgfShape{2, 0, 1, 1}};
  return {CgfShape{2, 0, 1, 1}, CgfShape{0, 0, 1, 0}, CgfShape{2, 0, 1, 0}, CgfShape{3, 0, 1, 1},
          CgfShape{2, 1, 1, 1}, CgfShape{4, 0, 2, 1}, CgfShape{8, 0, 4, 1}};
}

std::string shape_str(const CgfShape& c) {
  char buf[96];
  std::snprintf(buf, sizeof buf, "stages=%d keep=%d unroll=%d pdl=%d", c.stages, c.keep, c.unroll, c.pdl);
  return buf;
}

// The cached form of a choice: "stages keep unroll pdl k1 k5 k6".
std::string choice_str(const mfem_batch* b) {
  char buf[96];
  std::snprintf(buf, sizeof buf, "%d %d %d %d %d %d %d", b->cgf_shape.stages, b->cgf_shape.keep,
                b->cgf_shape.unroll, b->cgf_shape.pdl, b->var_elem, b->var_local, b->var_ls);
  return buf;
}
bool parse_choice(const std::string& v, mfem_batch* b) {
  int a[7];
  if (std::sscanf(v.c_str(), "%d %d %d %d %d %d %d", &a[0], &a[1], &a[2], &a[3], &a[4], &a[5], &a[6]) != 7)
    return false;
  if (a[4] < 0 || a[4] >= elem_update_variants(b->fp64, b->fem) || a[5] < 0 ||
      a[5] >= local_solve_variants(b->fp64) || a[6] < 0 || a[6] >= ls_energy_variants(b->fp64))
    return false;
  b->cgf_shape = CgfShape{a[0], a[1], a[2], a[3]};
  b->var_elem = a[4];
  b->var_local = a[5];
  b->var_ls = a[6];
  return true;
}

void json_kernel(std::string& out, const char* name, const std::vector<std::string>& names,
                 const std::vector<float>& t, int chosen) {
  char buf[256];
  std::snprintf(buf, sizeof buf,
                "\"%s\": {\"chosen\": \"%s\", \"default_ms\": %.6f, \"tuned_ms\": %.6f, \"candidates\": {", name,
                names[chosen].c_str(), t[0], t[chosen]);
  out += buf;
  for (size_t i = 0; i < t.size(); ++i) {
    std::snprintf(buf, sizeof buf, "%s\"%s\": %.6f", i ? ", " : "", names[i].c_str(), t[i]);
    out += buf;
  }
  out += "}}";
}

int batch_autotune(mfem_batch* b) {
  const int mode = tune_mode();
  if (mode == 0) return MFEM_OK;
  const std::string key = tune_key(b);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    tune_load_locked();
    auto it = g_tune_mem.find(key);
    if (mode == 1 && it != g_tune_mem.end() && parse_choice(it->second, b)) {
      b->tune_report = "{\"source\": \"cache\", \"key\": \"" + key + "\", \"choice\": \"" + it->second + "\"}";
      return MFEM_OK;
    }
  }
  const int n = (int)b->scenes.size();
  // the rotation warm starts that K1 overwrites
  size_t qbytes = 0;
  for (mfem_scene* s : b->scenes) qbytes += 4 * (size_t)s->ntp * s->rsz;
  char* qsave = nullptr;
  CUDA_OR(cudaMalloc(&qsave, std::max<size_t>(qbytes, 1)), MFEM_ERR_OOM);
  struct Free {
    char* p;
    ~Free() { cudaFree(p); }
  } free_q{qsave};
  {
    size_t off = 0;
    for (mfem_scene* s : b->scenes) {
      const size_t nb = 4 * (size_t)s->ntp * s->rsz;
      CUDA_OR(cudaMemcpyAsync(qsave + off, s->dev.quat, nb, cudaMemcpyDeviceToDevice, b->stream), MFEM_ERR_CUDA);
      off += nb;
    }
  }
  // a PCG that never stops: tolerance 0, no iteration limit
  std::vector<SceneDev> tsd = b->h_sds;
  for (SceneDev& d : tsd) {
    d.cg_tol = 0.0;
    d.max_cg = 1 << 30;
  }
  CUDA_OR(cudaMemcpyAsync(b->d_sds, tsd.data(), sizeof(SceneDev) * n, cudaMemcpyHostToDevice, b->stream),
          MFEM_ERR_CUDA);
  const Launch Lev = make_launch(b, TB_EV);
  launch_scalars_begin(Lev, n);
  launch_step_begin(Lev);
  int rc;
  std::string rep = "{\"source\": \"tuned\", \"key\": \"" + key + "\", \"kernels\": {";
  bool first = true;
  auto sep = [&]() {
    if (!first) rep += ", ";
    first = false;
  };
  // K1
  {
    const int nv = elem_update_variants(b->fp64, b->fem);
    std::vector<float> t(nv);
    std::vector<std::string> names;
    for (int v = 0; v < nv; ++v) {
      Launch l = make_launch(b, TB_ELEM);
      l.variant = v;
      if ((rc = time_calls(b, 3, [&]() { launch_elem_update(l, nullptr); }, &t[v]))) return rc;
      names.push_back(elem_update_variant_name(v));
    }
    b->var_elem = pick(t);
    if (nv > 1) {
      sep();
      json_kernel(rep, "k_elem_update", names, t, b->var_elem);
    }
  }
  launch_assemble(make_launch(b, TB_ROW));
  // the fused PCG iteration: chunks of 8 launches as graphs, as a step runs them
  bool have_dx = false;
  if (b->pcg_kernel == MFEM_PCG_KERNEL_FUSED && !b->minres && b->ntiles[TB_CG] >= 8) {
    const Launch Lcg = make_launch(b, TB_CG);
    launch_cgf_init(Lcg);
    const std::vector<CgfShape> cand = cgf_candidates(b->fp64);
    std::vector<float> t(cand.size());
    std::vector<std::string> names;
    for (size_t c = 0; c < cand.size(); ++c) {
      b->cgf_shape = cand[c];
      cudaGraphExec_t g = nullptr;
      if ((rc = capture_cg_graph(b, Lcg, true, &g))) return rc;
      rc = time_calls(b, 3, [&]() { cudaGraphLaunch(g, b->stream); }, &t[c]);
      cudaGraphExecDestroy(g);
      if (rc) return rc;
      t[c] /= 8.f;  // per iteration
      names.push_back(shape_str(cand[c]));
    }
    const int best = pick(t);
    b->cgf_shape = cand[best];
    sep();
    json_kernel(rep, "k_cgf_iter", names, t, best);
    have_dx = true;
  }
  if (!have_dx) {
    for (mfem_scene* s : b->scenes)
      CUDA_OR(cudaMemsetAsync(s->dev.cg_x, 0, 4 * (size_t)std::max(s->M.nf, 1) * s->rsz, b->stream),
              MFEM_ERR_CUDA);
  }
  if (!b->minres) {
    std::vector<float> t5(local_solve_variants(b->fp64)), t6(ls_energy_variants(b->fp64));
    std::vector<std::string> n5, n6;
    for (int v = 0; v < (int)t5.size(); ++v) {
      Launch l = Lev;
      l.variant = v;
      if ((rc = time_calls(b, 3, [&]() { launch_local_solve(l); }, &t5[v]))) return rc;
      n5.push_back(local_solve_variant_name(v));
    }
    for (int v = 0; v < (int)t6.size(); ++v) {
      Launch l = Lev;
      l.variant = v;
      if ((rc = time_prepped(b, 3, [&]() { launch_local_solve(Lev); }, [&]() { launch_ls_energy(l); }, &t6[v])))
        return rc;
      n6.push_back(ls_energy_variant_name(v));
    }
    b->var_local = pick(t5);
    b->var_ls = pick(t6);
    sep();
    json_kernel(rep, "k_local_solve", n5, t5, b->var_local);
    sep();
    json_kernel(rep, "k_ls_energy", n6, t6, b->var_ls);
  }
  rep += "}}";
  // restore: rotations, the real scene parameters, counters
  {
    size_t off = 0;
    for (mfem_scene* s : b->scenes) {
      const size_t nb = 4 * (size_t)s->ntp * s->rsz;
      CUDA_OR(cudaMemcpyAsync(s->dev.quat, qsave + off, nb, cudaMemcpyDeviceToDevice, b->stream), MFEM_ERR_CUDA);
      off += nb;
    }
  }
  CUDA_OR(cudaMemsetAsync(b->d_ctr, 0, sizeof(BatchCounters), b->stream), MFEM_ERR_CUDA);
  if ((rc = upload_sds(b))) return rc;  // synchronises the stream
  b->tune_report = rep;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  tune_store_locked(key, choice_str(b));
  return MFEM_OK;
}

}  // namespace

int batch_build(mfem_scene* const* scenes, int n, mfem_batch** out) {
  if (!scenes || n <= 0 || !out) return MFEM_ERR_INVALID;
  auto b = std::make_unique<mfem_batch>();
  b->fp64 = scenes[0]->fp64;
  for (int i = 0; i < n; ++i) {
    if (!scenes[i] || scenes[i]->fp64 != b->fp64) return MFEM_ERR_INVALID;
    b->scenes.push_back(scenes[i]);
  }
  // tile tables
  std::vector<Tile> tabs[TB_COUNT];
  b->h_sds.resize(n);
  for (int i = 0; i < n; ++i) {
    mfem_scene* s = scenes[i];
    SceneDev D = s->dev;
    auto add = [&](int tb, int kind, int count, int per) {
      for (int beg = 0; beg < count; beg += per) tabs[tb].push_back(Tile{i, kind, beg, std::min(count, beg + per)});
    };
    for (int tb = 0; tb < TB_COUNT; ++tb) D.tile_first[tb] = (int)tabs[tb].size();
    add(TB_ELEM, 0, s->M.nt, kElemTile);
    add(TB_ROW, 0, s->M.nf, kRowTile);
    add(TB_CG, 0, s->M.nf, kCgRows);
    add(TB_EV, 0, s->M.nt, kElemTile);
    add(TB_EV, 1, s->M.nv, kVertTile);
    for (int tb = 0; tb < TB_COUNT; ++tb) D.tile_count[tb] = (int)tabs[tb].size() - D.tile_first[tb];
    b->h_sds[i] = D;
    b->max_newton = std::max(b->max_newton, s->cfg.max_newton_iterations);
    b->max_ls = std::max(b->max_ls, s->cfg.max_linesearch_iterations);
    b->max_cg = std::max(b->max_cg, s->cfg.max_iterative_solver_iters);
  }
  size_t maxt = 1;
  for (int tb = 0; tb < TB_COUNT; ++tb) {
    b->ntiles[tb] = (int)tabs[tb].size();
    maxt = std::max(maxt, tabs[tb].size());
  }
  // the fused iteration's matrix staged through two shared-memory buffers
  // per warp, each iteration a programmatic dependent launch (measured
  // fastest on the 1M-tet cube); the autotuner may choose another shape for
  // the batch's size class
  b->cgf_shape = b->fp64 ? CgfShape{0, 0, 1, 0} : CgfShape{2, 0, 1, 1};
  b->pcg_kernel = scenes[0]->cfg.pcg_kernel;
  // MFEM_GB300_CG_LOOP=0: the PCG loop as chunks with host checks instead
  // of the device-driven WHILE graph
  if (const char* e = std::getenv("MFEM_GB300_CG_LOOP")) b->cg_loop_on = std::atoi(e) != 0;
  b->minres = scenes[0]->dev.minres;
  b->fem = scenes[0]->dev.fem;
  b->jacobi = 1;
  for (int i = 0; i < n; ++i)
    if (scenes[i]->dev.block_jacobi) b->jacobi = 0;
  for (int i = 1; i < n; ++i)
    if (scenes[i]->cfg.pcg_kernel != b->pcg_kernel || scenes[i]->dev.minres != b->minres ||
        scenes[i]->dev.fem != b->fem)
      return MFEM_ERR_INVALID;
  int sms = 0;
  {
    int dev = 0;
    CUDA_OR(cudaGetDevice(&dev), MFEM_ERR_CUDA);
    CUDA_OR(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), MFEM_ERR_CUDA);
  }
  if (b->pcg_kernel == MFEM_PCG_KERNEL_AUTO)
    b->pcg_kernel = (b->ntiles[TB_CG] >= 2 * sms || b->ntiles[TB_CG] <= 4) ? MFEM_PCG_KERNEL_FUSED
                                                                          : MFEM_PCG_KERNEL_SPLIT;
  if (b->pcg_kernel == MFEM_PCG_KERNEL_PERSISTENT) {
    const int per_sm = cg_solve_blocks_per_sm(b->fp64);
    if (per_sm <= 0) return MFEM_ERR_CUDA;
    b->coop_grid = std::min(b->ntiles[TB_CG], per_sm * sms);
  }
  Arena A;
  auto lay = [&](Arena& a) {
    for (int tb = 0; tb < TB_COUNT; ++tb) {
      b->d_tiles[tb] = a.take<Tile>(std::max<size_t>(tabs[tb].size(), 1));
      b->d_tiles_c[tb] = a.take<Tile>(std::max<size_t>(tabs[tb].size(), 1));
    }
    b->d_sds = a.take<SceneDev>(n);
    b->d_partials = a.take<double>(maxt * kNumPartials);
    b->pstride = (int)maxt;
    b->d_ctr = a.take<BatchCounters>(1);
    b->d_step_ns = a.take<unsigned long long>((size_t)n * kMaxCallSteps + 1);
  };
  lay(A);
  CUDA_OR(cudaMalloc(&b->dmem, A.used), MFEM_ERR_OOM);
  Arena B;
  B.base = b->dmem;
  lay(B);
  b->full_first.resize((size_t)n * TB_COUNT);
  b->full_count.resize((size_t)n * TB_COUNT);
  for (int tb = 0; tb < TB_COUNT; ++tb) {
    b->cur_tiles[tb] = b->d_tiles[tb];
    b->cur_ntiles[tb] = b->ntiles[tb];
    b->h_tiles[tb] = tabs[tb];
    for (int i = 0; i < n; ++i) {
      b->full_first[(size_t)i * TB_COUNT + tb] = b->h_sds[i].tile_first[tb];
      b->full_count[(size_t)i * TB_COUNT + tb] = b->h_sds[i].tile_count[tb];
    }
  }
  for (int i = 0; i < n; ++i) {
    b->h_sds[i].step_ns = b->d_step_ns + (size_t)i * kMaxCallSteps;
    b->h_sds[i].pin_traj = nullptr;
  }
  CUDA_OR(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), MFEM_ERR_CUDA);
  CUDA_OR(cudaEventCreate(&b->ev0), MFEM_ERR_CUDA);
  CUDA_OR(cudaEventCreate(&b->ev1), MFEM_ERR_CUDA);
  CUDA_OR(cudaMallocHost(&b->h_ctr, sizeof(BatchCounters)), MFEM_ERR_OOM);
  CUDA_OR(cudaMallocHost(&b->h_ctr_pipe, 2 * sizeof(BatchCounters)), MFEM_ERR_OOM);
  for (int k = 0; k < 2; ++k)
    CUDA_OR(cudaEventCreateWithFlags(&b->ev_pipe[k], cudaEventDisableTiming), MFEM_ERR_CUDA);
  CUDA_OR(cudaMallocHost(&b->h_sc, sizeof(SceneScalars) * n), MFEM_ERR_OOM);
  for (int tb = 0; tb < TB_COUNT; ++tb)
    if (!tabs[tb].empty())
      CUDA_OR(cudaMemcpyAsync(b->d_tiles[tb], tabs[tb].data(), sizeof(Tile) * tabs[tb].size(),
                              cudaMemcpyHostToDevice, b->stream),
              MFEM_ERR_CUDA);
  CUDA_OR(cudaMemsetAsync(b->d_ctr, 0, sizeof(BatchCounters), b->stream), MFEM_ERR_CUDA);
  int rc = upload_sds(b.get());
  if (rc) return rc;
  std::call_once(g_configured, configure_kernels);
  if ((rc = batch_autotune(b.get()))) return rc;
  *out = b.release();
  return MFEM_OK;
}

void batch_free(mfem_batch* b) {
  if (!b) return;
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->dmem) cudaFree(b->dmem);
  if (b->h_ctr) cudaFreeHost(b->h_ctr);
  if (b->h_ctr_pipe) cudaFreeHost(b->h_ctr_pipe);
  if (b->cg_graph) cudaGraphExecDestroy(b->cg_graph);
  if (b->cg_loop) cudaGraphExecDestroy(b->cg_loop);
  for (int k = 0; k < 2; ++k)
    if (b->ev_pipe[k]) cudaEventDestroy(b->ev_pipe[k]);
  if (b->h_sc) cudaFreeHost(b->h_sc);
  for (cudaEvent_t e : b->ev_pool) cudaEventDestroy(e);
  if (b->tick_graph) cudaGraphExecDestroy(b->tick_graph);
  if (b->tick_graph_c) cudaGraphExecDestroy(b->tick_graph_c);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

int scene_layout_bytes(mfem_scene* s, size_t* bytes) {
  Arena A;
  layout_scene(s, A);
  *bytes = A.used;
  return MFEM_OK;
}

int scene_init_device(mfem_scene* s) {
  const HostMesh& M = s->M;
  Arena A;
  layout_scene(s, A);
  s->dbytes = A.used;
  CUDA_OR(cudaMalloc(&s->dmem, s->dbytes), MFEM_ERR_OOM);
  Arena B;
  B.base = s->dmem;
  layout_scene(s, B);
  SceneDev& D = s->dev;
  D.nv = M.nv;
  D.nt = M.nt;
  D.nf = M.nf;
  D.nnzb = M.nnzb;
  D.ntp = s->ntp;
  D.npin = M.npin;
  D.material_uniform = M.material_uniform;
  D.block_jacobi = s->cfg.linear_solver == MFEM_SOLVER_GPU_PCG_BLOCK ? 1 : 0;
  D.minres = s->cfg.linear_solver == MFEM_SOLVER_MINRES_ID ? 1 : 0;
  D.fem = s->cfg.formulation == MFEM_FORMULATION_STRETCH ? 1 : 0;
  D.fp64 = s->fp64;
  D.h2 = s->h2;
  D.h2x = split_df(D.h2);
  D.dt = s->dt;
  D.newton_tol = s->cfg.newton_tol;
  D.res_tol = s->cfg.newton_residual_tolerance;
  D.cg_tol = s->cfg.iterative_solver_tolerance;
  D.max_newton = s->cfg.max_newton_iterations;
  D.max_ls = s->cfg.max_linesearch_iterations;
  D.max_cg = s->cfg.max_iterative_solver_iters;
  D.bdf_order = s->cfg.bdf_order;
  static const double alphas[7][6] = {
      {0},
      {1.0},
      {4.0 / 3, -1.0 / 3},
      {18.0 / 11, -9.0 / 11, 2.0 / 11},
      {48.0 / 25, -36.0 / 25, 16.0 / 25, -3.0 / 25},
      {300.0 / 137, -300.0 / 137, 200.0 / 137, -75.0 / 137, 12.0 / 137},
      {360.0 / 147, -450.0 / 147, 400.0 / 147, -225.0 / 147, 72.0 / 147, -10.0 / 147}};
  for (int i = 0; i < 6; ++i) D.bdf_alpha[i] = alphas[D.bdf_order][i];
  // SimConfig::ext is float[3]; the reference casts it to double (displacement.cpp:96).
  for (int k = 0; k < 3; ++k) D.body[k] = double(float(s->cfg.body_force[k]));
  {
    double acc = 0;
    for (int v = 0; v < M.nv; ++v) {
      if (M.free_map[v] < 0) continue;
      double m = 0;
      for (int q = M.m_ptr[v]; q < M.m_ptr[v + 1]; ++q) m += M.m_val[q];
      for (int k = 0; k < 3; ++k) acc += (s->h2 * m * D.body[k]) * (s->h2 * m * D.body[k]);
    }
    D.load_norm = std::sqrt(acc);
  }
  cudaStream_t st = nullptr;
  CUDA_OR(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), MFEM_ERR_CUDA);
  auto put = [&](const void* dst, const void* src, size_t bytes) -> int {
    if (bytes == 0) return MFEM_OK;
    CUDA_OR(cudaMemcpyAsync(const_cast<void*>(dst), src, bytes, cudaMemcpyHostToDevice, st), MFEM_ERR_CUDA);
    return MFEM_OK;
  };
  int rc = 0;
  CUDA_OR(cudaMemsetAsync(s->dmem, 0, s->dbytes, st), MFEM_ERR_CUDA);
  rc |= put(D.tets, M.T.data(), sizeof(int) * M.T.size());
  if (D.mat) rc |= put(D.mat, M.mat.data(), M.mat.size());
  const std::vector<double> x0e = to_ext(M.V0.data(), M.V0.size(), s->fp64);
  const std::vector<double> v0e = to_ext(M.v0.data(), M.v0.size(), s->fp64);
  rc |= put(D.x, x0e.data(), 8 * x0e.size());
  for (int i = 0; i < D.bdf_order; ++i) {
    rc |= put(byte_ptr(D.xhist, 24 * (size_t)M.nv * i), x0e.data(), 8 * x0e.size());
    rc |= put(byte_ptr(D.vhist, 24 * (size_t)M.nv * i), v0e.data(), 8 * v0e.size());
  }
  rc |= put(D.free_map, M.free_map.data(), sizeof(int) * M.nv);
  rc |= put(D.free_vert, M.free_vert.data(), sizeof(int) * M.nf);
  rc |= put(D.pin_vert, M.pin_vert.data(), sizeof(int) * M.npin);
  rc |= put(s->d_pin_pos, s->pin_pos.data(), sizeof(double) * s->pin_pos.size());
  rc |= put(D.m_ptr, M.m_ptr.data(), sizeof(int) * M.m_ptr.size());
  rc |= put(D.m_col, M.m_col.data(), sizeof(int) * M.m_col.size());
  rc |= put(D.b_ptr, M.b_ptr.data(), sizeof(int) * M.b_ptr.size());
  rc |= put(D.b_col, M.b_col.data(), sizeof(int) * M.b_col.size());
  rc |= put(D.slice_off, M.slice_off.data(), sizeof(int) * M.slice_off.size());
  rc |= put(D.inc_ptr, M.inc_ptr.data(), sizeof(int) * M.inc_ptr.size());
  rc |= put(D.inc, M.inc.data(), sizeof(int2) * M.inc.size());
  std::vector<double> mlinv;
  if (D.minres) {
    // inverse lumped projected mass per free row: 1 / sum_{b free} m_ab
    mlinv.assign(std::max(M.nf, 1), 1.0);
    for (int v = 0; v < M.nv; ++v) {
      const int f = M.free_map[v];
      if (f < 0) continue;
      double m = 0;
      for (int q = M.m_ptr[v]; q < M.m_ptr[v + 1]; ++q)
        if (M.free_map[M.m_col[q]] >= 0) m += M.m_val[q];
      mlinv[f] = 1.0 / m;
    }
    rc |= put(D.mr_mlinv, mlinv.data(), sizeof(double) * mlinv.size());
  }
  if (rc) return MFEM_ERR_CUDA;
  CUDA_OR(cudaStreamSynchronize(st), MFEM_ERR_CUDA);
  rc = s->fp64 ? upload_scene_reals<double>(s, st) : upload_scene_reals<float>(s, st);
  cudaStreamDestroy(st);
  return rc;
}

template <typename T>
void download_soa(const void* dsrc, int nt, int ntp, int ncomp, double* out, cudaStream_t st) {
  std::vector<T> tmp((size_t)ncomp * ntp);
  cudaMemcpyAsync(tmp.data(), dsrc, tmp.size() * sizeof(T), cudaMemcpyDeviceToHost, st);
  cudaStreamSynchronize(st);
  for (int e = 0; e < nt; ++e)
    for (int k = 0; k < ncomp; ++k) out[(size_t)ncomp * e + k] = double(tmp[(size_t)k * ntp + e]);
}

template <typename T>
void upload_soa(void* ddst, int nt, int ntp, int ncomp, const double* in, cudaStream_t st) {
  std::vector<T> tmp((size_t)ncomp * ntp, T(0));
  for (int e = 0; e < nt; ++e)
    for (int k = 0; k < ncomp; ++k) tmp[(size_t)k * ntp + e] = T(in[(size_t)ncomp * e + k]);
  cudaMemcpyAsync(ddst, tmp.data(), tmp.size() * sizeof(T), cudaMemcpyHostToDevice, st);
  cudaStreamSynchronize(st);
}

// Gauss-Jordan inverse with partial pivoting of a column-major 6x6 (the
// Hinv output of the element parity entry point).
void inverse6_host(const double* A, double* Ai) {
  double a[36];
  for (int i = 0; i < 36; ++i) {
    a[i] = A[i];
    Ai[i] = (i % 7 == 0) ? 1.0 : 0.0;
  }
  for (int k = 0; k < 6; ++k) {
    int p = k;
    for (int i = k + 1; i < 6; ++i)
      if (std::fabs(a[i + 6 * k]) > std::fabs(a[p + 6 * k])) p = i;
    for (int j = 0; j < 6; ++j) {
      std::swap(a[k + 6 * j], a[p + 6 * j]);
      std::swap(Ai[k + 6 * j], Ai[p + 6 * j]);
    }
    const double inv = 1.0 / a[k + 6 * k];
    for (int j = 0; j < 6; ++j) {
      a[k + 6 * j] *= inv;
      Ai[k + 6 * j] *= inv;
    }
    for (int i = 0; i < 6; ++i)
      if (i != k) {
        const double f = a[i + 6 * k];
        for (int j = 0; j < 6; ++j) {
          a[i + 6 * j] -= f * a[k + 6 * j];
          Ai[i + 6 * j] -= f * Ai[k + 6 * j];
        }
      }
  }
}

void quat_to_rot_h(const double q[4], double* R) {
  const double w = q[0], x = q[1], y = q[2], z = q[3];
  const double n = w * w + x * x + y * y + z * z;
  const double s = n > 0 ? 2.0 / n : 0.0;
  R[0] = 1 - s * (y * y + z * z);
  R[3] = s * (x * y - w * z);
  R[6] = s * (x * z + w * y);
  R[1] = s * (x * y + w * z);
  R[4] = 1 - s * (x * x + z * z);
  R[7] = s * (y * z - w * x);
  R[2] = s * (x * z - w * y);
  R[5] = s * (y * z + w * x);
  R[8] = 1 - s * (x * x + y * y);
}

void rot_to_quat_h(const double* R, double q[4]) {
  const double t = R[0] + R[4] + R[8];
  if (t > 0) {
    const double s = std::sqrt(t + 1) * 2;
    q[0] = 0.25 * s; q[1] = (R[5] - R[7]) / s; q[2] = (R[6] - R[2]) / s; q[3] = (R[1] - R[3]) / s;
  } else if (R[0] > R[4] && R[0] > R[8]) {
    const double s = std::sqrt(1 + R[0] - R[4] - R[8]) * 2;
    q[0] = (R[5] - R[7]) / s; q[1] = 0.25 * s; q[2] = (R[3] + R[1]) / s; q[3] = (R[6] + R[2]) / s;
  } else if (R[4] > R[8]) {
    const double s = std::sqrt(1 + R[4] - R[0] - R[8]) * 2;
    q[0] = (R[6] - R[2]) / s; q[1] = (R[3] + R[1]) / s; q[2] = 0.25 * s; q[3] = (R[7] + R[5]) / s;
  } else {
    const double s = std::sqrt(1 + R[8] - R[0] - R[4]) * 2;
    q[0] = (R[1] - R[3]) / s; q[1] = (R[6] + R[2]) / s; q[2] = (R[7] + R[5]) / s; q[3] = 0.25 * s;
  }
  const double n = 1.0 / std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  for (int i = 0; i < 4; ++i) q[i] *= n;
}

}  // namespace

// ================================================================ C ABI ===
extern "C" {

int mfem_gpu_abi_version(void) { return MFEM_ABI_VERSION; }

int mfem_gpu_set_device(int device) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return MFEM_ERR_NO_DEVICE;
  if (device < 0 || device >= n) return MFEM_ERR_INVALID;
  CUDA_OR(cudaSetDevice(device), MFEM_ERR_CUDA);
  return MFEM_OK;
}

const char* mfem_gpu_status_string(int status) {
  switch (status) {
    case MFEM_OK: return "ok";
    case MFEM_ERR_INVALID: return "invalid argument";
    case MFEM_ERR_OOM: return "out of device memory";
    case MFEM_ERR_CUDA: return g_last_error[0] ? g_last_error : "CUDA error";
    case MFEM_ERR_NONFINITE: return "non-finite value";
    case MFEM_ERR_CG_MAXITER: return "PCG reached max iterations";
    case MFEM_ERR_LS_FAILED: return "line search reached max iterations";
    case MFEM_ERR_PROCRUSTES: return "singular rotation Hessian";
    case MFEM_ERR_TIMEOUT: return "bounded device wait timed out";
    case MFEM_ERR_NO_DEVICE: return "no CUDA device";
    case MFEM_ERR_UNSUPPORTED: return "unsupported option";
    case MFEM_ERR_CAPACITY: return "capacity exceeded";
    default: return "unknown status";
  }
}

int mfem_gpu_selftest_bounded_wait(double* waited_ms) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return MFEM_ERR_NO_DEVICE;
  BatchCounters* d = nullptr;
  CUDA_OR(cudaMalloc(&d, sizeof(BatchCounters)), MFEM_ERR_OOM);
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  BatchCounters h{};
  int rc = MFEM_OK;
  float ms = 0.f;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
      cudaEventCreate(&e1) != cudaSuccess || cudaMemsetAsync(d, 0, sizeof(BatchCounters), st) != cudaSuccess ||
      cudaEventRecord(e0, st) != cudaSuccess || launch_barrier_selftest(d, st) != cudaSuccess ||
      cudaEventRecord(e1, st) != cudaSuccess ||
      cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
    rc = MFEM_ERR_CUDA;
  } else {
    // the wait ran out as designed: the persistent PCG reports this status
    rc = h.error ? MFEM_ERR_TIMEOUT : MFEM_OK;
    // and the context stays usable
    if (cudaMemsetAsync(d, 0, sizeof(BatchCounters), st) != cudaSuccess || cudaStreamSynchronize(st) != cudaSuccess)
      rc = MFEM_ERR_CUDA;
  }
  if (waited_ms) *waited_ms = ms;
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  cudaFree(d);
  return rc;
}

int mfem_gpu_device_info(char* name, int name_len, int* sm_count) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return MFEM_ERR_NO_DEVICE;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceProp p;
  CUDA_OR(cudaGetDeviceProperties(&p, dev), MFEM_ERR_CUDA);
  if (name && name_len > 0) {
    strncpy(name, p.name, name_len - 1);
    name[name_len - 1] = 0;
  }
  if (sm_count) *sm_count = p.multiProcessorCount;
  return MFEM_OK;
}

static int scene_prepare(const mfem_scene_desc* desc, std::unique_ptr<mfem_scene>& s) {
  s.reset(new (std::nothrow) mfem_scene());
  if (!s) return MFEM_ERR_OOM;
  int rc = build_host_mesh(desc, s->M);
  if (rc) return rc;
  if (desc->precision != MFEM_PRECISION_FP64 && desc->precision != MFEM_PRECISION_MIXED)
    return MFEM_ERR_INVALID;
  if (desc->linear_solver != MFEM_SOLVER_EIGEN_CG_DIAG &&
      desc->linear_solver != MFEM_SOLVER_GPU_PCG_BLOCK && desc->linear_solver != MFEM_SOLVER_MINRES_ID)
    return MFEM_ERR_UNSUPPORTED;
  if (desc->max_newton_iterations < 0 || desc->max_linesearch_iterations < 0 ||
      desc->max_iterative_solver_iters < 0)
    return MFEM_ERR_INVALID;
  if (desc->pcg_kernel != MFEM_PCG_KERNEL_PERSISTENT && desc->pcg_kernel != MFEM_PCG_KERNEL_SPLIT &&
      desc->pcg_kernel != MFEM_PCG_KERNEL_FUSED && desc->pcg_kernel != MFEM_PCG_KERNEL_AUTO)
    return MFEM_ERR_INVALID;
  if (desc->formulation != MFEM_FORMULATION_MIXED_STRETCH && desc->formulation != MFEM_FORMULATION_STRETCH)
    return MFEM_ERR_INVALID;
  if (desc->formulation == MFEM_FORMULATION_STRETCH) {
    // the standard-FEM variable has no MINRES form, and only SNH and NH
    // define the 9-vector energy (the others print "unimplemented")
    if (desc->linear_solver == MFEM_SOLVER_MINRES_ID) return MFEM_ERR_UNSUPPORTED;
    if (desc->material)
      for (int e = 0; e < desc->n_tets; ++e)
        if (desc->material[e] != MFEM_MATERIAL_SNH && desc->material[e] != MFEM_MATERIAL_NH)
          return MFEM_ERR_UNSUPPORTED;
  }
  s->cfg = *desc;
  // pointers in the copied descriptor are not kept
  s->cfg.V_rest = s->cfg.V_init = s->cfg.v_init = nullptr;
  s->cfg.tets = s->cfg.material = s->cfg.is_fixed = nullptr;
  s->cfg.mu = s->cfg.lambda = s->cfg.density = nullptr;
  s->fp64 = desc->precision == MFEM_PRECISION_FP64 ? 1 : 0;
  s->rsz = s->fp64 ? 8 : 4;
  s->ntp = (int)align_up((size_t)s->M.nt, 32);
  static const double beta[7] = {0, 1.0, 2.0 / 3, 6.0 / 11, 12.0 / 25, 60.0 / 137, 60.0 / 147};
  s->h = desc->dt;
  s->dt = beta[desc->bdf_order] * desc->dt;
  s->h2 = s->dt * s->dt;
  s->nnzb = s->M.nnzb;
  s->pin_pos.resize(3 * (size_t)s->M.npin);
  for (int p = 0; p < s->M.npin; ++p)
    for (int k = 0; k < 3; ++k) s->pin_pos[3 * p + k] = s->M.V0[3 * s->M.pin_vert[p] + k];
  return MFEM_OK;
}

int mfem_gpu_scene_footprint(const mfem_scene_desc* desc, int64_t* bytes) {
  if (!bytes) return MFEM_ERR_INVALID;
  std::unique_ptr<mfem_scene> s;
  int rc = scene_prepare(desc, s);
  if (rc) return rc;
  size_t b = 0;
  scene_layout_bytes(s.get(), &b);
  // plus the single-scene batch (tile tables, partials)
  const size_t tiles = (size_t)(s->M.nt / kElemTile + 1) * 2 + s->M.nf / kRowTile + s->M.nf / kCgRows +
                       s->M.nv / kVertTile + 8;  // tile tables of the single-scene batch
  *bytes = (int64_t)(b + tiles * (sizeof(Tile) + kNumPartials * sizeof(double)) + 4096);
  return MFEM_OK;
}

int mfem_gpu_scene_create(const mfem_scene_desc* desc, mfem_scene** out) {
  if (!desc || !out) return MFEM_ERR_INVALID;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return MFEM_ERR_NO_DEVICE;
  std::call_once(g_configured, configure_kernels);
  std::unique_ptr<mfem_scene> s;
  int rc = scene_prepare(desc, s);
  if (rc) return rc;
  rc = scene_init_device(s.get());
  if (rc) {
    if (s->dmem) cudaFree(s->dmem);
    return rc;
  }
  mfem_scene* raw = s.get();
  rc = batch_build(&raw, 1, &s->solo);
  if (rc) {
    cudaFree(s->dmem);
    return rc;
  }
  // s0 = polar(F0), R0 (MixedStretch::reset)
  launch_elem_init(make_launch(s->solo, TB_ELEM));
  CUDA_OR(cudaStreamSynchronize(s->solo->stream), MFEM_ERR_CUDA);
  CUDA_OR(cudaGetLastError(), MFEM_ERR_CUDA);
  *out = s.release();
  return MFEM_OK;
}

int mfem_gpu_scene_destroy(mfem_scene* scene) {
  if (!scene) return MFEM_ERR_INVALID;
  batch_free(scene->solo);
  if (scene->dmem) cudaFree(scene->dmem);
  if (scene->ckpt) cudaFree(scene->ckpt);
  if (scene->d_pin_traj) cudaFree(scene->d_pin_traj);
  delete scene;
  return MFEM_OK;
}

int mfem_gpu_scene_step(mfem_scene* scene, mfem_step_stats* stats) {
  if (!scene) return MFEM_ERR_INVALID;
  mfem_step_stats st{};
  int rc = batch_step_impl(scene->solo, &st);
  if (stats) *stats = st;
  return rc;
}

int mfem_gpu_scene_sizes(const mfem_scene* scene, int32_t* nv, int32_t* nt, int32_t* nf) {
  if (!scene) return MFEM_ERR_INVALID;
  if (nv) *nv = scene->M.nv;
  if (nt) *nt = scene->M.nt;
  if (nf) *nf = scene->M.nf;
  return MFEM_OK;
}

int mfem_gpu_scene_get_state(mfem_scene* s, double* x, double* v, double* sv, double* R,
                             double* la) {
  if (!s) return MFEM_ERR_INVALID;
  cudaStream_t st = s->solo->stream;
  CUDA_OR(cudaStreamSynchronize(st), MFEM_ERR_CUDA);
  const HostMesh& M = s->M;
  int rc;
  if (x && (rc = get_ext(x, s->dev.x, 3 * (size_t)M.nv, s->fp64))) return rc;
  if (v) {
    SceneScalars sc;
    CUDA_OR(cudaMemcpy(&sc, s->d_sc, sizeof(sc), cudaMemcpyDeviceToHost), MFEM_ERR_CUDA);
    if ((rc = get_ext(v, byte_ptr(s->dev.vhist, 24 * (size_t)M.nv * sc.hist_head), 3 * (size_t)M.nv,
                      s->fp64)))
      return rc;
  }
  if (sv) {
    std::vector<double> t(6 * (size_t)s->ntp);
    if ((rc = get_ext(t.data(), s->dev.s, t.size(), s->fp64))) return rc;
    for (int e = 0; e < M.nt; ++e)
      for (int k = 0; k < 6; ++k) sv[6 * (size_t)e + k] = t[(size_t)k * s->ntp + e];
  }
  if (la) {
    if (s->fp64) download_soa<double>(s->dev.la, M.nt, s->ntp, 6, la, st);
    else download_soa<float>(s->dev.la, M.nt, s->ntp, 6, la, st);
  }
  if (R) {
    std::vector<double> q(4 * (size_t)M.nt);
    if (s->fp64) download_soa<double>(s->dev.quat, M.nt, s->ntp, 4, q.data(), st);
    else download_soa<float>(s->dev.quat, M.nt, s->ntp, 4, q.data(), st);
    for (int e = 0; e < M.nt; ++e) quat_to_rot_h(&q[4 * (size_t)e], &R[9 * (size_t)e]);
  }
  return MFEM_OK;
}

// ---- snapshots ----------------------------------------------------------
namespace {
struct SnapHeader {
  char magic[4];  // "MFSN"
  int32_t version, nv, nt, bdf_order, npin, reserved[2];
};
size_t snapshot_doubles(const mfem_scene* s) {
  const HostMesh& M = s->M;
  const size_t I = s->cfg.bdf_order;
  return 3 * (size_t)M.nv * (1 + 2 * I) + 10 * (size_t)M.nt + 3 * (size_t)M.npin;
}
int read_head(mfem_scene* s, int* head) {
  CUDA_OR(cudaMemcpy(head, reinterpret_cast<char*>(s->d_sc) + offsetof(SceneScalars, hist_head), sizeof(int),
                     cudaMemcpyDeviceToHost),
          MFEM_ERR_CUDA);
  return MFEM_OK;
}
int write_head(mfem_scene* s, int head) {
  CUDA_OR(cudaMemcpy(reinterpret_cast<char*>(s->d_sc) + offsetof(SceneScalars, hist_head), &head, sizeof(int),
                     cudaMemcpyHostToDevice),
          MFEM_ERR_CUDA);
  return MFEM_OK;
}
// byte sizes of the raw state buffers: x, one history slot, s, quat
void state_sizes(const mfem_scene* s, size_t* bx, size_t* bslot, size_t* bs, size_t* bq) {
  *bx = 24 * (size_t)s->M.nv;
  *bslot = 24 * (size_t)s->M.nv;
  *bs = 6 * (size_t)s->ntp * 8;
  *bq = 4 * (size_t)s->ntp * s->rsz;
}
}  // namespace

int mfem_gpu_scene_snapshot_bytes(mfem_scene* s, int64_t* bytes) {
  if (!s || !bytes) return MFEM_ERR_INVALID;
  *bytes = (int64_t)(sizeof(SnapHeader) + 8 * snapshot_doubles(s));
  return MFEM_OK;
}

// Positions, history and s are stored as the scene holds them (an FP64
// value, or a float pair in the mixed path: 8 bytes either way), so that a
// restore into a scene of the same precision is bitwise; a restore into the
// other precision converts them.  Quaternions are stored as doubles.
int mfem_gpu_scene_snapshot(mfem_scene* s, void* buf, int64_t bytes) {
  int64_t need = 0;
  if (!s || !buf || mfem_gpu_scene_snapshot_bytes(s, &need) || bytes < need) return MFEM_ERR_INVALID;
  CUDA_OR(cudaStreamSynchronize(s->solo->stream), MFEM_ERR_CUDA);
  const HostMesh& M = s->M;
  const int I = s->cfg.bdf_order;
  SnapHeader h{};
  std::memcpy(h.magic, "MFSN", 4);
  h.version = 1;
  h.nv = M.nv;
  h.nt = M.nt;
  h.bdf_order = I;
  h.npin = M.npin;
  h.reserved[0] = s->fp64;
  std::memcpy(buf, &h, sizeof(h));
  double* out = reinterpret_cast<double*>(static_cast<char*>(buf) + sizeof(h));
  int head = 0, rc;
  if ((rc = read_head(s, &head))) return rc;
  const size_t n3 = 3 * (size_t)M.nv;
  CUDA_OR(cudaMemcpy(out, s->dev.x, 8 * n3, cudaMemcpyDeviceToHost), MFEM_ERR_CUDA);
  out += n3;
  for (int i = 0; i < I; ++i, out += n3)
    CUDA_OR(cudaMemcpy(out, byte_ptr(s->dev.xhist, 8 * n3 * ((head + i) % I)), 8 * n3, cudaMemcpyDeviceToHost),
            MFEM_ERR_CUDA);
  for (int i = 0; i < I; ++i, out += n3)
    CUDA_OR(cudaMemcpy(out, byte_ptr(s->dev.vhist, 8 * n3 * ((head + i) % I)), 8 * n3, cudaMemcpyDeviceToHost),
            MFEM_ERR_CUDA);
  {
    std::vector<double> t(6 * (size_t)s->ntp);
    CUDA_OR(cudaMemcpy(t.data(), s->dev.s, 8 * t.size(), cudaMemcpyDeviceToHost), MFEM_ERR_CUDA);
    for (int e = 0; e < M.nt; ++e)
      for (int k = 0; k < 6; ++k) out[6 * (size_t)e + k] = t[(size_t)k * s->ntp + e];
    out += 6 * (size_t)M.nt;
  }
  if (s->fp64) download_soa<double>(s->dev.quat, M.nt, s->ntp, 4, out, s->solo->stream);
  else download_soa<float>(s->dev.quat, M.nt, s->ntp, 4, out, s->solo->stream);
  out += 4 * (size_t)M.nt;
  std::memcpy(out, s->pin_pos.data(), 8 * s->pin_pos.size());
  return MFEM_OK;
}

int mfem_gpu_scene_restore(mfem_scene* s, const void* buf, int64_t bytes) {
  int64_t need = 0;
  if (!s || !buf || mfem_gpu_scene_snapshot_bytes(s, &need) || bytes < need) return MFEM_ERR_INVALID;
  const HostMesh& M = s->M;
  const int I = s->cfg.bdf_order;
  SnapHeader h;
  std::memcpy(&h, buf, sizeof(h));
  if (std::memcmp(h.magic, "MFSN", 4) != 0 || h.version != 1 || h.nv != M.nv || h.nt != M.nt ||
      h.bdf_order != I || h.npin != M.npin || (h.reserved[0] != 0 && h.reserved[0] != 1))
    return MFEM_ERR_INVALID;
  CUDA_OR(cudaStreamSynchronize(s->solo->stream), MFEM_ERR_CUDA);
  const double* in = reinterpret_cast<const double*>(static_cast<const char*>(buf) + sizeof(h));
  const int src64 = h.reserved[0];
  // an array of stored values into the scene's representation
  auto put = [&](void* dst, const double* v, size_t n) -> int {
    if (src64 == s->fp64) {
      CUDA_OR(cudaMemcpy(dst, v, 8 * n, cudaMemcpyHostToDevice), MFEM_ERR_CUDA);
      return MFEM_OK;
    }
    std::vector<double> t(n);
    from_ext(v, n, src64, t.data());
    return put_ext(dst, t.data(), n, s->fp64);
  };
  const size_t n3 = 3 * (size_t)M.nv;
  int rc;
  if ((rc = put(s->dev.x, in, n3))) return rc;
  in += n3;
  for (int i = 0; i < I; ++i, in += n3)
    if ((rc = put(byte_ptr(s->dev.xhist, 8 * n3 * i), in, n3))) return rc;
  for (int i = 0; i < I; ++i, in += n3)
    if ((rc = put(byte_ptr(s->dev.vhist, 8 * n3 * i), in, n3))) return rc;
  if ((rc = write_head(s, 0))) return rc;
  {
    std::vector<double> t(6 * (size_t)s->ntp, 0.0);
    for (int e = 0; e < M.nt; ++e)
      for (int k = 0; k < 6; ++k) t[(size_t)k * s->ntp + e] = in[6 * (size_t)e + k];
    if ((rc = put(s->dev.s, t.data(), t.size()))) return rc;
    in += 6 * (size_t)M.nt;
  }
  if (s->fp64) upload_soa<double>(s->dev.quat, M.nt, s->ntp, 4, in, s->solo->stream);
  else upload_soa<float>(s->dev.quat, M.nt, s->ntp, 4, in, s->solo->stream);
  in += 4 * (size_t)M.nt;
  std::memcpy(s->pin_pos.data(), in, 8 * s->pin_pos.size());
  if (M.npin)
    CUDA_OR(cudaMemcpy(s->d_pin_pos, s->pin_pos.data(), 8 * s->pin_pos.size(), cudaMemcpyHostToDevice),
            MFEM_ERR_CUDA);
  s->pins_driven = false;
  CUDA_OR(cudaGetLastError(), MFEM_ERR_CUDA);
  return MFEM_OK;
}

int mfem_gpu_scene_checkpoint(mfem_scene* s) {
  if (!s) return MFEM_ERR_INVALID;
  size_t bx, bslot, bs, bq;
  state_sizes(s, &bx, &bslot, &bs, &bq);
  const size_t I = s->cfg.bdf_order;
  if (!s->ckpt) CUDA_OR(cudaMalloc(&s->ckpt, bx + 2 * I * bslot + bs + bq), MFEM_ERR_OOM);
  cudaStream_t st = s->solo->stream;
  CUDA_OR(cudaStreamSynchronize(st), MFEM_ERR_CUDA);
  int rc;
  if ((rc = read_head(s, &s->ckpt_head))) return rc;
  char* d = s->ckpt;
  CUDA_OR(cudaMemcpyAsync(d, s->dev.x, bx, cudaMemcpyDeviceToDevice, st), MFEM_ERR_CUDA);
  d += bx;
  CUDA_OR(cudaMemcpyAsync(d, s->dev.xhist, I * bslot, cudaMemcpyDeviceToDevice, st), MFEM_ERR_CUDA);
  d += I * bslot;
  CUDA_OR(cudaMemcpyAsync(d, s->dev.vhist, I * bslot, cudaMemcpyDeviceToDevice, st), MFEM_ERR_CUDA);
  d += I * bslot;
  CUDA_OR(cudaMemcpyAsync(d, s->dev.s, bs, cudaMemcpyDeviceToDevice, st), MFEM_ERR_CUDA);
  d += bs;
  CUDA_OR(cudaMemcpyAsync(d, s->dev.quat, bq, cudaMemcpyDeviceToDevice, st), MFEM_ERR_CUDA);
  CUDA_OR(cudaStreamSynchronize(st), MFEM_ERR_CUDA);
  s->ckpt_pins = s->pin_pos;
  return MFEM_OK;
}

int mfem_gpu_scene_rollback(mfem_scene* s) {
  if (!s || !s->ckpt) return MFEM_ERR_INVALID;
  size_t bx, bslot, bs, bq;
  state_sizes(s, &bx, &bslot, &bs, &bq);
  const size_t I = s->cfg.bdf_order;
  cudaStream_t st = s->solo->stream;
  // the scene's batches return only when their streams are idle; the copies
  // go on the scene's own stream (no device-wide wait: another thread may be
  // capturing a graph on its batch's stream meanwhile)
  CUDA_OR(cudaStreamSynchronize(st), MFEM_ERR_CUDA);
  const char* d = s->ckpt;
  CUDA_OR(cudaMemcpyAsync(s->dev.x, d, bx, cudaMemcpyDeviceToDevice, st), MFEM_ERR_CUDA);
  d += bx;
  CUDA_OR(cudaMemcpyAsync(s->dev.xhist, d, I * bslot, cudaMemcpyDeviceToDevice, st), MFEM_ERR_CUDA);
  d += I * bslot;
  CUDA_OR(cudaMemcpyAsync(s->dev.vhist, d, I * bslot, cudaMemcpyDeviceToDevice, st), MFEM_ERR_CUDA);
  d += I * bslot;
  CUDA_OR(cudaMemcpyAsync(s->dev.s, d, bs, cudaMemcpyDeviceToDevice, st), MFEM_ERR_CUDA);
  d += bs;
  CUDA_OR(cudaMemcpyAsync(s->dev.quat, d, bq, cudaMemcpyDeviceToDevice, st), MFEM_ERR_CUDA);
  CUDA_OR(cudaStreamSynchronize(st), MFEM_ERR_CUDA);
  int rc;
  if ((rc = write_head(s, s->ckpt_head))) return rc;
  s->pin_pos = s->ckpt_pins;
  if (s->M.npin)
    CUDA_OR(cudaMemcpy(s->d_pin_pos, s->pin_pos.data(), 8 * s->pin_pos.size(), cudaMemcpyHostToDevice),
            MFEM_ERR_CUDA);
  s->pins_driven = false;
  return MFEM_OK;
}

int mfem_gpu_scene_set_state(mfem_scene* s, const double* x, const double* v, const double* sv,
                             const double* R) {
  if (!s) return MFEM_ERR_INVALID;
  cudaStream_t st = s->solo->stream;
  const HostMesh& M = s->M;
  SceneScalars sc;
  CUDA_OR(cudaMemcpy(&sc, s->d_sc, sizeof(sc), cudaMemcpyDeviceToHost), MFEM_ERR_CUDA);
  int rc;
  if (x) {
    if ((rc = put_ext(s->dev.x, x, 3 * (size_t)M.nv, s->fp64))) return rc;
    if ((rc = put_ext(byte_ptr(s->dev.xhist, 24 * (size_t)M.nv * sc.hist_head), x, 3 * (size_t)M.nv,
                      s->fp64)))
      return rc;
    for (int p = 0; p < M.npin; ++p)
      for (int k = 0; k < 3; ++k) s->pin_pos[3 * p + k] = x[3 * M.pin_vert[p] + k];
    if (M.npin)
      CUDA_OR(cudaMemcpy(s->d_pin_pos, s->pin_pos.data(), sizeof(double) * s->pin_pos.size(),
                         cudaMemcpyHostToDevice),
              MFEM_ERR_CUDA);
  }
  if (v && (rc = put_ext(byte_ptr(s->dev.vhist, 24 * (size_t)M.nv * sc.hist_head), v, 3 * (size_t)M.nv,
                         s->fp64)))
    return rc;
  if (sv) {
    std::vector<double> t(6 * (size_t)s->ntp, 0.0);
    for (int e = 0; e < M.nt; ++e)
      for (int k = 0; k < 6; ++k) t[(size_t)k * s->ntp + e] = sv[6 * (size_t)e + k];
    if ((rc = put_ext(s->dev.s, t.data(), t.size(), s->fp64))) return rc;
  }
  if (R) {
    std::vector<double> q(4 * (size_t)M.nt);
    for (int e = 0; e < M.nt; ++e) rot_to_quat_h(&R[9 * (size_t)e], &q[4 * (size_t)e]);
    if (s->fp64) upload_soa<double>(s->dev.quat, M.nt, s->ntp, 4, q.data(), st);
    else upload_soa<float>(s->dev.quat, M.nt, s->ntp, 4, q.data(), st);
  }
  return MFEM_OK;
}

int mfem_gpu_scene_pinned(mfem_scene* s, int32_t* n_pinned, int32_t* vertices) {
  if (!s) return MFEM_ERR_INVALID;
  if (n_pinned) *n_pinned = s->M.npin;
  if (vertices) std::memcpy(vertices, s->M.pin_vert.data(), sizeof(int) * s->M.npin);
  return MFEM_OK;
}

int mfem_gpu_scene_set_pins(mfem_scene* s, const double* positions) {
  if (!s || (!positions && s->M.npin)) return MFEM_ERR_INVALID;
  if (s->M.npin == 0) return MFEM_OK;
  std::memcpy(s->pin_pos.data(), positions, sizeof(double) * 3 * s->M.npin);
  CUDA_OR(cudaMemcpyAsync(s->d_pin_pos, s->pin_pos.data(), sizeof(double) * 3 * s->M.npin,
                          cudaMemcpyHostToDevice, s->solo->stream),
          MFEM_ERR_CUDA);
  s->pins_driven = true;
  return MFEM_OK;
}

int mfem_gpu_scene_solo_batch(mfem_scene* s, mfem_batch** batch) {
  if (!s || !batch) return MFEM_ERR_INVALID;
  *batch = s->solo;
  return MFEM_OK;
}

int mfem_gpu_batch_set_profiling(mfem_batch* b, int enable) {
  if (!b) return MFEM_ERR_INVALID;
  b->profiling = enable != 0;
  for (int k = 0; k < MFEM_K_COUNT; ++k) {
    b->k_ms[k] = 0;
    b->k_launches[k] = 0;
  }
  return MFEM_OK;
}

int mfem_gpu_set_tuning(int32_t mode) {
  if (mode < -1 || mode > 2) return MFEM_ERR_INVALID;
  g_tune_override.store(mode);
  return MFEM_OK;
}

int mfem_gpu_batch_set_priority(mfem_batch* b, int32_t priority) {
  if (!b) return MFEM_ERR_INVALID;
  int least = 0, greatest = 0;  // CUDA: numerically lower is the higher priority
  CUDA_OR(cudaDeviceGetStreamPriorityRange(&least, &greatest), MFEM_ERR_CUDA);
  const int p = std::max(greatest, std::min(least, least - (int)priority));
  cudaStream_t st = nullptr;
  CUDA_OR(cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, p), MFEM_ERR_CUDA);
  CUDA_OR(cudaStreamSynchronize(b->stream), MFEM_ERR_CUDA);
  cudaStreamDestroy(b->stream);
  b->stream = st;
  return MFEM_OK;
}

int mfem_gpu_batch_set_pcg_shape(mfem_batch* b, int32_t stages, int32_t keep, int32_t unroll, int32_t pdl) {
  if (!b || stages < 0 || (stages > 4 && stages != 8) || stages == 1 || keep < 0 || keep > 1 || unroll < 1 ||
      (unroll != 1 && unroll != 2 && unroll != 4) || (unroll == 2 && stages != 4) || (unroll == 4 && stages != 8) ||
      (stages == 8 && unroll != 4) || pdl < 0 || pdl > 1 || (pdl && stages == 0))
    return MFEM_ERR_INVALID;
  if (b->fp64 && stages > 2) stages = 2;
  if (b->fp64) unroll = 1;
  const CgfShape sh{stages, keep, unroll, pdl};
  if (b->cgf_shape.stages == sh.stages && b->cgf_shape.keep == sh.keep && b->cgf_shape.unroll == sh.unroll &&
      b->cgf_shape.pdl == sh.pdl)
    return MFEM_OK;
  b->cgf_shape = sh;
  if (b->cg_graph || b->cg_loop || b->tick_graph || b->tick_graph_c) {  // captured with the old shape
    CUDA_OR(cudaStreamSynchronize(b->stream), MFEM_ERR_CUDA);
    if (b->cg_graph) cudaGraphExecDestroy(b->cg_graph);
    if (b->cg_loop) cudaGraphExecDestroy(b->cg_loop);
    if (b->tick_graph) cudaGraphExecDestroy(b->tick_graph);
    if (b->tick_graph_c) cudaGraphExecDestroy(b->tick_graph_c);
    b->cg_graph = nullptr;
    b->cg_loop = nullptr;
    b->tick_graph = nullptr;
    b->tick_graph_c = nullptr;
  }
  return MFEM_OK;
}

int mfem_gpu_batch_get_pcg_shape(mfem_batch* b, int32_t* stages, int32_t* keep, int32_t* unroll,
                                 int32_t* pdl) {
  if (!b) return MFEM_ERR_INVALID;
  if (stages) *stages = b->cgf_shape.stages;
  if (keep) *keep = b->cgf_shape.keep;
  if (unroll) *unroll = b->cgf_shape.unroll;
  if (pdl) *pdl = b->cgf_shape.pdl;
  return MFEM_OK;
}

int mfem_gpu_batch_set_variants(mfem_batch* b, int32_t elem_update, int32_t local_solve, int32_t ls_energy) {
  if (!b || elem_update < 0 || elem_update >= elem_update_variants(b->fp64, b->fem) || local_solve < 0 ||
      local_solve >= local_solve_variants(b->fp64) || ls_energy < 0 || ls_energy >= ls_energy_variants(b->fp64))
    return MFEM_ERR_INVALID;
  b->var_elem = elem_update;
  b->var_local = local_solve;
  b->var_ls = ls_energy;
  if (b->tick_graph) {  // captured with the old variants
    CUDA_OR(cudaStreamSynchronize(b->stream), MFEM_ERR_CUDA);
    cudaGraphExecDestroy(b->tick_graph);
    b->tick_graph = nullptr;
  }
  return MFEM_OK;
}

int mfem_gpu_batch_tune_report(mfem_batch* b, char* buf, int32_t len) {
  if (!b || !buf || len <= 0) return MFEM_ERR_INVALID;
  if ((int32_t)b->tune_report.size() + 1 > len) return MFEM_ERR_CAPACITY;
  std::memcpy(buf, b->tune_report.c_str(), b->tune_report.size() + 1);
  return MFEM_OK;
}

int mfem_gpu_batch_kernel_stats(mfem_batch* b, int kernel, double* total_ms, int64_t* launches) {
  if (!b || kernel < 0 || kernel >= MFEM_K_COUNT) return MFEM_ERR_INVALID;
  if (total_ms) *total_ms = b->k_ms[kernel];
  if (launches) *launches = b->k_launches[kernel];
  return MFEM_OK;
}

int mfem_gpu_kernel_name(int kernel, char* name, int name_len) {
  static const char* names[MFEM_K_COUNT] = {
      "k_elem_update", "k_assemble", "k_cg_init", "k_cg_spmv", "k_cg_update", "k_local_solve",
      "k_ls_energy", "k_apply", "k_step_begin", "k_step_end", "k_scalars_begin",
      "k_cg_solve", "k_cgf_iter", "k_cg_replace", "k_mr_init", "k_mr_elem", "k_mr_vert",
      "k_mr_update", "k_mr_export", "k_cg_loop"};
  if (kernel < 0 || kernel >= MFEM_K_COUNT || !name || name_len <= 0) return MFEM_ERR_INVALID;
  strncpy(name, names[kernel], name_len - 1);
  name[name_len - 1] = 0;
  return MFEM_OK;
}

int mfem_gpu_batch_create(mfem_scene* const* scenes, int32_t n, mfem_batch** out) {
  std::call_once(g_configured, configure_kernels);
  return batch_build(scenes, n, out);
}

int mfem_gpu_batch_destroy(mfem_batch* batch) {
  if (!batch) return MFEM_ERR_INVALID;
  batch_free(batch);
  return MFEM_OK;
}

int mfem_gpu_batch_step_n(mfem_batch* batch, int32_t steps, mfem_step_stats* stats, double* step_done_ms) {
  if (!batch || steps < 1 || steps > MFEM_BATCH_MAX_STEPS) return MFEM_ERR_INVALID;
  return batch_step_n_impl(batch, steps, stats, step_done_ms);
}

int mfem_gpu_batch_step(mfem_batch* batch, mfem_step_stats* stats) {
  if (!batch) return MFEM_ERR_INVALID;
  return batch_step_impl(batch, stats);
}

int mfem_gpu_batches_step_n(mfem_batch* const* batches, int32_t nbatch, int32_t steps, mfem_step_stats* stats,
                            double* step_done_ms) {
  if (!batches || nbatch < 1 || steps < 1 || steps > MFEM_BATCH_MAX_STEPS) return MFEM_ERR_INVALID;
  std::vector<size_t> first(nbatch + 1, 0);
  std::vector<const mfem_scene*> seen;
  for (int k = 0; k < nbatch; ++k) {
    if (!batches[k]) return MFEM_ERR_INVALID;
    for (int j = 0; j < k; ++j)
      if (batches[j] == batches[k]) return MFEM_ERR_INVALID;
    first[k + 1] = first[k] + batches[k]->scenes.size();
    seen.insert(seen.end(), batches[k]->scenes.begin(), batches[k]->scenes.end());
  }
  // a scene in two of the batches would be stepped by two threads at once
  std::sort(seen.begin(), seen.end());
  if (std::adjacent_find(seen.begin(), seen.end()) != seen.end()) return MFEM_ERR_INVALID;
  int dev = 0;
  CUDA_OR(cudaGetDevice(&dev), MFEM_ERR_CUDA);
  // one host thread per batch, each driving its batch's stream; the GPU
  // runs the batches' launches side by side
  std::vector<int> rc(nbatch, MFEM_OK);
  std::vector<std::thread> th;
  th.reserve(nbatch);
  for (int k = 0; k < nbatch; ++k)
    th.emplace_back([&, k]() {
      if (cudaSetDevice(dev) != cudaSuccess) {
        rc[k] = MFEM_ERR_CUDA;
        return;
      }
      rc[k] = batch_step_n_impl(batches[k], steps, stats ? stats + first[k] : nullptr,
                                step_done_ms ? step_done_ms + first[k] * (size_t)steps : nullptr);
    });
  for (std::thread& t : th) t.join();
  // the first failure of the call in batch order; a retired scene's
  // non-finite status as the single-batch call reports it
  for (int k = 0; k < nbatch; ++k)
    if (rc[k] != MFEM_OK && rc[k] != MFEM_ERR_NONFINITE) return rc[k];
  for (int k = 0; k < nbatch; ++k)
    if (rc[k] != MFEM_OK) return rc[k];
  return MFEM_OK;
}

int mfem_gpu_scene_elem_update(mfem_scene* s, const double* x, double h, double* R, double* S,
                               double* dSdF, double* g, double* H, double* Hinv, double* Aloc,
                               double* gl) {
  if (!s || !x) return MFEM_ERR_INVALID;
  mfem_batch* b = s->solo;
  const int nt = s->M.nt;
  int rc0 = put_ext(s->dev.x, x, 3 * (size_t)s->M.nv, s->fp64);
  if (rc0) return rc0;
  // run K1 with h^2 = h*h and FP64 debug outputs
  SceneDev D = b->h_sds[0];
  D.h2 = h * h;
  D.h2x = split_df(D.h2);
  CUDA_OR(cudaMemcpy(b->d_sds, &D, sizeof(D), cudaMemcpyHostToDevice), MFEM_ERR_CUDA);
  const size_t per = 9 + 6 + 54 + 6 + 36 + 36 + 144 + 6;
  double* dbuf = nullptr;
  CUDA_OR(cudaMalloc(&dbuf, sizeof(double) * per * nt), MFEM_ERR_OOM);
  ElemDebug dbg;
  double* p = dbuf;
  dbg.R = p; p += 9 * (size_t)nt;
  dbg.S = p; p += 6 * (size_t)nt;
  dbg.dSdF = p; p += 54 * (size_t)nt;
  dbg.g = p; p += 6 * (size_t)nt;
  dbg.H = p; p += 36 * (size_t)nt;
  dbg.Hinv = nullptr; p += 36 * (size_t)nt;
  dbg.Aloc = p; p += 144 * (size_t)nt;
  dbg.gl = p;
  launch_scalars_begin(make_launch(b, TB_EV), 1);
  launch_elem_update(make_launch(b, TB_ELEM), &dbg);
  cudaError_t e1 = cudaStreamSynchronize(b->stream);
  cudaError_t e2 = cudaGetLastError();
  std::vector<double> host(per * (size_t)nt);
  cudaMemcpy(host.data(), dbuf, sizeof(double) * host.size(), cudaMemcpyDeviceToHost);
  cudaFree(dbuf);
  cudaMemcpy(b->d_sds, &b->h_sds[0], sizeof(SceneDev), cudaMemcpyHostToDevice);
  if (e1 != cudaSuccess || e2 != cudaSuccess) {
    set_error("elem_update", e1 != cudaSuccess ? e1 : e2);
    return MFEM_ERR_CUDA;
  }
  const double* q = host.data();
  auto out = [&](double* dst, size_t n) {
    if (dst) std::memcpy(dst, q, sizeof(double) * n);
    q += n;
  };
  out(R, 9 * (size_t)nt);
  out(S, 6 * (size_t)nt);
  out(dSdF, 54 * (size_t)nt);
  out(g, 6 * (size_t)nt);
  const double* Hsrc = q;
  out(H, 36 * (size_t)nt);
  q += 36 * (size_t)nt;  // the Hinv slot is filled on the host below
  if (Hinv)
    for (int e = 0; e < nt; ++e) inverse6_host(Hsrc + 36 * (size_t)e, Hinv + 36 * (size_t)e);
  out(Aloc, 144 * (size_t)nt);
  out(gl, 6 * (size_t)nt);
  return MFEM_OK;
}

int mfem_gpu_scene_bcsr_sizes(mfem_scene* s, int32_t* nf, int32_t* nnzb) {
  if (!s) return MFEM_ERR_INVALID;
  if (nf) *nf = s->M.nf;
  if (nnzb) *nnzb = s->M.nnzb;
  return MFEM_OK;
}

// Real vector of the device (4 Real per free row, device row order) to
// FP64 in the reference's free order (3 per row, vertex order).
// The mixed path's df64 solution vector (4 float pairs per row, device row
// order) to FP64 in the reference's free order.
int fetch_rows_df64(const mfem_scene* s, const void* src, double* dst) {
  const HostMesh& M = s->M;
  const size_t n8 = 8 * (size_t)M.nf;
  std::vector<float> f(n8);
  CUDA_OR(cudaMemcpy(f.data(), src, n8 * 4, cudaMemcpyDeviceToHost), MFEM_ERR_CUDA);
  for (int r = 0; r < M.nf; ++r)
    for (int c = 0; c < 3; ++c)
      dst[3 * (size_t)M.ref_of_row[r] + c] = double(f[8 * (size_t)r + 2 * c]) + double(f[8 * (size_t)r + 2 * c + 1]);
  return MFEM_OK;
}

int fetch_rows(const mfem_scene* s, const void* src, double* dst) {
  const HostMesh& M = s->M;
  const size_t n4 = 4 * (size_t)M.nf;
  std::vector<double> t(n4);
  if (s->fp64) {
    CUDA_OR(cudaMemcpy(t.data(), src, n4 * 8, cudaMemcpyDeviceToHost), MFEM_ERR_CUDA);
  } else {
    std::vector<float> f(n4);
    CUDA_OR(cudaMemcpy(f.data(), src, n4 * 4, cudaMemcpyDeviceToHost), MFEM_ERR_CUDA);
    for (size_t i = 0; i < n4; ++i) t[i] = f[i];
  }
  for (int r = 0; r < M.nf; ++r)
    for (int c = 0; c < 3; ++c) dst[3 * (size_t)M.ref_of_row[r] + c] = t[4 * (size_t)r + c];
  return MFEM_OK;
}

int put_rows(const mfem_scene* s, const double* src, void* dst) {
  const HostMesh& M = s->M;
  const size_t n4 = 4 * (size_t)M.nf;
  std::vector<double> t(n4, 0.0);
  for (int r = 0; r < M.nf; ++r)
    for (int c = 0; c < 3; ++c) t[4 * (size_t)r + c] = src[3 * (size_t)M.ref_of_row[r] + c];
  if (s->fp64) {
    CUDA_OR(cudaMemcpy(dst, t.data(), n4 * 8, cudaMemcpyHostToDevice), MFEM_ERR_CUDA);
  } else {
    std::vector<float> f(t.begin(), t.end());
    CUDA_OR(cudaMemcpy(dst, f.data(), n4 * 4, cudaMemcpyHostToDevice), MFEM_ERR_CUDA);
  }
  return MFEM_OK;
}

// The assembled system as FP64 BCSR in the reference's free order: rows
// and columns by vertex order of the free vertices (the Assembler's sorted
// pairs), blocks row-major.
int system_to_host(const mfem_scene* s, int32_t* row_ptr, int32_t* col, double* val, double* rhs) {
  const HostMesh& M = s->M;
  std::vector<double> ell;
  if (val) {
    const size_t nw = 10 * M.ell_col.size();
    ell.resize(nw);
    if (s->fp64) {
      CUDA_OR(cudaMemcpy(ell.data(), s->dev.ell, nw * 8, cudaMemcpyDeviceToHost), MFEM_ERR_CUDA);
    } else {
      std::vector<float> f(nw);
      CUDA_OR(cudaMemcpy(f.data(), s->dev.ell, nw * 4, cudaMemcpyDeviceToHost), MFEM_ERR_CUDA);
      for (size_t i = 0; i < nw; ++i) ell[i] = f[i];
    }
  }
  int32_t pos = 0;
  if (row_ptr) row_ptr[0] = 0;
  std::vector<std::pair<int, int>> cols;  // (reference column, block k of the device row)
  for (int i = 0; i < M.nf; ++i) {
    const int r = M.row_of_ref[i];
    const int sl = r / 32, rs = r % 32, soff = M.slice_off[sl];
    const int rb = M.b_ptr[r], nb = M.b_ptr[r + 1] - rb;
    cols.clear();
    for (int k = 0; k < nb; ++k) cols.push_back({M.ref_of_row[M.b_col[rb + k]], k});
    std::sort(cols.begin(), cols.end());
    for (int j = 0; j < nb; ++j) {
      if (col) col[pos + j] = cols[j].first;
      if (val)
        for (int e = 0; e < 9; ++e) val[9 * (size_t)(pos + j) + e] = ell[ell_entry(soff, cols[j].second, rs, e)];
    }
    pos += nb;
    if (row_ptr) row_ptr[i + 1] = pos;
  }
  if (rhs) return fetch_rows(s, s->dev.rhs, rhs);
  return MFEM_OK;
}

// Assembles LHS and RHS at the current state (update_system + pre_solve).
int mfem_gpu_scene_get_system(mfem_scene* s, int32_t* row_ptr, int32_t* col, double* val,
                              double* rhs) {
  if (!s) return MFEM_ERR_INVALID;
  mfem_batch* b = s->solo;
  launch_scalars_begin(make_launch(b, TB_EV), 1);
  launch_step_begin(make_launch(b, TB_EV));
  launch_elem_update(make_launch(b, TB_ELEM), nullptr);
  launch_assemble(make_launch(b, TB_ROW));
  CUDA_OR(cudaStreamSynchronize(b->stream), MFEM_ERR_CUDA);
  CUDA_OR(cudaGetLastError(), MFEM_ERR_CUDA);
  return system_to_host(s, row_ptr, col, val, rhs);
}

int mfem_gpu_scene_pcg(mfem_scene* s, const double* bvec, double* dx, int32_t* iterations,
                       double* rel_residual) {
  if (!s || !bvec || !dx) return MFEM_ERR_INVALID;
  mfem_batch* b = s->solo;
  int rc = put_rows(s, bvec, s->dev.rhs);
  if (rc) return rc;
  launch_scalars_begin(make_launch(b, TB_EV), 1);
  if ((rc = run_pcg(b, make_launch(b, TB_CG)))) return rc;
  if ((rc = sync_counters(b))) return rc;
  if (b->h_ctr->error) return MFEM_ERR_TIMEOUT;
  CUDA_OR(cudaGetLastError(), MFEM_ERR_CUDA);
  // the mixed path keeps the solution in df64 (x_e); FP64: x itself
  if ((rc = s->dev.cg_xe ? fetch_rows_df64(s, s->dev.cg_xe, dx) : fetch_rows(s, s->dev.cg_x, dx))) return rc;
  SceneScalars sc;
  CUDA_OR(cudaMemcpy(&sc, s->d_sc, sizeof(sc), cudaMemcpyDeviceToHost), MFEM_ERR_CUDA);
  if (iterations) *iterations = sc.cg_total;
  if (rel_residual) *rel_residual = sc.cg_err;
  return sc.cg_status;
}

}  // extern "C"
