// Device-side layout of a scene and of a batch of scenes, and the launch
// wrappers of every kernel of the Newton timestep.
//
// A batch concatenates any number of independent scenes.  Each kernel runs
// over a tile table; a tile covers a contiguous range of ONE scene's elements,
// rows or vertices, so per-scene reductions are tile partials summed in a
// fixed order by the last tile of that scene to finish (deterministic, and
// identical whether the scene runs alone or in a batch).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace mfem_gpu {

// Tile tables of a batch.
enum TableKind {
  TB_ELEM = 0,  // element tiles (kElemTile elements)               : K1
  TB_ROW = 1,   // free-row tiles, one warp per row (kRowTile rows)  : assembly
  TB_CG = 2,    // free-row tiles for PCG (kCgRows rows)              : PCG
  TB_EV = 3,    // element tiles then vertex tiles of each scene      : local solve,
                //                                                      line search, apply
  TB_COUNT = 4
};

constexpr int kElemTile = 128;   // elements per element tile (one thread each)
constexpr int kVertTile = 128;   // vertices per vertex tile (TB_EV: same block size)
constexpr int kRowTile = 32;     // rows per assembly tile (8 warps, 4 rows each)
constexpr int kCgThreads = 256;  // threads per PCG tile
constexpr int kCgRows = 256;     // rows per PCG tile
constexpr int kTicketGroup = 32; // tiles per first-level ticket counter
// Mixed path: every kCgReplace PCG iterations the recursive residual is
// replaced by b - A x computed with x in df64 and exact products (reliable
// updates), so FP32 rounding does not leave the true residual far above the
// tolerance the recursion reports.
constexpr int kCgReplace = 25;
// Packed sliced-ELL addressing (see SceneDev::ell): the Real index of
// entry e (row-major 3x3) of block k of the row in lane rs of the slice at
// slot offset soff.
__host__ __device__ constexpr size_t ell_pair(int soff, int k, int rs, int w) {
  return 5 * (size_t)(soff + 32 * k) + 32 * (size_t)w + (size_t)rs;
}
__host__ __device__ constexpr size_t ell_entry(int soff, int k, int rs, int e) {
  return 2 * ell_pair(soff, k, rs, (e + 1) >> 1) + (size_t)((e + 1) & 1);
}

// Per-element record written by K1 and gathered by the assembly: the 78
// upper-triangle entries of the 12x12 element block (Real) followed, at a
// 16-byte boundary, by the element's 12 right-hand-side shares (double).
__host__ __device__ constexpr int rec_rhs_offset(int real_bytes) { return real_bytes == 4 ? 320 : 624; }
__host__ __device__ constexpr int rec_bytes(int real_bytes) { return rec_rhs_offset(real_bytes) + 96; }
constexpr int kMaxRowBlocks = 126;  // 7-bit column slots in the incidence code
constexpr int kNumPartials = 8;  // partial quantities per tile

struct Tile {
  int scene;  // slot in the batch
  int kind;   // 0 element range, 1 vertex range (TB_EV); row range otherwise
  int begin;
  int end;
};

// Per-scene scalars: the state machine of the Newton iteration, the PCG and
// the line search, kept on the device so no step needs a host round trip
// to decide what the next kernel does.
struct SceneScalars {
  // Newton (NewtonOptimizer::step, newton_optimizer.cpp:11-89)
  int newton_active;
  int newton_iter;
  int converged_by_residual;
  int status;
  double rhs_norm0, rhs_norm;
  double E, E_prev, eres, decrement;
  // PCG (Eigen ConjugateGradient semantics)
  int cg_active, cg_iter, cg_total, cg_status;
  double cg_rhs_norm2, cg_threshold, rz, alpha, beta, cg_err;
  double rz_prev;    // rz of the previous iteration (residual replacement)
  // single-reduction PCG: (r, u) and alpha of iteration i in slot i & 1
  // (kernel i reads slot (i+1) & 1 and its first block writes slot i & 1)
  double cgf_gamma[2], cgf_alpha[2];
  // mixed path: verification phase of the single-reduction PCG (0: iterate;
  // 1: r = b - A (x_e + x) exactly; 2: fold x into x_e, w = A u and the
  // inner products of the true residual; 3: write the rounded solution)
  int cgf_phase, cgf_rounds;  // verifications that failed in this solve
  // mixed path: the single-reduction PCG solves for 2^cg_scale_exp b (a
  // power of two from max |b_i|, so that the float-float inner products of
  // tiny or huge right-hand sides stay inside FP32's exponent range); the
  // solution is scaled back when it is written
  int cg_scale_exp, cg_pad;
  // line search (linesearch.h:80-129 with c = 0, p = 0.5)
  int ls_active, ls_iter, ls_ok, ls_total;
  double fx0, alpha_ls, E_trial;
  double E_abs;      // sum of |element energy terms| at alpha = 0 (rounding bound)
  double max_ds, max_dx;
  // BDF ring head
  int hist_head;
  int procrustes_fail;
  // last-tile counters, one per table
  unsigned int ctr[TB_COUNT];
  // float copies of the step lengths every thread reads (the mixed path
  // converts nothing per thread); alpha_ls is a power of two, exact in float
  float alpha_f, beta_f, alpha_ls_f, pad_f;
  // MINRES (cg_active / cg_iter / cg_total / cg_status / cg_err shared with
  // the PCG): Lanczos beta, Givens state, the pending p / x update of
  // iteration mr_slot (r1, r2, r3 and coef = beta_one c eta), and the
  // recursive squared residual estimate against its threshold
  double mr_beta, mr_beta_one, mr_alpha, mr_c, mr_c_old, mr_s, mr_s_old, mr_eta;
  double mr_r1, mr_r2, mr_r3, mr_coef, mr_resid2, mr_thr2;
  int mr_pending, mr_slot;
  // several timesteps in one call (mfem_gpu_batch_step_n): the scene's own
  // count of steps (0: one step, the plain form), the steps it finished, a
  // flag raised by the Newton loop's end until the step is turned over, and
  // the statistics of its finished steps
  int steps_target, steps_done, turn;
  int acc_newton, acc_cg, acc_ls, acc_status;
  // the ticked multi-step form: every kernel acts only on the scenes in its
  // phase of the Newton iteration (nph, kPh* in reduce.cuh), so that a scene
  // never waits for another scene's PCG or line search
  int ticked, nph;
};

// Counters of a batch: scenes still active in each loop.
struct BatchCounters {
  int newton_active;
  int cg_active;
  int ls_active;
  int error;                // a bounded wait of the persistent PCG ran out
  unsigned int bar_count;   // grid barrier of the persistent PCG: arrivals
  unsigned int bar_gen;     //   and generation
  int cg_bodies;            // bodies of the device-driven PCG loop run in this solve
  int pad;
};

// One scene as the kernels see it (pointers into the scene's arena).
struct SceneDev {
  int nv, nt, nf, nnzb;
  int ntp;           // element SoA stride (nt rounded up)
  int npin;
  int material_uniform;  // material id when uniform, -1 when per element
  int block_jacobi;  // 0: Jacobi (eigen-pcg-diag), 1: 3x3 block Jacobi
  int fp64;          // 1: all-FP64 path, 0: FP32 element work
  int fem;           // 1: the standard-FEM "stretch" variable, 0: mixed stretch
  // parameters
  double h2;         // (beta*h)^2
  double dt;         // beta*h
  float2 h2x;        // h2 as a float pair (df64), and float(h2) in .x
  double newton_tol, res_tol, cg_tol;
  double load_norm;  // |h^2 P M f| over the free dofs (scale of the residual test)
  int max_newton, max_ls, max_cg, bdf_order;
  double bdf_alpha[6];
  double body[3];    // body force (float-rounded, as SimConfig::ext is float)
  // geometry
  const int4* tets;
  const void* dphi;  // 9 x ntp Real: [(3*(k-1)+c)*ntp + e] = dphi_k/dX_c, k = 1..3
  const void* vol;   // ntp Real
  const void* mu;
  const void* lam;
  const int8_t* mat; // ntp or null
  // element state (Real SoA, stride ntp)
  void* quat;        // 4 x ntp
  void* s;           // 6 x ntp  mixed stretch variable (Ext: float pairs / double)
  void* la;          // 6 x ntp
  void* dS;          // 6 x ntp  S(x) - s of the current x (K1 output)
  void* ds;          // 6 x ntp
  unsigned char* rec;  // nt x rec_bytes  (AoS element records)
  // vertices (Ext: float pairs in the mixed path, double in the FP64 path)
  void* x;           // 3 nv current positions; pinned entries hold b
  void* xt;          // 3 nv  x_tilde + h^2 f_ext (the inertial target)
  void* xhist;       // bdf_order x 3 nv ring
  void* vhist;       // bdf_order x 3 nv ring
  const int* free_map;   // nv: free index, or -1-pin_index when pinned
  const int* free_vert;  // nf
  const int* pin_vert;   // npin
  const double* pin_pos; // 3 npin  pinned positions after the next BC step
  const int* m_ptr;  // nv+1 scalar mass CSR over all vertices
  const int* m_col;
  const void* m_val;   // Real
  // Block pattern over free vertices (sorted columns per row, the BCSR of
  // the Assembler) and the sliced-ELL layout the values are stored in.
  // Free rows are numbered so that within each window of kCgRows rows they
  // run by decreasing block count (SELL-C-sigma with C = 32, sigma =
  // kCgRows), which leaves slices of 32 rows almost without padding.  Block
  // k of row r of slice s is slot slice_off[s] + 32 k + (r mod 32); a slot
  // is 10 Real words packed as 5 pairs (col, a00) (a01, a02) (a10, a11)
  // (a12, a20) (a21, a22), pair w of slot (s, k, r) at pair index
  // 5 (slice_off[s] + 32 k) + 32 w + (r mod 32): a warp loads pair w of
  // block k of 32 rows as one coalesced access, and the column arrives with
  // the first pair.  Blocks k >= the row's length are zero and point at the
  // row itself.
  const int* b_ptr;  // nf+1
  const int* b_col;  // nnzb
  const void* b_mass;  // nnzb Real: free-free mass m_ab
  const int* slice_off;  // nslices+1 (in blocks)
  void* ell;             // 10 * slice_off[nslices] Real
  void* dinv;        // 9 nf Real (block) or 4 nf (Jacobi, padded like the vectors)
  const int* inc_ptr;  // nf+1 incidences (element, local vertex) per free row
  const int2* inc;     // (element, code): code = i | slot_j << (2+7j), slot 127 = pinned
  // PCG vectors (Real, 4 nf: x, y, z of a row and a zero pad, so that a
  // row is one 16-byte (FP32) or two 16-byte (FP64) accesses)
  void* rhs;
  void* cg_x;
  void* cg_xe;       // mixed path: the PCG's x in df64 (4 float pairs per row)
  void* cg_r;
  void* cg_z;
  void* cg_p[2];
  void* cg_Ap;
  // single-reduction PCG (Chronopoulos-Gear): r, w = A u and s by
  // iteration parity (scaled by the Jacobi M^-1 when every scene of the
  // batch uses it); x, p (= cg_p[0]) and, unscaled, u (= cg_z) single
  void* cgf_r[2];
  void* cgf_w[2];
  void* cgf_s[2];
  // "minres-indefinite-block" (null unless the scene uses it): per element
  // ds/dx (72: [12 i + 3 a + l] = d s_i / d x_{a,l}) and the upper triangle
  // of h^2 hess psi (21) from K1, Real SoA; eight FP64 (x, s, lambda)
  // vectors of mr_len doubles (v, vn, wn, w, p0..p2, x); the x-row shares
  // of each element (12 x ntp); the preconditioner blocks (vol H)^-1 and
  // S_ee^-1 (21 x ntp each) and the inverse lumped free mass (nf).
  int minres;
  void* mr_B;
  void* mr_H;
  double* mr_vec;
  size_t mr_len;
  double* mr_y;
  double* mr_hinv;
  double* mr_sinv;
  double* mr_mlinv;
  // tiles of this scene in each table
  int tile_first[TB_COUNT];
  int tile_count[TB_COUNT];
  // mfem_gpu_batch_step_n: pinned positions after each of the call's BC
  // steps (3 npin per step; null when the pins do not move) and, per step,
  // the Newton round of the call in which the scene finished it
  const double* pin_traj;
  unsigned long long* step_ns;  // global-timer ns at which each step was done
  int gmax;                // ticket groups per table (capacity of gctr rows)
  unsigned int* gctr;      // TB_COUNT x gmax first-level ticket counters
  SceneScalars* sc;
};

// Optional FP64 per-element outputs of K1 (parity entry point only).
struct ElemDebug {
  double* R;     // 9 per tet
  double* S;     // 6
  double* dSdF;  // 54 (9x6 column-major)
  double* g;     // 6
  double* H;     // 36
  double* Hinv;  // 36
  double* Aloc;  // 144 (12x12 column-major)
  double* gl;    // 6
};

struct Launch {
  cudaStream_t stream;
  const Tile* tiles;
  int ntiles;
  const SceneDev* sds;
  double* partials;   // kNumPartials x pstride (quantity-major)
  int pstride;
  BatchCounters* counters;
  int fp64;
  int fem;     // the batch's scenes use the standard-FEM variable
  int jacobi;  // no scene of the batch uses the 3x3 block-Jacobi preconditioner
  int variant = 0;  // kernel variant chosen by the autotuner (same bits in each)
};

// Element kernels (k_elem.cu)
void launch_elem_init(const Launch& L);                        // s0 = polar(F0), R
void launch_elem_update(const Launch& L, const ElemDebug* dbg); // K1
void launch_local_solve(const Launch& L);                      // K5 + E(0)   (TB_EV)
void launch_ls_energy(const Launch& L);                        // K6          (TB_EV)
void launch_apply(const Launch& L);                            // x,s update  (TB_EV)
void launch_step_begin(const Launch& L);                       // x_tilde     (TB_EV)
void launch_step_end(const Launch& L);                         // BDF, la = 0 (TB_EV)
// Several timesteps in one call: the turnover of every scene whose Newton
// loop has ended (step end, and the next step's begin unless it was its
// last), recording the time the step was done (TB_EV).
void launch_step_turn(const Launch& L);
// Row kernels (k_rows.cu)
void launch_assemble(const Launch& L);  // K2 + K3 (TB_ROW)
void launch_cg_init(const Launch& L);   // r = b, z, rz  (TB_CG)
void launch_cg_spmv(const Launch& L);   // Ap, pAp, alpha (TB_CG)
void launch_cg_update(const Launch& L); // x, r, z, beta  (TB_CG)
void launch_scalars_begin(const Launch& L, int nscenes);        // reset Newton state
// The same for a call of `steps` timesteps per scene (steps_target);
// ticked: every kernel gated by the scene's phase.
void launch_scalars_begin_n(const Launch& L, int nscenes, int steps, int ticked);
// The device's global timer (ns) into *ns.
void launch_stamp(unsigned long long* ns, cudaStream_t st);
// The whole PCG in one cooperative launch of `grid` co-resident blocks.
cudaError_t launch_cg_solve(const Launch& L, int grid, int max_iters);
void launch_cg_replace(const Launch& L);  // r = b - A x in df64 (mixed path)
// Single-reduction PCG: init (r0, u0, w0 = A u0) and one launch per iteration.
// The iteration's shape: stages = 0 streams the matrix through registers;
// stages = 2..4 (or 8) stages each warp's ELL slots through a ring of that many
// shared-memory buffers filled by bulk copies (the FP64 path uses 2);
// keep = 1 marks half of the matrix lines evict-last in L2 (0: all
// evict-first); unroll = 2 puts two slots' gathers in flight together
// (four stages, four resident blocks of 64 registers; FP32 only), unroll =
// 4 four (eight stages, two resident blocks).  Every shape computes the
// same bits.
struct CgfShape {
  int stages;
  int keep;
  int unroll;
  int pdl;  // 1 (staged shapes): each iteration a programmatic dependent
            // launch of the previous one, its prologue (barriers, the first
            // slots' copies) overlapping the previous iteration's tail
};
void launch_cgf_init(const Launch& L);
// Mixed path, before launch_cgf_init: the power-of-two scale of b.
void launch_cgf_scale(const Launch& L);
void launch_cgf_iter(const Launch& L, const CgfShape& sh);
// The condition of the device-driven PCG loop (a WHILE node of a CUDA
// graph whose body is a chunk of iterations): another body while a scene of
// the batch is still iterating, no wait has run out and fewer than
// max_bodies bodies have run (counted in ctrs->cg_bodies).
void launch_cg_continue(const Launch& L, cudaGraphConditionalHandle h, int max_bodies);
// The loop's entry: its condition from the batch's counters, before the
// first body.
void launch_cg_enter(const Launch& L, cudaGraphConditionalHandle h);
int cg_solve_blocks_per_sm(int fp64);
// Two-block cooperative launch whose grid barrier has a missing arrival.
cudaError_t launch_barrier_selftest(BatchCounters* ctrs, cudaStream_t st);
// MINRES on the (x, s, lambda) system (k_minres.cu, all TB_EV)
void launch_mr_init(const Launch& L);    // rhs, preconditioner blocks, v1, w1
void launch_mr_elem(const Launch& L);    // A1: pending update, element rows of K w
void launch_mr_vert(const Launch& L);    // A2: vertex rows of K w, alpha
void launch_mr_update(const Launch& L);  // B: vn, wn = P vn, Givens, convergence
void launch_mr_export(const Launch& L);  // dx -> the PCG solution vector

// Register-budget variants of the element kernels the autotuner may pick
// (Launch::variant, 0 the default); each computes the default's bits.
int elem_update_variants(int fp64, int fem);
int local_solve_variants(int fp64);
int ls_energy_variants(int fp64);
const char* elem_update_variant_name(int v);
const char* local_solve_variant_name(int v);
const char* ls_energy_variant_name(int v);

// Maximum dynamic shared memory the element kernels need.
int elem_update_smem_bytes(int fp64);
void configure_kernels();

}  // namespace mfem_gpu
