/*
 * mfem_gb300 — C ABI of the GB300 mixed-FEM Newton timestep.
 *
 * The library owns every device allocation it makes; host buffers passed in
 * are caller-owned and copied.  Every entry point returns an int status
 * (MFEM_OK = 0).  Calls on distinct scenes/batches are thread-safe; calls on
 * one object are not re-entrant (the reference optimizer is not either).
 *
 * The entry points replace these reference interfaces (tytrusty/mfem):
 *   scene create/destroy  <- SimState<3>::load(json)  src/simulation_state.cpp:92-341
 *                            + NewtonOptimizer<3>::reset()  src/optimizers/newton_optimizer.cpp:127-140
 *   scene step            <- NewtonOptimizer<3>::step()  src/optimizers/newton_optimizer.cpp:11-89
 *   batch step            <- (no counterpart: many independent NewtonOptimizer::step calls)
 *   get/set state         <- Displacement::value(), MixedStretch::value()
 *                            src/variables/displacement.h:93-95, mixed_stretch.h:47-49
 *   elem_update           <- MixedStretch::update_rotations + update_derivatives
 *                            src/variables/mixed_stretch.cpp:133-204
 *   assemble              <- Assembler<double,3,-1>::update_matrix  src/utils/sparse_utils.cpp:141-203
 *   pcg solve             <- EigenIterativeSolver<ConjugateGradient<..,Lower|Upper>> ("eigen-pcg-diag")
 *                            src/linear_solvers/eigen_iterative_solver.h:20-29
 */
#ifndef MFEM_GB300_H
#define MFEM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MFEM_ABI_VERSION 1

/* ---- status codes ---------------------------------------------------- */
enum {
  MFEM_OK = 0,
  MFEM_ERR_INVALID = 1,      /* bad argument or descriptor                    */
  MFEM_ERR_OOM = 2,          /* device allocation failed                      */
  MFEM_ERR_CUDA = 3,         /* CUDA runtime error                            */
  MFEM_ERR_NONFINITE = 4,    /* NaN/Inf in the state or a reduction           */
  MFEM_ERR_CG_MAXITER = 5,   /* PCG stopped at max_iterative_solver_iters     */
  MFEM_ERR_LS_FAILED = 6,    /* line search hit max_linesearch_iterations     */
  MFEM_ERR_PROCRUSTES = 7,   /* singular rotation Hessian (reference exit(1)) */
  MFEM_ERR_TIMEOUT = 8,      /* a bounded device wait ran out                 */
  MFEM_ERR_NO_DEVICE = 9,    /* no CUDA device visible                        */
  MFEM_ERR_UNSUPPORTED = 10, /* option not implemented on this path           */
  MFEM_ERR_CAPACITY = 11     /* request exceeds a fixed capacity              */
};

/* ---- material models: MaterialModelType, src/config.h:61-68 ----------- */
enum {
  MFEM_MATERIAL_SNH = 0,   /* "Stable-Neohookean" */
  MFEM_MATERIAL_NH = 1,    /* "Neohookean"        */
  MFEM_MATERIAL_COROT = 2, /* "Corot"             */
  MFEM_MATERIAL_FCR = 3,   /* "FixedCorot"        */
  MFEM_MATERIAL_ARAP = 4,  /* "ARAP"              */
  MFEM_MATERIAL_FUNG = 5   /* "Fung"              */
};

/* ---- linear solvers: LinearSolverType, src/config.h:45-59 -------------- */
enum {
  MFEM_SOLVER_EIGEN_LLT = 0,       /* direct: oracle only                */
  MFEM_SOLVER_EIGEN_CG_DIAG = 5,   /* "eigen-pcg-diag" -> GPU Jacobi PCG  */
  MFEM_SOLVER_MINRES_ID = 8,       /* "minres-indefinite-block"          */
  MFEM_SOLVER_GPU_PCG_BLOCK = 100  /* "gpu-pcg-block": 3x3 block-Jacobi  */
};

/* ---- scripted boundary conditions: BCScriptType, src/config.h:70-87 ---- */
enum {
  MFEM_BC_NULL = 0, MFEM_BC_SCALEF = 1, MFEM_BC_HANG = 2, MFEM_BC_HANGENDS = 3,
  MFEM_BC_STRETCH = 4, MFEM_BC_BEND = 7, MFEM_BC_TWIST = 8,
  MFEM_BC_ONEPOINT = 13, MFEM_BC_RANDOM = 14,
  /* additions (no reference counterpart) */
  MFEM_BC_PINMIN = 16,   /* "pinmin": min-side group pinned, static            */
  MFEM_BC_COMPRESS = 17  /* "compress": min side pinned, max side moves along
                            the axis at `velocity` (m/s)                         */
};

enum { MFEM_PRECISION_FP64 = 0, MFEM_PRECISION_MIXED = 1 };

/* ---- the elastic variable: "mixed_variables": ["mixed-stretch"]
 * (MixedStretch, src/variables/mixed_stretch.cpp) or "variables":
 * ["stretch"] (standard FEM, Stretch, src/variables/stretch.cpp; materials
 * with a 9-vector energy only: Stable-Neohookean, Neohookean) ------------ */
enum { MFEM_FORMULATION_MIXED_STRETCH = 0, MFEM_FORMULATION_STRETCH = 1 };

/* How the PCG runs.  PERSISTENT: one cooperative (co-resident,
 * grid-synchronised) launch per solve; SPLIT: two launches per iteration
 * with a host check for convergence every few iterations (same arithmetic
 * and bitwise the same results as PERSISTENT: Eigen's PCG iteration).
 * FUSED: the single-reduction form of the same PCG (Chronopoulos and Gear,
 * 1989), one launch per iteration; equal to the others in exact arithmetic,
 * not bitwise.  AUTO: the batch picks FUSED when its PCG tiles (256 rows
 * each) fill at least two per SM or fit in a few blocks, SPLIT in between,
 * where the system sits in L2 and FUSED's extra gathers per neighbour set
 * the pace (a 30^3 cube: 117 tiles, SPLIT 20% faster; a 60^3 cube: 873
 * tiles, FUSED faster; a 200-tet beam: one tile, FUSED's single launch per
 * iteration faster). */
enum { MFEM_PCG_KERNEL_PERSISTENT = 0, MFEM_PCG_KERNEL_SPLIT = 1, MFEM_PCG_KERNEL_FUSED = 2,
       MFEM_PCG_KERNEL_AUTO = 3 };

/* Scene descriptor.  One tetrahedral object (or several concatenated by the
 * caller, as Meshes does in src/mesh/meshes.cpp:11-56).  Arrays are
 * row-major: vertex i at [3*i .. 3*i+2], tet e at [4*e .. 4*e+3].         */
typedef struct mfem_scene_desc {
  int32_t n_vertices;
  int32_t n_tets;
  const double*  V_rest;       /* 3*n_vertices  rest positions (Vref_)           */
  const double*  V_init;       /* 3*n_vertices  initial positions (NULL = rest)  */
  const double*  v_init;       /* 3*n_vertices  initial velocities (NULL = 0)    */
  const int32_t* tets;         /* 4*n_tets                                       */
  const double*  mu;           /* n_tets  Lame mu per tet                        */
  const double*  lambda;       /* n_tets  Lame lambda per tet                    */
  const int32_t* material;     /* n_tets  MFEM_MATERIAL_* (NULL = all SNH)       */
  const double*  density;      /* n_tets  mass density (NULL = density_const)    */
  double         density_const;
  const int32_t* is_fixed;     /* n_vertices 0/1 override (NULL = from BC script) */
  int32_t bc_type;             /* MFEM_BC_*                                       */
  int32_t bc_axis;
  double  bc_ratio;
  double  bc_velocity;
  double  dt;                  /* SimConfig::h                                    */
  double  body_force[3];       /* SimConfig::ext (acceleration)                   */
  int32_t bdf_order;           /* 1..6                                            */
  int32_t max_newton_iterations;      /* SimConfig::outer_steps                   */
  int32_t max_linesearch_iterations;  /* SimConfig::ls_iters                      */
  int32_t max_iterative_solver_iters; /* SimConfig::max_iterative_solver_iters    */
  double  iterative_solver_tolerance; /* SimConfig::itr_tol                       */
  double  newton_tol;                 /* SimConfig::newton_tol (max |delta|_inf)  */
  double  newton_residual_tolerance;  /* >0: also stop when |rhs_k| <= it times
                                         max(|rhs_0|, |h^2 P M f|)             */
  int32_t linear_solver;              /* MFEM_SOLVER_*                            */
  int32_t precision;                  /* MFEM_PRECISION_*                         */
  int32_t pcg_kernel;                 /* MFEM_PCG_KERNEL_* (a batch uses the first
                                         scene's choice)                         */
  int32_t formulation;                /* MFEM_FORMULATION_*                       */
  int32_t reserved[6];
} mfem_scene_desc;

/* Per-step statistics (the reference prints these as its per-iteration
 * table, src/optimizers/optimizer_data.cpp:28-123).                        */
typedef struct mfem_step_stats {
  int32_t status;              /* worst status seen during the step            */
  int32_t newton_iterations;
  int32_t cg_iterations;       /* summed over Newton iterations                */
  int32_t ls_iterations;       /* summed backtracking halvings                 */
  double  energy;              /* energy_func(0) of the last Newton iteration  */
  double  energy_residual;     /* |E - E_prev| / (E + 1e-6)                    */
  double  decrement;           /* max(|dx|_inf, |ds|_inf) of the last solve    */
  double  alpha;               /* last accepted line-search step               */
  double  residual0;           /* |rhs| at the first Newton iteration          */
  double  residual;            /* |rhs| at the last evaluated iterate          */
  double  cg_error;            /* |r|/|b| at the end of the last PCG solve     */
  double  device_ms;           /* device time of the step (CUDA events)        */
} mfem_step_stats;

typedef struct mfem_scene mfem_scene;   /* one resident simulation instance */
typedef struct mfem_batch mfem_batch;   /* a set of scenes stepped together */

/* ---- library ------------------------------------------------------------ */
int mfem_gpu_abi_version(void);
/* Makes `device` current for the calling thread (one process per GPU). */
int mfem_gpu_set_device(int device);
/* Writes the device name and SM count; fails with MFEM_ERR_NO_DEVICE. */
int mfem_gpu_device_info(char* name, int name_len, int* sm_count);
/* Failure-detection self-test of the bounded device wait the persistent PCG
 * uses between its phases: a two-block cooperative launch whose grid
 * barrier misses one arrival.  The wait runs out after its limit (2 s),
 * the kernel returns, and the call reports MFEM_ERR_TIMEOUT (the status a
 * step returns in that case) with the time waited; the context stays usable. */
int mfem_gpu_selftest_bounded_wait(double* waited_ms);
const char* mfem_gpu_status_string(int status);

/* ---- scenes ---------------------------------------------------------------
 * mfem_gpu_scene_create replaces SimState<3>::load + NewtonOptimizer::reset
 * (src/simulation_state.cpp:92-341, src/optimizers/newton_optimizer.cpp:127-140):
 * builds the mesh quantities (Mesh::init, src/mesh/mesh.cpp:124-159), the
 * BDF history, s0 = polar(F0) and lambda = 0 (mixed_stretch.cpp:261-304), and
 * uploads everything once; state stays resident until destroy.           */
int mfem_gpu_scene_create(const mfem_scene_desc* desc, mfem_scene** out);
int mfem_gpu_scene_destroy(mfem_scene* scene);
/* One timestep: NewtonOptimizer<3>::step, src/optimizers/newton_optimizer.cpp:11-89. */
int mfem_gpu_scene_step(mfem_scene* scene, mfem_step_stats* stats);
/* Bytes of device memory the scene holds (admission control). */
int mfem_gpu_scene_footprint(const mfem_scene_desc* desc, int64_t* bytes);
int mfem_gpu_scene_sizes(const mfem_scene* scene, int32_t* n_vertices,
                         int32_t* n_tets, int32_t* n_free);
/* Full vertex positions / velocities (3*n_vertices doubles), per-tet s
 * (6*n_tets), R (9*n_tets, column-major 3x3) and lambda (6*n_tets). Any
 * output pointer may be NULL.                                              */
int mfem_gpu_scene_get_state(mfem_scene* scene, double* x, double* v,
                             double* s, double* R, double* la);
int mfem_gpu_scene_set_state(mfem_scene* scene, const double* x,
                             const double* v, const double* s, const double* R);

/* ---- snapshots (resume): the whole dynamic state of a scene between steps --
 * positions, the BDF history of positions and velocities (bdf_order slots,
 * most recent first), the stretch variable s, the rotations (as unit
 * quaternions) and the scripted pin positions -- the state a run carries
 * from one NewtonOptimizer::step to the next (SimState x_, mixed_vars_ and
 * the BDF integrator, src/simulation_state.cpp:263-308, BDF.cpp:6-93).
 * Positions, history and s are stored as the scene holds them (8 bytes a
 * value: an FP64 number or the mixed path's float pair), so a restore into
 * a scene of the same precision is bitwise, and one into the other
 * precision converts them (same mesh, BDF order and pins).
 * snapshot_bytes gives the size; restore checks the header and returns
 * MFEM_ERR_INVALID for a snapshot of another mesh.                        */
int mfem_gpu_scene_snapshot_bytes(mfem_scene* scene, int64_t* bytes);
int mfem_gpu_scene_snapshot(mfem_scene* scene, void* buf, int64_t bytes);
int mfem_gpu_scene_restore(mfem_scene* scene, const void* buf, int64_t bytes);
/* Device-resident checkpoint of the same state (raw copies inside device
 * memory, allocated on first use): rollback returns the scene to its last
 * checkpoint.  No counterpart in the reference.                          */
int mfem_gpu_scene_checkpoint(mfem_scene* scene);
int mfem_gpu_scene_rollback(mfem_scene* scene);

/* ---- batches: many independent scenes stepped by one launch per phase ----- */
int mfem_gpu_batch_create(mfem_scene* const* scenes, int32_t n, mfem_batch** out);
int mfem_gpu_batch_destroy(mfem_batch* batch);
/* Steps every scene in the batch once; stats[i] belongs to scenes[i]. */
int mfem_gpu_batch_step(mfem_batch* batch, mfem_step_stats* stats);
/* Steps every scene `steps` timesteps (1..MFEM_BATCH_MAX_STEPS), each at its
 * own pace: a scene whose Newton loop has ended turns over to its next
 * timestep at once and joins the next round of launches, instead of waiting
 * for the batch's slowest scene (no counterpart in the reference, where
 * each scene is its own NewtonOptimizer::step loop).  The results are those
 * of `steps` calls of mfem_gpu_batch_step, bitwise.  stats[i]: status the
 * worst of scene i's steps, Newton / PCG / line-search iterations summed
 * over them, energy and residuals of its last step, device_ms the call's
 * time.  step_done_ms (optional; steps doubles per scene, scene-major): the
 * device time from the call's start at which each step of each scene was
 * done (-1 for a step not taken).  A scene whose step ends non-finite or
 * with a singular rotation solve is retired: its remaining steps are not
 * taken and its status is that step's.  Scripted boundary motion is
 * precomputed on the host for the call's steps. */
#define MFEM_BATCH_MAX_STEPS 1024
int mfem_gpu_batch_step_n(mfem_batch* batch, int32_t steps, mfem_step_stats* stats,
                          double* step_done_ms);
/* mfem_gpu_batch_step_n for several batches at once (no counterpart in the
 * reference): each batch on its own stream, driven by its own host thread,
 * so that the GPU runs the batches' launches side by side -- a latency-bound
 * small scene then waits only for the launches of its own batch.  The
 * batches must be distinct and on the calling thread's device (no scene in
 * two of them).  stats and step_done_ms are laid out batch after batch, each
 * batch's scenes in its order; step_done_ms is measured from each batch's
 * own start.  Returns the first failure in batch order (MFEM_ERR_NONFINITE
 * only if nothing else failed). */
int mfem_gpu_batches_step_n(mfem_batch* const* batches, int32_t nbatch, int32_t steps,
                            mfem_step_stats* stats, double* step_done_ms);

/* Prescribed positions of the pinned vertices for the next step (3*n_pinned
 * doubles in the order of mfem_gpu_scene_pinned), replacing the scripted
 * boundary motion for that step (the role of Mesh::update_bcs,
 * src/mesh/mesh.h:130-132, when the caller drives the pins).           */
int mfem_gpu_scene_pinned(mfem_scene* scene, int32_t* n_pinned, int32_t* vertices);
int mfem_gpu_scene_set_pins(mfem_scene* scene, const double* positions);

/* ---- instrumentation (the reference's Timer keys, optimizer_data.cpp:125-183) --
 * With profiling on, every kernel launch of the batch is bracketed by CUDA
 * events on the batch's stream; kernel_stats returns the summed device time
 * and the launch count of kernel `kernel` since profiling was switched on.
 * Launches are counted whether or not profiling is on.                    */
enum {
  MFEM_K_ELEM_UPDATE = 0, MFEM_K_ASSEMBLE = 1, MFEM_K_CG_INIT = 2, MFEM_K_CG_SPMV = 3,
  MFEM_K_CG_UPDATE = 4, MFEM_K_LOCAL_SOLVE = 5, MFEM_K_LS_ENERGY = 6, MFEM_K_APPLY = 7,
  MFEM_K_STEP_BEGIN = 8, MFEM_K_STEP_END = 9, MFEM_K_SCALARS = 10, MFEM_K_CG_SOLVE = 11,
  MFEM_K_CGF_ITER = 12, MFEM_K_CG_REPLACE = 13, MFEM_K_MR_INIT = 14, MFEM_K_MR_ELEM = 15,
  MFEM_K_MR_VERT = 16, MFEM_K_MR_UPDATE = 17, MFEM_K_MR_EXPORT = 18, MFEM_K_CG_LOOP = 19,
  MFEM_K_COUNT = 20
};
int mfem_gpu_scene_solo_batch(mfem_scene* scene, mfem_batch** batch);
int mfem_gpu_batch_set_profiling(mfem_batch* batch, int enable);
/* Scheduling priority of the batch's stream against other batches' streams
 * on the device (no counterpart in the reference): 0 the default, 1, 2, ...
 * higher (clamped to the device's range).  Waits for the batch's work in
 * flight. */
int mfem_gpu_batch_set_priority(mfem_batch* batch, int32_t priority);
int mfem_gpu_batch_kernel_stats(mfem_batch* batch, int kernel, double* total_ms,
                                int64_t* launches);
int mfem_gpu_kernel_name(int kernel, char* name, int name_len);

/* ---- kernel shapes (no counterpart in the reference) ---------------------
 * Shape of the batch's fused PCG iteration: stages = 0 streams the matrix
 * through registers; 2..4 or 8 stage each warp's ELL slots through that many
 * shared-memory buffers filled by bulk copies; keep = 1 marks half of the
 * matrix's L2 lines evict-last, 0 all evict-first; unroll = 2 (with
 * stages = 4) puts two slots' gathers in flight together, unroll = 4
 * (with stages = 8) four, for systems too small to fill the GPU; unroll = 1 one;
 * pdl = 1 (staged shapes only) launches each iteration as a programmatic
 * dependent of the previous one.  FP64 batches use stages <= 2 and
 * unroll 1.  Every shape computes the same bits; the autotuner picks one
 * per batch.  Changing the shape re-captures the batch's PCG graph. */
int mfem_gpu_batch_set_pcg_shape(mfem_batch* batch, int32_t stages, int32_t keep,
                                 int32_t unroll, int32_t pdl);
int mfem_gpu_batch_get_pcg_shape(mfem_batch* batch, int32_t* stages, int32_t* keep,
                                 int32_t* unroll, int32_t* pdl);
/* The autotuner's record for the batch as a JSON object: "source"
 * ("tuned", "cache" or "default"), the cache key and, when tuned, for each
 * tuned kernel the candidates' measured times per launch (per iteration for
 * the PCG), the default's and the chosen one's.  At batch (and scene)
 * creation the tuner times register-budget variants of K1, K5 and K6 and
 * the fused PCG shapes on the batch's own system and keeps the fastest;
 * every candidate computes the same bits.  MFEM_GB300_TUNE=0 keeps the
 * built-in defaults, =force re-times on every creation;
 * MFEM_GB300_TUNE_CACHE names the cache file.  MFEM_ERR_CAPACITY if len is
 * too small. */
int mfem_gpu_batch_tune_report(mfem_batch* batch, char* buf, int32_t len);
/* The autotuner's mode for batches created from now on, process-wide (no
 * counterpart in the reference): 0 built-in defaults, 1 time on a cache
 * miss, 2 always time, -1 back to MFEM_GB300_TUNE.  A serving loop that
 * creates batches as requests come and go sets 0 (or relies on a warm
 * cache) so that no batch creation pays for timing runs. */
int mfem_gpu_set_tuning(int32_t mode);
/* Sets the register-budget variants of K1 (0..1; FP64 and the standard-FEM
 * variable have only 0), K5 (0..2) and K6 (0..1) by hand, overriding the
 * autotuner; 0 is the built-in default.  Every variant computes the same
 * bits. */
int mfem_gpu_batch_set_variants(mfem_batch* batch, int32_t elem_update, int32_t local_solve,
                                int32_t ls_energy);

/* ---- per-kernel parity entry points (host buffers in, host buffers out) ----
 * elem_update: MixedStretch::update_rotations + update_derivatives for the
 * current state at positions x (3*n_vertices, full) and time step h
 * (mixed_stretch.cpp:133-204).  Outputs per tet (any may be NULL):
 *   S[6], dSdF[54] (9x6 column-major, = Js^T*Sym), g[6] = h^2 grad psi,
 *   H[36] = h^2 hess psi (psd-fixed), Hinv[36], Aloc[144] (12x12 col-major),
 *   gl[6] (MixedStretch::rhs, :219-220), R[9] (updated rotation).       */
int mfem_gpu_scene_elem_update(mfem_scene* scene, const double* x, double h,
                               double* R, double* S, double* dSdF, double* g,
                               double* H, double* Hinv, double* Aloc,
                               double* gl);
/* Assembled LHS = PMP + A_mixed as 3x3 BCSR over free vertices after the
 * last elem_update/step iteration (Assembler::update_matrix + the sparse
 * add of SystemMatrixPD::pre_solve, linear_system.h:18-31) and the RHS.
 * row_ptr: n_free+1, col: nnzb, val: 9*nnzb (row-major 3x3), rhs: 3*n_free. */
int mfem_gpu_scene_bcsr_sizes(mfem_scene* scene, int32_t* n_free, int32_t* nnzb);
int mfem_gpu_scene_get_system(mfem_scene* scene, int32_t* row_ptr,
                              int32_t* col, double* val, double* rhs);
/* Solves LHS * dx = b with the scene's PCG on the last assembled matrix.
 * b, dx: 3*n_free.  Returns iterations and |r|/|b|.  In the mixed path dx
 * is the solver's float-float (df64) solution and |r|/|b| the residual it
 * stopped on: the single-reduction form verifies its recursive residual
 * against b - A dx before it stops; the two-reduction forms replace the
 * recursive residual by b - A dx every 25 iterations. */
int mfem_gpu_scene_pcg(mfem_scene* scene, const double* b, double* dx,
                       int32_t* iterations, double* rel_residual);

/* ---- allocation-free PCG (no counterpart in the reference) ------------
 * Block-Jacobi PCG on a caller-owned 3x3 block-CSR matrix already in device
 * memory (the layout mfem_gpu_scene_get_system returns: row_ptr n+1, col
 * nnzb, val 9*nnzb row-major blocks, all FP64), solving A x = b from x = 0
 * with the stopping rule of mfem_gpu_scene_pcg: |r|^2 < tol^2 |b|^2, or
 * MFEM_ERR_CG_MAXITER after max_iters iterations.  It calls no allocator:
 * its scratch (five vectors, the inverted diagonal blocks, tile partials,
 * tickets and scalars, about 6 MiB) is one static __device__ array sized for
 * MFEM_NOALLOC_PCG_MAX_ROWS block rows; larger systems are rejected with
 * MFEM_ERR_CAPACITY.  It exists for callers that must not allocate device
 * memory at solve time: a host framework that hands out all device memory
 * from its own budget or pool, or a real-time loop where cudaMalloc's
 * implicit device synchronisation would stall other streams.
 * The first call on a device (with that device current) looks up the
 * scratch address with cudaGetSymbolAddress; that first call should come
 * before any stream capture.  Every call waits for its stream
 * (cudaStreamSynchronize) and copies the solver's scalars to the host
 * between chunks of iterations.  Calls on one device share the scratch,
 * so overlapping calls would race: they are serialised by a per-device
 * lock held until the call's stream has drained.  All
 * pointers must be device memory of the current device; `stream` is a
 * cudaStream_t (NULL: the legacy default stream).  Returns iterations and
 * |r|/|b| like mfem_gpu_scene_pcg. */
#define MFEM_NOALLOC_PCG_MAX_ROWS 32768
int mfem_gpu_bsr_pcg_noalloc(int32_t n_block_rows, int32_t nnzb,
                             const int32_t* row_ptr, const int32_t* col,
                             const double* val, const double* b, double* x,
                             int32_t max_iters, double tol, void* stream,
                             int32_t* iterations, double* rel_residual);

/* ---- 2-D scenes: triangle meshes in the plane -----------------------------
 * The DIM = 2 instantiation of the same timestep: Tri2DMesh
 * (src/mesh/tri2d_mesh.cpp), MixedStretch<2> with polar_svd<2>
 * (src/variables/mixed_stretch.cpp:43-78, dsvd src/svd/dsvd.cpp:140-189),
 * the 3-vector materials (Stable-Neohookean, Corot, FixedCorot, ARAP:
 * the Vector3d sections of the src/energies files), Displacement<2>, BDF<2>,
 * NewtonOptimizer<2> with "eigen-pcg-diag".  FP64 throughout.
 * s per triangle is [S00, S11, (S10+S01)/2]; R is 2x2 column-major.
 * "Volumes" are igl::doublearea, twice the triangle area, as in
 * Tri2DMesh::volumes (tri2d_mesh.cpp:30-32); triangles must be
 * counter-clockwise (a clockwise one has a negative doublearea and is
 * rejected with MFEM_ERR_INVALID).  Every BC script of the 3-D path
 * applies, with BEND and TWIST turning by Rotation2D (about the group's
 * last vertex and the bounding-box centre, bend_boundary_condition.h:45,
 * twist_boundary_condition.h:45).  Neohookean and Fung (no Vector3d energy
 * in the reference) and solvers other than MFEM_SOLVER_EIGEN_CG_DIAG
 * return MFEM_ERR_UNSUPPORTED.                                             */
typedef struct mfem_tri2d_desc {
  int32_t n_vertices;
  int32_t n_tris;
  const double*  V_rest;       /* 2*n_vertices rest positions                  */
  const double*  V_init;       /* 2*n_vertices initial positions (NULL = rest) */
  const double*  v_init;       /* 2*n_vertices initial velocities (NULL = 0)   */
  const int32_t* tris;         /* 3*n_tris, counter-clockwise                  */
  const double*  mu;           /* n_tris                                        */
  const double*  lambda;       /* n_tris                                        */
  const int32_t* material;     /* n_tris MFEM_MATERIAL_* (NULL = all SNH)      */
  const double*  density;      /* n_tris (NULL = density_const)                */
  double         density_const;
  const int32_t* is_fixed;     /* n_vertices 0/1 override (NULL = from BC)     */
  int32_t bc_type;
  int32_t bc_axis;             /* 0 or 1                                        */
  double  bc_ratio;
  double  bc_velocity;
  double  dt;
  double  body_force[2];
  int32_t bdf_order;           /* 1..6 */
  int32_t max_newton_iterations;
  int32_t max_linesearch_iterations;
  int32_t max_iterative_solver_iters;
  double  iterative_solver_tolerance;
  double  newton_tol;
  double  newton_residual_tolerance;
  int32_t linear_solver;       /* MFEM_SOLVER_EIGEN_CG_DIAG */
  int32_t reserved[7];
} mfem_tri2d_desc;

typedef struct mfem_tri2d mfem_tri2d;

/* SimState<2>::load + NewtonOptimizer<2>::reset. */
int mfem_gpu_tri2d_create(const mfem_tri2d_desc* desc, mfem_tri2d** out);
int mfem_gpu_tri2d_destroy(mfem_tri2d* scene);
/* NewtonOptimizer<2>::step. */
int mfem_gpu_tri2d_step(mfem_tri2d* scene, mfem_step_stats* stats);
int mfem_gpu_tri2d_sizes(const mfem_tri2d* scene, int32_t* n_vertices,
                         int32_t* n_tris, int32_t* n_free, int32_t* nnzb);
/* x, v: 2*n_vertices; s, la: 3*n_tris; R: 4*n_tris.  Any may be NULL. */
int mfem_gpu_tri2d_get_state(mfem_tri2d* scene, double* x, double* v,
                             double* s, double* R, double* la);
/* MixedStretch<2>::update_rotations + update_derivatives at positions x
 * (2*n_vertices) and step h.  Per triangle: R[4], S[3], dSdF[12] (4x3
 * column-major), g[3], H[9], Hinv[9], Aloc[36] (6x6 column-major), gl[3]. */
int mfem_gpu_tri2d_elem_update(mfem_tri2d* scene, const double* x, double h,
                               double* R, double* S, double* dSdF, double* g,
                               double* H, double* Hinv, double* Aloc,
                               double* gl);
/* LHS = PMP + A as 2x2 BCSR over free vertices (row_ptr n_free+1, col nnzb,
 * val 4*nnzb row-major blocks) and the RHS (2*n_free) of the last
 * elem_update or Newton iteration. */
int mfem_gpu_tri2d_get_system(mfem_tri2d* scene, int32_t* row_ptr,
                              int32_t* col, double* val, double* rhs);
/* Instrumentation of the 2-D kernels: launches are counted always; with
 * profiling on, every launch is bracketed by CUDA events on the scene's
 * stream and kernel_stats returns the summed device time since profiling
 * was switched on (times are collected at the end of each step). */
enum {
  MFEM_T2_K_ELEM = 0, MFEM_T2_K_ROWS = 1, MFEM_T2_K_NORM = 2, MFEM_T2_K_PCG = 3,
  MFEM_T2_K_LOCAL = 4, MFEM_T2_K_ENERGY = 5, MFEM_T2_K_ESUM = 6, MFEM_T2_K_APPLY = 7,
  MFEM_T2_K_HISTORY = 8, MFEM_T2_K_COUNT = 9
};
int mfem_gpu_tri2d_set_profiling(mfem_tri2d* scene, int enable);
int mfem_gpu_tri2d_kernel_stats(mfem_tri2d* scene, int kernel, double* total_ms,
                                int64_t* launches);

#ifdef __cplusplus
}
#endif
#endif /* MFEM_GB300_H */
