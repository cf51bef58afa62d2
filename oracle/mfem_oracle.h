/*
 * TEST INFRASTRUCTURE ONLY — the FP64 CPU oracle of the mixed-FEM Newton
 * timestep of tytrusty/mfem.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / --impl reference legs of bench.py may load it, and only to
 * check the GPU path's results or as the timed CPU baseline, never as the
 * product path.
 *
 * Parity status: the reference (C++17 on Eigen/libigl/Bartels/CHOLMOD) cannot
 * be built here — those libraries are absent — so this is a restatement.
 * It is pinned where the reference holds checks: the Procrustes dR/dF against
 * central differences (tests/test_dsvd.cpp:204-238) and the SVD dR/dF at a
 * fixed F (tests/test_dsvd.cpp:74-110); every energy derivative and the
 * Newton system are pinned by finite-difference checks in tests/.  The
 * reference holds no golden outputs of a whole timestep, so step-level
 * parity is "parity unpinned" beyond those checks.
 */
#ifndef MFEM_ORACLE_H
#define MFEM_ORACLE_H

#include "../include/mfem_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

int oracle_set_threads(int n);
int oracle_get_threads(void);

/* newton_procrustes, src/svd/newton_procrustes.h:108-189.  R (in/out, 3x3
 * column-major), A, B 3x3 column-major; dRdF 81 column-major (may be NULL). */
int oracle_procrustes(double* R, const double* A, const double* B,
                      int compute_gradients, double* dRdF, double tol,
                      int max_iter, int* iterations);
/* dsvd dR/dF, src/svd/dsvd.cpp:69-138 (column 3s+r = vec(dR/dF_rs)). */
int oracle_dsvd_dRdF(const double* F, double* dRdF);
/* polar_svd<3>, src/variables/mixed_stretch.cpp:14-42. */
int oracle_polar(double* R, const double* F, int compute_gradients,
                 double* s, double* dsdF);

double oracle_material_energy(int type, double mu, double la, const double* s);
void oracle_material_gradient(int type, double mu, double la, const double* s,
                              double* g);
void oracle_material_hessian(int type, double mu, double la, const double* s,
                             int psd_fix, double* H);
void oracle_psd_fix(double* H, int n, double tol);

void* oracle_scene_create(const mfem_scene_desc* desc, int* status);
void oracle_scene_destroy(void* scene);
int oracle_scene_step(void* scene, mfem_step_stats* stats);
int oracle_scene_sizes(void* scene, int* nv, int* nt, int* nfree, int* nnzb);
int oracle_scene_get_state(void* scene, double* x, double* v, double* s,
                           double* R, double* la);
int oracle_scene_set_state(void* scene, const double* x, const double* v,
                           const double* s, const double* R,
                           const double* la);
/* Positions only (free and pinned), leaving the BDF history unchanged. */
int oracle_scene_set_positions(void* scene, const double* x);
int oracle_scene_elem_update(void* scene, const double* x, double h, double* R,
                             double* S, double* dSdF, double* g, double* H,
                             double* Hinv, double* Aloc, double* gl);
/* BCSR (3x3 blocks, row-major block values) of LHS = PMP + A and the RHS
 * after the last update_system. */
int oracle_scene_get_system(void* scene, int* row_ptr, int* col, double* val,
                            double* rhs);
/* energy_func(alpha) of src/optimizers/newton_optimizer.cpp:34-49 at the
 * current state and the last (dx, ds). */
double oracle_scene_energy(void* scene, double alpha);
/* PCG on the last assembled LHS (Eigen ConjugateGradient semantics). */
int oracle_scene_pcg(void* scene, const double* b, double* x, int* iters,
                     double* rel_residual);
double oracle_material9(int type, double mu, double la, const double* F, double* g, double* H, int fix);
int oracle_scene_kkt_size(void* scene);
int oracle_scene_kkt_rhs(void* scene, double* rhs);
int oracle_scene_kkt_mul(void* scene, const double* w, double* out);
int oracle_scene_minres(void* scene, const double* b, double* x, int* iters, double* rel);
int oracle_scene_schur_solve(void* scene, double* x, int* iters, double* rel);
int oracle_scene_update_system(void* scene);

/* ---- the 2-D path (mfem_oracle2d.cpp): triangle meshes, DIM = 2 ---------- */
/* polar_svd<2,3> (mixed_stretch.cpp:43-78): R 2x2 column-major, s[3], dsdF
 * 3x4 column-major (NULL: no derivative).  Returns MFEM_ERR_PROCRUSTES when
 * sig0 + sig1 = 0 (no unique nearest rotation). */
int oracle2d_polar(double* R, const double* F, double* s, double* dsdF);
/* svd<double,2> with the sign fix (svd_eigen.h:7-32). */
int oracle2d_svd(const double* F, double* sig, double* U, double* V);
/* psi of a 3-vector material; g[3], H[9] (may be NULL); fix: psd projection. */
double oracle2d_material(int type, double mu, double la, const double* s, double* g,
                         double* H, int fix);
void* oracle2d_create(const mfem_tri2d_desc* desc, int* status);
void oracle2d_destroy(void* scene);
int oracle2d_step(void* scene, mfem_step_stats* stats);
int oracle2d_sizes(void* scene, int* nv, int* nt, int* nfree, int* nnzb);
int oracle2d_get_state(void* scene, double* x, double* v, double* s, double* R, double* la);
int oracle2d_elem_update(void* scene, const double* x, double h, double* R, double* S,
                         double* dSdF, double* g, double* H, double* Hinv, double* Aloc,
                         double* gl);
int oracle2d_get_system(void* scene, int* row_ptr, int* col, double* val, double* rhs);
double oracle2d_energy(void* scene, double alpha);
/* One Newton direction at the current state, without stepping: the system,
 * its PCG solve and the local solve.  dx: 2*n_vertices (0 at pinned
 * vertices), ds and la: 3*n_tris. */
int oracle2d_direction(void* scene, double* dx, double* ds, double* la, int* iters);

#ifdef __cplusplus
}
#endif
#endif
