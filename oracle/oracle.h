/*
 * oracle.h -- C API of the FP64 CPU oracle (TEST INFRASTRUCTURE ONLY).
 *
 * The oracle is a plain C++17/OpenMP restatement of ssim's FEM time-stepping
 * path (per-tet F, stable Neo-Hookean energy / PK1 / 9x9 Hessian, SPD
 * projection by a textbook cyclic-Jacobi eigensolver, 12x12 element stiffness,
 * CSR pattern + assembly, consistent mass, Dirichlet filtering, backward-Euler
 * state machine, Newton / Jacobi-PCG / backtracking line search, L-BFGS and the
 * Laplacian-preconditioned L-BFGS ("PD") stepper).  Every function cites the
 * reference file:line it restates.  It is the checker for the CUDA library and
 * the timed CPU baseline; it is never linked into, called by, or shipped with
 * the product library.
 *
 * Parity pins: the reference cannot be built (its numeric core `mathprim` is an
 * unpinned, absent dependency), so the oracle is pinned against the
 * known-answer and finite-difference tests the reference's own test suite
 * holds (tests/fem_intro, tests/fem_local_global, tests/fem_time_step_diff).
 * Optimizer trajectories (Newton / CG / L-BFGS iterates) have no pin in the
 * reference: parity unpinned for those.
 */
#ifndef SSIM_ORACLE_H
#define SSIM_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------- mesh generators ---------- */
/* ssim::mesh::unit_box (common_shapes.hpp:67-132): vertex COUNTS nx,ny,nz, 5 tets per cell. */
int orc_unit_box_sizes(int nx, int ny, int nz, int* nv, int* nt);
void orc_unit_box(int nx, int ny, int nz, double* X, int32_t* cells);
/* ssim::mesh::tetra (common_shapes.hpp:134-145). */
void orc_tetra(double* X, int32_t* cells);

/* ---------- element-level math ---------- */
void orc_lame(double E, double nu, double* lambda, double* mu);
double orc_snh_energy(const double F[9], double lambda, double mu);
double orc_snh_stress(const double F[9], double lambda, double mu, double P[9]);
void orc_snh_hessian(const double F[9], double lambda, double mu, double H[81]);
/* cyclic Jacobi eigen-decomposition of a symmetric n x n (n<=12), row-major */
int orc_sym_eigen(int n, const double* A, double* evals, double* evecs /* columns */);
void orc_project_spd(const double H[81], double eps, double Hp[81]);
void orc_dminv(const double x0[3], const double x1[3], const double x2[3], const double x3[3], double Dminv[9],
               double* vol);
void orc_element_stiffness(const double F[9], const double Dminv[9], double lambda, double mu, int make_spsd,
                           double K[144]);

/* ---------- time-step object ---------- */
typedef struct orc_ts orc_ts;

enum orc_buffer {
  ORC_DEFORMATION = 0,
  ORC_PREV_DEFORM = 1,
  ORC_INERTIA_DEFORM = 2,
  ORC_NEXT_DEFORM = 3,
  ORC_VELOCITY = 4,
  ORC_EXT_ACCEL = 5,
  ORC_FORCES = 6,
  ORC_DBC_VALUES = 7
};

enum orc_matrix { ORC_SYSMATRIX = 0, ORC_MASS = 1, ORC_MASS_FILTERED = 2 };

typedef struct {
  int max_newton_iters;  /* reference: 1000 (backward_euler.hpp:21) */
  double armijo;         /* reference: 0.3 (backward_euler.hpp:22) */
  double ls_shrink;      /* backtracking factor */
  int max_ls_iters;      /* line-search trials before giving up */
  int cg_max_iters;      /* PCG iteration cap */
  double cg_rtol;        /* PCG stop: |r| <= cg_rtol * |b| (fixed mode) */
  int cg_forcing;        /* 0: fixed cg_rtol; 1: eta_k = min(cg_rtol, max(cg_eta_min, |g_k|/|g_0|)) */
  double cg_eta_min;     /* lower clamp of the adaptive forcing term */
  int stop_mode;         /* 0: |g| < rtol*sum|M|/3 (reference); 1: |g| <= rel_tol*|g_0| */
  double rel_tol;        /* used when stop_mode == 1 */
  int precond;           /* 0: none, 1: Jacobi (diagonal), 2: block-Jacobi (3x3) */
  int lbfgs_history;     /* L-BFGS memory m */
  double lbfgs_armijo;   /* L-BFGS Armijo constant */
  int max_lbfgs_iters;
  double ls_energy_slack; /* Armijo accepts E_t <= E + c a g.d + slack S_E, S_E = sum of |energy terms| */
  int ncg_max_iters;      /* nonlinear CG: reference 1000 (nonlinear_cg.hpp:20) */
  double ncg_step0;       /* first trial step of the first iteration: reference learning_rate 1e-2 (:21) */
  double ncg_eta;         /* Dai-Kou truncation beta >= eta g.d / |d|^2 */
  int ncg_expand;         /* line-search expansions toward the parabola's minimiser */
  double stop_floor;      /* stop_mode 1 also stops at |g| <= stop_floor * sum|M| / 3 */
} orc_params;

typedef struct {
  int converged;
  int newton_iters;
  int cg_iters_total;
  int ls_steps_total;
  double grad_norm;
  double grad_norm0;
  double energy;
  double last_change;
} orc_stats;

void orc_default_params(orc_params* p);

orc_ts* orc_create(const double* X, int nv, const int32_t* cells, int nt, double dt, double E, double nu,
                   double rho);
/* 2D triangles in the plane (basic_time_step<Scalar, Device, 2, 3, ...>): X2 [nv][2], tris [nt][3]; the
 * state vectors keep 3 entries per vertex with z identically zero */
orc_ts* orc_create_2d(const double* X2, int nv, const int32_t* tris, int nt, double dt, double E, double nu,
                      double rho);
/* 2D element models on a row-major 2x2 F (Hessian flat index r*2+c) */
double orc_snh2_energy(const double F[4], double lambda, double mu);
double orc_snh2_stress(const double F[4], double lambda, double mu, double P[4]);
void orc_snh2_hessian(const double F[4], double lambda, double mu, double H[16]);
double orc_linear2_stress(const double F[4], double lambda, double mu, double P[4]);
void orc_linear2_hessian(double lambda, double mu, double H[16]);
/* 6x6 triangle stiffness embedded in 9x9 (3 dofs per vertex), Dm^-1 row-major 2x2 */
void orc_element_stiffness_2d(const double F[4], const double Dminv[4], double lambda, double mu, int make_spsd,
                              int model, double K[81]);
/* a mass-spring system (no reference counterpart): springs [ns][2], rest lengths from X, stiffness k, vertex
 * masses vmass[nv] (or m each), lumped mass, energy 1/2|x - x~|_M^2 + dt^2 sum k/2 (|x_i - x_j| - L)^2 */
orc_ts* orc_create_springs(const double* X, int nv, const int32_t* springs, int ns, double k, const double* vmass,
                           double m, double dt);
void orc_destroy(orc_ts* ts);
int orc_num_vertices(const orc_ts* ts);
int orc_num_cells(const orc_ts* ts);
int orc_nnz(const orc_ts* ts);
double orc_threshold_abs(const orc_ts* ts);

/* setters (time_step.hpp:316-347); return 0 or -1 on invalid argument */
int orc_set_time_step(orc_ts* ts, double dt);
int orc_set_youngs(orc_ts* ts, double E);
int orc_set_poisson(orc_ts* ts, double nu);
int orc_set_density(orc_ts* ts, double rho);
int orc_set_damping(orc_ts* ts, double d);
int orc_set_threshold(orc_ts* ts, double rtol);
/* per-element material (an extension over the reference's uniform E, nu); NULL restores uniform */
void orc_set_material(orc_ts* ts, const double* E_elem, const double* nu_elem);
/* per-(vertex,dof) boundary type (0 general, 1 dirichlet) and values, both [nv*3] */
void orc_set_dof_type(orc_ts* ts, const int8_t* types);
void orc_get_dof_type(const orc_ts* ts, int8_t* types);
int orc_add_ext_force_dof(orc_ts* ts, int dof, double a);
/* the PD stepper's diffusivity: 0 = as ssim computes it (time_step.hpp:356 builds the model from (E, nu)
 * in the (lambda, mu) slots), 1 = from the Lame parameters */
void orc_set_pd_diffusivity_mode(orc_ts* ts, int mode);

void orc_reset(orc_ts* ts);
void orc_prepare_step(orc_ts* ts);
double orc_update_energy_and_gradients(orc_ts* ts, int F_updated);
double orc_energy_at(orc_ts* ts, const double* u /* [nv*3] */);
void orc_update_hessian(orc_ts* ts, int F_updated, int make_spsd, int filter_dbc);
double orc_compute_step_newton(orc_ts* ts, const orc_params* p, orc_stats* st);
double orc_compute_step_lbfgs(orc_ts* ts, const orc_params* p, orc_stats* st);
double orc_compute_step_pd(orc_ts* ts, const orc_params* p, orc_stats* st);
double orc_compute_step_h0(orc_ts* ts, const orc_params* p, orc_stats* st);
double orc_compute_step_forward_euler(orc_ts* ts, const orc_params* p, orc_stats* st);
/* time_step_solver_ncg (nonlinear_cg.hpp:9-38) and _with_ext_prec (:40-97): nonlinear CG, the latter
 * preconditioned by x = L L^T g with L on the system matrix's CSR pattern (identity until set) */
double orc_compute_step_ncg(orc_ts* ts, const orc_params* p, orc_stats* st);
double orc_compute_step_ncg_prec(orc_ts* ts, const orc_params* p, orc_stats* st);
/* L's values in the CSR order of the system matrix (orc_get_csr); NULL restores the identity */
void orc_set_ncg_matrix(orc_ts* ts, const double* values);
/* elastic model of the time step: 0 stable Neo-Hookean (stable_neohookean.hpp), 1 linear (linear.hpp) */
void orc_set_model(orc_ts* ts, int model);
double orc_linear_stress(const double F[9], double lambda, double mu, double P[9]);
void orc_linear_hessian(double lambda, double mu, double H[81]);
void orc_element_stiffness_model(const double F[9], const double Dminv[9], double lambda, double mu, int make_spsd,
                                 int model, double K[144]);
void orc_step_next(orc_ts* ts);
void orc_restore(orc_ts* ts);
int orc_check_convergence(orc_ts* ts);

void orc_get(const orc_ts* ts, int which, double* out);
void orc_set(orc_ts* ts, int which, const double* in);
void orc_get_dminv(const orc_ts* ts, double* out /* [nt*9] */);
void orc_get_rest_vol(const orc_ts* ts, double* out /* [nt] */);
void orc_get_def_grad(const orc_ts* ts, double* out /* [nt*9] */);
void orc_get_local_stiffness(const orc_ts* ts, double* out /* [nt*144] */);
void orc_get_csr(const orc_ts* ts, int32_t* row_ptr, int32_t* col_idx);
void orc_get_values(const orc_ts* ts, int which, double* vals);
void orc_spmv(const orc_ts* ts, int which, const double* x, double* y);
/* PD matrix (projective_dynamics.hpp:53-93), values on the same CSR pattern as the system matrix */
void orc_pd_matrix_values(orc_ts* ts, double* vals);
/* Jacobi-PCG on the current system matrix; returns iterations */
int orc_pcg(const orc_ts* ts, const double* b, double* x, double rtol, int max_iters, int precond, double* rel_res);

/* gather semantics (global_composer.hpp:36-128): external local arrays, weights = rest volume */
void orc_gather_force(const orc_ts* ts, const double* local_force /* [nt*12] */, double alpha, double* f);
void orc_gather_hessian(const orc_ts* ts, const double* local_K /* [nt*144] */, double alpha, double* vals);

/* element integrals (bilinears.hpp:191-264): [nt*16] local 4x4 matrices, mass scaled by rho = alpha */
void orc_local_mass(const orc_ts* ts, double alpha, double* out);
void orc_local_laplace(const orc_ts* ts, double alpha, double* out);

int orc_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
