/*
 * ssim_gb.h -- C ABI of the GB300-native FEM time-stepping library (libssim_gb300.so).
 *
 * One handle is one ssim::fem::basic_time_step<double, cuda, 3, 4, stable_neohookean, ...> object
 * (ssim/include/ssim/finite_elements/time_step.hpp:168-715) together with the stepper chosen at
 * reset (Newton / L-BFGS / PD, stepper/backward_euler.hpp, stepper/projective_dynamics.hpp).  Every
 * entry point takes plain pointers and sizes; host arrays use the reference's layouts:
 *   vertices  [V,3] float64 row-major      (bindings/src/fem_host.cpp:56 VertNb)
 *   cells     [T,4] int32 row-major         (bindings/src/fem_host.cpp:57 CellNb, index_t == int32)
 *   per-vertex fields (deformation, velocity, forces ...) [V,3] float64
 *   Dirichlet targets [n,3] float64 (the memory of Eigen::Matrix3Xd, fem_host.cpp:123)
 *   CSR matrices: row_ptr [3V+1] int32, col_idx [nnz] int32, values [nnz] float64, full storage,
 *   columns strictly ascending per row (global_composer.hpp:68-100)
 * All functions return an ssim_gb_status; on failure ssim_gb_last_error(h) describes the cause.
 * A handle is not thread-safe: calls on one handle must be serialised (the reference object is
 * single-threaded too, time_step.hpp:679).  Different handles may run concurrently on different
 * CUDA streams.  No entry point falls back to the CPU: with no usable CUDA device they fail with
 * SSIM_GB_ERR_CUDA.
 */
#ifndef SSIM_GB_H
#define SSIM_GB_H
#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define SSIM_GB_API __attribute__((visibility("default")))
#else
#define SSIM_GB_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  SSIM_GB_OK = 0,
  SSIM_GB_ERR_INVALID_ARGUMENT = 1, /* where the reference throws std::invalid_argument */
  SSIM_GB_ERR_NOT_CONVERGED = 2,    /* only returned when strict convergence is requested */
  SSIM_GB_ERR_CUDA = 3,             /* CUDA runtime error (message in last_error) */
  SSIM_GB_ERR_NUMERICAL = 4,        /* NaN/Inf in energy or gradient, or an inverted element */
  SSIM_GB_ERR_STATE = 5,            /* call out of order (e.g. compute_step before prepare_step) */
  SSIM_GB_ERR_OUT_OF_MEMORY = 6,
  SSIM_GB_ERR_DEVICE_TIMEOUT = 7    /* a bounded device-side wait gave up; the CUDA context stays usable */
} ssim_gb_status;

/* Precision of the Hessian, assembly and inner PCG.  Energy, gradient, state and every reduction are
 * FP64 in both modes. */
typedef enum { SSIM_GB_FP64 = 0, SSIM_GB_MIXED = 1 } ssim_gb_precision;

typedef enum {
  SSIM_GB_STEPPER_NEWTON = 0, /* time_step_solver_backward_euler<cg<diagonal>> (backward_euler.hpp:9-41) */
  SSIM_GB_STEPPER_LBFGS = 1,  /* time_step_solver_lbfgs (backward_euler.hpp:43-67) */
  SSIM_GB_STEPPER_PD = 2,     /* time_step_solver_pd (projective_dynamics.hpp:9-97) */
  SSIM_GB_STEPPER_NONE = 3,   /* time_step_solver_nothing (time_step.hpp:131-142) */
  SSIM_GB_STEPPER_FORWARD_EULER = 4, /* time_step_solver_forward_euler (time_step.hpp:717-736) */
  SSIM_GB_STEPPER_H0 = 5,     /* time_step_solver_h0 (projective_dynamics.hpp:100-150) */
  SSIM_GB_STEPPER_NCG = 6,    /* time_step_solver_ncg (nonlinear_cg.hpp:9-38) */
  SSIM_GB_STEPPER_NCG_EXT = 7 /* time_step_solver_ncg_with_ext_prec (nonlinear_cg.hpp:40-97): x = L L^T g */
} ssim_gb_stepper;

/* The ElastModel template argument of basic_time_step */
typedef enum {
  SSIM_GB_MODEL_STABLE_NEOHOOKEAN = 0, /* elast::stable_neohookean (stable_neohookean.hpp:11-112) */
  SSIM_GB_MODEL_LINEAR = 1             /* elast::linear (linear.hpp:7-70) */
} ssim_gb_elastic_model;

typedef enum {
  SSIM_GB_DEFORMATION = 0,
  SSIM_GB_PREV_DEFORM = 1,
  SSIM_GB_INERTIA_DEFORM = 2,
  SSIM_GB_NEXT_DEFORM = 3,
  SSIM_GB_VELOCITY = 4,
  SSIM_GB_EXT_ACCEL = 5,
  SSIM_GB_FORCES = 6,
  SSIM_GB_DBC_VALUES = 7
} ssim_gb_field;

typedef enum {
  SSIM_GB_SYSMATRIX = 0,
  SSIM_GB_MASS = 1,
  SSIM_GB_MASS_FILTERED = 2,
  SSIM_GB_SYSMATRIX_HALF = 3 /* ssim_gb_spmv only, mixed precision: the FP16 copy of pcg_half_matrix */
} ssim_gb_matrix;

/* Solver settings.  Defaults (ssim_gb_default_params) follow the reference where it fixes a value:
 * max 1000 Newton iterations and Armijo 0.3 (backward_euler.hpp:21-22), stopping rule
 * |g| < rtol * sum|M| / 3 (time_step.hpp:490-491, 660-664), Jacobi-preconditioned CG
 * (tests/fem_cu/main.cu:52-54). */
typedef struct {
  int32_t max_newton_iters;
  double armijo;
  double ls_shrink;
  int32_t max_ls_iters;
  int32_t cg_max_iters;
  double cg_rtol;      /* PCG stop |r| <= eta |b| */
  int32_t cg_forcing;  /* 0: eta = cg_rtol; 1: eta = min(cg_rtol, max(cg_eta_min, |g_k|/|g_0|)) */
  double cg_eta_min;
  int32_t stop_mode;   /* 0: |g| < rtol*sum|M|/3 (reference); 1: |g| <= rel_tol*|g_0| */
  double rel_tol;
  int32_t precond;     /* 0 none, 1 Jacobi (the reference's diagonal preconditioner), 2 block-Jacobi (3x3) */
  int32_t lbfgs_history;
  double lbfgs_armijo;
  int32_t max_lbfgs_iters;
  int32_t cg_check_every; /* PCG iterations launched between host convergence checks */
  double ls_energy_slack; /* Armijo accepts E_t <= E + c a g.d + slack * sum|energy terms| (round-off) */
  int32_t pd_kappa_mode;  /* PD matrix diffusivity: 0 as ssim builds it (time_step.hpp:356), 1 from the Lame
                             parameters, 2 from each element's own Lame parameters (per-element materials) */
  int32_t pcg_persistent; /* 0: two launches per PCG iteration, host checks every cg_check_every iterations;
                             1: the same PCG in one cooperative launch per solve (grid barriers, no host
                             round trips; bitwise the iterates of 0); 2: Chronopoulos-Gear PCG in one
                             launch (one reduction per iteration; equal to 0 up to rounding);
                             3 (default): in mixed precision 4 for the solves on the FP16 copy of the
                             scaled matrix (pcg_half_matrix, whose true-residual check covers the drift
                             below) and 2 on the FP32 values; 0 in FP64 (the faster on GB300);
                             4: pipelined PCG in one launch (one grid barrier per iteration, two more vertex
                             vectors, Chronopoulos-Gear after pcg_pipe_iters iterations; equal to 0 up to
                             rounding, but in FP32 its true residual drifts from the recursive one with the
                             iterations and the condition number: for loose solves of well-conditioned
                             systems only) */
  int64_t pcg_spin_limit; /* polls before a grid-barrier wait gives up (SSIM_GB_ERR_DEVICE_TIMEOUT); 0 = default
                             (2^25 polls, about a second) */
  int32_t pcg_barrier_extra; /* test hook: arrivals a grid barrier waits for beyond the grid; 0 in normal use,
                                > 0 makes every wait run out after pcg_spin_limit polls */
  int32_t pcg_max_blocks; /* cap on the persistent PCG grid (0: as many 256-thread blocks as are resident) */
  int32_t ncg_max_iters;  /* nonlinear CG iteration cap: 1000 as the reference (nonlinear_cg.hpp:20) */
  double ncg_step0;       /* first trial step of the first NCG iteration: the reference's learning rate 1e-2 */
  double ncg_eta;         /* Dai-Kou truncation: beta >= ncg_eta * g.d / |d|^2 (0.5) */
  int32_t ncg_expand;     /* line-search expansions toward the fitted parabola's minimiser (3) */
  double stop_floor;      /* stop_mode 1 also stops when |g| <= stop_floor * sum|M| / 3 (the reference's absolute
                             rule with rtol = stop_floor; default 1e-12), so a step starting at rest, whose
                             gradient is round-off, does not chase a fraction of it */
  int32_t mixed_elem32;   /* mixed precision, Newton and L-BFGS: 1 (default) evaluates energy and forces with FP32
                             element arithmetic while the residual is above elem32_switch times the target, then
                             in FP64 (the stopping test always sees an FP64 residual); the FP32 phase also ends
                             when its residual stalls (Newton: two iterations without halving; L-BFGS: within 1e3
                             times the target, no halving in max(100, 3 x the phase's longest halving interval)
                             iterations, or a line search that runs out); 0 keeps every evaluation FP64 */
  double ls_energy_slack32; /* Armijo round-off slack of the FP32 evaluations, times their term-magnitude sum */
  double elem32_switch;   /* residual / target below which the FP32 phase ends (10) */
  int32_t pcg_pipe_iters; /* pipelined PCG (pcg_persistent 4) continues as Chronopoulos-Gear PCG after this many
                             iterations (80), bounding the drift of its recursive residual in long solves */
  int32_t fused_assembly; /* tets: 0 (default) runs the element Hessian and the assembly as two kernels through a
                             per-element block buffer; 1 evaluates the element Hessians inside the assembly, each
                             CTA summing the blocks of its own rows in shared memory (no per-element blocks in
                             memory, but every element is evaluated by each CTA whose rows it touches: 2.3x the
                             element work on a lexicographically numbered box, measured slower on GB300).  Both
                             give the same values bit for bit (each slot sums its blocks in element order) */
  int32_t mixed_delta;    /* mixed precision, Newton, tets with stable Neo-Hookean: 1 (default) evaluates the
                             iterations after the FP32 phase as FP32 increments from the FP64 evaluation made at
                             the switch (energy and forces = that evaluation's + increments whose rounding is
                             relative to the increment); 0 evaluates them in FP64 */
  int32_t pcg_half_matrix; /* mixed precision: 1 (default) runs the persistent Chronopoulos-Gear PCG solves whose relative
                             tolerance is at least half_matrix_min_rtol on an FP16 copy of the Jacobi-scaled system
                             matrix (S K S, S = diag(K)^-1/2, both triangles, one 16-byte load per block; remade
                             after each assembly): the same iterates up to the FP16 rounding of the scaled values
                             (~5e-4 relative), about 60% of the FP32 symmetric format's SpMV time on a 1M-tet
                             mesh; ssim_gb_autotune turns it off where its per-assembly conversion costs more than
                             it saves.  0 keeps every solve on the FP32 values */
  double half_matrix_min_rtol; /* tighter solves (adjoint, tight forcing) stay on the FP32 values (1e-2) */
  int32_t half_hessian_blocks; /* tets: 1 (default) writes the element Hessian blocks of the assemblies whose solve
                             runs on the FP16 copy in FP16 (a power-of-two scale per 3x3 block, 24 bytes a block
                             instead of 36, three 8-byte loads in the assembly, FP32 sums); 0 keeps FP32 blocks */
  double half_check_slack; /* after every Newton solve on the FP16 copy the true residual |g + K d| on the FP32
                             values is computed with g . d (one fused kernel, about 25 us more than g . d alone
                             at 1M tets); above half_check_slack (1.2) times the forcing eta
                             times |g| the copy is too coarse for the system's conditioning and the handle's
                             later solves use the FP32 values (until reset() or ssim_gb_set_params).  Measured
                             ratios: 0.8-1.05 on the beams, bar and cube, up to 1.46 (2.7 with FP32 element
                             blocks) on the reference's light, stiff unit box, where the copy costs Newton
                             iterations */
  int32_t speculative_hessian; /* mixed precision, tets, Newton: 1 assembles the next iteration's Hessian at the
                             full step u + d on a second stream while the line search runs on the handle's
                             stream; a full step accepted finds its matrix ready (the same values: the same FP32
                             positions), a shorter one assembles again.  0 (default): after the line search.
                             Measured on GB300: 304 against 299 steps/s on the 192k-tet bar, but 62.2 against
                             63.9 on the 1.02M-tet beam and 9.37 against 9.83 on the 6.5M-tet batch (the
                             Hessian's many small blocks hold the SMs the line search's kernels wait for) */
} ssim_gb_params;

/* Per compute_step statistics (the optim_result fields of backward_euler.hpp:28-32 and more). */
typedef struct {
  int32_t converged;
  int32_t newton_iters;
  int32_t cg_iters_total;
  int32_t ls_steps_total;
  double grad_norm;
  double grad_norm0;
  double energy;
  double last_change;
  double elapsed_ms;
  int32_t half_solves;    /* mixed Newton: solves of this step that ran on the FP16 copy of the scaled matrix */
  double half_check;      /* the largest |g + K d| / (eta |g|) on the FP32 values among those solves (0: none) */
  int32_t spec_hits;      /* Newton iterations whose matrix was assembled ahead of the line search (speculative_hessian) */
} ssim_gb_step_stats;

/* Launch shapes chosen by ssim_gb_autotune (extension: the reference has no GPU kernels of its own) */
typedef struct {
  int32_t elem_block;     /* threads per block of the FP32 element passes (0: not tuned, the default 128) */
  int32_t hessian_block;  /* threads per block of the element Hessian kernel (default 64) */
  int32_t assembly_block; /* threads per block of the assembly kernel (default 256) */
  int32_t gather_block;   /* threads per block of the FP32 force gathers (0: not tuned, the default 256) */
  int32_t pcg_persistent; /* the PCG variant chosen (ssim_gb_params.pcg_persistent) */
  int32_t pcg_max_blocks; /* the persistent PCG's grid cap chosen (ssim_gb_params.pcg_max_blocks) */
  int32_t fused_assembly; /* ssim_gb_params.fused_assembly chosen */
  int32_t from_cache;     /* 1: an earlier sweep of the same shape in this process decided (nothing timed) */
  double elem_us;         /* per launch of the chosen element pass (0 when not timed) */
  double hessian_us;      /* Hessian + assembly with the chosen shapes */
  double pcg_solve_ms;    /* one PCG solve to 5e-2 relative residual with the chosen variant and grid */
  int32_t pcg_iterations; /* iterations of that solve */
  int32_t candidates;     /* configurations timed */
  int32_t pcg_half_matrix; /* ssim_gb_params.pcg_half_matrix chosen (mixed: the persistent Chronopoulos-Gear
                              solve timed on the FP16 copy, its conversion included, and on the FP32 values) */
  int32_t elem_regcap;    /* 1: the FP32 element pass's variant capped at 64 registers a thread (more resident
                             warps for its dependent gathers) */
} ssim_gb_tuning;

typedef struct ssim_gb_timestep ssim_gb_timestep;

/* ---- library ---- */
SSIM_GB_API const char* ssim_gb_version(void);
/* count of CUDA kernels this library has launched in this process */
SSIM_GB_API uint64_t ssim_gb_launch_count(void);
/* ABI check for bindings that mirror the public structs: sizeof of ssim_gb_params (0), ssim_gb_step_stats (1)
 * and ssim_gb_tuning (2); 0 for anything else.  Needs no GPU. */
SSIM_GB_API size_t ssim_gb_struct_size(int32_t which);
SSIM_GB_API void ssim_gb_default_params(ssim_gb_params* p);
SSIM_GB_API const char* ssim_gb_last_error(const ssim_gb_timestep* h);

/* ---- mesh utilities (host only, no GPU needed) ---- */
/* sizes / pattern of the Hessian CSR of a tet mesh, the pattern local_global_composer::hessian builds
 * (global_composer.hpp:68-100): row_ptr [3V+1], col_idx [nnz] */
SSIM_GB_API ssim_gb_status ssim_gb_mesh_csr_nnz(const int32_t* cells, int32_t num_cells, int32_t num_vertices, int64_t* nnz);
SSIM_GB_API ssim_gb_status ssim_gb_mesh_csr_pattern(const int32_t* cells, int32_t num_cells, int32_t num_vertices,
                                        int32_t* row_ptr, int32_t* col_idx);

/* ---- construction: basic_time_step(mesh, dt, E, nu, rho) (time_step.hpp:260-265),
 *      timestep_wrapper_cuda(vert, cell, time_step, youngs, poisson, density) (fem_cuda.cu:61-71) ---- */
SSIM_GB_API ssim_gb_status ssim_gb_create(const double* vertices, int32_t num_vertices, const int32_t* cells,
                              int32_t num_cells, double time_step, double youngs, double poisson,
                              double density, ssim_gb_timestep** out);
/* A mass-spring system (cloth) stepped by the same object: springs [num_springs][2] vertex pairs with rest
 * lengths from the vertices, stiffness k, vertex masses (vertex_mass[num_vertices], or `mass` for every
 * vertex when NULL), energy 1/2 |x - x~|^2_M + dt^2 sum k/2 (|x_i - x_j| - L)^2 with the lumped mass.  No
 * reference counterpart (the reference has no spring model); Newton, L-BFGS, PD (mass + dt^2 k spring
 * Laplacian), NCG and forward Euler apply, the adjoint does not. */
SSIM_GB_API ssim_gb_status ssim_gb_create_springs(const double* vertices, int32_t num_vertices, const int32_t* springs,
                                                  int32_t num_springs, double stiffness, const double* vertex_mass,
                                                  double mass, double time_step, ssim_gb_timestep** out);
/* 2D triangles in the plane: basic_time_step<Scalar, Device, 2, 3, ElastModel, ...> (time_step.hpp:168-715
 * with PhysicalDim 2, TopologyDim 3; rest shape def_grad.hpp:56-91 and rest_vol.hpp:34-54 in 2D, consistent
 * mass p1_element_2d bilinears.hpp:45-96, stable_neohookean<2> / linear<2>).  vertices [V][2], triangles
 * [T][3].  The handle keeps 3 dofs per vertex: fields are [V,3] with z identically zero, the system matrix
 * carries the mass alone on the z dofs; ssim_gb_get_csr_2d gives the reference's 2-dof CSR.  The adjoint
 * and the FP32 element phase of the mixed steppers are tets only. */
SSIM_GB_API ssim_gb_status ssim_gb_create_2d(const double* vertices, int32_t num_vertices, const int32_t* triangles,
                                             int32_t num_triangles, double time_step, double youngs, double poisson,
                                             double density, ssim_gb_timestep** out);
/* physical dimension of a handle: 3 (tets, springs) or 2 (triangles) */
SSIM_GB_API ssim_gb_status ssim_gb_get_dim(const ssim_gb_timestep* h, int32_t* dim);
/* the reference's 2-dof CSR of a 2D handle's matrix `which` (SSIM_GB_SYSTEM, _MASS, _MASS_FILTERED):
 * row 2u+a holds columns {2w+b : w in N(u) sorted, b < 2}; row_ptr [2V+1], col_idx and values [nnz2] with
 * nnz2 = 4/9 of ssim_gb_sizes' nnz; any of the three outputs may be NULL */
SSIM_GB_API ssim_gb_status ssim_gb_get_csr_2d(ssim_gb_timestep* h, int32_t which, int32_t* row_ptr, int32_t* col_idx,
                                              double* values);
SSIM_GB_API ssim_gb_status ssim_gb_destroy(ssim_gb_timestep* h);
SSIM_GB_API ssim_gb_status ssim_gb_sizes(const ssim_gb_timestep* h, int32_t* num_vertices, int32_t* num_cells,
                             int32_t* num_dofs, int64_t* nnz);
/* use an existing CUDA stream (cudaStream_t); NULL restores the handle's own stream */
SSIM_GB_API ssim_gb_status ssim_gb_set_stream(ssim_gb_timestep* h, void* stream);

/* ---- setters (time_step.hpp:316-347); applied at the next reset() ---- */
SSIM_GB_API ssim_gb_status ssim_gb_set_time_step(ssim_gb_timestep* h, double dt);
SSIM_GB_API ssim_gb_status ssim_gb_set_youngs(ssim_gb_timestep* h, double E);
SSIM_GB_API ssim_gb_status ssim_gb_set_poisson(ssim_gb_timestep* h, double nu);
SSIM_GB_API ssim_gb_status ssim_gb_set_density(ssim_gb_timestep* h, double rho);
SSIM_GB_API ssim_gb_status ssim_gb_set_damping(ssim_gb_timestep* h, double damping);
/* set_threshold (time_step.hpp:343-347) == set_rtol (fem_cuda.cu:132) */
SSIM_GB_API ssim_gb_status ssim_gb_set_threshold(ssim_gb_timestep* h, double rtol);
SSIM_GB_API ssim_gb_status ssim_gb_set_precision(ssim_gb_timestep* h, int32_t precision);
SSIM_GB_API ssim_gb_status ssim_gb_set_params(ssim_gb_timestep* h, const ssim_gb_params* p);
SSIM_GB_API ssim_gb_status ssim_gb_get_params(const ssim_gb_timestep* h, ssim_gb_params* p);
/* per-element Young's modulus and Poisson ratio [T] (extension: the reference's elastic model has the
 * per-call (lambda, mu) overloads of basic_elast.hpp:74-81 but the time step only uses uniform values);
 * NULL restores the uniform material */
SSIM_GB_API ssim_gb_status ssim_gb_set_material(ssim_gb_timestep* h, const double* youngs_per_cell,
                                    const double* poisson_per_cell);

/* ---- boundary conditions (fem_cuda.cu:115-150, boundary.hpp:13-106) ---- */
/* The arrays are copied before the call returns (the caller may reuse them at once); the upload and the
 * marking run on the handle's stream ahead of its next work, without a host wait. */
SSIM_GB_API ssim_gb_status ssim_gb_mark_dirichlet_batched(ssim_gb_timestep* h, const int32_t* verts, int32_t n,
                                              const double* targ_deform /* [n,3] */);
SSIM_GB_API ssim_gb_status ssim_gb_mark_general_batched(ssim_gb_timestep* h, const int32_t* verts, int32_t n);
SSIM_GB_API ssim_gb_status ssim_gb_set_dof_type(ssim_gb_timestep* h, const int8_t* dof_type /* [V,3] */);
SSIM_GB_API ssim_gb_status ssim_gb_get_dof_type(const ssim_gb_timestep* h, int8_t* dof_type /* [V,3] */);
/* add_ext_force_dof (time_step.hpp:550-557); add_gravity (fem_cuda.cu:134-138) */
SSIM_GB_API ssim_gb_status ssim_gb_add_ext_force_dof(ssim_gb_timestep* h, int32_t dof, double accel);
SSIM_GB_API ssim_gb_status ssim_gb_add_gravity(ssim_gb_timestep* h, const double gravity[3]);

/* ---- loop (time_step.hpp:363-543) ---- */
SSIM_GB_API ssim_gb_status ssim_gb_reset(ssim_gb_timestep* h, int32_t stepper);
SSIM_GB_API ssim_gb_status ssim_gb_prepare_step(ssim_gb_timestep* h);
/* compute_step: runs the stepper, re-evaluates the gradient, returns |g| (time_step.hpp:520-528) */
SSIM_GB_API ssim_gb_status ssim_gb_compute_step(ssim_gb_timestep* h, double* residual_norm);
SSIM_GB_API ssim_gb_status ssim_gb_step_next(ssim_gb_timestep* h);
/* prepare + compute + next with the host wall time in ms (fem_cuda.cu:92-101) */
SSIM_GB_API ssim_gb_status ssim_gb_step(ssim_gb_timestep* h, double* elapsed_ms);
SSIM_GB_API ssim_gb_status ssim_gb_restore(ssim_gb_timestep* h);
SSIM_GB_API ssim_gb_status ssim_gb_get_step_stats(const ssim_gb_timestep* h, ssim_gb_step_stats* st);
/* elastic model (the reference picks it as basic_time_step's ElastModel template argument); takes effect
 * immediately for every energy, gradient and Hessian evaluation */
SSIM_GB_API ssim_gb_status ssim_gb_set_elastic_model(ssim_gb_timestep* h, int32_t model);
/* NCG preconditioner factor L of SSIM_GB_STEPPER_NCG_EXT (x = L L^T g; timestep_ncg::set_matrix,
 * fem_cuda.cu:206): nnz values in the CSR order of ssim_gb_get_csr_pattern; NULL restores the identity,
 * which reset() installs (fem_cuda.cu:174-204).  Unlike the reference wrapper, whose solver never
 * receives the matrix (fem_cuda.cu:177-204 vs nonlinear_cg.hpp:73), the values set here are used. */
SSIM_GB_API ssim_gb_status ssim_gb_set_ncg_matrix(ssim_gb_timestep* h, const double* values);
/* PCG iteration counts of every solve since the last reset, oldest first: *count = number logged, the
 * first min(count, capacity) copied to iters (diagnostics; no reference counterpart) */
SSIM_GB_API ssim_gb_status ssim_gb_get_solve_log(const ssim_gb_timestep* h, int32_t* iters, int32_t capacity,
                                                 int32_t* count);
SSIM_GB_API ssim_gb_status ssim_gb_check_convergence(ssim_gb_timestep* h, int32_t* converged);
SSIM_GB_API ssim_gb_status ssim_gb_threshold_abs(const ssim_gb_timestep* h, double* abs_tol);

/* ---- energy / gradient / Hessian (time_step.hpp:577-658) ---- */
SSIM_GB_API ssim_gb_status ssim_gb_update_energy_and_gradients(ssim_gb_timestep* h, int32_t is_deform_grad_updated,
                                                   double* energy);
SSIM_GB_API ssim_gb_status ssim_gb_update_hessian(ssim_gb_timestep* h, int32_t is_deform_grad_updated, int32_t make_spsd,
                                      int32_t filter_dbc);
/* the incremental potential at an arbitrary displacement [V,3] (value only) */
SSIM_GB_API ssim_gb_status ssim_gb_energy_at(ssim_gb_timestep* h, const double* deform, double* energy);

/* ---- state and matrices (copies; views of time_step.hpp:275-311) ---- */
SSIM_GB_API ssim_gb_status ssim_gb_get_field(const ssim_gb_timestep* h, int32_t field, double* out /* [V,3] */);
SSIM_GB_API ssim_gb_status ssim_gb_set_field(ssim_gb_timestep* h, int32_t field, const double* in /* [V,3] */);
/* device address of a field ([V,3] float64 on the handle's device) for zero-copy interop */
SSIM_GB_API ssim_gb_status ssim_gb_field_device_ptr(ssim_gb_timestep* h, int32_t field, void** dptr);
SSIM_GB_API ssim_gb_status ssim_gb_get_csr_pattern(const ssim_gb_timestep* h, int32_t* row_ptr, int32_t* col_idx);
SSIM_GB_API ssim_gb_status ssim_gb_get_matrix_values(ssim_gb_timestep* h, int32_t which, double* values /* [nnz] */);
SSIM_GB_API ssim_gb_status ssim_gb_get_rest_volume(const ssim_gb_timestep* h, double* out /* [T] */);
SSIM_GB_API ssim_gb_status ssim_gb_get_dminv(const ssim_gb_timestep* h, double* out /* [T,3,3]; 2D: [T,2,2] */);
/* y = A x with the current system matrix (or mass) in the handle's precision, host buffers [V,3] */
SSIM_GB_API ssim_gb_status ssim_gb_spmv(ssim_gb_timestep* h, int32_t which, const double* x, double* y);
/* PCG on the current system matrix: x [V,3] in/out (initial guess zero if x_is_guess == 0) */
SSIM_GB_API ssim_gb_status ssim_gb_pcg(ssim_gb_timestep* h, const double* b, double* x, double rtol, int32_t max_iters,
                           int32_t* iters, double* rel_residual);

/* ---- batched instances (extension; e.g. 256 cubes of 4-24 hexes a side in one handle): the mesh handed
 * to ssim_gb_create is a disjoint union of independent meshes whose vertices occupy the contiguous ranges
 * vertex_offsets[i] ..
 * vertex_offsets[i+1]-1 (num_instances + 1 offsets, first 0, last V).  Every kernel runs over the whole
 * union; with stop_mode 1 each instance must meet |g_i| <= rel_tol |g_i0| on its own. */
SSIM_GB_API ssim_gb_status ssim_gb_set_instances(ssim_gb_timestep* h, const int32_t* vertex_offsets,
                                                 int32_t num_instances);
/* per-instance |g_i| of the last gradient and |g_i0| at the start of the last compute_step [num_instances] */
SSIM_GB_API ssim_gb_status ssim_gb_get_instance_residuals(ssim_gb_timestep* h, double* grad_norm, double* grad_norm0);

/* ---- adjoint of one backward-Euler step (extension: the reference has no differentiation) ----
 * The handle's next_deform must hold u_{n+1}, the state after forward step n.  ubar, vbar (device [V,3]
 * float64) hold dL/du_{n+1}, dL/dv_{n+1} on entry and dL/du_n, dL/dv_n on exit; ebar (device [T] float64)
 * accumulates dL/dE_e (Young's modulus per cell).  The linear solve H lambda = ubar uses the exact filtered
 * Hessian at u_{n+1} and PCG to rtol; *projected = 1 reports a fall-back to the SPD-projected Hessian. */
SSIM_GB_API ssim_gb_status ssim_gb_adjoint_step(ssim_gb_timestep* h, double* ubar, double* vbar, double* ebar,
                                                double rtol, int32_t max_iters, int32_t* cg_iters,
                                                int32_t* projected);
/* device-to-device copies of a field ([V,3] float64 device buffers), ordered on the handle's stream */
SSIM_GB_API ssim_gb_status ssim_gb_get_field_device(ssim_gb_timestep* h, int32_t field, double* dst);
SSIM_GB_API ssim_gb_status ssim_gb_set_field_device(ssim_gb_timestep* h, int32_t field, const double* src);

/* ---- allocation-free energy (no counterpart in the reference) ----
 * The incremental potential 1/2 |u - x~|^2_M + dt^2 sum_e V_e Psi(F_e) (the value update_energy_and_gradients
 * returns, time_step.hpp:577-624) of a tet mesh given entirely by caller-owned device arrays, computed
 * without allocating device memory.  For callers that cannot call cudaMalloc: code whose device memory is
 * all owned by another allocator (a framework's caching allocator, a fixed budget taken at start-up) or a
 * loop that must not pay an allocation's latency or risk its failure.
 * Inputs (device): X, u, x_tilde [V,3] float64; cells [T,4] int32, 16-byte aligned; dminv [T,3,3] (rows of
 * Dm^-1, ssim_gb_get_dminv's layout); rest_volume, lambda, mu [T].  Output: *energy_out (device, one
 * double), written on `stream` (a cudaStream_t; NULL = the legacy default stream).
 * Scratch: a fixed 64 KiB array inside the library, held by every GPU that loads it until the process
 * exits.  num_cells above SSIM_GB_NOALLOC_MAX_CELLS is rejected (SSIM_GB_ERR_INVALID_ARGUMENT).  The first
 * call on a device, and the first in each further CUDA context of it (a non-primary context, or the primary
 * context re-created after cudaDeviceReset), looks up that array's device address; make that first call
 * before any stream capture.
 * All calls share the array: calls that overlap on the GPU (different streams, or different host threads
 * without ordering) race and give wrong results; calls queued on one stream are safe. */
#define SSIM_GB_NOALLOC_MAX_CELLS (1 << 20)
SSIM_GB_API ssim_gb_status ssim_gb_energy_noalloc(const double* X, const double* u, const double* x_tilde,
                                                  const int32_t* cells, const double* dminv,
                                                  const double* rest_volume, const double* lambda_,
                                                  const double* mu, int32_t num_cells, double time_step,
                                                  double density, void* stream, double* energy_out);

/* ---- launch-shape autotuning (extension) ----
 * A one-time sweep on this handle's own data (call after reset(), between steps): the block sizes of the
 * FP32 element pass (64 / 128 / 256), the element Hessian (32 / 64 / 128), the assembly (128 / 256 / 512)
 * and the FP32 force gather (128 / 256 / 512), the persistent PCG's variant (mixed: standard or
 * Chronopoulos-Gear; FP64: two launches or Chronopoulos-Gear) and grid (one block per 256 rows or four per
 * SM), and the fused or two-kernel Hessian assembly.  Each candidate runs once untimed and then timed by
 * CUDA events on the handle's stream; the fastest is applied to the handle (the shapes, and pcg_persistent,
 * pcg_max_blocks, fused_assembly in its parameters).  The choice is cached for the process by (vertices,
 * cells, nonzero blocks, precision, instances, cell kind): a later handle of the same shape gets it without
 * timing (from_cache = 1).  The deformation and the other state are left as they were; the forces view is
 * restored. */
SSIM_GB_API ssim_gb_status ssim_gb_autotune(ssim_gb_timestep* h, ssim_gb_tuning* out);
/* Applies a tuning found earlier (by ssim_gb_autotune in this or another process) without timing anything:
 * elem_block in {0, 64, 128, 256}, hessian_block in {0, 32, 64, 128}, assembly_block and gather_block in
 * {0, 128, 256, 512} (0: the compiled default), pcg_persistent 0..4, pcg_max_blocks >= 0, fused_assembly,
 * pcg_half_matrix and elem_regcap 0 or 1; the timing and cache fields are ignored.  Anything else: SSIM_GB_ERR_INVALID_ARGUMENT, nothing
 * applied. */
SSIM_GB_API ssim_gb_status ssim_gb_set_tuning(ssim_gb_timestep* h, const ssim_gb_tuning* t);

/* ---- profiling (CUDA events on the handle's stream around the element, assembly and PCG launches) ---- */
SSIM_GB_API ssim_gb_status ssim_gb_profile_enable(ssim_gb_timestep* h, int32_t enable);
/* kernel: 0 = PCG SpMV, 1 = element Hessian, 2 = assembly, 3 = gradient element, 4 = PCG update (the
 * two-launch PCG), 5 = persistent PCG: launches = iterations, total_ms over all solves, bytes per iteration */
SSIM_GB_API ssim_gb_status ssim_gb_profile_read(ssim_gb_timestep* h, int32_t kernel, int64_t* launches, double* total_ms,
                                    double* bytes_per_launch);
SSIM_GB_API ssim_gb_status ssim_gb_synchronize(ssim_gb_timestep* h);

#ifdef __cplusplus
}
#endif
#endif
