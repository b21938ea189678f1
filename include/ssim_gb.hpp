/*
 * ssim_gb.hpp -- the C++ face of libssim_gb300.so: ssim::fem::basic_time_step's method names
 * (ssim/include/ssim/finite_elements/time_step.hpp:168-715) over the C ABI of ssim_gb.h.
 *
 * Header-only, C++17, no CUDA headers: a host program includes this file and links libssim_gb300.so.
 *
 *   ssim::fem::basic_time_step ts(vertices, nv, cells, nt, 1e-2, 1e5, 0.45, 1000.0);  // calls reset()
 *   ts.mark_dirichlet_batched(fixed, targets).add_gravity({0, 0, -9.8});
 *   ts.reset(ssim::fem::stepper::newton);
 *   ts.prepare_step(); double g = ts.compute_step(); ts.step_next();
 *   std::vector<double> u = ts.deformation();                                      // [V,3] copy
 *
 * Differences from the reference class, all forced by the device boundary:
 *  - the class is not a template: Scalar = double, Device = cuda, 3D tets (ssim_gb_create_2d and
 *    ssim_gb_create_springs remain reachable through handle());
 *  - the reference's views (deformation(), forces(), sysmatrix() ...) return host copies here (the Python
 *    bindings copy too, bindings/src/fem_cuda.cu:156-168); set_* writes them back;
 *  - the stepper is chosen by reset(stepper) instead of a solver object (time_step.hpp:363-494).
 * Errors: SSIM_GB_ERR_INVALID_ARGUMENT throws std::invalid_argument, as the reference does
 * (time_step.hpp:316-374,500-501,551-552); out of memory throws std::bad_alloc; every other failure throws
 * ssim::gb300::error (status() tells which), with the subclasses cuda_error, numerical_error, state_error,
 * device_timeout and not_converged.
 */
#ifndef SSIM_GB_HPP
#define SSIM_GB_HPP

#include <array>
#include <cstdint>
#include <initializer_list>
#include <new>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "ssim_gb.h"

namespace ssim {
namespace gb300 {

class error : public std::runtime_error {
 public:
  error(ssim_gb_status s, const std::string& msg) : std::runtime_error(msg), status_(s) {}
  ssim_gb_status status() const noexcept { return status_; }

 private:
  ssim_gb_status status_;
};
struct cuda_error : error {
  using error::error;
};
struct numerical_error : error {
  using error::error;
};
struct state_error : error {
  using error::error;
};
struct device_timeout : error {
  using error::error;
};
struct not_converged : error {
  using error::error;
};

// Turns a status into the exception a caller of the reference class would see (no-op for SSIM_GB_OK).
inline void throw_on_error(ssim_gb_status s, const ssim_gb_timestep* h = nullptr) {
  if (s == SSIM_GB_OK) return;
  const char* m = ssim_gb_last_error(h);
  const std::string msg = m ? m : "";
  switch (s) {
    case SSIM_GB_ERR_INVALID_ARGUMENT:
      throw std::invalid_argument(msg);
    case SSIM_GB_ERR_OUT_OF_MEMORY:
      throw std::bad_alloc();
    case SSIM_GB_ERR_CUDA:
      throw cuda_error(s, "CUDA error: " + msg);
    case SSIM_GB_ERR_NUMERICAL:
      throw numerical_error(s, msg);
    case SSIM_GB_ERR_STATE:
      throw state_error(s, msg);
    case SSIM_GB_ERR_DEVICE_TIMEOUT:
      throw device_timeout(s, msg);
    case SSIM_GB_ERR_NOT_CONVERGED:
      throw not_converged(s, msg);
    default:
      throw error(s, "status " + std::to_string(static_cast<int>(s)) + ": " + msg);
  }
}

inline ssim_gb_params default_params() {
  ssim_gb_params p;
  ssim_gb_default_params(&p);
  return p;
}

// A CSR matrix in the reference's layout: full storage, row_ptr [n+1], columns ascending per row.
struct csr_matrix {
  std::vector<int32_t> row_ptr, col_idx;
  std::vector<double> values;
};

// The Hessian pattern of a tet mesh (global_composer.hpp:68-100) on the host; no GPU needed.
inline csr_matrix mesh_csr_pattern(const int32_t* cells, int32_t num_cells, int32_t num_vertices) {
  int64_t nnz = 0;
  throw_on_error(ssim_gb_mesh_csr_nnz(cells, num_cells, num_vertices, &nnz));
  csr_matrix m;
  m.row_ptr.resize(3 * (size_t)num_vertices + 1);
  m.col_idx.resize((size_t)nnz);
  throw_on_error(ssim_gb_mesh_csr_pattern(cells, num_cells, num_vertices, m.row_ptr.data(), m.col_idx.data()));
  return m;
}

}  // namespace gb300

namespace fem {

// The steppers of stepper/backward_euler.hpp, stepper/projective_dynamics.hpp, stepper/nonlinear_cg.hpp
// and time_step.hpp:717-736, chosen at reset().
enum class stepper : int32_t {
  newton = SSIM_GB_STEPPER_NEWTON,
  lbfgs = SSIM_GB_STEPPER_LBFGS,
  pd = SSIM_GB_STEPPER_PD,
  none = SSIM_GB_STEPPER_NONE,
  forward_euler = SSIM_GB_STEPPER_FORWARD_EULER,
  h0 = SSIM_GB_STEPPER_H0,
  ncg = SSIM_GB_STEPPER_NCG,
  ncg_ext = SSIM_GB_STEPPER_NCG_EXT
};

// basic_time_step<double, cuda, 3, 4, stable_neohookean, ...> on the GPU: owns one library handle
// (move-only, like the reference object, time_step.hpp:259).
class basic_time_step {
 public:
  // basic_time_step(mesh, dt = 1e-3, E = 1e6, nu = 0.33, rho = 1e3) (time_step.hpp:260-265): vertices
  // [V,3] float64, cells [T,4] int32; the handle is reset on construction
  basic_time_step(const double* vertices, int32_t num_vertices, const int32_t* cells, int32_t num_cells,
                  double time_step = 1e-3, double youngs = 1e6, double poisson = 0.33, double density = 1e3) {
    gb300::throw_on_error(
        ssim_gb_create(vertices, num_vertices, cells, num_cells, time_step, youngs, poisson, density, &h_));
    nv_ = num_vertices;
    nt_ = num_cells;
  }
  basic_time_step(const std::vector<double>& vertices, const std::vector<int32_t>& cells, double time_step = 1e-3,
                  double youngs = 1e6, double poisson = 0.33, double density = 1e3)
      : basic_time_step(vertices.data(), static_cast<int32_t>(vertices.size() / 3), cells.data(),
                        static_cast<int32_t>(cells.size() / 4), time_step, youngs, poisson, density) {}
  basic_time_step(const basic_time_step&) = delete;
  basic_time_step& operator=(const basic_time_step&) = delete;
  basic_time_step(basic_time_step&& o) noexcept : h_(std::exchange(o.h_, nullptr)), nv_(o.nv_), nt_(o.nt_) {}
  basic_time_step& operator=(basic_time_step&& o) noexcept {
    if (this != &o) {
      if (h_) ssim_gb_destroy(h_);
      h_ = std::exchange(o.h_, nullptr);
      nv_ = o.nv_;
      nt_ = o.nt_;
    }
    return *this;
  }
  ~basic_time_step() {
    if (h_) ssim_gb_destroy(h_);
  }

  ssim_gb_timestep* handle() noexcept { return h_; }
  int32_t num_vertices() const noexcept { return nv_; }
  int32_t num_cells() const noexcept { return nt_; }

  // ---- setters (time_step.hpp:316-347), each returning *this; they take effect at the next reset()
  basic_time_step& set_time_step(double v) { return chk(ssim_gb_set_time_step(h_, v)); }
  basic_time_step& set_youngs(double v) { return chk(ssim_gb_set_youngs(h_, v)); }
  basic_time_step& set_poisson(double v) { return chk(ssim_gb_set_poisson(h_, v)); }
  basic_time_step& set_density(double v) { return chk(ssim_gb_set_density(h_, v)); }
  basic_time_step& set_damping(double v) { return chk(ssim_gb_set_damping(h_, v)); }
  basic_time_step& set_threshold(double v) { return chk(ssim_gb_set_threshold(h_, v)); }
  // extensions: precision of the Hessian / assembly / PCG, solver settings, per-cell material, stream
  basic_time_step& set_precision(ssim_gb_precision p) { return chk(ssim_gb_set_precision(h_, p)); }
  basic_time_step& set_params(const ssim_gb_params& p) { return chk(ssim_gb_set_params(h_, &p)); }
  ssim_gb_params params() const {
    ssim_gb_params p;
    gb300::throw_on_error(ssim_gb_get_params(h_, &p), h_);
    return p;
  }
  basic_time_step& set_material(const double* youngs_per_cell, const double* poisson_per_cell) {
    return chk(ssim_gb_set_material(h_, youngs_per_cell, poisson_per_cell));
  }
  basic_time_step& set_stream(void* cuda_stream) { return chk(ssim_gb_set_stream(h_, cuda_stream)); }

  // ---- boundary conditions and external acceleration (fem_cuda.cu:115-150, time_step.hpp:550-557)
  basic_time_step& mark_dirichlet_batched(const std::vector<int32_t>& verts, const std::vector<double>& targets) {
    if (targets.size() != 3 * verts.size()) throw std::invalid_argument("targets must hold [n,3] values");
    return chk(ssim_gb_mark_dirichlet_batched(h_, verts.data(), static_cast<int32_t>(verts.size()),
                                              targets.data()));
  }
  basic_time_step& mark_general_batched(const std::vector<int32_t>& verts) {
    return chk(ssim_gb_mark_general_batched(h_, verts.data(), static_cast<int32_t>(verts.size())));
  }
  basic_time_step& add_ext_force_dof(int32_t dof, double accel) { return chk(ssim_gb_add_ext_force_dof(h_, dof, accel)); }
  basic_time_step& add_gravity(const std::array<double, 3>& g) { return chk(ssim_gb_add_gravity(h_, g.data())); }

  // ---- the loop (time_step.hpp:363-569)
  basic_time_step& reset(stepper s = stepper::none) { return chk(ssim_gb_reset(h_, static_cast<int32_t>(s))); }
  basic_time_step& prepare_step() { return chk(ssim_gb_prepare_step(h_)); }
  // runs the stepper and returns |g| after it (time_step.hpp:520-528)
  double compute_step() {
    double r = 0;
    chk(ssim_gb_compute_step(h_, &r));
    return r;
  }
  basic_time_step& step_next() { return chk(ssim_gb_step_next(h_)); }
  basic_time_step& restore() { return chk(ssim_gb_restore(h_)); }
  // prepare_step + compute_step + step_next; returns the host wall time in ms (fem_cuda.cu:92-101)
  double step() {
    double ms = 0;
    chk(ssim_gb_step(h_, &ms));
    return ms;
  }
  ssim_gb_step_stats stats() const {
    ssim_gb_step_stats st;
    gb300::throw_on_error(ssim_gb_get_step_stats(h_, &st), h_);
    return st;
  }
  bool check_convergence() {
    int32_t c = 0;
    chk(ssim_gb_check_convergence(h_, &c));
    return c != 0;
  }
  double grad_convergence_threshold_abs() const {
    double t = 0;
    gb300::throw_on_error(ssim_gb_threshold_abs(h_, &t), h_);
    return t;
  }

  // ---- launch shapes (extension): sweep once, or apply a tuning saved from an earlier sweep
  ssim_gb_tuning autotune() {
    ssim_gb_tuning t{};
    chk(ssim_gb_autotune(h_, &t));
    return t;
  }
  basic_time_step& set_tuning(const ssim_gb_tuning& t) { return chk(ssim_gb_set_tuning(h_, &t)); }

  // ---- energy, gradient, Hessian (time_step.hpp:577-658)
  double update_energy_and_gradients(bool is_deform_grad_updated = false) {
    double e = 0;
    chk(ssim_gb_update_energy_and_gradients(h_, is_deform_grad_updated ? 1 : 0, &e));
    return e;
  }
  basic_time_step& update_hessian(bool is_deform_grad_updated = false, bool make_spsd = false, bool filter_dbc = true) {
    return chk(ssim_gb_update_hessian(h_, is_deform_grad_updated ? 1 : 0, make_spsd ? 1 : 0, filter_dbc ? 1 : 0));
  }

  // ---- state (copies of the reference's views, time_step.hpp:275-311): [V,3] float64 row-major
  std::vector<double> deformation() const { return field(SSIM_GB_DEFORMATION); }
  std::vector<double> prev_deform() const { return field(SSIM_GB_PREV_DEFORM); }
  std::vector<double> inertia_deform() const { return field(SSIM_GB_INERTIA_DEFORM); }
  std::vector<double> next_deform() const { return field(SSIM_GB_NEXT_DEFORM); }
  std::vector<double> velocity() const { return field(SSIM_GB_VELOCITY); }
  std::vector<double> ext_accel() const { return field(SSIM_GB_EXT_ACCEL); }
  std::vector<double> forces() const { return field(SSIM_GB_FORCES); }
  std::vector<double> dbc_values() const { return field(SSIM_GB_DBC_VALUES); }
  std::vector<double> field(ssim_gb_field f) const {
    std::vector<double> out(3 * (size_t)nv_);
    gb300::throw_on_error(ssim_gb_get_field(h_, f, out.data()), h_);
    return out;
  }
  basic_time_step& set_field(ssim_gb_field f, const std::vector<double>& v) {
    if (v.size() != 3 * (size_t)nv_) throw std::invalid_argument("a field holds [V,3] values");
    return chk(ssim_gb_set_field(h_, f, v.data()));
  }
  std::vector<double> rest_vol() const {
    std::vector<double> out((size_t)nt_);
    gb300::throw_on_error(ssim_gb_get_rest_volume(h_, out.data()), h_);
    return out;
  }
  std::vector<double> dminv() const {
    std::vector<double> out(9 * (size_t)nt_);
    gb300::throw_on_error(ssim_gb_get_dminv(h_, out.data()), h_);
    return out;
  }
  gb300::csr_matrix sysmatrix() { return matrix(SSIM_GB_SYSMATRIX); }
  gb300::csr_matrix mass_matrix() { return matrix(SSIM_GB_MASS); }
  gb300::csr_matrix mass_matrix_filtered() { return matrix(SSIM_GB_MASS_FILTERED); }

 private:
  basic_time_step& chk(ssim_gb_status s) {
    gb300::throw_on_error(s, h_);
    return *this;
  }
  gb300::csr_matrix matrix(ssim_gb_matrix which) {
    int32_t nv = 0, nc = 0, nd = 0;
    int64_t nnz = 0;
    chk(ssim_gb_sizes(h_, &nv, &nc, &nd, &nnz));
    gb300::csr_matrix m;
    m.row_ptr.resize((size_t)nd + 1);
    m.col_idx.resize((size_t)nnz);
    m.values.resize((size_t)nnz);
    chk(ssim_gb_get_csr_pattern(h_, m.row_ptr.data(), m.col_idx.data()));
    chk(ssim_gb_get_matrix_values(h_, which, m.values.data()));
    return m;
  }

  ssim_gb_timestep* h_ = nullptr;
  int32_t nv_ = 0, nt_ = 0;
};

}  // namespace fem
}  // namespace ssim

#endif
