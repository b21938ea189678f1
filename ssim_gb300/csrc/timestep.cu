// timestep.cu -- the C ABI of include/ssim_gb.h over the time-step object of timestep.cuh.
#include <initializer_list>
#include "timestep.cuh"

// ==================================================================== C ABI
using ssim_gb::TimeStep;

struct ssim_gb_timestep {
  TimeStep ts;
};

namespace {
thread_local std::string g_global_error;

}  // namespace

void ssim_gb::set_global_error(const std::string& msg) { g_global_error = msg; }

namespace {
ssim_gb_status fail(ssim_gb_timestep* h, ssim_gb_status s, const std::string& msg) {
  if (h)
    h->ts.last_error = msg;
  else
    g_global_error = msg;
  return s;
}
}  // namespace

#define API_TRY try {
#define API_CATCH(h)                                                                             \
  }                                                                                              \
  catch (const std::invalid_argument& e) {                                                       \
    return fail(h, SSIM_GB_ERR_INVALID_ARGUMENT, e.what());                                      \
  }                                                                                              \
  catch (const ssim_gb::state_error& e) {                                                        \
    return fail(h, SSIM_GB_ERR_STATE, e.what());                                                 \
  }                                                                                              \
  catch (const ssim_gb::numerical_error& e) {                                                    \
    return fail(h, SSIM_GB_ERR_NUMERICAL, e.what());                                             \
  }                                                                                              \
  catch (const ssim_gb::device_timeout& e) {                                                     \
    return fail(h, SSIM_GB_ERR_DEVICE_TIMEOUT, e.what());                                        \
  }                                                                                              \
  catch (const ssim_gb::cuda_error& e) {                                                         \
    return fail(h, SSIM_GB_ERR_CUDA, e.what());                                                  \
  }                                                                                              \
  catch (const std::bad_alloc&) {                                                                \
    return fail(h, SSIM_GB_ERR_OUT_OF_MEMORY, "out of memory");                                  \
  }                                                                                              \
  catch (const std::exception& e) {                                                              \
    return fail(h, SSIM_GB_ERR_CUDA, e.what());                                                  \
  }                                                                                              \
  return SSIM_GB_OK;

#define CHECK_H(h) \
  if (!(h)) return fail(nullptr, SSIM_GB_ERR_INVALID_ARGUMENT, "null handle");

static ssim_gb::DBuf<double>* field_buf(TimeStep& t, int f) {
  switch (f) {
    case SSIM_GB_DEFORMATION: return &t.deformation;
    case SSIM_GB_PREV_DEFORM: return &t.prev_deform;
    case SSIM_GB_INERTIA_DEFORM: return &t.inertia;
    case SSIM_GB_NEXT_DEFORM: return &t.next;
    case SSIM_GB_VELOCITY: return &t.velocity;
    case SSIM_GB_EXT_ACCEL: return &t.ext_accel;
    case SSIM_GB_FORCES: return &t.forces;
    case SSIM_GB_DBC_VALUES: return &t.dbc_values;
  }
  return nullptr;
}

template <typename S>
static void export_values(TimeStep& t, int which, double* out) {
  ssim_gb::Solver<S>& s = t.solver<S>();
  const S* src = s.vals.p;
  if (which == SSIM_GB_MASS || which == SSIM_GB_MASS_FILTERED) {
    s.mvals.alloc(9 * (size_t)t.topo.nslots);
    ssim_gb::launch_assemble<S>(t.A(), t.cptr.p, t.csrc.p, nullptr, s.slot_mass.p, t.mask.p,
                                which == SSIM_GB_MASS_FILTERED, s.mvals.p, nullptr, 0, t.stream);
    src = s.mvals.p;
  }
  t.csr_out.alloc(9 * (size_t)t.topo.nnzb);
  ssim_gb::launch_export_csr<S>(t.A(), t.bptr.p, t.slot_k.p, t.slot_kt.p, src, t.csr_out.p, t.stream);
  SSIM_CUDA(cudaMemcpyAsync(out, t.csr_out.p, sizeof(double) * 9 * t.topo.nnzb, cudaMemcpyDeviceToHost, t.stream));
  SSIM_CUDA(cudaStreamSynchronize(t.stream));
}

template <typename S>
static void do_spmv(TimeStep& t, int which, const double* x, double* y) {
  ssim_gb::Solver<S>& s = t.solver<S>();
  const S* vals = s.vals.p;
  if (which == SSIM_GB_MASS || which == SSIM_GB_MASS_FILTERED) {
    s.mvals.alloc(9 * (size_t)t.topo.nslots);
    ssim_gb::launch_assemble<S>(t.A(), t.cptr.p, t.csrc.p, nullptr, s.slot_mass.p, t.mask.p,
                                which == SSIM_GB_MASS_FILTERED, s.mvals.p, nullptr, 0, t.stream);
    vals = s.mvals.p;
  }
  SSIM_CUDA(cudaMemcpyAsync(t.work.p, x, sizeof(double) * t.n, cudaMemcpyHostToDevice, t.stream));
  ssim_gb::launch_to_vec4<S>(t.nv, t.work.p, s.tmp.p, false, t.stream);
  ssim_gb::launch_spmv<S>(t.A(), vals, s.tmp.p, s.q.p, t.stream);
  ssim_gb::launch_from_vec4<S>(t.nv, s.q.p, t.work.p, t.stream);
  SSIM_CUDA(cudaMemcpyAsync(y, t.work.p, sizeof(double) * t.n, cudaMemcpyDeviceToHost, t.stream));
  SSIM_CUDA(cudaStreamSynchronize(t.stream));
}

template <typename S>
static int do_pcg(TimeStep& t, const double* b, double* x, double rtol, int max_iters, double* rr) {
  SSIM_CUDA(cudaMemcpyAsync(t.work.p, b, sizeof(double) * t.n, cudaMemcpyHostToDevice, t.stream));
  const int it = t.pcg<S>(t.work.p, false, rtol, max_iters, rr);
  ssim_gb::launch_from_vec4<S>(t.nv, t.solver<S>().x.p, t.work.p, t.stream);
  SSIM_CUDA(cudaMemcpyAsync(x, t.work.p, sizeof(double) * t.n, cudaMemcpyDeviceToHost, t.stream));
  SSIM_CUDA(cudaStreamSynchronize(t.stream));
  return it;
}

extern "C" {

const char* ssim_gb_version(void) { return "ssim_gb300 0.1.0 (sm_103a)"; }

uint64_t ssim_gb_launch_count(void) { return ssim_gb::g_launches.load(); }

size_t ssim_gb_struct_size(int32_t which) {
  switch (which) {
    case 0: return sizeof(ssim_gb_params);
    case 1: return sizeof(ssim_gb_step_stats);
    case 2: return sizeof(ssim_gb_tuning);
    default: return 0;
  }
}

void ssim_gb_default_params(ssim_gb_params* p) {
  if (!p) return;
  p->max_newton_iters = 1000;
  p->armijo = 0.3;
  p->ls_shrink = 0.5;
  p->max_ls_iters = 30;
  p->cg_max_iters = 10000;
  p->cg_rtol = 1e-8;
  p->cg_forcing = 0;
  p->cg_eta_min = 1e-6;
  p->stop_mode = 0;
  p->rel_tol = 1e-6;
  p->precond = 1;
  p->lbfgs_history = 8;
  p->lbfgs_armijo = 1e-4;
  p->max_lbfgs_iters = 1000;
  p->cg_check_every = 8;
  p->ls_energy_slack = 1e-14;
  p->pd_kappa_mode = 0;
  p->pcg_persistent = 3;
  p->pcg_spin_limit = 0;
  p->pcg_barrier_extra = 0;
  p->pcg_max_blocks = 0;
  p->ncg_max_iters = 1000;
  p->ncg_step0 = 1e-2;
  p->ncg_eta = 0.5;
  p->ncg_expand = 3;
  p->stop_floor = 1e-12;
  p->mixed_elem32 = 1;
  p->ls_energy_slack32 = 1e-6;
  p->pcg_pipe_iters = 80;
  p->fused_assembly = 0;
  p->mixed_delta = 1;
  p->pcg_half_matrix = 1;
  p->half_matrix_min_rtol = 1e-2;
  p->half_hessian_blocks = 1;
  p->half_check_slack = 1.2;
  p->speculative_hessian = 0;
  p->elem32_switch = 10.0;
}

ssim_gb_status ssim_gb_mesh_csr_nnz(const int32_t* cells, int32_t nt, int32_t nv, int64_t* nnz) {
  API_TRY
  if (!cells || !nnz) throw ssim_gb::invalid_argument("null pointer");
  ssim_gb::Topology t;
  ssim_gb::build_topology(nv, nt, cells, t);
  *nnz = 9 * t.nnzb;
  API_CATCH(nullptr)
}

ssim_gb_status ssim_gb_mesh_csr_pattern(const int32_t* cells, int32_t nt, int32_t nv, int32_t* row_ptr,
                                        int32_t* col_idx) {
  API_TRY
  if (!cells || !row_ptr || !col_idx) throw ssim_gb::invalid_argument("null pointer");
  ssim_gb::Topology t;
  ssim_gb::build_topology(nv, nt, cells, t);
  ssim_gb::csr_pattern(t, row_ptr, col_idx);
  API_CATCH(nullptr)
}

const char* ssim_gb_last_error(const ssim_gb_timestep* h) {
  return h ? h->ts.last_error.c_str() : g_global_error.c_str();
}

ssim_gb_status ssim_gb_create(const double* vertices, int32_t num_vertices, const int32_t* cells, int32_t num_cells,
                              double time_step, double youngs, double poisson, double density,
                              ssim_gb_timestep** out) {
  if (!out) return fail(nullptr, SSIM_GB_ERR_INVALID_ARGUMENT, "null output handle");
  *out = nullptr;
  std::unique_ptr<ssim_gb_timestep> h(new ssim_gb_timestep());
  try {
    h->ts.create(vertices, num_vertices, cells, num_cells, time_step, youngs, poisson, density);
  } catch (const std::invalid_argument& e) {
    return fail(nullptr, SSIM_GB_ERR_INVALID_ARGUMENT, e.what());
  } catch (const ssim_gb::cuda_error& e) {
    return fail(nullptr, SSIM_GB_ERR_CUDA, e.what());
  } catch (const std::bad_alloc&) {
    return fail(nullptr, SSIM_GB_ERR_OUT_OF_MEMORY, "out of memory");
  } catch (const std::exception& e) {
    return fail(nullptr, SSIM_GB_ERR_CUDA, e.what());
  }
  *out = h.release();
  return SSIM_GB_OK;
}

ssim_gb_status ssim_gb_create_springs(const double* vertices, int32_t num_vertices, const int32_t* springs,
                                      int32_t num_springs, double stiffness, const double* vertex_mass,
                                      double mass, double time_step, ssim_gb_timestep** out) {
  if (!out) return fail(nullptr, SSIM_GB_ERR_INVALID_ARGUMENT, "null output handle");
  *out = nullptr;
  std::unique_ptr<ssim_gb_timestep> h(new ssim_gb_timestep());
  try {
    h->ts.create_springs(vertices, num_vertices, springs, num_springs, stiffness, vertex_mass, mass, time_step);
  } catch (const std::invalid_argument& e) {
    return fail(nullptr, SSIM_GB_ERR_INVALID_ARGUMENT, e.what());
  } catch (const ssim_gb::cuda_error& e) {
    return fail(nullptr, SSIM_GB_ERR_CUDA, e.what());
  } catch (const std::bad_alloc&) {
    return fail(nullptr, SSIM_GB_ERR_OUT_OF_MEMORY, "out of memory");
  } catch (const std::exception& e) {
    return fail(nullptr, SSIM_GB_ERR_CUDA, e.what());
  }
  *out = h.release();
  return SSIM_GB_OK;
}

ssim_gb_status ssim_gb_destroy(ssim_gb_timestep* h) {
  if (!h) return SSIM_GB_OK;
  if (h->ts.stream) cudaStreamSynchronize(h->ts.stream);
  delete h;
  return SSIM_GB_OK;
}

ssim_gb_status ssim_gb_create_2d(const double* vertices, int32_t num_vertices, const int32_t* triangles,
                                 int32_t num_triangles, double time_step, double youngs, double poisson,
                                 double density, ssim_gb_timestep** out) {
  if (!out) return fail(nullptr, SSIM_GB_ERR_INVALID_ARGUMENT, "null output handle");
  *out = nullptr;
  std::unique_ptr<ssim_gb_timestep> h(new ssim_gb_timestep());
  try {
    h->ts.create_2d(vertices, num_vertices, triangles, num_triangles, time_step, youngs, poisson, density);
  } catch (const std::invalid_argument& e) {
    return fail(nullptr, SSIM_GB_ERR_INVALID_ARGUMENT, e.what());
  } catch (const ssim_gb::cuda_error& e) {
    return fail(nullptr, SSIM_GB_ERR_CUDA, e.what());
  } catch (const std::bad_alloc&) {
    return fail(nullptr, SSIM_GB_ERR_OUT_OF_MEMORY, "out of memory");
  } catch (const std::exception& e) {
    return fail(nullptr, SSIM_GB_ERR_CUDA, e.what());
  }
  *out = h.release();
  return SSIM_GB_OK;
}

ssim_gb_status ssim_gb_get_dim(const ssim_gb_timestep* h, int32_t* dim) {
  CHECK_H(h);
  if (!dim) return fail(const_cast<ssim_gb_timestep*>(h), SSIM_GB_ERR_INVALID_ARGUMENT, "null output");
  *dim = h->ts.tri2d ? 2 : 3;
  return SSIM_GB_OK;
}

ssim_gb_status ssim_gb_sizes(const ssim_gb_timestep* h, int32_t* nv, int32_t* nt, int32_t* ndofs, int64_t* nnz) {
  CHECK_H(h);
  if (nv) *nv = h->ts.nv;
  if (nt) *nt = h->ts.nt;
  if (ndofs) *ndofs = h->ts.n;
  if (nnz) *nnz = 9 * h->ts.topo.nnzb;
  return SSIM_GB_OK;
}

ssim_gb_status ssim_gb_set_stream(ssim_gb_timestep* h, void* stream) {
  CHECK_H(h);
  API_TRY
  SSIM_CUDA(cudaStreamSynchronize(h->ts.stream));
  h->ts.stream = stream ? (cudaStream_t)stream : h->ts.own_stream;
  API_CATCH(h)
}

#define SETTER(name, field, cond, msg)                                       \
  ssim_gb_status name(ssim_gb_timestep* h, double v) {                       \
    CHECK_H(h);                                                              \
    if (!(cond)) return fail(h, SSIM_GB_ERR_INVALID_ARGUMENT, msg);          \
    h->ts.field = v;                                                         \
    return SSIM_GB_OK;                                                       \
  }
// time_step.hpp:316-347
SETTER(ssim_gb_set_time_step, dt, v > 0, "Time step must be positive.")
SETTER(ssim_gb_set_youngs, E, v > 0, "Young's modulus must be positive.")
SETTER(ssim_gb_set_poisson, nu, v > 0 && v < 0.5, "Poisson's ratio must be in (0, 0.5).")
SETTER(ssim_gb_set_density, rho, v > 0, "Density must be positive.")
SETTER(ssim_gb_set_damping, damping, 0 <= v && v < 1, "Damping must be in [0, 1).")
SETTER(ssim_gb_set_threshold, rtol, 0 < v && v < 1, "Threshold must be positive.")

ssim_gb_status ssim_gb_set_precision(ssim_gb_timestep* h, int32_t precision) {
  CHECK_H(h);
  if (precision != SSIM_GB_FP64 && precision != SSIM_GB_MIXED)
    return fail(h, SSIM_GB_ERR_INVALID_ARGUMENT, "precision must be SSIM_GB_FP64 or SSIM_GB_MIXED");
  if (precision != h->ts.precision) {
    h->ts.precision = precision;
    h->ts.has_reset = false;  // buffers of the other precision are allocated at reset()
  }
  return SSIM_GB_OK;
}

ssim_gb_status ssim_gb_set_params(ssim_gb_timestep* h, const ssim_gb_params* p) {
  CHECK_H(h);
  if (!p) return fail(h, SSIM_GB_ERR_INVALID_ARGUMENT, "null params");
  if (p->max_newton_iters < 0 || p->cg_max_iters < 0 || p->max_ls_iters < 1 || !(p->ls_shrink > 0 && p->ls_shrink < 1) ||
      !(p->ls_energy_slack >= 0) || p->precond < 0 || p->precond > 2 || p->pd_kappa_mode < 0 || p->pd_kappa_mode > 2 ||
      p->pcg_persistent < 0 || p->pcg_persistent > 4 || p->pcg_spin_limit < 0 || p->pcg_barrier_extra < 0 ||
      p->pcg_max_blocks < 0 || p->ncg_max_iters < 0 || !(p->ncg_step0 > 0) || !(p->ncg_eta >= 0) ||
      p->ncg_expand < 0 || !(p->stop_floor >= 0) || p->mixed_elem32 < 0 || p->mixed_elem32 > 1 ||
      !(p->ls_energy_slack32 >= 0) || !(p->elem32_switch >= 1) || p->pcg_pipe_iters < 0 || (p->fused_assembly != 0 && p->fused_assembly != 1) ||
      (p->mixed_delta != 0 && p->mixed_delta != 1) || (p->pcg_half_matrix != 0 && p->pcg_half_matrix != 1) ||
      !(p->half_matrix_min_rtol >= 0) || (p->half_hessian_blocks != 0 && p->half_hessian_blocks != 1) ||
      !(p->half_check_slack > 0) || (p->speculative_hessian != 0 && p->speculative_hessian != 1) ||
      !(p->cg_rtol >= 0) || p->cg_check_every < 1 || p->lbfgs_history < 1)
    return fail(h, SSIM_GB_ERR_INVALID_ARGUMENT, "invalid solver parameters");
  h->ts.params = *p;
  h->ts.half_off = false;
  return SSIM_GB_OK;
}

ssim_gb_status ssim_gb_get_params(const ssim_gb_timestep* h, ssim_gb_params* p) {
  CHECK_H(h);
  if (p) *p = h->ts.params;
  return SSIM_GB_OK;
}

ssim_gb_status ssim_gb_set_material(ssim_gb_timestep* h, const double* Ee, const double* ne) {
  CHECK_H(h);
  TimeStep& t = h->ts;
  if (t.springs) return fail(h, SSIM_GB_ERR_STATE, "a spring system has no elastic material");
  if (Ee) {
    for (int e = 0; e < t.nt; ++e)
      if (!(Ee[e] > 0)) return fail(h, SSIM_GB_ERR_INVALID_ARGUMENT, "Young's modulus must be positive.");
    t.E_elem.assign(Ee, Ee + t.nt);
  } else {
    t.E_elem.clear();
  }
  if (ne) {
    for (int e = 0; e < t.nt; ++e)
      if (!(ne[e] > 0 && ne[e] < 0.5)) return fail(h, SSIM_GB_ERR_INVALID_ARGUMENT, "Poisson's ratio must be in (0, 0.5).");
    t.nu_elem.assign(ne, ne + t.nt);
  } else {
    t.nu_elem.clear();
  }
  t.has_reset = false;
  return SSIM_GB_OK;
}

ssim_gb_status ssim_gb_mark_dirichlet_batched(ssim_gb_timestep* h, const int32_t* verts, int32_t n,
                                              const double* targ) {
  CHECK_H(h);
  API_TRY
  TimeStep& t = h->ts;
  if (n < 0 || (n > 0 && (!verts || !targ))) throw ssim_gb::invalid_argument("invalid vertex list");
  for (int i = 0; i < n; ++i)
    if (verts[i] < 0 || verts[i] >= t.nv) throw ssim_gb::invalid_argument("vertex index out of range");
  if (n == 0) return SSIM_GB_OK;
  if (t.mark_verts.n < (size_t)n) t.mark_verts.alloc(n);
  if (t.mark_targ.n < 3 * (size_t)n) t.mark_targ.alloc(3 * (size_t)n);
  // the caller's arrays are copied before the return; the upload and the marking run on the handle's
  // stream ahead of the next step without a host wait
  t.stage_marks(verts, targ, n);
  SSIM_CUDA(cudaMemcpyAsync(t.mark_verts.p, t.mark_verts_h, sizeof(int32_t) * n, cudaMemcpyHostToDevice, t.stream));
  SSIM_CUDA(cudaMemcpyAsync(t.mark_targ.p, t.mark_targ_h, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, t.stream));
  SSIM_CUDA(cudaEventRecord(t.ev_mark, t.stream));
  t.mark_in_flight = true;
  ssim_gb::launch_mark_dofs(n, t.mark_verts.p, t.mark_targ.p, 1, t.dof_type.p, t.dbc_values.p, t.stream);
  ssim_gb::launch_build_mask(t.nv, t.dof_type.p, t.mask.p, t.stream);
  API_CATCH(h)
}

ssim_gb_status ssim_gb_mark_general_batched(ssim_gb_timestep* h, const int32_t* verts, int32_t n) {
  CHECK_H(h);
  API_TRY
  TimeStep& t = h->ts;
  if (n < 0 || (n > 0 && !verts)) throw ssim_gb::invalid_argument("invalid vertex list");
  for (int i = 0; i < n; ++i)
    if (verts[i] < 0 || verts[i] >= t.nv) throw ssim_gb::invalid_argument("vertex index out of range");
  if (n == 0) return SSIM_GB_OK;
  if (t.mark_verts.n < (size_t)n) t.mark_verts.alloc(n);
  SSIM_CUDA(cudaMemcpyAsync(t.mark_verts.p, verts, sizeof(int32_t) * n, cudaMemcpyHostToDevice, t.stream));
  ssim_gb::launch_mark_dofs(n, t.mark_verts.p, nullptr, 0, t.dof_type.p, t.dbc_values.p, t.stream);
  ssim_gb::launch_build_mask(t.nv, t.dof_type.p, t.mask.p, t.stream);
  SSIM_CUDA(cudaStreamSynchronize(t.stream));
  API_CATCH(h)
}

ssim_gb_status ssim_gb_set_dof_type(ssim_gb_timestep* h, const int8_t* types) {
  CHECK_H(h);
  API_TRY
  TimeStep& t = h->ts;
  if (!types) throw ssim_gb::invalid_argument("null dof types");
  for (int i = 0; i < t.n; ++i)
    if (types[i] != 0 && types[i] != 1) throw ssim_gb::invalid_argument("dof type must be 0 (general) or 1 (dirichlet)");
  SSIM_CUDA(cudaMemcpyAsync(t.dof_type.p, types, t.n, cudaMemcpyHostToDevice, t.stream));
  ssim_gb::launch_build_mask(t.nv, t.dof_type.p, t.mask.p, t.stream);
  SSIM_CUDA(cudaStreamSynchronize(t.stream));
  API_CATCH(h)
}

ssim_gb_status ssim_gb_get_dof_type(const ssim_gb_timestep* hc, int8_t* types) {
  ssim_gb_timestep* h = const_cast<ssim_gb_timestep*>(hc);
  CHECK_H(h);
  API_TRY
  if (!types) throw ssim_gb::invalid_argument("null output");
  SSIM_CUDA(cudaMemcpyAsync(types, h->ts.dof_type.p, h->ts.n, cudaMemcpyDeviceToHost, h->ts.stream));
  SSIM_CUDA(cudaStreamSynchronize(h->ts.stream));
  API_CATCH(h)
}

ssim_gb_status ssim_gb_add_ext_force_dof(ssim_gb_timestep* h, int32_t dof, double a) {
  CHECK_H(h);
  API_TRY
  // time_step.hpp:550-557
  if (!(-3 < dof && dof < 3)) throw ssim_gb::invalid_argument("|dof_idx| must be less than PhysicalDim.");
  if (dof < 0) dof += 3;
  ssim_gb::launch_add_ext(h->ts.nv, dof, a, h->ts.ext_accel.p, h->ts.stream);
  API_CATCH(h)
}

ssim_gb_status ssim_gb_add_gravity(ssim_gb_timestep* h, const double g[3]) {
  CHECK_H(h);
  if (!g) return fail(h, SSIM_GB_ERR_INVALID_ARGUMENT, "null gravity");
  for (int d = 0; d < 3; ++d) {
    ssim_gb_status s = ssim_gb_add_ext_force_dof(h, d, g[d]);
    if (s != SSIM_GB_OK) return s;
  }
  return SSIM_GB_OK;
}

ssim_gb_status ssim_gb_reset(ssim_gb_timestep* h, int32_t stepper) {
  CHECK_H(h);
  API_TRY
  h->ts.reset(stepper);
  API_CATCH(h)
}

ssim_gb_status ssim_gb_prepare_step(ssim_gb_timestep* h) {
  CHECK_H(h);
  API_TRY
  TimeStep& t = h->ts;
  if (!t.has_reset) {
    // fem_cuda.cu:78-86: the wrapper resets with a warning when prepare_step comes first
    fprintf(stderr, "Warning: prepare_step() called before reset(), bad logic.\n");
    t.reset(t.stepper);
  }
  t.prepare_step();
  API_CATCH(h)
}

ssim_gb_status ssim_gb_compute_step(ssim_gb_timestep* h, double* residual) {
  CHECK_H(h);
  API_TRY
  const double r = h->ts.compute_step();
  if (residual) *residual = r;
  API_CATCH(h)
}

ssim_gb_status ssim_gb_step_next(ssim_gb_timestep* h) {
  CHECK_H(h);
  API_TRY
  h->ts.step_next();
  API_CATCH(h)
}

ssim_gb_status ssim_gb_step(ssim_gb_timestep* h, double* elapsed_ms) {
  CHECK_H(h);
  const auto t0 = std::chrono::high_resolution_clock::now();
  ssim_gb_status s = ssim_gb_prepare_step(h);
  if (s != SSIM_GB_OK) return s;
  s = ssim_gb_compute_step(h, nullptr);
  if (s != SSIM_GB_OK) return s;
  s = ssim_gb_step_next(h);
  if (s != SSIM_GB_OK) return s;
  API_TRY
  SSIM_CUDA(cudaStreamSynchronize(h->ts.stream));
  const auto t1 = std::chrono::high_resolution_clock::now();
  if (elapsed_ms) *elapsed_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  API_CATCH(h)
}

ssim_gb_status ssim_gb_restore(ssim_gb_timestep* h) {
  CHECK_H(h);
  API_TRY
  h->ts.restore();
  API_CATCH(h)
}

ssim_gb_status ssim_gb_get_step_stats(const ssim_gb_timestep* h, ssim_gb_step_stats* st) {
  CHECK_H(h);
  if (st) *st = h->ts.stats;
  return SSIM_GB_OK;
}

ssim_gb_status ssim_gb_set_elastic_model(ssim_gb_timestep* h, int32_t model) {
  CHECK_H(h);
  if (model != SSIM_GB_MODEL_STABLE_NEOHOOKEAN && model != SSIM_GB_MODEL_LINEAR)
    return fail(h, SSIM_GB_ERR_INVALID_ARGUMENT, "unknown elastic model");
  h->ts.elastic_model = model;
  return SSIM_GB_OK;
}

ssim_gb_status ssim_gb_set_ncg_matrix(ssim_gb_timestep* h, const double* values) {
  CHECK_H(h);
  API_TRY
  h->ts.set_ncg_matrix(values);
  API_CATCH(h)
}

ssim_gb_status ssim_gb_get_solve_log(const ssim_gb_timestep* h, int32_t* iters, int32_t capacity, int32_t* count) {
  CHECK_H(h);
  const auto& log = h->ts.solve_log;
  if (count) *count = (int32_t)log.size();
  if (iters && capacity > 0)
    std::copy(log.begin(), log.begin() + std::min<size_t>(log.size(), (size_t)capacity), iters);
  return SSIM_GB_OK;
}

ssim_gb_status ssim_gb_check_convergence(ssim_gb_timestep* h, int32_t* converged) {
  CHECK_H(h);
  API_TRY
  // time_step.hpp:660-664, on the forces of the last evaluation
  TimeStep& t = h->ts;
  std::vector<double> f(t.n);
  SSIM_CUDA(cudaMemcpyAsync(f.data(), t.forces.p, sizeof(double) * t.n, cudaMemcpyDeviceToHost, t.stream));
  SSIM_CUDA(cudaStreamSynchronize(t.stream));
  double s = 0;
  for (double v : f) s += v * v;
  if (converged) *converged = std::sqrt(s) < t.abs_tol ? 1 : 0;
  API_CATCH(h)
}

ssim_gb_status ssim_gb_threshold_abs(const ssim_gb_timestep* h, double* abs_tol) {
  CHECK_H(h);
  if (abs_tol) *abs_tol = h->ts.abs_tol;
  return SSIM_GB_OK;
}

ssim_gb_status ssim_gb_update_energy_and_gradients(ssim_gb_timestep* h, int32_t, double* energy) {
  CHECK_H(h);
  API_TRY
  const double E = h->ts.energy_grad();
  if (energy) *energy = E;
  API_CATCH(h)
}

ssim_gb_status ssim_gb_update_hessian(ssim_gb_timestep* h, int32_t, int32_t make_spsd, int32_t filter_dbc) {
  CHECK_H(h);
  API_TRY
  if (!h->ts.has_reset) throw ssim_gb::state_error("update_hessian() before reset()");
  h->ts.hessian_any(make_spsd != 0, filter_dbc != 0);
  SSIM_CUDA(cudaStreamSynchronize(h->ts.stream));
  API_CATCH(h)
}

ssim_gb_status ssim_gb_energy_at(ssim_gb_timestep* h, const double* deform, double* energy) {
  CHECK_H(h);
  API_TRY
  TimeStep& t = h->ts;
  if (!deform) throw ssim_gb::invalid_argument("null deformation");
  SSIM_CUDA(cudaMemcpyAsync(t.work.p, deform, sizeof(double) * t.n, cudaMemcpyHostToDevice, t.stream));
  const double E = t.energy_at(t.work.p);
  if (energy) *energy = E;
  API_CATCH(h)
}


ssim_gb_status ssim_gb_get_field(const ssim_gb_timestep* hc, int32_t field, double* out) {
  ssim_gb_timestep* h = const_cast<ssim_gb_timestep*>(hc);
  CHECK_H(h);
  API_TRY
  auto* b = field_buf(h->ts, field);
  if (!b || !out) throw ssim_gb::invalid_argument("unknown field or null output");
  SSIM_CUDA(cudaMemcpyAsync(out, b->p, sizeof(double) * h->ts.n, cudaMemcpyDeviceToHost, h->ts.stream));
  SSIM_CUDA(cudaStreamSynchronize(h->ts.stream));
  API_CATCH(h)
}

ssim_gb_status ssim_gb_set_field(ssim_gb_timestep* h, int32_t field, const double* in) {
  CHECK_H(h);
  API_TRY
  auto* b = field_buf(h->ts, field);
  if (!b || !in) throw ssim_gb::invalid_argument("unknown field or null input");
  SSIM_CUDA(cudaMemcpyAsync(b->p, in, sizeof(double) * h->ts.n, cudaMemcpyHostToDevice, h->ts.stream));
  SSIM_CUDA(cudaStreamSynchronize(h->ts.stream));
  API_CATCH(h)
}

ssim_gb_status ssim_gb_field_device_ptr(ssim_gb_timestep* h, int32_t field, void** dptr) {
  CHECK_H(h);
  auto* b = field_buf(h->ts, field);
  if (!b || !dptr) return fail(h, SSIM_GB_ERR_INVALID_ARGUMENT, "unknown field or null output");
  *dptr = b->p;
  return SSIM_GB_OK;
}

ssim_gb_status ssim_gb_get_csr_pattern(const ssim_gb_timestep* h, int32_t* row_ptr, int32_t* col_idx) {
  CHECK_H(h);
  if (!row_ptr || !col_idx) return fail(const_cast<ssim_gb_timestep*>(h), SSIM_GB_ERR_INVALID_ARGUMENT, "null output");
  ssim_gb::csr_pattern(h->ts.topo, row_ptr, col_idx);
  return SSIM_GB_OK;
}


ssim_gb_status ssim_gb_get_matrix_values(ssim_gb_timestep* h, int32_t which, double* values) {
  CHECK_H(h);
  API_TRY
  TimeStep& t = h->ts;
  if (!values || which < 0 || which > 2) throw ssim_gb::invalid_argument("invalid matrix or null output");
  if (!t.has_reset) throw ssim_gb::state_error("matrix values before reset()");
  if (t.mixed())
    export_values<float>(t, which, values);
  else
    export_values<double>(t, which, values);
  API_CATCH(h)
}

ssim_gb_status ssim_gb_get_csr_2d(ssim_gb_timestep* h, int32_t which, int32_t* row_ptr, int32_t* col_idx,
                                  double* values) {
  CHECK_H(h);
  API_TRY
  TimeStep& t = h->ts;
  if (!t.tri2d) throw ssim_gb::state_error("the 2-dof CSR is for 2D handles");
  if (which < 0 || which > 2) throw ssim_gb::invalid_argument("invalid matrix");
  const ssim_gb::Topology& tp = t.topo;
  // 3-dof row 3u+a starts at 9 bptr[u] + 3 deg(u) a; 2-dof row 2u+a at 4 bptr[u] + 2 deg(u) a
  std::vector<double> v3;
  if (values) {
    if (!t.has_reset) throw ssim_gb::state_error("matrix values before reset()");
    v3.resize(9 * (size_t)tp.nnzb);
    if (t.mixed())
      export_values<float>(t, which, v3.data());
    else
      export_values<double>(t, which, v3.data());
  }
  for (int u = 0; u < t.nv; ++u) {
    const int deg = tp.bptr[u + 1] - tp.bptr[u];
    for (int a = 0; a < 2; ++a) {
      const long long r2 = 4LL * tp.bptr[u] + 2LL * deg * a, r3 = 9LL * tp.bptr[u] + 3LL * deg * a;
      if (row_ptr) row_ptr[2 * u + a] = (int32_t)r2;
      for (int k = 0; k < deg; ++k)
        for (int b = 0; b < 2; ++b) {
          if (col_idx) col_idx[r2 + 2 * k + b] = 2 * tp.bcol[tp.bptr[u] + k] + b;
          if (values) values[r2 + 2 * k + b] = v3[r3 + 3 * k + b];
        }
    }
  }
  if (row_ptr) row_ptr[2 * t.nv] = (int32_t)(4 * tp.nnzb);
  API_CATCH(h)
}

ssim_gb_status ssim_gb_get_rest_volume(const ssim_gb_timestep* h, double* out) {
  CHECK_H(h);
  if (!out) return fail(const_cast<ssim_gb_timestep*>(h), SSIM_GB_ERR_INVALID_ARGUMENT, "null output");
  if (h->ts.springs) return fail(const_cast<ssim_gb_timestep*>(h), SSIM_GB_ERR_STATE, "a spring system has no cells");
  std::copy(h->ts.vol_h.begin(), h->ts.vol_h.end(), out);
  return SSIM_GB_OK;
}

ssim_gb_status ssim_gb_get_dminv(const ssim_gb_timestep* hc, double* out) {
  ssim_gb_timestep* h = const_cast<ssim_gb_timestep*>(hc);
  CHECK_H(h);
  API_TRY
  TimeStep& t = h->ts;
  if (!out) throw ssim_gb::invalid_argument("null output");
  if (t.springs) throw ssim_gb::state_error("a spring system has no cells");
  std::vector<double> soa(9 * (size_t)t.nt);
  SSIM_CUDA(cudaMemcpyAsync(soa.data(), t.dminv.p, sizeof(double) * soa.size(), cudaMemcpyDeviceToHost, t.stream));
  SSIM_CUDA(cudaStreamSynchronize(t.stream));
  const int per = t.tri2d ? 4 : 9;
  for (int e = 0; e < t.nt; ++e)
    for (int k = 0; k < per; ++k) out[per * (size_t)e + k] = soa[(size_t)k * t.nt + e];
  API_CATCH(h)
}


ssim_gb_status ssim_gb_spmv(ssim_gb_timestep* h, int32_t which, const double* x, double* y) {
  CHECK_H(h);
  API_TRY
  TimeStep& t = h->ts;
  if (!x || !y || which < 0 || which > 3) throw ssim_gb::invalid_argument("invalid matrix or null buffer");
  if (!t.has_reset) throw ssim_gb::state_error("spmv before reset()");
  if (which == SSIM_GB_SYSMATRIX_HALF) {
    if (!t.mixed()) throw ssim_gb::invalid_argument("the FP16 system matrix exists in mixed precision only");
    if (!t.half_ready()) throw ssim_gb::invalid_argument("the pattern does not fit the FP16 matrix's indices");
    t.half_refresh();
    ssim_gb::Solver<float>& s = t.sf;
    SSIM_CUDA(cudaMemcpyAsync(t.work.p, x, sizeof(double) * t.n, cudaMemcpyHostToDevice, t.stream));
    ssim_gb::launch_to_vec4<float>(t.nv, t.work.p, s.tmp.p, false, t.stream);
    ssim_gb::launch_half_spmv(t.half_matrix(), s.tmp.p, s.r.p, s.q.p, t.stream);
    ssim_gb::launch_from_vec4<float>(t.nv, s.q.p, t.work.p, t.stream);
    SSIM_CUDA(cudaMemcpyAsync(y, t.work.p, sizeof(double) * t.n, cudaMemcpyDeviceToHost, t.stream));
    SSIM_CUDA(cudaStreamSynchronize(t.stream));
    return SSIM_GB_OK;
  }
  if (t.mixed())
    do_spmv<float>(t, which, x, y);
  else
    do_spmv<double>(t, which, x, y);
  API_CATCH(h)
}


ssim_gb_status ssim_gb_pcg(ssim_gb_timestep* h, const double* b, double* x, double rtol, int32_t max_iters,
                           int32_t* iters, double* rel_residual) {
  CHECK_H(h);
  API_TRY
  TimeStep& t = h->ts;
  if (!b || !x) throw ssim_gb::invalid_argument("null buffer");
  if (!t.has_reset) throw ssim_gb::state_error("pcg before reset()");
  double rr = 0;
  const int it = t.mixed() ? do_pcg<float>(t, b, x, rtol, max_iters, &rr) : do_pcg<double>(t, b, x, rtol, max_iters, &rr);
  if (iters) *iters = it;
  if (rel_residual) *rel_residual = rr;
  API_CATCH(h)
}

ssim_gb_status ssim_gb_set_instances(ssim_gb_timestep* h, const int32_t* vertex_offsets, int32_t num_instances) {
  CHECK_H(h);
  API_TRY
  TimeStep& t = h->ts;
  if (num_instances < 0 || (num_instances > 0 && !vertex_offsets)) throw ssim_gb::invalid_argument("invalid instances");
  if (num_instances > 0) {
    if (vertex_offsets[0] != 0 || vertex_offsets[num_instances] != t.nv)
      throw ssim_gb::invalid_argument("instance offsets must run from 0 to the number of vertices");
    for (int i = 0; i < num_instances; ++i)
      if (vertex_offsets[i + 1] <= vertex_offsets[i]) throw ssim_gb::invalid_argument("instance offsets must increase");
  }
  t.ninst = num_instances;
  t.inst_off_h.assign(vertex_offsets, vertex_offsets + (num_instances > 0 ? num_instances + 1 : 0));
  t.inst_off.upload(t.inst_off_h, t.stream);
  t.inst_g2.alloc(std::max(1, num_instances));
  t.inst_g2_h.assign(std::max(1, num_instances), 0.0);
  t.inst_g0_h.assign(std::max(1, num_instances), 0.0);
  t.instance_masses();
  SSIM_CUDA(cudaStreamSynchronize(t.stream));
  API_CATCH(h)
}

ssim_gb_status ssim_gb_get_instance_residuals(ssim_gb_timestep* h, double* grad_norm, double* grad_norm0) {
  CHECK_H(h);
  API_TRY
  TimeStep& t = h->ts;
  if (t.ninst <= 0) throw ssim_gb::state_error("no instances set");
  t.instance_norms();
  for (int i = 0; i < t.ninst; ++i) {
    if (grad_norm) grad_norm[i] = std::sqrt(t.inst_g2_h[i]);
    if (grad_norm0) grad_norm0[i] = t.inst_g0_h[i];
  }
  API_CATCH(h)
}

ssim_gb_status ssim_gb_adjoint_step(ssim_gb_timestep* h, double* ubar, double* vbar, double* ebar, double rtol,
                                    int32_t max_iters, int32_t* cg_iters, int32_t* projected) {
  CHECK_H(h);
  API_TRY
  TimeStep& t = h->ts;
  if (!ubar || !vbar || !ebar) throw ssim_gb::invalid_argument("null adjoint buffer");
  if (!(rtol > 0) || max_iters <= 0) throw ssim_gb::invalid_argument("invalid adjoint solve tolerance");
  if (!t.has_reset) throw ssim_gb::state_error("adjoint_step() before reset()");
  if (t.springs || t.tri2d) throw ssim_gb::state_error("the adjoint is built for the tet models");
  int proj = 0;
  const int it = t.mixed() ? t.adjoint_step<float>(ubar, vbar, ebar, rtol, max_iters, &proj)
                           : t.adjoint_step<double>(ubar, vbar, ebar, rtol, max_iters, &proj);
  if (cg_iters) *cg_iters = it;
  if (projected) *projected = proj;
  API_CATCH(h)
}

ssim_gb_status ssim_gb_autotune(ssim_gb_timestep* h, ssim_gb_tuning* out) {
  CHECK_H(h);
  API_TRY
  const ssim_gb_tuning r = h->ts.autotune();
  if (out) *out = r;
  API_CATCH(h)
}

ssim_gb_status ssim_gb_set_tuning(ssim_gb_timestep* h, const ssim_gb_tuning* t) {
  CHECK_H(h);
  if (!t) return fail(h, SSIM_GB_ERR_INVALID_ARGUMENT, "null tuning");
  auto one_of = [](int v, std::initializer_list<int> set) {
    for (int x : set)
      if (v == x) return true;
    return false;
  };
  if (!one_of(t->elem_block, {0, 64, 128, 256}) || !one_of(t->hessian_block, {0, 32, 64, 128}) ||
      !one_of(t->assembly_block, {0, 128, 256, 512}) || !one_of(t->gather_block, {0, 128, 256, 512}) ||
      t->pcg_persistent < 0 || t->pcg_persistent > 4 || t->pcg_max_blocks < 0 ||
      (t->fused_assembly != 0 && t->fused_assembly != 1) || (t->pcg_half_matrix != 0 && t->pcg_half_matrix != 1) ||
      (t->elem_regcap != 0 && t->elem_regcap != 1))
    return fail(h, SSIM_GB_ERR_INVALID_ARGUMENT, "invalid tuning (block size outside its candidate set)");
  h->ts.apply_tuning(*t);
  return SSIM_GB_OK;
}

ssim_gb_status ssim_gb_get_field_device(ssim_gb_timestep* h, int32_t field, double* dst) {
  CHECK_H(h);
  API_TRY
  auto* b = field_buf(h->ts, field);
  if (!b || !dst) throw ssim_gb::invalid_argument("unknown field or null output");
  SSIM_CUDA(cudaMemcpyAsync(dst, b->p, sizeof(double) * h->ts.n, cudaMemcpyDeviceToDevice, h->ts.stream));
  SSIM_CUDA(cudaStreamSynchronize(h->ts.stream));
  API_CATCH(h)
}

ssim_gb_status ssim_gb_set_field_device(ssim_gb_timestep* h, int32_t field, const double* src) {
  CHECK_H(h);
  API_TRY
  auto* b = field_buf(h->ts, field);
  if (!b || !src) throw ssim_gb::invalid_argument("unknown field or null input");
  SSIM_CUDA(cudaMemcpyAsync(b->p, src, sizeof(double) * h->ts.n, cudaMemcpyDeviceToDevice, h->ts.stream));
  SSIM_CUDA(cudaStreamSynchronize(h->ts.stream));
  API_CATCH(h)
}

ssim_gb_status ssim_gb_profile_enable(ssim_gb_timestep* h, int32_t enable) {
  CHECK_H(h);
  API_TRY
  h->ts.set_profiling(enable != 0);
  API_CATCH(h)
}

ssim_gb_status ssim_gb_profile_read(ssim_gb_timestep* h, int32_t kernel, int64_t* launches, double* total_ms,
                                    double* bytes_per_launch) {
  CHECK_H(h);
  if (kernel < 0 || kernel >= ssim_gb::PK_COUNT) return fail(h, SSIM_GB_ERR_INVALID_ARGUMENT, "unknown kernel id");
  if (launches) *launches = h->ts.prof_launch[kernel];
  if (total_ms) *total_ms = h->ts.prof_ms[kernel];
  if (bytes_per_launch) *bytes_per_launch = h->ts.prof_bytes[kernel];
  return SSIM_GB_OK;
}

ssim_gb_status ssim_gb_synchronize(ssim_gb_timestep* h) {
  CHECK_H(h);
  API_TRY
  SSIM_CUDA(cudaStreamSynchronize(h->ts.stream));
  API_CATCH(h)
}

}  // extern "C"
