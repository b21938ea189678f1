// A host program written against include/ssim_gb.hpp, as a user of ssim::fem::basic_time_step would write
// it (time_step.hpp:168-715).  Driven by tests/test_cpp_drop_in.py.
//   drop_in cpu                 -- no GPU: host-only utilities work, construction throws ssim::gb300::cuda_error,
//                                  an invalid argument maps to std::invalid_argument
//   drop_in gpu <in> <out> <n>  -- reads a scene (int32 V, T, nfixed; V*3 float64 vertices; T*4 int32 cells;
//                                  nfixed int32 vertex ids), steps it n times with Newton, writes the
//                                  deformation (V*3 float64) and checks the reference's argument errors
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <vector>

#include "ssim_gb.hpp"

static int fail(const char* what) {
  std::fprintf(stderr, "FAIL: %s\n", what);
  return 1;
}

static int run_cpu() {
  const ssim_gb_params p = ssim::gb300::default_params();
  if (p.max_newton_iters != 1000 || p.armijo != 0.3) return fail("default_params");
  // one tet: the pattern is the full 12 x 12 block
  const std::vector<int32_t> cells = {0, 1, 2, 3};
  const ssim::gb300::csr_matrix m = ssim::gb300::mesh_csr_pattern(cells.data(), 1, 4);
  if (m.row_ptr.size() != 13 || m.col_idx.size() != 144 || m.row_ptr.back() != 144) return fail("mesh_csr_pattern");
  try {
    ssim::gb300::throw_on_error(SSIM_GB_ERR_INVALID_ARGUMENT);
    return fail("invalid argument did not throw");
  } catch (const std::invalid_argument&) {
  }
  const std::vector<double> X = {0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1};
  try {
    ssim::fem::basic_time_step ts(X, cells, 1e-2);
    return fail("construction without a GPU did not throw");
  } catch (const ssim::gb300::cuda_error& e) {
    if (e.status() != SSIM_GB_ERR_CUDA) return fail("cuda_error status");
  }
  std::puts("cpu ok");
  return 0;
}

static int run_gpu(const char* in, const char* out, int steps) {
  std::ifstream f(in, std::ios::binary);
  int32_t hdr[3];
  f.read(reinterpret_cast<char*>(hdr), sizeof(hdr));
  std::vector<double> X(3 * (size_t)hdr[0]);
  std::vector<int32_t> cells(4 * (size_t)hdr[1]), fixed((size_t)hdr[2]);
  f.read(reinterpret_cast<char*>(X.data()), X.size() * sizeof(double));
  f.read(reinterpret_cast<char*>(cells.data()), cells.size() * sizeof(int32_t));
  f.read(reinterpret_cast<char*>(fixed.data()), fixed.size() * sizeof(int32_t));
  if (!f) return fail("reading the scene");

  ssim::fem::basic_time_step made(X, cells, 1e-2, 1e5, 0.45, 1000.0);
  ssim::fem::basic_time_step ts = std::move(made);  // move-only, like the reference object
  if (made.handle() != nullptr) return fail("moved-from handle");
  // the reference's argument checks (time_step.hpp:316-347)
  try {
    ts.set_poisson(0.5);
    return fail("set_poisson(0.5) did not throw");
  } catch (const std::invalid_argument&) {
  }
  try {
    ts.set_time_step(0.0);
    return fail("set_time_step(0) did not throw");
  } catch (const std::invalid_argument&) {
  }
  ssim_gb_params p = ssim::gb300::default_params();
  p.stop_mode = 1;
  p.rel_tol = 1e-10;
  p.cg_rtol = 1e-12;
  ts.mark_dirichlet_batched(fixed, std::vector<double>(3 * fixed.size(), 0.0))
      .add_gravity({0.0, 0.0, -9.8})
      .set_params(p)
      .reset(ssim::fem::stepper::newton);
  for (int s = 0; s < steps; ++s) {
    ts.prepare_step();
    const double g = ts.compute_step();
    ts.step_next();
    const ssim_gb_step_stats st = ts.stats();
    if (!st.converged || g != st.grad_norm) return fail("Newton step did not converge");
  }
  const std::vector<double> u = ts.deformation();
  const ssim::gb300::csr_matrix K = ts.sysmatrix();
  if ((int64_t)K.values.size() != K.row_ptr.back()) return fail("sysmatrix");
  std::ofstream o(out, std::ios::binary);
  o.write(reinterpret_cast<const char*>(u.data()), u.size() * sizeof(double));
  std::puts("gpu ok");
  return o ? 0 : fail("writing the state");
}

int main(int argc, char** argv) {
  try {
    if (argc >= 2 && std::strcmp(argv[1], "cpu") == 0) return run_cpu();
    if (argc >= 5 && std::strcmp(argv[1], "gpu") == 0) return run_gpu(argv[2], argv[3], std::atoi(argv[4]));
  } catch (const std::exception& e) {
    std::fprintf(stderr, "FAIL: uncaught %s\n", e.what());
    return 1;
  }
  return fail("usage: drop_in cpu | drop_in gpu <scene> <out> <steps>");
}
