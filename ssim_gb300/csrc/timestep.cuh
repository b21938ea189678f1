// timestep.cuh -- the time-step object (ssim::fem::basic_time_step, time_step.hpp:168-715, Device = cuda)
// with its steppers, driving the kernels of kernels_*.cu; the C ABI over it is timestep.cu.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <type_traits>
#include <vector>

#include "../../include/ssim_gb.h"
#include "elem_math.cuh"
#include "kernels.cuh"
#include "topology.h"

namespace ssim_gb {

// ------------------------------------------------------------------ device buffer
template <typename T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  DBuf() = default;
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  ~DBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  void alloc(size_t count) {
    if (count == n && p) return;
    release();
    if (count == 0) return;
    SSIM_CUDA(cudaMalloc((void**)&p, count * sizeof(T)));
    n = count;
  }
  void zero(cudaStream_t st) {
    if (p) SSIM_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), st));
  }
  void upload(const T* h, size_t count, cudaStream_t st) {
    alloc(count);
    if (count) SSIM_CUDA(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, st));
  }
  void upload(const std::vector<T>& v, cudaStream_t st) { upload(v.data(), v.size(), st); }
};

template <typename S>
struct Solver {
  DBuf<S> K, vals, mvals;  // element blocks, system values, mass values (SELL)
  DBuf<uint2> K16;         // element blocks in FP16 (launch_elem_hessian16), mixed Newton only
  DBuf<S> slot_mass;
  DBuf<V4<S>> x, r, z, p0, p1, q, dinv, tmp;
  DBuf<V4<S>> pm;  // the pipelined PCG's double-buffered m = M w (2 nv), allocated on first use
  // L-BFGS / PD: direction, two-loop work vector, history ring, PD matrix and its preconditioner
  DBuf<V4<S>> ld, lq;
  std::vector<std::unique_ptr<DBuf<V4<S>>>> hs, hy;
  DBuf<S> pd_vals, slot_pd;
  DBuf<S> pd_svals;      // the PD matrix as (scalar) (x) I3: one value per slot, when its blocks allow
  bool pd_kron = false;
  DBuf<V4<S>> pd_dinv;
  DBuf<S> ncg_L, ncg_Lt;  // NCG preconditioner factor and its transpose on the CSR pattern
  long ncg_version = -1;
  void release() {
    for (DBuf<S>* b : {&K, &vals, &mvals, &slot_mass, &pd_vals, &slot_pd, &pd_svals, &ncg_L, &ncg_Lt}) b->release();
    K16.release();
    pd_kron = false;
    ncg_version = -1;
    for (DBuf<V4<S>>* b : {&x, &r, &z, &p0, &p1, &q, &dinv, &tmp, &pm, &ld, &lq, &pd_dinv}) b->release();
    hs.clear();
    hy.clear();
  }
};

// PK_PCG counts iterations of the persistent PCG kernel (one launch per solve), so total / count is the
// time of one PCG iteration
enum ProfileKernel { PK_SPMV = 0, PK_HESS = 1, PK_ASM = 2, PK_GRAD = 3, PK_UPD = 4, PK_PCG = 5, PK_COUNT = 6 };

struct TimeStep {
  // ---- configuration (time_step.hpp:683-708)
  int nv = 0, nt = 0, n = 0;
  double dt = 1e-3, E = 1e6, nu = 0.33, rho = 1e3, damping = 0.0, rtol = 1e-2, abs_tol = 1e-2;
  double mass_third = 0;  // sum |M_ij| / 3, the reference threshold's scale (abs_tol = rtol * mass_third)
  DBuf<int32_t> mark_verts;  // scratch of the mark_* calls (grown, never shrunk)
  DBuf<double> mark_targ;
  // pinned staging of the Dirichlet marks: the call copies the caller's arrays here and returns without
  // waiting for the upload (the next upload waits for this one's event before it reuses the staging)
  int32_t* mark_verts_h = nullptr;
  double* mark_targ_h = nullptr;
  size_t mark_cap_h = 0;
  cudaEvent_t ev_mark = nullptr;
  bool mark_in_flight = false;
  void stage_marks(const int32_t* verts, const double* targ, int n) {
    if (mark_in_flight) SSIM_CUDA(cudaEventSynchronize(ev_mark));
    mark_in_flight = false;
    if ((size_t)n > mark_cap_h) {
      if (mark_verts_h) cudaFreeHost(mark_verts_h);
      if (mark_targ_h) cudaFreeHost(mark_targ_h);
      mark_verts_h = nullptr;
      mark_targ_h = nullptr;
      mark_cap_h = 0;
      SSIM_CUDA(cudaMallocHost((void**)&mark_verts_h, sizeof(int32_t) * n));
      SSIM_CUDA(cudaMallocHost((void**)&mark_targ_h, sizeof(double) * 3 * n));
      mark_cap_h = n;
    }
    if (!ev_mark) SSIM_CUDA(cudaEventCreateWithFlags(&ev_mark, cudaEventDisableTiming));
    std::memcpy(mark_verts_h, verts, sizeof(int32_t) * n);
    std::memcpy(mark_targ_h, targ, sizeof(double) * 3 * n);
  }
  int precision = SSIM_GB_FP64;
  int stepper = SSIM_GB_STEPPER_NONE;
  ssim_gb_params params{};
  bool has_reset = false;
  std::vector<double> E_elem, nu_elem;
  std::vector<double> X;
  std::vector<int32_t> cells;
  std::vector<double> detJ, vol_h;
  Topology topo;
  bool topo_ready = false;
  cudaStream_t stream = nullptr;
  cudaStream_t own_stream = nullptr;
  std::string last_error;
  ssim_gb_step_stats stats{};
  // ---- device: mesh, element constants
  DBuf<double> dX;
  DBuf<int4> dcells;
  DBuf<double> dminv, vol, lam, mu, snh_alpha, snh_psi0, snh_delta;
  DBuf<float> fdminv, fvol, flam, fmu;
  DBuf<float> fdelta;  // triangles: the 2D stable Neo-Hookean delta per element in FP32
  // ---- device: state [n] (time_step.hpp:668-679)
  DBuf<double> deformation, prev_deform, inertia, next, velocity, ext_accel, forces, dbc_values, work;
  DBuf<int8_t> dof_type;
  DBuf<uint8_t> mask;
  DBuf<float4> xf;
  // ---- device: topology
  DBuf<int32_t> vptr, vinc, sl_off, sl_col, slot_row, cptr, csrc, bptr, slot_k, slot_kt, lo_off, lo_src, lo_col;
  // lists of the fused element-Hessian + assembly kernel (tets; topology.h FusedLists)
  DBuf<int32_t> fptr, felem;
  DBuf<uint16_t> fcode;
  int fused_ncta = 0, fused_spc = 0;
  bool fused_ok = false, fused_built = false;
  // FP16 copy of the scaled system matrix for the mixed Newton's loose PCG solves (kernels.cuh HalfMatrix):
  // pattern built on first use, values made from the FP32 assembly before the first solve that reads them
  DBuf<int32_t> h16off, h16col, h16src;
  DBuf<uint4> h16v8;
  DBuf<uint16_t> h16v1;
  DBuf<float4> h16scale, h16iscale, h16dinv;
  bool h16_ok = false, h16_built = false;
  long long nfs = 0;
  long long asm_count = 0, h16_count = -1;  // assemblies of the FP32 values; the one the copy was made from
  bool last_half = false;  // the last pcg() ran on the FP16 copy
  bool half_checked = false;  // ... and its kernel left g . d, |d|^2 and the true residual in the scalars
  // speculative assembly (speculative_hessian): the next Newton iteration's Hessian at the full step, built on
  // a second stream while the line search runs on the handle's stream
  cudaStream_t side = nullptr;
  cudaEvent_t ev_dir = nullptr, ev_spec = nullptr, ev_xf = nullptr;
  DBuf<float4> xf_spec;
  bool spec_pending = false;
  bool spec_k16 = false;  // the element-block precision of the speculative assembly
  bool half_off = false;   // a Newton solve on the copy missed its forcing on the FP32 values: not used again
                           // until reset() or new parameters
  DBuf<double> lf, csr_out;
  // ---- device: solver
  Solver<float> sf;
  Solver<double> sd;
  DBuf<double> partials;
  DBuf<unsigned int> counter;
  DBuf<unsigned long long> gsync;  // grid-barrier state of the persistent PCG (counters, release, groups)
  DBuf<DevScalars> sc;
  DevScalars* hsc = nullptr;  // pinned
  DBuf<double> gprev, dscal;   // previous gradient (L-BFGS), device scalars of vdot
  // batched instances: the mesh is a disjoint union of independent meshes with contiguous vertex ranges;
  // with stop_mode 1 every instance must meet |g_i| <= rel_tol |g_i0| on its own
  int ninst = 0;
  std::vector<int32_t> inst_off_h;
  DBuf<int32_t> inst_off;
  DBuf<double> inst_g2;
  std::vector<double> inst_g2_h, inst_g0_h;
  std::vector<double> inst_mass_third;  // sum |M_ij| / 3 of each instance (its stop floor's scale)

  // per-instance sums of |mass| (the instances are disjoint, so every block belongs to one instance)
  void instance_masses() {
    inst_mass_third.assign(std::max(1, ninst), 0.0);
    if (ninst <= 1) return;
    std::vector<double> smass;
    slot_mass_values(smass);
    for (int q = 0; q < topo.nslots; ++q) {
      const int u = topo.slot_row[q];
      if (u < 0) continue;
      const int i = (int)(std::upper_bound(inst_off_h.begin(), inst_off_h.end(), u) - inst_off_h.begin()) - 1;
      inst_mass_third[i] += (topo.sl_col[q] == u ? 1.0 : 2.0) * std::fabs(smass[q]);
    }
  }
  double* hscal = nullptr;     // pinned mirror of dscal
  // ---- profiling
  bool profiling = false;
  std::vector<cudaEvent_t> ev;
  int elastic_model = SSIM_GB_MODEL_STABLE_NEOHOOKEAN;  // ElastModel of basic_time_step
  // mass-spring system instead of tets (cells are the springs' vertex pairs)
  bool springs = false;
  // 2D triangles in the plane (cells are triangles; the z dof of every vertex carries no force)
  bool tri2d = false;
  DBuf<int2> sp_ends;
  DBuf<double> sp_rest, sp_k, vmass;
  DBuf<float4> sp_e0, sp_lf32;
  DBuf<float> sp_k32;
  std::vector<double> vmass_h, sp_k_h;
  SpringData spd() const { return SpringData{nt, sp_ends.p, dX.p, sp_rest.p, sp_k.p, sp_e0.p, sp_k32.p}; }
  // the FP32 passes' per-vertex split of next (hi + lo) and of next - x~; split32() refreshes it for the
  // current next (once per base point: every trial of a line search shares it), lf32t holds the tets'
  // FP32 local forces
  DBuf<float4> uh32, ul32, w32;
  DBuf<float> lf32t;
  Split32 s32() const { return Split32{uh32.p, ul32.p, w32.p}; }
  // block sizes chosen by autotune() for the element pass, the Hessian, the assembly and the gather (0: the
  // kernels' defaults)
  struct Shapes {
    int elem = 0, hess = 0, assem = 0, gather = 0;
    int elem_regcap = 0;  // the FP32 element pass's 64-register variant
  } shapes;
  // the reference of the increment evaluations (mixed Newton after the FP32 phase): u_r, its FP64 forces and
  // energy, and the base point offset u_b - u_r; the FP32 split of u_r lives in uh32 / ul32 / w32
  DBuf<double> uref, gref;
  DBuf<float4> db32;
  double e_ref = 0, escale_ref = 0;
  bool delta_supported() const {
    return !springs && !tri2d && elastic_model == SSIM_GB_MODEL_STABLE_NEOHOOKEAN && params.mixed_delta != 0;
  }
  // u_r = next, whose FP64 energy E and forces were just evaluated
  void set_delta_reference(double E, double Escale) {
    uref.alloc(n);
    gref.alloc(n);
    db32.alloc(nv);
    SSIM_CUDA(cudaMemcpyAsync(uref.p, next.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, stream));
    SSIM_CUDA(cudaMemcpyAsync(gref.p, forces.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, stream));
    split32();
    e_ref = E;
    escale_ref = Escale;
  }
  void delta_base() { launch_delta_base(nv, next.p, uref.p, db32.p, stream); }
  void delta_trial(const float4* d, double alpha) {
    launch_elem_delta32(e64(), e32s(), s32(), db32.p, d, alpha, dt * dt, rho, e_ref, escale_ref, lf32t.p, true, true,
                        red(), stream, shapes.elem);
  }
  void delta_gather() {
    launch_vertex_gather_delta32(nv, vptr.p, vinc.p, lf32t.p, mask.p, gref.p, forces.p, red(), stream, shapes.gather);
  }
  void split32() {
    uh32.alloc(nv);
    ul32.alloc(nv);
    w32.alloc(nv);
    if (!springs) lf32t.alloc((tri2d ? 9 : 12) * (size_t)nt);
    launch_split32(nv, next.p, inertia.p, uh32.p, ul32.p, w32.p, stream);
  }

  // element / spring pass at u = next (+ alpha d): energy (+ local forces into lf) into the trial scalars;
  // the per-triangle FP32 delta that the stable Neo-Hookean FP32 triangle pass reads (the linear model reads
  // none); refuses to hand the kernel a missing array
  const float* tri_delta32() const {
    if (elastic_model != SSIM_GB_MODEL_LINEAR && fdelta.p == nullptr)
      throw state_error("the FP32 triangle pass needs the per-element delta: the material is not uploaded");
    return fdelta.p;
  }

  // fp32: the FP32 element / spring arithmetic of the mixed path's early iterations
  template <typename S>
  void launch_trial(const V4<S>* d, double alpha, bool forces, bool fp32 = false) {
    if (fp32) {
      if constexpr (std::is_same<S, float>::value) {
        if (springs)
          launch_spring_energy_grad32<float>(spd(), s32(), next.p, inertia.p, vmass.p, nv, d, alpha, dt * dt,
                                             forces ? sp_lf32.p : nullptr, forces, true, red(), stream);
        else if (tri2d)
          launch_tri_energy_grad32(e64(), e32s(), tri_delta32(), s32(), d, alpha, dt * dt, rho,
                                   forces ? lf32t.p : nullptr, forces, true, red(), stream);
        else
          launch_elem_energy_grad32(e64(), e32s(), s32(), d, alpha, dt * dt, rho, forces ? lf32t.p : nullptr,
                                    forces, true, red(), stream, shapes.elem, shapes.elem_regcap);
      } else {
        throw state_error("the FP32 element pass takes FP32 directions");
      }
    } else if (springs)
      launch_spring_energy_grad<S>(spd(), next.p, inertia.p, vmass.p, nv, d, alpha, dt * dt, forces ? lf.p : nullptr,
                                   forces, true, red(), stream);
    else if (tri2d)
      launch_tri_energy_grad<S>(e64(), next.p, inertia.p, d, alpha, dt * dt, rho, forces ? lf.p : nullptr, forces,
                                true, red(), stream);
    else
      launch_elem_energy_grad<S>(e64(), dX.p, next.p, inertia.p, d, alpha, dt * dt, rho, forces ? lf.p : nullptr,
                                 forces, true, red(), stream);
  }
  // forces at next (+ alpha d: the point of the last trial pass) from the last pass's local forces,
  // Dirichlet dofs zeroed, |g|^2
  template <typename S = double>
  void gather_forces(const V4<S>* d = nullptr, double alpha = 0.0, bool fp32 = false) {
    if (springs && fp32) {
      if constexpr (std::is_same<S, float>::value)
        launch_spring_gather32<float>(nv, vptr.p, vinc.p, sp_lf32.p, vmass.p, next.p, d, alpha, inertia.p, mask.p,
                                      forces.p, red(), stream);
      else
        throw state_error("the FP32 spring pass takes FP32 directions");
    } else if (springs)
      launch_spring_gather<S>(nv, vptr.p, vinc.p, lf.p, vmass.p, next.p, d, alpha, inertia.p, mask.p, forces.p, red(),
                              stream);
    else if (fp32)
      launch_vertex_gather32(nv, vptr.p, vinc.p, lf32t.p, mask.p, forces.p, red(), stream, shapes.gather);
    else
      launch_vertex_gather(nv, vptr.p, vinc.p, lf.p, mask.p, forces.p, red(), stream);
  }
  // mass per upper slot: consistent (tets) or lumped on the diagonal (springs)
  void slot_mass_values(std::vector<double>& smass) {
    if (tri2d) {
      slot_masses_2d(topo, detJ, rho, smass);
      return;
    }
    if (!springs) {
      slot_masses(topo, detJ, rho, smass);
      return;
    }
    smass.assign(topo.nslots, 0.0);
    for (int q = 0; q < topo.nslots; ++q)
      if (topo.slot_row[q] >= 0 && topo.slot_row[q] == topo.sl_col[q]) smass[q] = vmass_h[topo.slot_row[q]];
  }
  std::vector<int32_t> solve_log;  // PCG iterations of every solve since the last reset
  DBuf<double> lbc;                // L-BFGS two-loop coefficients a_i, b_i
  DBuf<double> lbtab, lbpart;      // compact L-BFGS: S^T Y / Y^T Y tables + coefficients; multidot partials
  // NCG preconditioner factor L (host copy; empty = identity), its CSR pattern on the device and the
  // position of each entry's transpose
  std::vector<double> ncg_vals;
  long ncg_ver = 0;
  DBuf<int32_t> ncg_rp, ncg_ci;
  std::vector<int64_t> ncg_tperm;
  long long prof_launch[PK_COUNT] = {0};
  double prof_ms[PK_COUNT] = {0};
  double prof_bytes[PK_COUNT] = {0};

  ~TimeStep() {
    if (mark_in_flight && ev_mark) cudaEventSynchronize(ev_mark);  // the staging is not freed under the upload
    if (mark_verts_h) cudaFreeHost(mark_verts_h);
    if (mark_targ_h) cudaFreeHost(mark_targ_h);
    if (ev_mark) cudaEventDestroy(ev_mark);
    if (side) cudaStreamSynchronize(side);
    if (side) cudaStreamDestroy(side);
    if (ev_dir) cudaEventDestroy(ev_dir);
    if (ev_spec) cudaEventDestroy(ev_spec);
    if (ev_xf) cudaEventDestroy(ev_xf);
    for (auto e : ev) cudaEventDestroy(e);
    if (hsc) cudaFreeHost(hsc);
    if (hscal) cudaFreeHost(hscal);
    if (own_stream) cudaStreamDestroy(own_stream);
  }

  bool mixed() const { return precision == SSIM_GB_MIXED; }
  Reduce red() { return Reduce{partials.p, counter.p, sc.p}; }
  ElemFP64 e64() const {
    return ElemFP64{nt, dcells.p, dminv.p, vol.p, lam.p, mu.p, snh_alpha.p, snh_psi0.p, elastic_model, snh_delta.p};
  }
  ElemFP32 e32() const { return ElemFP32{nt, dcells.p, fdminv.p, fvol.p, flam.p, fmu.p}; }
  ElemFP32 e32s() const { return e32(); }
  SellMatrix A() const {
    return SellMatrix{nv, topo.nslots, sl_off.p, sl_col.p, slot_row.p, lo_off.p, lo_src.p, lo_col.p};
  }

  void sync_scalars() {
    SSIM_CUDA(cudaMemcpyAsync(hsc, sc.p, sizeof(DevScalars), cudaMemcpyDeviceToHost, stream));
    SSIM_CUDA(cudaStreamSynchronize(stream));
  }

  // ------------------------------------------------------------------ construction
  void create(const double* Xh, int nv_, const int32_t* cells_h, int nt_, double dt_, double E_, double nu_,
              double rho_) {
    E = E_;
    nu = nu_;
    rho = rho_;
    init_common(Xh, nv_, cells_h, nt_, 4, dt_);
    std::vector<int4> c4(nt);
    std::memcpy(c4.data(), cells.data(), sizeof(int4) * nt);
    dcells.upload(c4, stream);
    // rest shape (dminv_task def_grad.hpp:56-91, rest_vol_task rest_vol.hpp:34-54)
    std::vector<double> dm(9 * (size_t)nt);
    detJ.assign(nt, 0);
    vol_h.assign(nt, 0);
    for (int e = 0; e < nt; ++e) {
      const double* x0 = &X[3 * (size_t)cells[4 * e + 0]];
      double D[9];
      for (int k = 0; k < 3; ++k) {
        const double* xk = &X[3 * (size_t)cells[4 * e + k + 1]];
        for (int r = 0; r < 3; ++r) D[r * 3 + k] = xk[r] - x0[r];
      }
      const double det = D[0] * (D[4] * D[8] - D[5] * D[7]) - D[1] * (D[3] * D[8] - D[5] * D[6]) +
                         D[2] * (D[3] * D[7] - D[4] * D[6]);
      const double id = 1.0 / det;
      const double B[9] = {(D[4] * D[8] - D[5] * D[7]) * id, (D[2] * D[7] - D[1] * D[8]) * id,
                           (D[1] * D[5] - D[2] * D[4]) * id, (D[5] * D[6] - D[3] * D[8]) * id,
                           (D[0] * D[8] - D[2] * D[6]) * id, (D[2] * D[3] - D[0] * D[5]) * id,
                           (D[3] * D[7] - D[4] * D[6]) * id, (D[1] * D[6] - D[0] * D[7]) * id,
                           (D[0] * D[4] - D[1] * D[3]) * id};
      for (int k = 0; k < 9; ++k) dm[(size_t)k * nt + e] = B[k];
      detJ[e] = std::fabs(det);
      vol_h[e] = std::fabs(det / 6);
    }
    dminv.upload(dm, stream);
    vol.upload(vol_h, stream);
    std::vector<float> f(dm.begin(), dm.end());
    fdminv.upload(f, stream);
    std::vector<float> fv(vol_h.begin(), vol_h.end());
    fvol.upload(fv, stream);
    reset(SSIM_GB_STEPPER_NONE);  // the constructor calls reset() (time_step.hpp:260-265)
  }

  // a mass-spring system: springs [ns][2] vertex pairs with rest lengths from X, stiffness k, vertex masses
  // (mass_h[nv], or m for every vertex); gravity and Dirichlet vertices as for tets
  void create_springs(const double* Xh, int nv_, const int32_t* ends_h, int ns_, double k, const double* mass_h,
                      double m, double dt_) {
    if (ns_ <= 0) throw invalid_argument("a spring system needs at least one spring");
    if (!(k > 0)) throw invalid_argument("spring stiffness must be positive");
    if (!mass_h && !(m > 0)) throw invalid_argument("vertex mass must be positive");
    springs = true;
    E = 1.0;  // unused by springs; keeps reset's material checks satisfied
    nu = 0.25;
    rho = 0.0;
    init_common(Xh, nv_, ends_h, ns_, 2, dt_);
    std::vector<double> rest(nt);
    std::vector<int2> e2(nt);
    for (int e = 0; e < nt; ++e) {
      const int i = cells[2 * e], j = cells[2 * e + 1];
      if (i == j) throw invalid_argument("a spring joins a vertex to itself");
      double l2 = 0;
      for (int q = 0; q < 3; ++q) l2 += (X[3 * i + q] - X[3 * j + q]) * (X[3 * i + q] - X[3 * j + q]);
      if (!(l2 > 0)) throw invalid_argument("a spring has zero rest length");
      rest[e] = std::sqrt(l2);
      e2[e] = make_int2(i, j);
    }
    sp_k_h.assign(nt, k);
    if (mass_h) {
      vmass_h.assign(mass_h, mass_h + nv);
      for (double mv : vmass_h)
        if (!(mv > 0)) throw invalid_argument("vertex masses must be positive");
    } else {
      vmass_h.assign(nv, m);
    }
    sp_ends.upload(e2, stream);
    sp_rest.upload(rest, stream);
    sp_k.upload(sp_k_h, stream);
    vmass.upload(vmass_h, stream);
    std::vector<float4> e0(nt);
    for (int e = 0; e < nt; ++e) {
      const int i = cells[2 * e], j = cells[2 * e + 1];
      e0[e] = make_float4((float)(X[3 * i] - X[3 * j]), (float)(X[3 * i + 1] - X[3 * j + 1]),
                          (float)(X[3 * i + 2] - X[3 * j + 2]), (float)rest[e]);
    }
    sp_e0.upload(e0, stream);
    std::vector<float> k32(sp_k_h.begin(), sp_k_h.end());
    sp_k32.upload(k32, stream);
    sp_lf32.alloc(nt);
    reset(SSIM_GB_STEPPER_NONE);
  }

  // 2D triangles: vertices [nv][2] (embedded at z = 0), triangles [nt][3] (basic_time_step with
  // PhysicalDim 2, TopologyDim 3); Dm^-1 row-major 2x2 in dminv rows 0..3, vol = area, detJ = 2 area
  void create_2d(const double* X2, int nv_, const int32_t* tris, int nt_, double dt_, double E_, double nu_,
                 double rho_) {
    if (!X2) throw invalid_argument("null mesh pointer");
    if (nv_ <= 0) throw invalid_argument("mesh must have at least one vertex and one cell");
    E = E_;
    nu = nu_;
    rho = rho_;
    tri2d = true;
    std::vector<double> X3(3 * (size_t)nv_, 0.0);
    for (int v = 0; v < nv_; ++v) {
      X3[3 * (size_t)v] = X2[2 * (size_t)v];
      X3[3 * (size_t)v + 1] = X2[2 * (size_t)v + 1];
    }
    init_common(X3.data(), nv_, tris, nt_, 3, dt_);
    std::vector<int4> c4(nt);
    for (int e = 0; e < nt; ++e) c4[e] = make_int4(cells[3 * e], cells[3 * e + 1], cells[3 * e + 2], cells[3 * e]);
    dcells.upload(c4, stream);
    std::vector<double> dm(9 * (size_t)nt, 0.0);
    detJ.assign(nt, 0);
    vol_h.assign(nt, 0);
    for (int e = 0; e < nt; ++e) {
      const double* x0 = &X[3 * (size_t)cells[3 * e]];
      const double* x1 = &X[3 * (size_t)cells[3 * e + 1]];
      const double* x2 = &X[3 * (size_t)cells[3 * e + 2]];
      const double D[4] = {x1[0] - x0[0], x2[0] - x0[0], x1[1] - x0[1], x2[1] - x0[1]};
      const double det = D[0] * D[3] - D[1] * D[2];
      if (!(det != 0)) throw invalid_argument("degenerate triangle " + std::to_string(e));
      const double B[4] = {D[3] / det, -D[1] / det, -D[2] / det, D[0] / det};
      for (int k = 0; k < 4; ++k) dm[(size_t)k * nt + e] = B[k];
      detJ[e] = std::fabs(det);
      vol_h[e] = std::fabs(det / 2);
    }
    dminv.upload(dm, stream);
    vol.upload(vol_h, stream);
    std::vector<float> f(dm.begin(), dm.end());
    fdminv.upload(f, stream);
    std::vector<float> fv(vol_h.begin(), vol_h.end());
    fvol.upload(fv, stream);
    reset(SSIM_GB_STEPPER_NONE);
  }

  void init_common(const double* Xh, int nv_, const int32_t* cells_h, int nt_, int cv, double dt_) {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
      cudaGetLastError();
      throw cuda_error("no CUDA device available (this library has no CPU path)");
    }
    if (!Xh || !cells_h) throw invalid_argument("null mesh pointer");
    nv = nv_;
    nt = nt_;
    n = 3 * nv;
    dt = dt_;
    X.assign(Xh, Xh + (size_t)n);
    cells.assign(cells_h, cells_h + (size_t)cv * nt);
    build_topology(nv, nt, cells.data(), topo, cv);  // validates indices
    topo_ready = true;
    ssim_gb_default_params(&params);
    SSIM_CUDA(cudaStreamCreateWithFlags(&own_stream, cudaStreamNonBlocking));
    stream = own_stream;
    SSIM_CUDA(cudaMallocHost((void**)&hsc, sizeof(DevScalars)));
    SSIM_CUDA(cudaMallocHost((void**)&hscal, 8 * sizeof(double)));
    dscal.alloc(8);
    gprev.alloc(n);
    // state buffers (zero_if_not_valid, time_step.hpp:396-413)
    for (DBuf<double>* b : {&deformation, &prev_deform, &inertia, &next, &velocity, &ext_accel, &forces,
                            &dbc_values, &work}) {
      b->alloc(n);
      b->zero(stream);
    }
    dof_type.alloc(n);
    dof_type.zero(stream);
    mask.alloc(nv);
    mask.zero(stream);
    xf.alloc(nv);
    sc.alloc(1);
    sc.zero(stream);
    counter.alloc(1);
    counter.zero(stream);
    gsync.alloc(grid_sync_words(nv));
    gsync.zero(stream);
    const size_t maxgrid = (size_t)std::max(div_up(nt, 64), div_up(std::max(3 * nv, topo.nslots), 256)) + 1;
    partials.alloc(maxgrid * 4);
    dX.upload(X, stream);
    vptr.upload(topo.vptr, stream);
    vinc.upload(topo.vinc, stream);
    sl_off.upload(topo.sl_off, stream);
    sl_col.upload(topo.sl_col, stream);
    slot_row.upload(topo.slot_row, stream);
    cptr.upload(topo.cptr, stream);
    csrc.upload(topo.csrc, stream);
    bptr.upload(topo.bptr, stream);
    slot_k.upload(topo.slot_k, stream);
    slot_kt.upload(topo.slot_kt, stream);
    lo_off.upload(topo.lo_off, stream);
    lo_src.upload(topo.lo_src, stream);
    lo_col.upload(topo.lo_col, stream);
    lf.alloc((size_t)3 * cv * nt);
  }

  // the fused kernel's lists, built on its first use (4 slices = 128 block rows per CTA); false if the mesh
  // is not a tet mesh or does not fit the lists' codes
  bool fused_ready() {
    if (fused_built) return fused_ok;
    fused_built = true;
    if (topo.cv != 4) return false;
    FusedLists fl;
    build_fused_lists(topo, cells.data(), 4, fused_chunk(), fl);
    fused_ok = fl.ok;
    if (fl.ok) {
      fptr.upload(fl.ptr, stream);
      felem.upload(fl.elem, stream);
      fcode.upload(fl.code, stream);
      fused_ncta = fl.ncta;
      fused_spc = fl.slices_per_cta;
      SSIM_CUDA(cudaStreamSynchronize(stream));  // the host lists go out of scope
    }
    return fused_ok;
  }

  bool half_ready() {
    if (h16_built) return h16_ok;
    h16_built = true;
    std::vector<int32_t> off, col, src;
    h16_ok = build_full_sell(topo, off, col, src);
    if (!h16_ok) return false;
    nfs = (long long)col.size();
    h16off.upload(off, stream);
    h16col.upload(col, stream);
    h16src.upload(src, stream);
    SSIM_CUDA(cudaStreamSynchronize(stream));  // the host lists go out of scope
    return true;
  }
  HalfMatrix half_matrix() const {
    return HalfMatrix{nv, h16off.p, h16col.p, h16v8.p, h16v1.p, h16scale.p, h16iscale.p};
  }
  // the FP16 copy of the current FP32 system values (remade only after a new assembly)
  void half_refresh() {
    h16v8.alloc((size_t)nfs);
    h16v1.alloc((size_t)nfs);
    h16scale.alloc(nv);
    h16iscale.alloc(nv);
    h16dinv.alloc(3 * (size_t)nv);
    if (h16_count == asm_count) return;
    launch_half_prepare(A(), sf.vals.p, params.precond, h16scale.p, h16iscale.p, h16dinv.p, stream);
    launch_half_convert(A(), h16off.p, h16col.p, h16src.p, sf.vals.p, h16scale.p, h16v8.p, h16v1.p, stream);
    h16_count = asm_count;
  }
  // the FP16 copy serves a solve when it is enabled, the tolerance is loose enough for its rounding, the
  // solve would run the persistent Chronopoulos-Gear kernel, and the pattern fits
  bool use_half(double rtol) {
    if (half_off || !mixed() || params.pcg_half_matrix != 1 || !(rtol >= params.half_matrix_min_rtol)) return false;
    const int variant = params.pcg_persistent;
    return (variant == 2 || variant == 3 || variant == 4) && half_ready();
  }

  // material: per element Lame parameters (basic_elast.hpp:10-20) and the stable Neo-Hookean constants
  void upload_material() {
    std::vector<double> l(nt), m(nt);
    for (int e = 0; e < nt; ++e) {
      const double Ee = E_elem.empty() ? E : E_elem[e];
      const double ne = nu_elem.empty() ? nu : nu_elem[e];
      m[e] = Ee / (2 * (1 + ne));
      l[e] = Ee * ne / ((1 + ne) * (1 - 2 * ne));
    }
    lam.upload(l, stream);
    mu.upload(m, stream);
    std::vector<double> al(nt), p0(nt);
    if (tri2d) {
      // stable_neohookean<2> (stable_neohookean.hpp:30-35, 93-100): delta the positive root of
      // (2t+1) d^2 + (2t+2) d - 2t = 0 with t = mu / lambda, alpha = (1 - 1/(2 + delta)) mu/lambda + 1
      std::vector<double> dl(nt);
      for (int e = 0; e < nt; ++e) {
        const double t = m[e] / l[e], a = 2 * t + 1, b = 2 * t + 2, c = -2 * t;
        dl[e] = (-b + std::sqrt(b * b - 4 * a * c)) / (2 * a);
        al[e] = (1 - 1 / (2 + dl[e])) * m[e] / l[e] + 1;
        p0[e] = 0.5 * (l[e] * (1 - al[e]) * (1 - al[e]) - m[e] * std::log(2 + dl[e]));
      }
      snh_delta.upload(dl, stream);
      std::vector<float> df(dl.begin(), dl.end());
      fdelta.upload(df, stream);
    } else {
      for (int e = 0; e < nt; ++e) snh_constants<double>(l[e], m[e], al[e], p0[e]);
    }
    snh_alpha.upload(al, stream);
    snh_psi0.upload(p0, stream);
    std::vector<float> lf32(l.begin(), l.end()), mf32(m.begin(), m.end());
    flam.upload(lf32, stream);
    fmu.upload(mf32, stream);
  }

  // ------------------------------------------------------------------ reset (time_step.hpp:363-494)
  void reset(int stepper_kind) {
    if (!(E >= 0)) throw invalid_argument("Young's modulus must be positive, got " + std::to_string(E));
    if (!(nu > 0 && nu < 0.5)) throw invalid_argument("Poisson's ratio must be in (0, 0.5), got " + std::to_string(nu));
    if (!(rho >= 0)) throw invalid_argument("Density must be positive, got " + std::to_string(rho));
    if (stepper_kind < 0 || stepper_kind > SSIM_GB_STEPPER_NCG_EXT) throw invalid_argument("unknown stepper");
    stepper = stepper_kind;
    half_off = false;
    if (side) SSIM_CUDA(cudaStreamSynchronize(side));  // no speculative assembly outlives the buffers it writes
    spec_pending = false;
    for (DBuf<double>* b : {&inertia, &next, &forces, &work}) b->zero(stream);
    if (!springs) upload_material();
    // consistent mass per slot (time_step.hpp:437-461) and the threshold (time_step.hpp:490-491):
    // rtol * asum(mass CSR values) / 3; each slot's scalar appears on the 3 diagonal dofs of its block
    std::vector<double> smass;
    slot_mass_values(smass);
    double asum = 0;  // the full CSR holds every off-diagonal block twice (the store keeps the upper one)
    for (int q = 0; q < topo.nslots; ++q)
      if (topo.slot_row[q] >= 0) asum += (topo.sl_col[q] == topo.slot_row[q] ? 3.0 : 6.0) * std::fabs(smass[q]);
    abs_tol = asum / 3.0 * rtol;
    mass_third = asum / 3.0;
    instance_masses();
    if (mixed()) {
      std::vector<float> sm(smass.begin(), smass.end());
      sf.slot_mass.upload(sm, stream);
      alloc_solver(sf);
      sd.release();
    } else {
      sd.slot_mass.upload(smass, stream);
      alloc_solver(sd);
      sf.release();
      h16v8.release();
      h16v1.release();
      h16_count = -1;
    }
    launch_build_mask(nv, dof_type.p, mask.p, stream);
    if (stepper == SSIM_GB_STEPPER_PD) {
      if (mixed())
        pd_setup<float>(sf);
      else
        pd_setup<double>(sd);
    }
    SSIM_CUDA(cudaStreamSynchronize(stream));
    has_reset = true;
    solve_log.clear();
    ncg_vals.clear();  // timestep_ncg::reset installs the identity (fem_cuda.cu:174-204)
    ++ncg_ver;
  }

  // time_step_solver_pd::reset_impl (projective_dynamics.hpp:53-93): (mass(rho) + laplace(dt^2 kappa)) (x) I3
  // with the Dirichlet identity filter, assembled once into the symmetric block store.  kappa is
  // approximated_diffusivity (stable_neohookean.hpp:106-111) of uniform_elasticity() (time_step.hpp:356),
  // which builds the model as ElastModel{E, nu}, i.e. with (E, nu) in its (lambda, mu) slots; mode 1 uses the
  // Lame parameters instead, mode 2 each element's own Lame parameters (per-element materials).
  template <typename S>
  void pd_setup(Solver<S>& s) {
    if (springs) {
      // mass-spring projective dynamics (Liu et al. 2013): (M + dt^2 sum_s k_s A_s^T A_s) (x) I3, A_s the
      // edge difference, with the Dirichlet identity filter
      std::vector<double> pd;
      slot_mass_values(pd);
      for (int e = 0; e < nt; ++e) {
        const int i = cells[2 * e], j = cells[2 * e + 1];
        const double w = dt * dt * sp_k_h[e];
        pd[upper_slot(topo, i, i)] += w;
        pd[upper_slot(topo, j, j)] += w;
        if (i != j) pd[upper_slot(topo, std::min(i, j), std::max(i, j))] -= w;
      }
      std::vector<S> pds(pd.begin(), pd.end());
      s.slot_pd.upload(pds, stream);
      s.pd_vals.alloc(9 * (size_t)topo.nslots);
      s.pd_dinv.alloc(3 * (size_t)nv);
      launch_assemble<S>(A(), cptr.p, csrc.p, nullptr, s.slot_pd.p, mask.p, true, s.pd_vals.p, s.pd_dinv.p, 2, stream);
      pd_kron_form<S>(s);
      return;
    }
    double lam_slot = E, mu_slot = nu;
    if (params.pd_kappa_mode == 1) {
      mu_slot = E / (2 * (1 + nu));
      lam_slot = E * nu / ((1 + nu) * (1 - 2 * nu));
    }
    const double kappa = (lam_slot + 5.0 / 6.0 * mu_slot) + 2.0 * (4.0 / 3.0 * mu_slot);
    std::vector<double> pd, alpha_e;
    if (params.pd_kappa_mode == 2) {
      alpha_e.resize(nt);
      for (int e = 0; e < nt; ++e) {
        const double Ee = E_elem.empty() ? E : E_elem[e], ne = nu_elem.empty() ? nu : nu_elem[e];
        const double m = Ee / (2 * (1 + ne)), l = Ee * ne / ((1 + ne) * (1 - 2 * ne));
        alpha_e[e] = dt * dt * ((l + 5.0 / 6.0 * m) + 2.0 * (4.0 / 3.0 * m));
      }
    }
    if (tri2d)
      slot_pd_values_2d(topo, cells.data(), X.data(), detJ, rho, dt * dt * kappa, pd,
                        params.pd_kappa_mode == 2 ? &alpha_e : nullptr);
    else
      slot_pd_values(topo, cells.data(), X.data(), detJ, rho, dt * dt * kappa, pd,
                     params.pd_kappa_mode == 2 ? &alpha_e : nullptr);
    std::vector<S> pds(pd.begin(), pd.end());
    s.slot_pd.upload(pds, stream);
    s.pd_vals.alloc(9 * (size_t)topo.nslots);
    s.pd_dinv.alloc(3 * (size_t)nv);
    launch_assemble<S>(A(), cptr.p, csrc.p, nullptr, s.slot_pd.p, mask.p, true, s.pd_vals.p, s.pd_dinv.p, 2, stream);
    pd_kron_form<S>(s);
  }

  // the PD matrix is (M + dt^2 kappa L) (x) I3 with the Dirichlet identity on whole vertices; when every
  // block is a multiple of I3 (no vertex is only partly fixed) the PCG reads it with one value per block
  template <typename S>
  void pd_kron_form(Solver<S>& s) {
    s.pd_svals.alloc(std::max(topo.nslots, 1));
    SSIM_CUDA(cudaMemsetAsync(&sc.p->status, 0, sizeof(int32_t), stream));
    launch_kron_extract<S>(A(), s.pd_vals.p, s.pd_svals.p, &sc.p->status, stream);
    sync_scalars();
    s.pd_kron = hsc->status == 0;
  }

  template <typename S>
  void alloc_solver(Solver<S>& s) {
    s.vals.alloc(9 * (size_t)topo.nslots);
    s.vals.zero(stream);
    s.mvals.release();
    for (DBuf<V4<S>>* b : {&s.x, &s.r, &s.z, &s.p0, &s.p1, &s.q, &s.tmp}) {
      b->alloc(nv);
      b->zero(stream);
    }
    s.dinv.alloc(3 * (size_t)nv);
    s.dinv.zero(stream);
    s.ld.alloc(nv);
    s.lq.alloc(nv);
    s.hs.clear();
    s.hy.clear();
    for (int i = 0; i < params.lbfgs_history; ++i) {
      s.hs.emplace_back(new DBuf<V4<S>>());
      s.hy.emplace_back(new DBuf<V4<S>>());
      s.hs.back()->alloc(nv);
      s.hy.back()->alloc(nv);
    }
  }

  // ------------------------------------------------------------------ loop
  void prepare_step() {
    if (!(0 <= damping && damping < 1)) throw invalid_argument("velocity damping must be in [0, 1).");
    launch_prepare_step(n, dt, deformation.p, velocity.p, ext_accel.p, dof_type.p, dbc_values.p, inertia.p,
                        next.p, stream);
  }

  void step_next() { launch_step_next(n, dt, damping, prev_deform.p, deformation.p, next.p, velocity.p, stream); }

  void restore() { launch_restore(n, dt, dof_type.p, dbc_values.p, prev_deform.p, deformation.p, velocity.p, stream); }

  // energy + gradient at next (update_energy_and_gradients, time_step.hpp:577-624); synchronous
  double energy_grad() {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (profiling) prof_begin(e0, e1);
    if (springs)
      launch_spring_energy_grad<double>(spd(), next.p, inertia.p, vmass.p, nv, nullptr, 0.0, dt * dt, lf.p, true,
                                        false, red(), stream);
    else if (tri2d)
      launch_tri_energy_grad<double>(e64(), next.p, inertia.p, nullptr, 0.0, dt * dt, rho, lf.p, true, false, red(),
                                     stream);
    else if (mixed())
      launch_elem_energy_grad<float>(e64(), dX.p, next.p, inertia.p, nullptr, 0.0, dt * dt, rho, lf.p, true, false,
                                     red(), stream);
    else
      launch_elem_energy_grad<double>(e64(), dX.p, next.p, inertia.p, nullptr, 0.0, dt * dt, rho, lf.p, true, false,
                                      red(), stream);
    if (profiling) prof_end(e0, e1, PK_GRAD, 0);
    gather_forces();
    sync_scalars();
    if (!std::isfinite(hsc->energy) || !std::isfinite(hsc->gnorm2))
      throw numerical_error("non-finite energy or gradient (inverted or degenerate element?)");
    return hsc->energy;
  }

  // energy and forces with FP32 element arithmetic (mixed Newton's inner iterations), FP64 gather and sums
  double energy_grad32() {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (profiling) prof_begin(e0, e1);
    split32();
    if (springs)
      launch_spring_energy_grad32<float>(spd(), s32(), next.p, inertia.p, vmass.p, nv, nullptr, 0.0, dt * dt,
                                         sp_lf32.p, true, false, red(), stream);
    else if (tri2d)
      launch_tri_energy_grad32(e64(), e32s(), tri_delta32(), s32(), nullptr, 0.0, dt * dt, rho, lf32t.p, true, false,
                               red(), stream);
    else
      launch_elem_energy_grad32(e64(), e32s(), s32(), nullptr, 0.0, dt * dt, rho, lf32t.p, true, false, red(),
                                stream, shapes.elem, shapes.elem_regcap);
    if (profiling) prof_end(e0, e1, PK_GRAD, 0);
    gather_forces<float>(nullptr, 0.0, true);
    sync_scalars();
    if (!std::isfinite(hsc->energy) || !std::isfinite(hsc->gnorm2))
      throw numerical_error("non-finite energy or gradient (inverted or degenerate element?)");
    return hsc->energy;
  }

  double energy_at(const double* u_dev) {
    // value only: trial kernel with alpha = 0 against an arbitrary displacement
    if (mixed()) sf.tmp.zero(stream); else sd.tmp.zero(stream);
    if (springs && mixed())
      launch_spring_energy_grad<float>(spd(), u_dev, inertia.p, vmass.p, nv, sf.tmp.p, 0.0, dt * dt, nullptr, false,
                                       true, red(), stream);
    else if (springs)
      launch_spring_energy_grad<double>(spd(), u_dev, inertia.p, vmass.p, nv, sd.tmp.p, 0.0, dt * dt, nullptr, false,
                                        true, red(), stream);
    else if (tri2d && mixed())
      launch_tri_energy_grad<float>(e64(), u_dev, inertia.p, sf.tmp.p, 0.0, dt * dt, rho, nullptr, false, true, red(),
                                    stream);
    else if (tri2d)
      launch_tri_energy_grad<double>(e64(), u_dev, inertia.p, sd.tmp.p, 0.0, dt * dt, rho, nullptr, false, true,
                                     red(), stream);
    else if (mixed())
      launch_elem_energy_grad<float>(e64(), dX.p, u_dev, inertia.p, sf.tmp.p, 0.0, dt * dt, rho, nullptr, false,
                                     true, red(), stream);
    else
      launch_elem_energy_grad<double>(e64(), dX.p, u_dev, inertia.p, sd.tmp.p, 0.0, dt * dt, rho, nullptr, false,
                                      true, red(), stream);
    sync_scalars();
    return hsc->trial_energy;
  }

  template <typename S>
  Solver<S>& solver();

  // update_hessian (time_step.hpp:626-658)
  // k16: the element blocks in FP16 (tets, mixed precision; for assemblies whose solve runs on the FP16 copy)
  template <typename S>
  void hessian(bool spsd, bool filter, bool k16 = false, const float4* xfp = nullptr) {
    Solver<S>& s = solver<S>();
    ++asm_count;
    if (xfp == nullptr) xfp = xf.p;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (profiling) prof_begin(e0, e1);
    if (!springs && !tri2d && params.fused_assembly && fused_ready()) {
      launch_fused_hessian<S>(e64(), e32(), dX.p, next.p, mixed() ? xfp : nullptr, dt * dt, spsd, A(), topo.nslices,
                              fused_spc, fused_ncta, fptr.p, felem.p, fcode.p, s.slot_mass.p, mask.p, filter, s.vals.p,
                              s.dinv.p, params.precond, stream);
      if (profiling) prof_end(e0, e1, PK_HESS, 0);
      return;
    }
    if constexpr (std::is_same<S, float>::value) {
      if (k16 && !springs && !tri2d) {
        s.K16.alloc((size_t)30 * nt);
        launch_elem_hessian16(e64(), e32(), dX.p, next.p, xfp, dt * dt, spsd, s.K16.p, stream, shapes.hess);
        if (profiling) prof_end(e0, e1, PK_HESS, 0);
        if (profiling) prof_begin(e0, e1);
        launch_assemble16(A(), cptr.p, csrc.p, s.K16.p, s.slot_mass.p, mask.p, filter, s.vals.p, s.dinv.p,
                          params.precond, stream, shapes.assem);
        if (profiling) prof_end(e0, e1, PK_ASM, 0);
        return;
      }
    }
    // two kernels through the per-element block buffer (allocated on first use)
    s.K.alloc((size_t)9 * (topo.cv * (topo.cv + 1) / 2) * nt);
    if (springs)
      launch_spring_hessian<S>(spd(), next.p, dt * dt, spsd, s.K.p, stream);
    else if (tri2d)
      launch_tri_hessian<S>(e64(), next.p, dt * dt, spsd, s.K.p, stream);
    else
      launch_elem_hessian<S>(e64(), e32(), dX.p, next.p, mixed() ? xfp : nullptr, dt * dt, spsd, s.K.p, stream,
                             shapes.hess);
    if (profiling) prof_end(e0, e1, PK_HESS, 0);
    if (profiling) prof_begin(e0, e1);
    launch_assemble<S>(A(), cptr.p, csrc.p, s.K.p, s.slot_mass.p, mask.p, filter, s.vals.p, s.dinv.p,
                       params.precond, stream, shapes.assem);
    if (profiling) prof_end(e0, e1, PK_ASM, 0);
  }

  // the next Newton iteration's Hessian at u + d (the full step), on the side stream after the direction
  // is final: the same FP32 positions as launch_axpy_update(alpha = 1) and refresh_xf would make, so a
  // full step accepted by the line search finds its matrix assembled
  template <typename S>
  void spec_hessian(const V4<S>* d, bool k16) {
    if (!side) {
      SSIM_CUDA(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
      SSIM_CUDA(cudaEventCreateWithFlags(&ev_dir, cudaEventDisableTiming));
      SSIM_CUDA(cudaEventCreateWithFlags(&ev_spec, cudaEventDisableTiming));
      SSIM_CUDA(cudaEventCreateWithFlags(&ev_xf, cudaEventDisableTiming));
    }
    xf_spec.alloc(nv);
    SSIM_CUDA(cudaEventRecord(ev_dir, stream));
    SSIM_CUDA(cudaStreamWaitEvent(side, ev_dir, 0));
    launch_full_step_xf<S>(nv, d, dX.p, next.p, xf_spec.p, side);
    SSIM_CUDA(cudaEventRecord(ev_xf, side));  // the line search's update of u waits for this read of u
    std::swap(stream, side);  // hessian() launches on `stream`
    try {
      hessian<S>(true, true, k16, xf_spec.p);
    } catch (...) {
      std::swap(stream, side);
      throw;
    }
    std::swap(stream, side);
    SSIM_CUDA(cudaEventRecord(ev_spec, side));
    spec_pending = true;
  }
  // the handle's stream waits for a speculative assembly in flight (before anything reads or rewrites the
  // system values, the element blocks or the positions it used)
  void spec_join() {
    if (!spec_pending) return;
    SSIM_CUDA(cudaStreamWaitEvent(stream, ev_spec, 0));
    spec_pending = false;
  }

  void hessian_any(bool spsd, bool filter) {
    if (mixed()) {
      launch_refresh_xf(nv, dX.p, next.p, xf.p, stream);
      hessian<float>(spsd, filter);
    } else {
      hessian<double>(spsd, filter);
    }
  }

  // Jacobi-PCG on the current system values; rhs = (negate ? -b : b) with b an FP64 [n] device vector.
  // Result in solver().x.  Returns iterations.
  template <typename S>
  int pcg(const double* b, bool negate, double eta, int max_iters, double* rel_res) {
    Solver<S>& s = solver<S>();
    last_half = false;
    if constexpr (std::is_same<S, float>::value) {
      int it = 0;
      if (use_half(eta) && pcg_half(b, negate, eta, max_iters, rel_res, &it)) {
        last_half = true;
        return it;
      }
    }
    launch_pcg_setup<S>(nv, b, s.dinv.p, s.x.p, s.r.p, s.z.p, s.p0.p, eta, max_iters, negate, red(), stream);
    return pcg_loop<S>(s.vals.p, s.dinv.p, max_iters, rel_res, true);
  }

  // PCG on the FP16 copy of the scaled system matrix (Chronopoulos-Gear, one cooperative launch); false if
  // the device cannot launch it cooperatively (the caller then runs the FP32 matrix)
  bool pcg_half(const double* b, bool negate, double eta, int max_iters, double* rel_res, int* iters) {
    Solver<float>& s = sf;
    half_refresh();
    const HalfMatrix H = half_matrix();
    // the automatic choice (3) on the copy is the pipelined iteration: one reducing barrier per iteration
    // (21.1 against 23.8 us per iteration on the 1.02M-tet beam, the same iteration counts); its FP32
    // recursive-residual drift is covered by the true-residual check of every Newton solve, which that
    // kernel runs itself after the solve (with its set-up before it: one launch, one host wait)
    const bool pipe = (params.pcg_persistent == 3 || params.pcg_persistent == 4) && max_iters > 0;
    half_checked = false;
    HalfSolveArgs ha{b, negate ? 1 : 0, eta, max_iters, params.pcg_pipe_iters, negate ? 1 : 0, A(), s.vals.p};
    if (pipe) {
      if (s.pm.n < 2 * (size_t)nv) s.pm.alloc(2 * (size_t)nv);
    } else {
      launch_pcg_setup_half(H, b, h16dinv.p, s.x.p, s.r.p, s.z.p, s.p0.p, eta, max_iters, negate, red(), stream);
    }
    if (profiling) SSIM_CUDA(cudaEventRecord(ev[0], stream));
    const bool ran = launch_pcg_half(H, h16dinv.p, s.x.p, s.r.p, s.z.p, s.p0.p, s.p1.p, s.q.p, max_iters, red(),
                                     gsync.p, params.pcg_spin_limit, params.pcg_barrier_extra, params.pcg_max_blocks,
                                     stream, pipe ? s.pm.p : nullptr, pipe ? &ha : nullptr);
    if (!ran) return false;
    half_checked = pipe && ha.check;
    if (profiling) SSIM_CUDA(cudaEventRecord(ev[1], stream));
    sync_scalars();
    if (hsc->wait_failed) throw device_timeout("a grid-barrier wait of the persistent PCG kernel gave up");
    if (profiling) {
      float ms = 0;
      SSIM_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[1]));
      prof_ms[PK_PCG] += ms;
      prof_launch[PK_PCG] += hsc->iters;
      prof_bytes[PK_PCG] = half_spmv_bytes() + update_bytes(sizeof(float));
    }
    if (rel_res) *rel_res = hsc->rr0 > 0 ? std::sqrt(hsc->rr / hsc->rr0) : 0.0;
    if (hsc->status == 2) throw numerical_error("PCG produced a non-finite residual");
    if (solve_log.size() < (1u << 20)) solve_log.push_back(hsc->iters);
    *iters = hsc->iters;
    return true;
  }

  // PCG on another matrix of the same block pattern (the PD matrix) with an S right-hand side
  template <typename S>
  int pcg_on(const S* vals, const V4<S>* dinv, const V4<S>* b, double eta, int max_iters, double* rel_res,
             bool kron = false) {
    Solver<S>& s = solver<S>();
    launch_pcg_setup_v<S>(nv, b, dinv, s.x.p, s.r.p, s.z.p, s.p0.p, eta, max_iters, red(), stream);
    return pcg_loop<S>(vals, dinv, max_iters, rel_res, false, kron);
  }

  template <typename S>
  int pcg_loop(const S* vals, const V4<S>* dinv, int max_iters, double* rel_res, bool profile_spmv,
               bool kron = false) {
    Solver<S>& s = solver<S>();
    int variant = params.pcg_persistent;
    // automatic: FP64 runs two launches per iteration (its FP64 dots and updates make the persistent
    // kernels slower on GB300), FP32 Chronopoulos-Gear.  Pipelined PCG (4) is opt-in: its recursive
    // residual drifts from the true one in FP32 by an amount that grows with the iterations and the
    // condition number, which a loose tolerance does not cover for ill-conditioned systems (cloth, thin
    // sheets)
    if (variant == 3) variant = sizeof(S) == 4 ? 2 : 0;
    if (variant) {
      const bool prof = profiling && profile_spmv;
      if (prof) SSIM_CUDA(cudaEventRecord(ev[0], stream));
      if (variant == 4 && s.pm.n < 2 * (size_t)nv) s.pm.alloc(2 * (size_t)nv);
      const bool ran = launch_pcg_persistent<S>(A(), vals, dinv, s.x.p, s.r.p, s.z.p, s.p0.p, s.p1.p, s.q.p, max_iters,
                                                red(), gsync.p, params.pcg_spin_limit, params.pcg_barrier_extra,
                                                params.pcg_max_blocks, variant, stream, kron, s.pm.p,
                                                params.pcg_pipe_iters);
      if (ran) {
        if (prof) SSIM_CUDA(cudaEventRecord(ev[1], stream));
        sync_scalars();
        if (hsc->wait_failed) throw device_timeout("a grid-barrier wait of the persistent PCG kernel gave up");
        if (prof) {
          float ms = 0;
          SSIM_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[1]));
          prof_ms[PK_PCG] += ms;
          prof_launch[PK_PCG] += hsc->iters;
          prof_bytes[PK_PCG] = spmv_bytes(sizeof(S)) + update_bytes(sizeof(S));
        }
        if (rel_res) *rel_res = hsc->rr0 > 0 ? std::sqrt(hsc->rr / hsc->rr0) : 0.0;
        if (hsc->status == 2) throw numerical_error("PCG produced a non-finite residual");
        if (solve_log.size() < (1u << 20)) solve_log.push_back(hsc->iters);
        return hsc->iters;
      }
    }
    int k = 0;
    int chunk = std::max(1, params.cg_check_every);
    const bool prof = profiling && profile_spmv;
    int it_prev = 0;
    double rr_prev = 0;
    while (true) {
      const int k0 = k;
      for (int c = 0; c < chunk; ++c, ++k) {
        V4<S>* pold = (k & 1) ? s.p1.p : s.p0.p;
        V4<S>* pnew = (k & 1) ? s.p0.p : s.p1.p;
        if (prof) SSIM_CUDA(cudaEventRecord(ev[2 * c], stream));
        launch_pcg_spmv<S>(A(), vals, s.z.p, pold, pnew, s.q.p, k == 0, red(), stream, kron);
        if (prof) SSIM_CUDA(cudaEventRecord(ev[2 * c + 1], stream));
        launch_pcg_update<S>(nv, pnew, s.q.p, dinv, s.x.p, s.r.p, s.z.p, max_iters, red(), stream);
      }
      sync_scalars();
      if (prof) {
        const int valid = std::min(chunk, std::max(0, hsc->iters - k0));
        for (int c = 0; c < valid; ++c) {
          float ms = 0;
          SSIM_CUDA(cudaEventElapsedTime(&ms, ev[2 * c], ev[2 * c + 1]));
          prof_ms[PK_SPMV] += ms;
          prof_launch[PK_SPMV] += 1;
        }
        prof_bytes[PK_SPMV] = spmv_bytes(sizeof(S));
      }
      if (hsc->done || hsc->iters >= max_iters) break;
      // next chunk: the iterations still needed at the observed convergence rate (plus a margin), so few
      // launches run past convergence and few host round trips are spent
      const int it_now = hsc->iters;
      const double rr_now = hsc->rr;
      if (it_prev == 0) rr_prev = hsc->rr0;
      int next_chunk = 2 * chunk;
      if (it_now > it_prev && rr_now > 0 && rr_prev > 0 && rr_now < rr_prev && hsc->tol2 > 0) {
        const double rate = std::log(rr_now / rr_prev) / (it_now - it_prev);  // log decrease per iteration
        const double need = std::log(hsc->tol2 / rr_now) / rate;
        if (std::isfinite(need)) next_chunk = (int)std::ceil(1.1 * need) + 2;
      }
      it_prev = it_now;
      rr_prev = rr_now;
      chunk = std::max(4, std::min(next_chunk, 256));
      if ((int)ev.size() < 2 * chunk && prof) chunk = (int)ev.size() / 2;
    }
    if (rel_res) *rel_res = hsc->rr0 > 0 ? std::sqrt(hsc->rr / hsc->rr0) : 0.0;
    if (hsc->status == 2) throw numerical_error("PCG produced a non-finite residual");
    if (solve_log.size() < (1u << 20)) solve_log.push_back(hsc->iters);
    return hsc->iters;
  }

  // per-instance |g_i|^2 of the current forces (host copy in inst_g2_h)
  void instance_norms() {
    launch_instance_norms(ninst, inst_off.p, forces.p, inst_g2.p, stream);
    SSIM_CUDA(cudaMemcpyAsync(inst_g2_h.data(), inst_g2.p, sizeof(double) * ninst, cudaMemcpyDeviceToHost, stream));
    SSIM_CUDA(cudaStreamSynchronize(stream));
  }
  void start_instances() {
    if (ninst <= 1 || params.stop_mode != 1) return;
    instance_norms();
    for (int i = 0; i < ninst; ++i) inst_g0_h[i] = std::sqrt(inst_g2_h[i]);
  }
  // the stopping test: the reference's absolute rule (stop_mode 0), the relative rule on the whole vector,
  // or, for a batch, the relative rule on every instance
  bool stop_test(double gn, double g0) {
    if (params.stop_mode == 0) return gn < abs_tol;
    // relative rule, with the reference's absolute rule at rtol = stop_floor as a floor (per instance for a
    // batch): a step that starts at rest has a round-off gradient whose fraction cannot be reached
    if (ninst <= 1) return gn <= params.rel_tol * g0 || gn <= params.stop_floor * mass_third;
    instance_norms();
    for (int i = 0; i < ninst; ++i)
      if (std::sqrt(inst_g2_h[i]) > std::max(params.rel_tol * inst_g0_h[i], params.stop_floor * inst_mass_third[i]))
        return false;
    return true;
  }

  template <typename S>
  double vdot(const V4<S>* a, const V4<S>* b) {
    launch_vdot<S>(nv, a, b, dscal.p, red(), stream);
    SSIM_CUDA(cudaMemcpyAsync(hscal, dscal.p, sizeof(double), cudaMemcpyDeviceToHost, stream));
    SSIM_CUDA(cudaStreamSynchronize(stream));
    return hscal[0];
  }

  // L-BFGS stepper (backward_euler.hpp:43-67) over mathprim's l_bfgs_optimizer (absent from the reference
  // tree; the definition used is the oracle's: two-loop recursion, initial scaling s.y / y.y (1/|g| before
  // any history), backtracking Armijo line search).  With pd, the initial inverse Hessian is the PD matrix
  // solve (projective_dynamics.hpp:31-34), done here by PCG to pd tolerance instead of a factorisation.
  template <typename S>
  void lbfgs(ssim_gb_step_stats& st, bool pd, bool h0 = false) {
    Solver<S>& s = solver<S>();
    if (h0) {
      // time_step_solver_h0 (projective_dynamics.hpp:100-150): the projected Hessian at the step start is
      // the initial inverse Hessian (the reference factorises it; here it is applied by PCG)
      if (mixed()) launch_refresh_xf(nv, dX.p, next.p, xf.p, stream);
      hessian<S>(true, true);
      s.pd_vals.alloc(9 * (size_t)topo.nslots);
      s.pd_dinv.alloc(3 * (size_t)nv);
      SSIM_CUDA(cudaMemcpyAsync(s.pd_vals.p, s.vals.p, sizeof(S) * 9 * (size_t)topo.nslots, cudaMemcpyDeviceToDevice,
                                stream));
      SSIM_CUDA(cudaMemcpyAsync(s.pd_dinv.p, s.dinv.p, sizeof(V4<S>) * 3 * (size_t)nv, cudaMemcpyDeviceToDevice,
                                stream));
      s.pd_kron = false;  // the projected Hessian is not a multiple of I3 per block
      pd = true;
    }
    const int m = std::max(1, std::min(params.lbfgs_history, (int)s.hs.size()));
    // The two-loop coefficients a_i (lbc[i]) and b_i (lbc[m + i]) stay on the device; rho_i and the initial
    // scaling are known on the host from the pair's s.y and y.y, read with the trial point's energy.  One
    // host round trip per line-search trial: the trial pass also forms the forces at the trial point and
    // the curvature pair against the current gradient (kept in gprev), so an accepted trial needs no
    // further evaluation.
    lbc.alloc(2 * (size_t)m);
    double* al = lbc.p;
    double* bb = lbc.p + m;
    // without a PD/H0 solve and with at most kLbfgsMaxCompact pairs the direction comes from the compact
    // form of the same matrix: two passes instead of 2m dependent ones
    const bool compact = !pd && m <= kLbfgsMaxCompact;
    constexpr int MC = kLbfgsMaxCompact;
    if (compact) {
      lbtab.alloc(2 * MC * MC + 2 * MC + 1);
      lbpart.alloc((size_t)lbfgs_multidot_partials(nv));
    }
    std::vector<double> rho_h(m, 0.0);
    double gamma = 0.0;     // s.y / y.y of the newest pair
    int hsize = 0, head = 0;  // ring: entries head-hsize .. head-1 (mod m), oldest first
    // mixed precision: FP32 element / spring arithmetic until the residual is within elem32_switch times
    // the target, a line search runs out or the residual stalls within kLbfgsStallBand times the target
    // (its best value not halved in max(kLbfgsStall32, 3 x the longest halving interval of the phase so far)
    // iterations: the FP32 rounding floor of the O(|g0|) forces can lie above the switch, where the trials'
    // energy slack keeps accepting steps; the band and the phase's own pace keep slow but steady progress,
    // as on the cloth, in FP32), FP64 after that and for the stopping test
    constexpr int kLbfgsStall32 = 100;
    constexpr double kLbfgsStallBand = 1e3;
    bool e32 = mixed() && params.mixed_elem32 != 0, e32_stall = false;
    double best32 = 0.0;
    int since32 = 0, longest32 = 0;
    double E0 = e32 ? energy_grad32() : energy_grad();
    double gn = std::sqrt(hsc->gnorm2);
    const double g0 = gn;
    best32 = gn;
    st.grad_norm0 = g0;
    start_instances();
    SSIM_CUDA(cudaMemcpyAsync(gprev.p, forces.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, stream));
    const double pd_tol = mixed() ? std::max(params.cg_rtol, 1e-6) : params.cg_rtol;
    double E0_scale = hsc->energy_scale;
    auto to_fp64 = [&]() {
      e32 = false;
      E0 = energy_grad();
      E0_scale = hsc->energy_scale;
      gn = std::sqrt(hsc->gnorm2);
      SSIM_CUDA(cudaMemcpyAsync(gprev.p, forces.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, stream));
    };
    V4<S>* q = s.lq.p;
    V4<S>* d = s.ld.p;
    auto slot = [&](int j) { return (head - hsize + j + m) % m; };  // j-th oldest entry
    int it = 0;
    for (;; ++it) {
      const double tgt = params.stop_mode == 0 ? abs_tol : params.rel_tol * g0;
      if (e32 && (gn <= params.elem32_switch * tgt || e32_stall)) to_fp64();
      st.grad_norm = gn;
      st.energy = E0;
      if (stop_test(gn, g0)) {
        st.converged = 1;
        break;
      }
      if (it >= params.max_lbfgs_iters) break;
      if (compact) {
        LbfgsHist<S> hist{};
        hist.n = hsize;
        for (int j = 0; j < hsize; ++j) {
          hist.s[j] = s.hs[slot(j)]->p;
          hist.y[j] = s.hy[slot(j)]->p;
          hist.slot[j] = slot(j);
        }
        if (hsize > 0) launch_lbfgs_multidot<S>(nv, gprev.p, hist, lbpart.p, lbtab.p, counter.p, stream);
        launch_lbfgs_combine<S>(nv, gprev.p, hist, lbtab.p + 2 * MC * MC, 1.0 / std::max(gn, 1e-300), d, red(),
                                stream);
      } else {
        // first loop, newest pair first: a_i = rho_i s_i.q, q -= a_i y_i (q starts as g, read from gprev,
        // which holds the current gradient)
        for (int j = hsize - 1; j >= 0; --j) {
          const int i = slot(j), inext = j + 1 < hsize ? slot(j + 1) : -1;
          launch_lbfgs_pass<S>(nv, j == hsize - 1 ? nullptr : q, gprev.p, q, inext >= 0 ? s.hy[inext]->p : nullptr,
                               inext >= 0 ? al + inext : nullptr, nullptr, -1.0, nullptr, 1.0, s.hs[i]->p, rho_h[i],
                               al + i, red(), stream);
        }
        // z = H0 q (q -= a_0 y_0 folded in), then b_0 = rho_0 y_0.z
        V4<S>* z = pd ? s.x.p : d;
        const int i0 = hsize > 0 ? slot(0) : -1;
        if (pd) {
          launch_lbfgs_pass<S>(nv, hsize > 0 ? q : nullptr, gprev.p, q, i0 >= 0 ? s.hy[i0]->p : nullptr,
                               i0 >= 0 ? al + i0 : nullptr, nullptr, -1.0, nullptr, 1.0, nullptr, 0.0, nullptr, red(),
                               stream);
          double rr = 0;
          st.cg_iters_total += pcg_on<S>(s.pd_kron ? s.pd_svals.p : s.pd_vals.p, s.pd_dinv.p, q, pd_tol,
                                       params.cg_max_iters, &rr, s.pd_kron);
          if (i0 >= 0)
            launch_lbfgs_pass<S>(nv, z, nullptr, z, nullptr, nullptr, nullptr, 0.0, nullptr, 1.0, s.hy[i0]->p,
                                 rho_h[i0], bb + i0, red(), stream);
        } else {
          const double h0 = hsize > 0 ? gamma : 1.0 / std::max(gn, 1e-300);
          launch_lbfgs_pass<S>(nv, hsize > 0 ? q : nullptr, gprev.p, z, i0 >= 0 ? s.hy[i0]->p : nullptr,
                               i0 >= 0 ? al + i0 : nullptr, nullptr, -1.0, nullptr, h0,
                               i0 >= 0 ? s.hy[i0]->p : nullptr, i0 >= 0 ? rho_h[i0] : 0.0,
                               i0 >= 0 ? bb + i0 : nullptr, red(), stream);
        }
        // second loop, oldest pair first: z += (a_{j-1} - b_{j-1}) s_{j-1}, b_j = rho_j y_j.z
        for (int j = 1; j < hsize; ++j) {
          const int i = slot(j), ip = slot(j - 1);
          launch_lbfgs_pass<S>(nv, z, nullptr, z, s.hs[ip]->p, al + ip, bb + ip, 1.0, nullptr, 1.0, s.hy[i]->p,
                               rho_h[i], bb + i, red(), stream);
        }
        // d = -(z + (a - b) s) of the newest pair; g.d and |d|^2
        const int il = hsize > 0 ? slot(hsize - 1) : -1;
        launch_lbfgs_final<S>(nv, z, il >= 0 ? s.hs[il]->p : nullptr, il >= 0 ? al + il : nullptr,
                              il >= 0 ? bb + il : nullptr, gprev.p, d, red(), stream);
      }
      // backtracking line search; each trial forms energy, forces and the curvature pair at u + alpha d
      const double Escale = (e32 ? params.ls_energy_slack32 : params.ls_energy_slack) * E0_scale;
      if (e32) split32();  // the trials' base point
      double alpha = 1.0, gd = 0.0, dn = 0.0;
      bool have_gd = false, accepted = false;
      auto trial = [&](double a) {
        launch_trial<S>(d, a, true, e32);
        gather_forces<S>(d, a, e32);
        launch_lbfgs_pair<S>(nv, a, d, forces.p, gprev.p, s.hs[head]->p, s.hy[head]->p, red(), stream);
        sync_scalars();
        st.ls_steps_total++;
      };
      for (int ls = 0; ls < params.max_ls_iters; ++ls) {
        trial(alpha);
        if (!have_gd) {
          gd = hsc->gd;
          have_gd = true;
          if (!(gd < 0)) {  // not a descent direction: drop the history, normalised steepest descent
            hsize = 0;
            st.ls_steps_total--;
            launch_lbfgs_pass<S>(nv, nullptr, gprev.p, q, nullptr, nullptr, nullptr, 0.0, nullptr,
                                 1.0 / std::max(gn, 1e-300), nullptr, 0.0, nullptr, red(), stream);
            launch_lbfgs_final<S>(nv, q, nullptr, nullptr, nullptr, gprev.p, d, red(), stream);
            trial(alpha);
            gd = hsc->gd;
          }
          dn = std::sqrt(hsc->dnorm2);
        }
        if (hsc->trial_energy <= E0 + params.lbfgs_armijo * alpha * gd + Escale) {
          accepted = true;
          break;
        }
        alpha *= params.ls_shrink;
      }
      if (!accepted) {  // the search ran out: the step is taken at the last shrunk alpha
        trial(alpha);
        e32_stall = e32;
      }
      launch_lbfgs_accept<S>(nv, alpha, d, next.p, forces.p, gprev.p, stream);
      st.last_change = alpha * dn;
      E0 = hsc->trial_energy;
      E0_scale = hsc->trial_energy_scale;
      gn = std::sqrt(hsc->gnorm2);
      if (!std::isfinite(E0) || !std::isfinite(gn))
        throw numerical_error("non-finite energy or gradient (inverted or degenerate element?)");
      if (e32) {
        const double tgt32 = params.stop_mode == 0 ? abs_tol : params.rel_tol * g0;
        if (gn < 0.5 * best32) {
          longest32 = std::max(longest32, since32 + 1);
          best32 = gn;
          since32 = 0;
        } else if (++since32 >= std::max(kLbfgsStall32, 3 * longest32) && best32 <= kLbfgsStallBand * tgt32) {
          e32_stall = true;
        }
      }
      const double sy = hsc->pair_sy, yy = hsc->pair_yy;
      if (sy > 1e-300) {
        rho_h[head] = 1.0 / sy;
        gamma = sy / yy;
        head = (head + 1) % m;
        hsize = std::min(hsize + 1, m);
      } else if (hsize == m) {
        hsize = m - 1;  // the pair was formed in the oldest entry's storage: that entry is gone
      }
    }
    st.newton_iters = it;
  }

  // bytes one PCG SpMV launch must move in this storage format, each array counted once: upper values
  // + block columns (padding slots included: they are read), lower slot/column indices, slice offsets,
  // z and p_old read, p_new and q written (4-wide vectors).  The transposed re-reads of upper blocks for
  // the lower triangle and the repeated x gathers are cache traffic, not counted.
  double spmv_bytes(size_t s) const {
    const double up = topo.nslots, lo = topo.nlslots;
    return up * (9.0 * s + 4.0) + lo * 8.0 + 2.0 * (topo.nslices + 1) * 4 + 4.0 * nv * 4 * s;
  }

  // bytes one SpMV on the FP16 copy moves: 18 B of values and a 4-byte column per entry, the gathered vector
  // and the product once, the inverse scale for the unscaled residual norm
  double half_spmv_bytes() const { return 22.0 * (double)nfs + 3.0 * nv * 16.0; }
  // bytes one PCG update pass moves: p, q, x, r read, x, r, z written, the 3x3 preconditioner blocks
  double update_bytes(size_t s) const { return 7.0 * nv * 4 * s + 3.0 * nv * 4 * s; }

  // ------------------------------------------------------------------ adjoint of one step
  // The handle's next_deform holds u_{n+1}.  ubar, vbar (device [n]) hold the adjoint of (u_{n+1}, v_{n+1}) on
  // entry and of (u_n, v_n) on exit; ebar (device [T]) accumulates dL/dE_e.  Returns the PCG iterations;
  // *projected = 1 when the exact Hessian was not positive definite along the CG directions and the solve
  // fell back to the SPD-projected one.
  template <typename S>
  int adjoint_step(double* ubar, double* vbar, double* ebar, double rtol, int max_iters, int* projected) {
    Solver<S>& s = solver<S>();
    if (mixed()) launch_refresh_xf(nv, dX.p, next.p, xf.p, stream);
    hessian<S>(false, true);
    launch_adj_prep(n, (1.0 - damping) / dt, ubar, vbar, dof_type.p, work.p, gprev.p, stream);
    double rr = 0;
    int it = pcg<S>(work.p, false, rtol, max_iters, &rr);
    int proj = 0;
    if (hsc->status == 1) {  // indefinite along a CG direction: use the projected Hessian
      hessian<S>(true, true);
      it += pcg<S>(work.p, false, rtol, max_iters, &rr);
      proj = 1;
    }
    if (projected) *projected = proj;
    s.mvals.alloc(9 * (size_t)topo.nslots);
    launch_assemble<S>(A(), cptr.p, csrc.p, nullptr, s.slot_mass.p, mask.p, false, s.mvals.p, nullptr, 0, stream);
    launch_spmv<S>(A(), s.mvals.p, s.x.p, s.q.p, stream);
    launch_adj_finish<S>(nv, dt, s.q.p, dof_type.p, gprev.p, ubar, vbar, stream);
    launch_adj_material<S>(e64(), dX.p, next.p, s.x.p, dt * dt, ebar, stream);
    SSIM_CUDA(cudaStreamSynchronize(stream));
    return it;
  }

  // ------------------------------------------------------------------ Newton stepper
  // time_step_solver_backward_euler::solve_impl (backward_euler.hpp:15-33) over mathprim's
  // newton_optimizer (absent from the reference tree; the definition used is the one restated by the
  // oracle): evaluate; stop on the gradient test; H = update_hessian(true, make_spsd = true); d from
  // Jacobi-PCG on H d = -g; backtracking Armijo line search from alpha = 1 (with the energy round-off
  // slack ls_energy_slack * sum of |energy terms|); x += alpha d.
  template <typename S>
  void newton(ssim_gb_step_stats& st) {
    Solver<S>& s = solver<S>();
    // mixed precision: the inner iterations evaluate energy and forces with FP32 element arithmetic (the
    // small-strain forms); the stopping test is then confirmed with an FP64 evaluation, and if the FP64
    // residual is above the target (or the FP32 residual stalls) the remaining iterations run in FP64
    bool e32 = mixed() && params.mixed_elem32 != 0;
    // after the FP32 phase: FP32 increments from the FP64 evaluation at the switch (delta)
    bool delta = false;
    double E0 = e32 ? energy_grad32() : energy_grad();
    double Escale = hsc->energy_scale;
    double gn = std::sqrt(hsc->gnorm2);
    const double g0 = gn;
    st.grad_norm0 = g0;
    start_instances();
    double gn_prev = gn;
    int stall = 0;
    auto to_fp64 = [&]() {
      e32 = false;
      E0 = energy_grad();
      Escale = hsc->energy_scale;
      gn = std::sqrt(hsc->gnorm2);
      if constexpr (std::is_same<S, float>::value) {
        if (delta_supported()) {
          set_delta_reference(E0, Escale);
          delta = true;
        }
      }
    };
    int it = 0;
    // speculation: tets in mixed precision (the Hessian reads only the FP32 positions), not while profiling
    const bool can_spec = params.speculative_hessian == 1 && std::is_same<S, float>::value && !springs && !tri2d &&
                          !profiling;
    bool spec_ready = false;  // this iteration's matrix was assembled ahead, at the accepted full step
    for (;; ++it) {
      st.grad_norm = gn;
      st.energy = E0;
      // the FP32 phase ends once the residual is within elem32_switch times the target (FP32 rounding of
      // the O(|g0|) inertia and elastic forces is close to a 1e-6 target), or when it stalls
      const double tgt = params.stop_mode == 0 ? abs_tol : params.rel_tol * g0;
      if (e32 && (gn <= params.elem32_switch * tgt || stall >= 2)) {
        to_fp64();
        st.grad_norm = gn;
        st.energy = E0;
      } else if (delta && stall >= 3) {
        // the increments have grown with little progress: a fresh FP64 reference at the current state
        to_fp64();
        stall = 0;
        st.grad_norm = gn;
        st.energy = E0;
      }
      if (stop_test(gn, g0)) {
        st.converged = 1;
        break;
      }
      if (it >= params.max_newton_iters) break;
      double eta = params.cg_rtol;
      if (params.cg_forcing == 1 && g0 > 0) eta = std::min(params.cg_rtol, std::max(params.cg_eta_min, gn / g0));
      // a solve on the FP16 matrix copy can take FP16 element blocks too (half_hessian_blocks)
      const bool k16 = std::is_same<S, float>::value && params.half_hessian_blocks == 1 && use_half(eta);
      spec_join();
      if (!(spec_ready && spec_k16 == k16)) {
        if (mixed()) launch_refresh_xf(nv, dX.p, next.p, xf.p, stream);
        hessian<S>(true, true, k16);
      }
      spec_ready = false;
      double rr = 0;
      st.cg_iters_total += pcg<S>(forces.p, true, eta, params.cg_max_iters, &rr);
      // every solve on the copy is checked: on the reference's light, stiff unit box the first solves of a
      // step pass and later ones of the same step miss the forcing by 40%, so sampling (the first solves
      // after reset(), the first of each step) let the copy cost it a fifth more Newton iterations
      const bool checked = last_half;
      st.half_solves += last_half ? 1 : 0;
      if (!(checked && half_checked)) {  // the pipelined solve on the copy did this in its own launch
        if constexpr (std::is_same<S, float>::value) {
          if (checked)
            launch_dot_gd_check(A(), s.vals.p, forces.p, s.x.p, red(), stream);
          else
            launch_dot_gd<S>(nv, forces.p, s.x.p, red(), stream);
        } else {
          launch_dot_gd<S>(nv, forces.p, s.x.p, red(), stream);
        }
        sync_scalars();
      }
      // a solve on the FP16 copy whose true residual (FP32 values) misses the forcing by the slack: the copy's
      // rounding is too coarse for this system's conditioning; later solves use the FP32 values
      const double tr_max = params.half_check_slack * eta;
      if (checked && hsc->true_bb > 0) {
        st.half_check = std::max(st.half_check, std::sqrt(hsc->true_rr / hsc->true_bb) / eta);
        if (!(hsc->true_rr <= tr_max * tr_max * hsc->true_bb)) half_off = true;
      }
      double gd = hsc->gd;
      const double dn = std::sqrt(hsc->dnorm2);
      if (!(gd < 0)) {  // not a descent direction: steepest descent
        launch_to_vec4<S>(nv, forces.p, s.x.p, true, stream);
        gd = -gn * gn;
      }
      // the next iteration's matrix at the full step, on the side stream while the line search runs; its
      // element-block precision is the one the next forcing term will ask for (FP16 blocks only when every
      // possible next forcing term allows them)
      const bool spec = can_spec && it + 1 < params.max_newton_iters;
      if (spec) {
        const double eta_lo = std::min(params.cg_rtol, params.cg_forcing == 1 ? params.cg_eta_min : params.cg_rtol);
        spec_k16 = params.half_hessian_blocks == 1 && use_half(eta_lo);
        if constexpr (std::is_same<S, float>::value) spec_hessian<S>(s.x.p, spec_k16);
      }
      // backtracking line search; each trial evaluates energy and forces at u + alpha d in one element
      // pass, so the accepted trial's forces are the next gradient (no separate evaluation)
      double alpha = 1.0;
      double Et = 0, Et_scale = 0;
      const double slack = (e32 ? params.ls_energy_slack32 : params.ls_energy_slack) * Escale;
      if (e32) split32();  // the trials' base point
      if constexpr (std::is_same<S, float>::value) {
        if (delta) delta_base();
      }
      for (int ls = 0; ls < params.max_ls_iters; ++ls) {
        if constexpr (std::is_same<S, float>::value) {
          if (delta)
            delta_trial(s.x.p, alpha);
          else
            launch_trial<S>(s.x.p, alpha, true, e32);
        } else {
          launch_trial<S>(s.x.p, alpha, true, e32);
        }
        sync_scalars();
        st.ls_steps_total++;
        Et = hsc->trial_energy;
        Et_scale = hsc->trial_energy_scale;
        if (Et <= E0 + params.armijo * alpha * gd + slack) break;
        if (ls + 1 < params.max_ls_iters) alpha *= params.ls_shrink;
      }
      if (spec) SSIM_CUDA(cudaStreamWaitEvent(stream, ev_xf, 0));
      launch_axpy_update<S>(nv, alpha, s.x.p, dX.p, next.p, nullptr, stream);
      if (delta)
        delta_gather();
      else
        gather_forces<S>(nullptr, 0.0, e32);
      sync_scalars();
      if (!std::isfinite(Et) || !std::isfinite(hsc->gnorm2))
        throw numerical_error("non-finite energy or gradient (inverted or degenerate element?)");
      st.last_change = alpha * dn;
      E0 = Et;
      Escale = Et_scale;
      gn = std::sqrt(hsc->gnorm2);
      stall = gn > 0.5 * gn_prev ? stall + 1 : 0;
      gn_prev = gn;
      spec_ready = spec && alpha == 1.0;
      st.spec_hits += spec_ready ? 1 : 0;
    }
    spec_join();
    st.newton_iters = it;
  }

  // ------------------------------------------------------------------ nonlinear CG
  void set_ncg_matrix(const double* values) {
    if (!values) {
      ncg_vals.clear();
      ++ncg_ver;
      return;
    }
    const size_t nnz = 9 * (size_t)topo.nnzb;
    if (ncg_rp.n == 0) {
      std::vector<int32_t> rp(n + 1), ci(nnz);
      csr_pattern(topo, rp.data(), ci.data());
      ncg_tperm.assign(nnz, 0);
      for (int r = 0; r < n; ++r)
        for (int k = rp[r]; k < rp[r + 1]; ++k) {
          const int c = ci[k];
          ncg_tperm[k] = std::lower_bound(ci.begin() + rp[c], ci.begin() + rp[c + 1], r) - ci.begin();
        }
      ncg_rp.upload(rp, stream);
      ncg_ci.upload(ci, stream);
    }
    ncg_vals.assign(values, values + nnz);
    ++ncg_ver;
  }

  template <typename S>
  void ncg_sync(Solver<S>& s) {
    if (s.ncg_version == ncg_ver || ncg_vals.empty()) return;
    std::vector<S> L(ncg_vals.begin(), ncg_vals.end()), Lt(ncg_vals.size());
    for (size_t k = 0; k < ncg_vals.size(); ++k) Lt[k] = (S)ncg_vals[ncg_tperm[k]];
    s.ncg_L.upload(L, stream);
    s.ncg_Lt.upload(Lt, stream);
    s.ncg_version = ncg_ver;
  }

  // out = H in with H = L L^T (out = in without a factor); tmp is scratch
  template <typename S>
  void ncg_apply(Solver<S>& s, bool prec, const V4<S>* in, V4<S>* out, V4<S>* tmp) {
    if (!prec || ncg_vals.empty()) {
      if (out != in) launch_vaxpby<S>(nv, 0.0, out, 1.0, in, stream);
      return;
    }
    launch_csr_dof_spmv<S>(n, ncg_rp.p, ncg_ci.p, s.ncg_Lt.p, in, tmp, stream);
    launch_csr_dof_spmv<S>(n, ncg_rp.p, ncg_ci.p, s.ncg_L.p, tmp, out, stream);
  }

  // time_step_solver_ncg / _with_ext_prec (nonlinear_cg.hpp:9-97) over mathprim's ncg_optimizer (Dai-Kou,
  // backtracking, learning rate 1e-2, 1000 iterations).  mathprim is not in the reference tree: the
  // iteration is the published Dai-Kou method (Y.-H. Dai, C.-X. Kou, SIAM J. Optim. 23(1) 2013) with the
  // line search described at the FP64 oracle's ncg_core, which this follows step for step.
  template <typename S>
  void ncg(ssim_gb_step_stats& st, bool prec) {
    Solver<S>& s = solver<S>();
    if (prec) ncg_sync<S>(s);
    V4<S>* d = s.ld.p;   // direction
    V4<S>* z = s.lq.p;   // H g
    V4<S>* y = s.r.p;    // g - g_prev
    V4<S>* hy = s.x.p;   // H y
    V4<S>* gv = s.z.p;   // g, 4-wide
    V4<S>* t = s.tmp.p;  // scratch of ncg_apply
    double E = energy_grad();
    double Escale = hsc->energy_scale;
    double gn = std::sqrt(hsc->gnorm2);
    const double g0 = gn;
    st.grad_norm0 = g0;
    start_instances();
    SSIM_CUDA(cudaMemcpyAsync(gprev.p, forces.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, stream));
    launch_to_vec4<S>(nv, forces.p, gv, false, stream);
    ncg_apply<S>(s, prec, gv, z, t);
    launch_vaxpby<S>(nv, 0.0, d, -1.0, z, stream);
    auto dot_g = [&]() {  // g.d and |d|^2 of the current forces and direction
      launch_dot_gd<S>(nv, forces.p, d, red(), stream);
      sync_scalars();
    };
    dot_g();
    double gd = hsc->gd, dn2 = hsc->dnorm2;
    double alpha_init = params.ncg_step0;
    auto trial = [&](double a) {
      launch_trial<S>(d, a, false);
      sync_scalars();
      st.ls_steps_total++;
      return hsc->trial_energy;
    };
    int it = 0;
    for (;; ++it) {
      st.grad_norm = gn;
      st.energy = E;
      if (stop_test(gn, g0)) {
        st.converged = 1;
        break;
      }
      if (it >= params.ncg_max_iters) break;
      if (!(gd < 0)) {  // restart
        launch_vaxpby<S>(nv, 0.0, d, -1.0, z, stream);
        dot_g();
        gd = hsc->gd;
        dn2 = hsc->dnorm2;
        if (!(gd < 0)) {
          launch_to_vec4<S>(nv, forces.p, d, true, stream);
          dot_g();
          gd = hsc->gd;
          dn2 = hsc->dnorm2;
        }
        alpha_init = params.ncg_step0;
      }
      const double slack = params.ls_energy_slack * Escale;
      auto armijo = [&](double aa, double ee) { return ee <= E + params.lbfgs_armijo * aa * gd + slack; };
      double a = alpha_init, Et = trial(a);
      for (int ls = 1; ls < params.max_ls_iters && !armijo(a, Et); ++ls) {
        const double c2 = (Et - E - gd * a) / (a * a);
        double an = c2 > 0 ? -gd / (2 * c2) : 0.5 * a;
        if (!std::isfinite(an)) an = 0.5 * a;
        a = std::min(std::max(an, 0.1 * a), 0.5 * a);
        Et = trial(a);
      }
      for (int ex = 0; ex < params.ncg_expand && armijo(a, Et); ++ex) {
        const double c2 = (Et - E - gd * a) / (a * a);
        if (!(c2 > 0)) break;
        const double astar = -gd / (2 * c2);
        if (!(astar > 1.5 * a)) break;
        const double an = std::min(astar, 10 * a);
        const double En = trial(an);
        if (!(En < Et) || !armijo(an, En)) break;
        a = an;
        Et = En;
      }
      launch_axpy_update<S>(nv, a, d, dX.p, next.p, nullptr, stream);
      st.last_change = a * std::sqrt(dn2);
      E = energy_grad();
      Escale = hsc->energy_scale;
      gn = std::sqrt(hsc->gnorm2);
      launch_vdiff<S>(nv, forces.p, gprev.p, y, stream);
      SSIM_CUDA(cudaMemcpyAsync(gprev.p, forces.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, stream));
      launch_to_vec4<S>(nv, forces.p, gv, false, stream);
      ncg_apply<S>(s, prec, gv, z, t);
      const V4<S>* hyp = y;
      if (prec && !ncg_vals.empty()) {
        ncg_apply<S>(s, prec, y, hy, t);
        hyp = hy;
      }
      const double dy = vdot<S>(d, y), zy = vdot<S>(z, y), yhy = vdot<S>(y, hyp);
      dot_g();
      const double gdn = hsc->gd, dd = hsc->dnorm2;
      double beta = 0;
      if (dy > 1e-300) beta = zy / dy - yhy * gdn / (dy * dy);
      if (dd > 0) beta = std::max(beta, params.ncg_eta * gdn / dd);
      const double gd_old = gd;
      launch_vaxpby<S>(nv, beta, d, -1.0, z, stream);
      dot_g();
      gd = hsc->gd;
      dn2 = hsc->dnorm2;
      alpha_init = (gd < 0 && gd_old < 0) ? a * gd_old / gd : params.ncg_step0;
    }
    st.newton_iters = it;
  }

  // compute_step (time_step.hpp:520-528): run the stepper, then |g| at the result
  double compute_step() {
    if (!has_reset) throw state_error("compute_step() before reset()");
    ssim_gb_step_stats st{};
    const auto t0 = std::chrono::high_resolution_clock::now();
    if (stepper == SSIM_GB_STEPPER_NEWTON) {
      if (mixed())
        newton<float>(st);
      else
        newton<double>(st);
    } else if (stepper == SSIM_GB_STEPPER_LBFGS || stepper == SSIM_GB_STEPPER_PD) {
      if (mixed())
        lbfgs<float>(st, stepper == SSIM_GB_STEPPER_PD);
      else
        lbfgs<double>(st, stepper == SSIM_GB_STEPPER_PD);
    } else if (stepper == SSIM_GB_STEPPER_H0) {
      if (mixed())
        lbfgs<float>(st, false, true);
      else
        lbfgs<double>(st, false, true);
    } else if (stepper == SSIM_GB_STEPPER_NCG || stepper == SSIM_GB_STEPPER_NCG_EXT) {
      if (mixed())
        ncg<float>(st, stepper == SSIM_GB_STEPPER_NCG_EXT);
      else
        ncg<double>(st, stepper == SSIM_GB_STEPPER_NCG_EXT);
    } else if (stepper == SSIM_GB_STEPPER_FORWARD_EULER) {
      // time_step_solver_forward_euler (time_step.hpp:717-736): evaluate, next += dt^2 / 2 * forces; then
      // the re-evaluation of compute_step
      energy_grad();
      launch_axpy_d(n, 0.5 * dt * dt, forces.p, next.p, stream);
      st.energy = energy_grad();
      st.grad_norm = st.grad_norm0 = std::sqrt(hsc->gnorm2);
      st.converged = 1;
    } else {
      // time_step_solver_nothing: no solve; the gradient is still evaluated
      st.energy = energy_grad();
      st.grad_norm = st.grad_norm0 = std::sqrt(hsc->gnorm2);
    }
    const auto t1 = std::chrono::high_resolution_clock::now();
    st.elapsed_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    stats = st;
    return st.grad_norm;
  }

  // ------------------------------------------------------------------ launch-shape autotuning
  // ssim_gb_autotune: times candidate launch shapes on this handle's data and applies the fastest; the
  // choice is cached per process by the problem's shape (see ssim_gb.h).
  using TuneKey = std::tuple<int, int, long long, int, int, int>;
  static std::map<TuneKey, ssim_gb_tuning>& tune_cache() {
    static std::map<TuneKey, ssim_gb_tuning> m;
    return m;
  }
  static std::mutex& tune_mutex() {
    static std::mutex m;
    return m;
  }
  void apply_tuning(const ssim_gb_tuning& t) {
    shapes.elem = t.elem_block;
    shapes.hess = t.hessian_block;
    shapes.assem = t.assembly_block;
    shapes.gather = t.gather_block;
    shapes.elem_regcap = t.elem_regcap;
    params.pcg_persistent = t.pcg_persistent;
    params.pcg_max_blocks = t.pcg_max_blocks;
    params.fused_assembly = t.fused_assembly;
    params.pcg_half_matrix = t.pcg_half_matrix;
  }
  ssim_gb_tuning autotune() {
    if (!has_reset) throw state_error("autotune() before reset()");
    const TuneKey key{nv, nt, topo.nnzb, mixed() ? 1 : 0, ninst, springs ? 2 : (tri2d ? 1 : 0)};
    {
      std::lock_guard<std::mutex> lock(tune_mutex());
      auto it = tune_cache().find(key);
      if (it != tune_cache().end()) {
        ssim_gb_tuning t = it->second;
        apply_tuning(t);
        t.from_cache = 1;
        return t;
      }
    }
    ssim_gb_tuning t{};
    if (mixed())
      tune_impl<float>(t);
    else
      tune_impl<double>(t);
    apply_tuning(t);
    t.from_cache = 0;
    std::lock_guard<std::mutex> lock(tune_mutex());
    tune_cache()[key] = t;
    return t;
  }
  // mean time of f over reps launches after one untimed launch, CUDA events on the handle's stream (ms)
  template <typename F>
  double time_launches(F&& f, int reps = 3) {
    cudaEvent_t a, b;
    SSIM_CUDA(cudaEventCreate(&a));
    SSIM_CUDA(cudaEventCreate(&b));
    f();
    SSIM_CUDA(cudaEventRecord(a, stream));
    for (int r = 0; r < reps; ++r) f();
    SSIM_CUDA(cudaEventRecord(b, stream));
    SSIM_CUDA(cudaEventSynchronize(b));
    float ms = 0;
    SSIM_CUDA(cudaEventElapsedTime(&ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return ms / reps;
  }
  template <typename S>
  void tune_impl(ssim_gb_tuning& t) {
    Solver<S>& s = solver<S>();
    const bool tets = !springs && !tri2d;
    DBuf<double> keep, rhs;
    keep.alloc(n);
    SSIM_CUDA(cudaMemcpyAsync(keep.p, forces.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, stream));
    int count = 0;
    // FP32 element pass and force gather (the mixed path's tet kernels)
    if constexpr (std::is_same<S, float>::value) {
      if (tets) {
        split32();
        double best = 1e300;
        for (int b : {64, 128, 256})
          for (int cap : {0, 1}) {
            const double ms = time_launches([&] {
              launch_elem_energy_grad32(e64(), e32s(), s32(), s.x.p, 0.0, dt * dt, rho, lf32t.p, true, true, red(),
                                        stream, b, cap);
            });
            ++count;
            if (ms < best) best = ms, t.elem_block = b, t.elem_regcap = cap;
          }
        t.elem_us = best * 1e3;
        best = 1e300;
        for (int b : {128, 256, 512}) {
          const double ms = time_launches(
              [&] { launch_vertex_gather32(nv, vptr.p, vinc.p, lf32t.p, mask.p, forces.p, red(), stream, b); });
          ++count;
          if (ms < best) best = ms, t.gather_block = b;
        }
      }
    }
    // element Hessian and assembly: block sizes of the two kernels, against the fused kernel
    if (mixed()) launch_refresh_xf(nv, dX.p, next.p, xf.p, stream);
    const float4* xfp = mixed() ? xf.p : nullptr;
    t.hessian_block = 0;
    t.assembly_block = 0;
    double hbest = 1e300, abest = 1e300;
    s.K.alloc((size_t)9 * (topo.cv * (topo.cv + 1) / 2) * nt);
    if (tets) {
      for (int b : {32, 64, 128}) {
        const double ms = time_launches(
            [&] { launch_elem_hessian<S>(e64(), e32(), dX.p, next.p, xfp, dt * dt, true, s.K.p, stream, b); });
        ++count;
        if (ms < hbest) hbest = ms, t.hessian_block = b;
      }
    } else {
      hbest = 0;
      hessian<S>(true, true);  // the springs' / triangles' element blocks for the assembly timings
    }
    for (int b : {128, 256, 512}) {
      const double ms = time_launches([&] {
        launch_assemble<S>(A(), cptr.p, csrc.p, s.K.p, s.slot_mass.p, mask.p, true, s.vals.p, s.dinv.p,
                           params.precond, stream, b);
      });
      ++count;
      if (ms < abest) abest = ms, t.assembly_block = b;
    }
    ++asm_count;  // the timed assemblies rewrote the system values
    t.hessian_us = (hbest + abest) * 1e3;
    t.fused_assembly = 0;
    if (tets && fused_ready()) {
      const double ms = time_launches([&] {
        launch_fused_hessian<S>(e64(), e32(), dX.p, next.p, xfp, dt * dt, true, A(), topo.nslices, fused_spc,
                                fused_ncta, fptr.p, felem.p, fcode.p, s.slot_mass.p, mask.p, true, s.vals.p, s.dinv.p,
                                params.precond, stream);
      });
      ++count;
      if (ms < hbest + abest) t.fused_assembly = 1, t.hessian_us = ms * 1e3;
    }
    // PCG on the assembled matrix: variant and persistent grid, one solve to 5e-2 from a fixed right-hand side
    std::vector<double> ones(n, 1.0);
    rhs.upload(ones, stream);
    int nsm = 0, dev = 0;
    SSIM_CUDA(cudaGetDevice(&dev));
    SSIM_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    // mixed: Chronopoulos-Gear or standard PCG on the FP32 values, and on the FP16 copy (when enabled) the
    // automatic choice (pipelined, variant 3) or Chronopoulos-Gear
    const std::vector<int> variants = mixed() ? std::vector<int>{2, 1, 3} : std::vector<int>{0, 2};
    std::vector<int> grids = {0};
    if (4 * nsm < div_up(nv, 256)) grids.push_back(4 * nsm);
    const int keep_variant = params.pcg_persistent, keep_grid = params.pcg_max_blocks;
    const int keep_half = params.pcg_half_matrix;
    const size_t log0 = solve_log.size();
    double pbest = 1e300;
    t.pcg_persistent = keep_variant;
    t.pcg_max_blocks = keep_grid;
    t.pcg_half_matrix = keep_half;
    for (int v : variants)
      for (int gcap : grids)
        for (int half : {0, 1}) {
          if (v == 0 && gcap != 0) continue;  // the two-launch loop has no persistent grid
          // the FP16 copy serves only these, and only when enabled (the sweep may turn it off, never on)
          if (half && ((v != 2 && v != 3) || !mixed() || keep_half != 1 || !half_ready())) continue;
          if (v == 3 && !half) continue;  // on the FP32 values variant 3 is variant 2
          params.pcg_persistent = v;
          params.pcg_max_blocks = gcap;
          params.pcg_half_matrix = half;
          int iters = 0;
          // the FP16 candidate pays its conversion in every timed solve, as each Newton solve follows an assembly
          const double ms = time_launches([&] {
            h16_count = -1;
            iters = pcg<S>(rhs.p, false, 5e-2, params.cg_max_iters, nullptr);
          }, 2);
          ++count;
          if (ms < pbest)
            pbest = ms, t.pcg_persistent = v, t.pcg_max_blocks = gcap, t.pcg_iterations = iters, t.pcg_half_matrix = half;
        }
    params.pcg_persistent = keep_variant;
    params.pcg_max_blocks = keep_grid;
    params.pcg_half_matrix = keep_half;
    solve_log.resize(log0);
    t.pcg_solve_ms = pbest;
    t.candidates = count;
    SSIM_CUDA(cudaMemcpyAsync(forces.p, keep.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, stream));
    SSIM_CUDA(cudaStreamSynchronize(stream));
  }

  // ------------------------------------------------------------------ profiling
  void prof_begin(cudaEvent_t& a, cudaEvent_t& b) {
    SSIM_CUDA(cudaEventCreate(&a));
    SSIM_CUDA(cudaEventCreate(&b));
    SSIM_CUDA(cudaEventRecord(a, stream));
  }
  void prof_end(cudaEvent_t a, cudaEvent_t b, int kind, double bytes) {
    SSIM_CUDA(cudaEventRecord(b, stream));
    SSIM_CUDA(cudaEventSynchronize(b));
    float ms = 0;
    SSIM_CUDA(cudaEventElapsedTime(&ms, a, b));
    prof_ms[kind] += ms;
    prof_launch[kind] += 1;
    if (bytes > 0) prof_bytes[kind] = bytes;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
  }
  void set_profiling(bool on) {
    profiling = on;
    if (on && ev.empty()) {
      ev.resize(512);
      for (auto& e : ev) SSIM_CUDA(cudaEventCreate(&e));
    }
    for (int k = 0; k < PK_COUNT; ++k) {
      prof_launch[k] = 0;
      prof_ms[k] = 0;
    }
  }
};

template <>
inline Solver<float>& TimeStep::solver<float>() {
  return sf;
}
template <>
inline Solver<double>& TimeStep::solver<double>() {
  return sd;
}

}  // namespace ssim_gb

