// kernels.cuh -- launchers of the device kernels (definitions in kernels_elem.cu / kernels_sparse.cu).
//
// HBM layout of one time-step object (T tets, V vertices, S = float (mixed) or double (FP64)):
//   cells        int4[T]                       vertex ids of each tet
//   element SoA  dminv[9][T], vol[T], lam[T], mu[T]   (FP64, plus an FP32 copy for the mixed path)
//   state        [V*3] FP64 in the reference layout (deformation, next, inertia, velocity, ...)
//   xf           float4[V]  current positions X + u rounded to FP32 (mixed-path Hessian input)
//   matrix       symmetric 3x3-block SELL-32: slice s covers block rows 32s..32s+31; upper slot
//                (s, k, lane) holds block (row = 32s+lane, col = sl_col[slot] >= row); value c of a slot q
//                sits at vals[9*(q & ~31) + 32*c + (q & 31)] so that every component load of a warp is one
//                128-byte (FP32) or 256-byte (FP64) line; lower blocks are transposed upper slots
//   dinv         vec4<S>[3V]  rows of the inverse 3x3 diagonal block (block-Jacobi preconditioner)
//   Kbuf         S[T][10][9]  scaled element stiffness blocks (v <= w) awaiting assembly
//   lf           double[T][4][3] scaled element forces awaiting the vertex gather
//   vectors      vec4<S>[V]  CG vectors, one padded xyz triple per vertex
#pragma once
#include <type_traits>
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace ssim_gb {

template <typename S>
using V4 = typename vec4<S>::type;

// a 4-wide vector with w = 0
template <typename S>
__device__ __forceinline__ V4<S> mk4(S a, S b, S c) {
  V4<S> r;
  r.x = a;
  r.y = b;
  r.z = c;
  r.w = S(0);
  return r;
}

struct ElemFP64 {
  int nt;
  const int4* cells;
  const double* dminv;  // SoA [9][nt]
  const double* vol;
  const double* lam;
  const double* mu;
  const double* alpha;  // 1 + 3/4 mu / lambda
  const double* psi0;   // stable Neo-Hookean energy at F = I
  int model;            // 0 stable Neo-Hookean, 1 linear
  const double* delta;  // triangles: the 2D stable Neo-Hookean log offset per element (tets: 1, unused)
};

struct ElemFP32 {
  int nt;
  const int4* cells;
  const float* dminv;  // SoA [9][nt]
  const float* vol;
  const float* lam;
  const float* mu;
};

// per-vertex FP32 split of the state for the FP32 element / spring passes: uh + ul = u (to ~2^-48),
// w = u - x~ rounded once
// Calls fn(std::integral_constant<int, B>) for the block size B in the candidate list equal to `block`
// (the first candidate if none is): the run-time choice of a launch's block size among compiled variants
template <int... Bs, typename Fn>
inline void dispatch_block(int block, Fn&& fn) {
  bool done = false;
  ((!done && block == Bs ? (fn(std::integral_constant<int, Bs>{}), done = true) : false), ...);
  if (!done) {
    constexpr int first[] = {Bs...};
    fn(std::integral_constant<int, first[0]>{});
  }
}

struct Split32 {
  const float4* uh;
  const float4* ul;
  const float4* w;
};

// springs (2-vertex cells) of a mass-spring system
struct SpringData {
  int ns;
  const int2* ends;     // [ns] (i, j)
  const double* X;      // [V][3] rest positions
  const double* rest;   // [ns] rest lengths
  const double* k;      // [ns] stiffness
  const float4* e0;     // [ns] FP32 rest edge X_i - X_j and rest length (the FP32 spring pass)
  const float* k32;     // [ns] FP32 stiffness
};

struct Reduce {
  double* partials;       // [grid * 4] scratch
  unsigned int* counter;  // zero-initialised, restored by the last block
  DevScalars* sc;
};

// Symmetric 3x3-block matrix: upper blocks (w >= u) in SELL-32 slots; the lower blocks of row u are read
// as transposes of upper slots of other rows through a second SELL-32 index.
struct SellMatrix {
  int nv;
  int nslots;
  const int* sl_off;    // [nslices + 1] slot offset of each slice (multiple of 32)
  const int* sl_col;    // [nslots] block column (vertex); own row for padding
  const int* slot_row;  // [nslots] block row, -1 for padding
  const int* lo_off;    // [nslices + 1]
  const int* lo_src;    // [nlslots] upper slot holding the transposed block, -1 for padding
  const int* lo_col;    // [nlslots] block column (own row for padding)
};

// 3x3 preconditioner rows from a diagonal block a (row-major): 0 identity, 1 Jacobi, 2 block-Jacobi
// (inverse of the symmetric block by its adjugate; falls back to Jacobi if the block is singular).
template <typename S>
__device__ __forceinline__ void precond_rows(const S* a, int precond, V4<S>* out) {
  S m[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) m[i] = S(0);
  if (precond == 2) {
    const S c0 = a[4] * a[8] - a[5] * a[7], c1 = a[5] * a[6] - a[3] * a[8], c2 = a[3] * a[7] - a[4] * a[6];
    const S det = a[0] * c0 + a[1] * c1 + a[2] * c2;
    if (det > S(0) && isfinite(det)) {
      const S id = S(1) / det;
      m[0] = c0 * id;
      m[1] = (a[2] * a[7] - a[1] * a[8]) * id;
      m[2] = (a[1] * a[5] - a[2] * a[4]) * id;
      m[3] = c1 * id;
      m[4] = (a[0] * a[8] - a[2] * a[6]) * id;
      m[5] = (a[2] * a[3] - a[0] * a[5]) * id;
      m[6] = c2 * id;
      m[7] = (a[1] * a[6] - a[0] * a[7]) * id;
      m[8] = (a[0] * a[4] - a[1] * a[3]) * id;
      // symmetrise (the block is symmetric; keeps the preconditioner exactly symmetric)
      const S m01 = S(0.5) * (m[1] + m[3]), m02 = S(0.5) * (m[2] + m[6]), m12 = S(0.5) * (m[5] + m[7]);
      m[1] = m[3] = m01;
      m[2] = m[6] = m02;
      m[5] = m[7] = m12;
    } else {
      precond = 1;
    }
  }
  if (precond == 1) {
    m[0] = a[0] != S(0) ? S(1) / a[0] : S(1);
    m[4] = a[4] != S(0) ? S(1) / a[4] : S(1);
    m[8] = a[8] != S(0) ? S(1) / a[8] : S(1);
  } else if (precond == 0) {
    m[0] = m[4] = m[8] = S(1);
  }
  out[0] = mk4<S>(m[0], m[1], m[2]);
  out[1] = mk4<S>(m[3], m[4], m[5]);
  out[2] = mk4<S>(m[6], m[7], m[8]);
}

// ---------------- element kernels (FP64 energy / gradient) ----------------
// lf[e] = dt^2 V_e * local elastic force + element inertia force M_e (u - x_tilde); energy reduced into
// sc->energy.  When trial, u is replaced by u + alpha * d and the energy goes to sc->trial_energy (forces
// at the trial point are written when with_forces: an accepted line-search trial is the next gradient).
template <typename SD>
void launch_elem_energy_grad(const ElemFP64& el, const double* X, const double* u, const double* xt,
                             const V4<SD>* d, double alpha, double dt2, double rho, double* lf, bool with_forces,
                             bool trial, const Reduce& red, cudaStream_t st);
// g[v] = sum over incident (e, i) of lf[e][i], Dirichlet dofs zeroed; |g|^2 into sc->gnorm2
// the mixed steppers' FP32 element pass: per-vertex FP32 split of u (hi + lo) and of w = u - x~ (made by
// launch_split32 once per base point), FP32 element arithmetic, forces to lf32[t][4][3]
void launch_split32(int nv, const double* u, const double* xt, float4* uh, float4* ul, float4* w, cudaStream_t st);
void launch_elem_energy_grad32(const ElemFP64& el, const ElemFP32& ef, const Split32& sp, const float4* d,
                               double alpha, double dt2, double rho, float* lf32, bool with_forces, bool trial,
                               const Reduce& red, cudaStream_t st, int block = 0, int regcap = 0);
// increment evaluation from a reference u_r (the mixed Newton's iterations after the FP32 phase): ref = the
// FP32 split of u_r and w = u_r - x~, db = u_b - u_r; energy e_ref + increment into the (trial) energy,
// escale_ref as its round-off scale; local force increments into lf32 (see kernels_elem.cu)
void launch_elem_delta32(const ElemFP64& el, const ElemFP32& ef, const Split32& ref, const float4* db, const float4* d,
                         double alpha, double dt2, double rho, double e_ref, double escale_ref, float* lf32,
                         bool with_forces, bool trial, const Reduce& red, cudaStream_t st, int block = 0);
// g = gref + the gathered increments (Dirichlet dofs zeroed), |g|^2 into sc->gnorm2
void launch_vertex_gather_delta32(int nv, const int* vptr, const int* vinc, const float* lf32, const uint8_t* mask,
                                  const double* gref, double* g, const Reduce& red, cudaStream_t st, int block = 0);
void launch_delta_base(int nv, const double* u, const double* uref, float4* db, cudaStream_t st);
void launch_vertex_gather32(int nv, const int* vptr, const int* vinc, const float* lf32, const uint8_t* mask,
                            double* g, const Reduce& red, cudaStream_t st, int block = 0);
// mass-spring energy (+ spring forces into lf[s][2][3]) at u (+ alpha d), plus the lumped inertia energy
template <typename SD>
void launch_spring_energy_grad(const SpringData& sp, const double* u, const double* xt, const double* m, int nv,
                               const V4<SD>* d, double alpha, double dt2, double* lf, bool with_forces, bool trial,
                               const Reduce& red, cudaStream_t st);
// g = spring forces gathered per vertex + m (u - x~), Dirichlet dofs zeroed; |g|^2 into the scalars
template <typename SD>
void launch_spring_gather(int nv, const int* vptr, const int* vinc, const double* lf, const double* m,
                          const double* u, const V4<SD>* d, double alpha, const double* xt, const uint8_t* mask,
                          double* g, const Reduce& red, cudaStream_t st);
// FP32 spring pass (strain-relative: l - L = (2 E0.D + D.D) / (l + L) with D = the displacement difference
// formed in FP64): energy (+ the spring force vector f_s into lf32[s] when with_forces), FP64 sums
template <typename SD>
void launch_spring_energy_grad32(const SpringData& sp, const Split32& s3, const double* u, const double* xt,
                                 const double* m, int nv, const V4<SD>* d, double alpha, double dt2, float4* lf32,
                                 bool with_forces, bool trial, const Reduce& red, cudaStream_t st);
// g from the FP32 spring forces (vertex i of a spring receives +f_s, vertex j -f_s) + m (u (+ alpha d) - x~)
template <typename SD>
void launch_spring_gather32(int nv, const int* vptr, const int* vinc, const float4* lf32, const double* m,
                            const double* u, const V4<SD>* d, double alpha, const double* xt, const uint8_t* mask,
                            double* g, const Reduce& red, cudaStream_t st);
// spring Hessian blocks Kbuf[s][3][9] (scaled by dt^2), the compressed transverse part dropped when spsd
template <typename S>
void launch_spring_hessian(const SpringData& sp, const double* u, double dt2, bool spsd, S* Kbuf, cudaStream_t st);
void launch_vertex_gather(int nv, const int* vptr, const int* vinc, const double* lf, const uint8_t* mask,
                          double* g, const Reduce& red, cudaStream_t st);

// ---------------- 2D triangles (kernels_tri.cu) ----------------
// cells int4 (x, y, z = the triangle), dminv rows 0..3 = the row-major 2x2 Dm^-1, vol = area; local forces
// lf[t][3][3] (z = 0), element blocks Kbuf[t][6][9] (the 6 upper 3x3 vertex blocks, z rows/columns 0)
template <typename SD>
void launch_tri_energy_grad(const ElemFP64& el, const double* u, const double* xt, const V4<SD>* d, double alpha,
                            double dt2, double rho, double* lf, bool with_forces, bool trial, const Reduce& red,
                            cudaStream_t st);
template <typename S>
void launch_tri_hessian(const ElemFP64& el, const double* u, double dt2, bool spsd, S* Kbuf, cudaStream_t st);
// the FP32 pass of the mixed path for triangles (as launch_elem_energy_grad32): delta32 the per-element
// FP32 stable Neo-Hookean delta, forces lf32[t][3][3] for launch_vertex_gather32
void launch_tri_energy_grad32(const ElemFP64& el, const ElemFP32& ef, const float* delta32, const Split32& sp,
                              const float4* d, double alpha, double dt2, double rho, float* lf32, bool with_forces,
                              bool trial, const Reduce& red, cudaStream_t st);

// ---------------- element Hessian ----------------
template <typename S>
void launch_elem_hessian(const ElemFP64& e64, const ElemFP32& e32, const double* X, const double* u,
                         const float4* xf, double dt2, bool spsd, S* Kbuf, cudaStream_t st, int block = 0);

// ---------------- assembly / sparse ----------------
// precond: 0 identity, 1 Jacobi (diagonal of the diagonal block), 2 block-Jacobi (inverse 3x3 block)
// element Hessian and assembly in one pass for tets (kernels_fused.cu): CTA b owns the block rows of slices
// [spc b, spc (b + 1)); fptr / felem / fcode are the lists of topology.h's FusedLists.  Writes vals (and the
// preconditioner rows dinv) exactly as launch_elem_hessian followed by launch_assemble would, up to the
// order of the FP sums
template <typename S>
void launch_fused_hessian(const ElemFP64& e64, const ElemFP32& e32, const double* X, const double* u,
                          const float4* xf, double dt2, bool spsd, const SellMatrix& A, int nslices, int spc,
                          int ncta, const int* fptr, const int* felem, const uint16_t* fcode, const S* slot_mass,
                          const uint8_t* mask, bool filter, S* vals, V4<S>* dinv, int precond, cudaStream_t st);
// entries per chunk of the fused kernel's lists (the rank of a block counts within a chunk)
int fused_chunk();

template <typename S>
void launch_assemble(const SellMatrix& A, const int* cptr, const int* csrc, const S* Kbuf, const S* slot_mass,
                     const uint8_t* mask, bool filter, S* vals, V4<S>* dinv, int precond, cudaStream_t st, int block = 0);
// the element Hessian blocks in FP16 (per block a power-of-two scale; 24 bytes a block instead of 36) and the
// assembly that reads them (FP32 sums): the mixed Newton's assemblies whose solve runs on the FP16 matrix copy
void launch_elem_hessian16(const ElemFP64& e64, const ElemFP32& e32, const double* X, const double* u,
                           const float4* xf, double dt2, bool spsd, uint2* K16, cudaStream_t st, int block = 0);
void launch_assemble16(const SellMatrix& A, const int* cptr, const int* csrc, const uint2* K16, const float* slot_mass,
                       const uint8_t* mask, bool filter, float* vals, float4* dinv, int precond, cudaStream_t st,
                       int block = 0);
template <typename S>
void launch_spmv(const SellMatrix& A, const S* vals, const V4<S>* x, V4<S>* y, cudaStream_t st);
template <typename S>
void launch_export_csr(const SellMatrix& A, const int* bptr, const int* slot_k, const int* slot_kt, const S* vals,
                       double* csr_vals, cudaStream_t st);

// ---------------- PCG (fused) ----------------
template <typename S>
void launch_pcg_setup(int nv, const double* g, const V4<S>* dinv, V4<S>* x, V4<S>* r, V4<S>* z, V4<S>* p0,
                      double rtol, int max_iters, bool rhs_negate, const Reduce& red, cudaStream_t st);
template <typename S>
void launch_pcg_spmv(const SellMatrix& A, const S* vals, const V4<S>* z, const V4<S>* p_old, V4<S>* p_new,
                     V4<S>* q, bool first, const Reduce& red, cudaStream_t st, bool kron = false);
// the whole PCG loop (after launch_pcg_setup*) in one cooperative launch: variant 1 standard PCG (bitwise
// the two-launch iterates), 2 Chronopoulos-Gear PCG, 4 pipelined PCG (one grid barrier per iteration;
// pm: 2 nv vectors of scratch; Chronopoulos-Gear after pipe_iters iterations); gsync: grid_sync_words(nv)
// words of barrier state (zeroed by the launch); false if the device cannot launch it cooperatively (the
// caller runs the two-launch loop)
size_t grid_sync_words(int nv);
template <typename S>
bool launch_pcg_persistent(const SellMatrix& A, const S* vals, const V4<S>* dinv, V4<S>* x, V4<S>* r, V4<S>* z,
                           V4<S>* p0, V4<S>* p1, V4<S>* q, int max_iters, const Reduce& red, unsigned long long* gsync,
                           long long spin_limit, int extra, int max_blocks, int variant, cudaStream_t st,
                           bool kron = false, V4<S>* pm = nullptr, int pipe_iters = 0);
// FP16 copy of the Jacobi-scaled system matrix for the mixed Newton's loose PCG solves.  With s_a =
// 1/sqrt(K_aa) per dof and S = diag(s), the copy holds K~ = S K S (|K~_ij| <= 1 for an SPD K) in both
// triangles, full block SELL-32 (build_full_sell): per entry one 16-byte load of the block's first eight
// values and one 2-byte load of the ninth.  PCG on K~ with the scaled block-Jacobi (S B S)^-1 makes the
// same iterates as PCG on K with B^-1 up to the FP16 rounding of K~ (about 5e-4 relative per value): the
// scalars (r, u), (w, u) are invariant, the stop test uses (r, r) of the unscaled residual, and the
// solution is unscaled (x = S x~) before the kernel returns.
struct HalfMatrix {
  int nv;
  const int* off;       // [nslices + 1] entry offset of each slice (multiple of 32)
  const int* col;       // [nfs] block column, own row for padding
  const uint4* v8;      // [nfs] values 0..7 of the scaled block (row-major), FP16
  const uint16_t* v1;   // [nfs] value 8, FP16 bits
  const float4* scale;  // [nv] s_a
  const float4* iscale; // [nv] 1 / s_a
};
// scale, inverse scale and the scaled block-Jacobi rows (precond 0 / 1 / 2 on S B S) from the diagonal blocks
// of the FP32 symmetric values
void launch_half_prepare(const SellMatrix& A, const float* vals, int precond, float4* scale, float4* iscale,
                         float4* dinv16, cudaStream_t st);
// the FP16 values of every full entry from the FP32 symmetric values (src: build_full_sell's sources)
void launch_half_convert(const SellMatrix& A, const int* off, const int* col, const int* src, const float* vals,
                         const float4* scale, uint4* v8, uint16_t* v1, cudaStream_t st);
// PCG setup in the scaled space: r~ = S (negate ? -b : b), z~ = M~ r~, x = p0 = 0; partials (r~, z~) and
// (r, r) of the unscaled residual
void launch_pcg_setup_half(const HalfMatrix& H, const double* b, const float4* dinv16, float4* x, float4* r, float4* z,
                           float4* p0, double rtol, int max_iters, bool negate, const Reduce& red, cudaStream_t st);
// Chronopoulos-Gear PCG on the FP16 copy in one cooperative launch (as launch_pcg_persistent variant 2);
// x holds the unscaled solution on return.  false if the device cannot launch it cooperatively.
// the pipelined solve on the copy does its own set-up and, with check set, the solve's check on the FP32
// symmetric store (A32, vals32): g . x, |x|^2, |sign b - K x|^2, |b|^2 into sc->gd, dnorm2, true_rr, true_bb
struct HalfSolveArgs {
  const double* b;  // right-hand side sign * b (the Newton gradient g with negate = 1)
  int negate;
  double rtol;
  int max_iters;
  int pipe_iters;  // pipelined iterations before Chronopoulos-Gear
  int check;
  SellMatrix A32;
  const float* vals32;
};
// pm and pa non-null: the pipelined solve (pipe_persistent_kernel's scheme, 2 nv vectors of scratch in pm)
// with its set-up and check in the same launch (no launch_pcg_setup_half before it); otherwise
// Chronopoulos-Gear after launch_pcg_setup_half
bool launch_pcg_half(const HalfMatrix& H, const float4* dinv16, float4* x, float4* r, float4* z, float4* p0,
                     float4* p1, float4* q, int max_iters, const Reduce& red, unsigned long long* gsync,
                     long long spin_limit, int extra, int max_blocks, cudaStream_t st, float4* pm = nullptr,
                     const HalfSolveArgs* pa = nullptr);
// after a solve on the FP16 copy: g . d, |d|^2 (as launch_dot_gd) and the solve's true residual on the FP32
// symmetric values, |-g - K d|^2 and |g|^2 (sc->true_rr, sc->true_bb)
void launch_dot_gd_check(const SellMatrix& A, const float* vals, const double* g, const float4* d, const Reduce& red,
                         cudaStream_t st);
// y = S^-1 K~ S^-1 x (the FP16 copy applied in the unscaled space); xs: nv vectors of scratch
void launch_half_spmv(const HalfMatrix& H, const float4* x, float4* xs, float4* y, cudaStream_t st);
// kron: vals holds one value per slot (the matrix is (scalar) (x) I3); launch_kron_extract makes that form
// from a 9-value store and sets *not_kron when some block is not a multiple of I3
template <typename S>
void launch_kron_extract(const SellMatrix& A, const S* vals, S* svals, int* not_kron, cudaStream_t st);
// y = A x, A a scalar CSR matrix over dofs, x / y 4-wide vertex vectors
template <typename S>
void launch_csr_dof_spmv(int n, const int* rp, const int* ci, const S* vals, const V4<S>* x, V4<S>* y,
                         cudaStream_t st);
template <typename S>
void launch_pcg_update(int nv, const V4<S>* p, const V4<S>* q, const V4<S>* dinv, V4<S>* x, V4<S>* r, V4<S>* z,
                       int max_iters, const Reduce& red, cudaStream_t st);

// ---------------- vector kernels ----------------
template <typename S>
void launch_dot_gd(int nv, const double* g, const V4<S>* d, const Reduce& red, cudaStream_t st);
template <typename S>
void launch_axpy_update(int nv, double alpha, const V4<S>* d, const double* X, double* u, float4* xf,
                        cudaStream_t st);
// xf = float(X + (u + d)): the positions after a full step, for an assembly made ahead of the line search
template <typename S>
void launch_full_step_xf(int nv, const V4<S>* d, const double* X, const double* u, float4* xf, cudaStream_t st);
void launch_refresh_xf(int nv, const double* X, const double* u, float4* xf, cudaStream_t st);
void launch_prepare_step(int n, double dt, const double* u, const double* v, const double* a,
                         const int8_t* dof_type, const double* dbc, double* xt, double* next, cudaStream_t st);
void launch_step_next(int n, double dt, double damping, double* prev, double* u, const double* next, double* v,
                      cudaStream_t st);
void launch_restore(int n, double dt, const int8_t* dof_type, const double* dbc, double* prev, double* u,
                    double* v, cudaStream_t st);
void launch_add_ext(int nv, int dof, double val, double* a, cudaStream_t st);
void launch_mark_dofs(int n, const int* verts, const double* targ, int dirichlet, int8_t* dof_type, double* dbc,
                      cudaStream_t st);
void launch_build_mask(int nv, const int8_t* dof_type, uint8_t* mask, cudaStream_t st);
template <typename S>
void launch_to_vec4(int nv, const double* in, V4<S>* out, bool negate, cudaStream_t st);
// y += a x on FP64 [n] vectors
void launch_axpy_d(int n, double a, const double* x, double* y, cudaStream_t st);
// FP64 dot of two S vectors into *out (device), deterministic
template <typename S>
void launch_vdot(int nv, const V4<S>* a, const V4<S>* b, double* out, const Reduce& red, cudaStream_t st);
// y = alpha * y + beta * x
template <typename S>
void launch_vaxpby(int nv, double alpha, V4<S>* y, double beta, const V4<S>* x, cudaStream_t st);
// y = (S)(a - b) for FP64 [3V] a, b
template <typename S>
void launch_vdiff(int nv, const double* a, const double* b, V4<S>* y, cudaStream_t st);

// L-BFGS in compact form (history of at most kLbfgsMaxCompact pairs): the pairs in age order (oldest first)
// and their storage slots
constexpr int kLbfgsMaxCompact = 8;
template <typename S>
struct LbfgsHist {
  int n;
  const V4<S>* s[kLbfgsMaxCompact];
  const V4<S>* y[kLbfgsMaxCompact];
  int slot[kLbfgsMaxCompact];
};
// S^T g, Y^T g and the newest column of S^T Y, Y^T Y in one pass; tab = [S^T Y (M x M by slot) | Y^T Y |
// coefficients p (M), -gamma q (M), gamma]; partials: lbfgs_multidot_partials(nv) doubles
template <typename S>
void launch_lbfgs_multidot(int nv, const double* g, const LbfgsHist<S>& h, double* partials, double* tab,
                           unsigned int* counter, cudaStream_t st);
template <typename S>
void launch_lbfgs_combine(int nv, const double* g, const LbfgsHist<S>& h, const double* coef, double gamma_host,
                          V4<S>* d, const Reduce& red, cudaStream_t st);
int lbfgs_multidot_partials(int nv);
// L-BFGS two-loop recursion with device-resident coefficients (kernels_lbfgs.cu)
template <typename S>
void launch_lbfgs_pass(int nv, const V4<S>* vin, const double* g, V4<S>* vout, const V4<S>* w, const double* cA,
                       const double* cB, double csign, const double* scale_ptr, double scale, const V4<S>* a,
                       double rho, double* out, const Reduce& red, cudaStream_t st);
template <typename S>
void launch_lbfgs_final(int nv, const V4<S>* z, const V4<S>* w, const double* cA, const double* cB, const double* g,
                        V4<S>* d, const Reduce& red, cudaStream_t st);
template <typename S>
void launch_lbfgs_pair(int nv, double alpha, const V4<S>* d, const double* gnew, const double* gold, V4<S>* sv,
                       V4<S>* yv, const Reduce& red, cudaStream_t st);
template <typename S>
void launch_lbfgs_accept(int nv, double alpha, const V4<S>* d, double* u, const double* gnew, double* gold,
                         cudaStream_t st);
// per-instance |g|^2 over contiguous vertex ranges voff[i]..voff[i+1] (one block per instance, fixed order)
void launch_instance_norms(int ninst, const int* voff, const double* g, double* out, cudaStream_t st);
// PCG setup from an S right-hand side (the PD stepper's inner solve)
template <typename S>
void launch_pcg_setup_v(int nv, const V4<S>* b, const V4<S>* dinv, V4<S>* x, V4<S>* r, V4<S>* z, V4<S>* p0,
                        double rtol, int max_iters, const Reduce& red, cudaStream_t st);
template <typename S>
void launch_from_vec4(int nv, const V4<S>* in, double* out, cudaStream_t st);

// ---------------- adjoint (kernels_adjoint.cu) ----------------
void launch_adj_prep(int n, double kdt, const double* ubar, const double* vbar, const int8_t* dof_type, double* ub,
                     double* ubp, cudaStream_t st);
template <typename S>
void launch_adj_finish(int nv, double dt, const V4<S>* mlam, const int8_t* dof_type, const double* ubp, double* ubar,
                       double* vbar, cudaStream_t st);
template <typename S>
void launch_adj_material(const ElemFP64& el, const double* X, const double* u, const V4<S>* lam_adj, double dt2,
                         double* Ebar, cudaStream_t st);

}  // namespace ssim_gb
