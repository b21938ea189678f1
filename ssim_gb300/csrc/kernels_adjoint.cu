// kernels_adjoint.cu -- the reverse (adjoint) pass of one backward-Euler step.
//
// Forward step (time_step.hpp:499-543): x~ = u + dt v + dt^2 a on free dofs, u' = argmin E(x) with
// E = 1/2 |x - x~|_M^2 + dt^2 sum_e V_e Psi_e(x; E_e), v' = (u' - u) / dt * (1 - damping).
// At the minimiser the free rows of r = M (u' - x~) + dt^2 grad Psi vanish, so with H the filtered Hessian
// (identity on Dirichlet rows / columns, time_step.hpp:626-658 with make_spsd = false):
//   lambda = H^-1 ubar'            (ubar' zeroed on Dirichlet dofs)
//   xbar~  = M lambda              (unfiltered mass; zeroed on Dirichlet dofs, where x~ is a constant)
//   ubar   = -k/dt vbar' + xbar~,  vbar = dt xbar~          (k = 1 - damping)
//   Ebar_e -= dt^2 V_e <Lambda_e Dm^-1, P_e> / E_e
// The last line: the stable Neo-Hookean PK1 (stable_neohookean.hpp:38-62) is homogeneous of degree one in
// (lambda, mu) jointly (alpha depends on mu / lambda only), and so is the linear model's (linear.hpp:37-52);
// both Lame parameters scale with E, so dP/dE = P / E; the
// element's forces contracted with the adjoint are <Lambda Dm^-1, P> with Lambda = [l1-l0, l2-l0, l3-l0].
#include "elem_math.cuh"
#include "kernels.cuh"

namespace ssim_gb {
namespace {

constexpr int AB = 256;
constexpr int EB = 128;

// ub = (ubar + k/dt vbar) with Dirichlet dofs zeroed; ubp = -k/dt vbar (the part of ubar that does not
// pass through the solve)
__global__ void adj_prep_kernel(int n, double kdt, const double* __restrict__ ubar, const double* __restrict__ vbar,
                                const int8_t* __restrict__ dof_type, double* __restrict__ ub,
                                double* __restrict__ ubp) {
  const int i = blockIdx.x * AB + threadIdx.x;
  if (i >= n) return;
  const double v = kdt * vbar[i];
  ub[i] = dof_type[i] == 1 ? 0.0 : ubar[i] + v;
  ubp[i] = -v;
}

// ubar = ubp + xbar~ (free), vbar = dt xbar~ (free), xbar~ = M lambda
template <typename S>
__global__ void adj_finish_kernel(int nv, double dt, const V4<S>* __restrict__ mlam, const int8_t* __restrict__ dof_type,
                                  const double* __restrict__ ubp, double* __restrict__ ubar, double* __restrict__ vbar) {
  const int v = blockIdx.x * AB + threadIdx.x;
  if (v >= nv) return;
  const V4<S> m = mlam[v];
  const double xb[3] = {(double)m.x, (double)m.y, (double)m.z};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int i = 3 * v + k;
    const double x = dof_type[i] == 1 ? 0.0 : xb[k];
    ubar[i] = ubp[i] + x;
    vbar[i] = dt * x;
  }
}

template <typename S>
__global__ void __launch_bounds__(EB)
    adj_material_kernel(ElemFP64 el, const double* __restrict__ X, const double* __restrict__ u,
                        const V4<S>* __restrict__ lam_adj, double dt2, double* __restrict__ Ebar) {
  const int e = blockIdx.x * EB + threadIdx.x;
  if (e >= el.nt) return;
  const int4 c = el.cells[e];
  const int vid[4] = {c.x, c.y, c.z, c.w};
  double x[4][3], l[4][3];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const V4<S> a = lam_adj[vid[i]];
    l[i][0] = (double)a.x;
    l[i][1] = (double)a.y;
    l[i][2] = (double)a.z;
#pragma unroll
    for (int k = 0; k < 3; ++k) x[i][k] = X[vid[i] * 3 + k] + u[vid[i] * 3 + k];
  }
  double Dm[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) Dm[k] = el.dminv[(size_t)k * el.nt + e];
  double F[9], W[9];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int cc = 0; cc < 3; ++cc) {
      F[r * 3 + cc] = (x[1][r] - x[0][r]) * Dm[0 * 3 + cc] + (x[2][r] - x[0][r]) * Dm[1 * 3 + cc] +
                      (x[3][r] - x[0][r]) * Dm[2 * 3 + cc];
      W[r * 3 + cc] = (l[1][r] - l[0][r]) * Dm[0 * 3 + cc] + (l[2][r] - l[0][r]) * Dm[1 * 3 + cc] +
                      (l[3][r] - l[0][r]) * Dm[2 * 3 + cc];
    }
  const double lam = el.lam[e], mu = el.mu[e];
  double P[9];
  if (el.model == 1) {
    double G[9], sc;
#pragma unroll
    for (int k = 0; k < 9; ++k) G[k] = F[k] - ((k % 4 == 0) ? 1.0 : 0.0);
    linear_eval<double, true>(G, lam, mu, P, sc);
  } else {
    snh_stress<double>(F, lam, mu, P);
  }
  double wp = 0;
#pragma unroll
  for (int k = 0; k < 9; ++k) wp += W[k] * P[k];
  const double E = mu * (3 * lam + 2 * mu) / (lam + mu);
  Ebar[e] -= dt2 * el.vol[e] * wp / E;
}

}  // namespace

void launch_adj_prep(int n, double kdt, const double* ubar, const double* vbar, const int8_t* dof_type, double* ub,
                     double* ubp, cudaStream_t st) {
  adj_prep_kernel<<<div_up(n, AB), AB, 0, st>>>(n, kdt, ubar, vbar, dof_type, ub, ubp);
  after_launch("adj_prep");
}

template <typename S>
void launch_adj_finish(int nv, double dt, const V4<S>* mlam, const int8_t* dof_type, const double* ubp, double* ubar,
                       double* vbar, cudaStream_t st) {
  adj_finish_kernel<S><<<div_up(nv, AB), AB, 0, st>>>(nv, dt, mlam, dof_type, ubp, ubar, vbar);
  after_launch("adj_finish");
}

template <typename S>
void launch_adj_material(const ElemFP64& el, const double* X, const double* u, const V4<S>* lam_adj, double dt2,
                         double* Ebar, cudaStream_t st) {
  if (el.nt <= 0) return;
  adj_material_kernel<S><<<div_up(el.nt, EB), EB, 0, st>>>(el, X, u, lam_adj, dt2, Ebar);
  after_launch("adj_material");
}

template void launch_adj_finish<float>(int, double, const float4*, const int8_t*, const double*, double*, double*,
                                       cudaStream_t);
template void launch_adj_finish<double>(int, double, const double4_32a*, const int8_t*, const double*, double*,
                                        double*, cudaStream_t);
template void launch_adj_material<float>(const ElemFP64&, const double*, const double*, const float4*, double, double*,
                                         cudaStream_t);
template void launch_adj_material<double>(const ElemFP64&, const double*, const double*, const double4_32a*, double,
                                          double*, cudaStream_t);

}  // namespace ssim_gb
