// kernels_tri.cu -- 2D triangles in the plane (basic_time_step with PhysicalDim 2, TopologyDim 3, restated):
// the element pass (energy, PK1 -> vertex forces, consistent-mass inertia) and the element Hessian with its
// SPD projection.  Vertices keep 3 dofs (z carries no force and no stiffness), so assembly, gather and the
// solvers are the tet ones.
//
// Models (F row-major 2x2, flat index r*2+c):
//   stable Neo-Hookean 2D (stable_neohookean.hpp:23-104): Psi = (mu (Ic-2) + lambda (J-alpha)^2
//   - mu log(Ic+delta))/2 - psi0, P = lambda (J-alpha) dJ/dF + mu (1 - 1/(Ic+delta)) F,
//   H = mu (1 - 1/(Ic+delta)) I + 2 mu/(Ic+delta)^2 f f^T + lambda g g^T + lambda (J-alpha) d2J/dF2;
//   linear 2D (linear.hpp:23-68) from G = F - I.
// The projection clamps the eigenvalues of the 4x4 H at 1e-3 (time_step.hpp:44-52), eigenvectors by cyclic
// Jacobi rotations in registers.
#include "elem_math.cuh"
#include "kernels.cuh"

namespace ssim_gb {
namespace {

constexpr int TB = 128;

template <typename S>
__device__ __forceinline__ S comp3(const V4<S>& v, int k) {
  return k == 0 ? v.x : (k == 1 ? v.y : v.z);
}

template <typename S, bool STRESS>
__device__ __forceinline__ S snh2_eval(const S* F, S lam, S mu, S alpha, S delta, S psi0, S* P, S& scale) {
  const S Ic = F[0] * F[0] + F[1] * F[1] + F[2] * F[2] + F[3] * F[3];
  const S Jm = (F[0] * F[3] - F[1] * F[2]) - alpha;
  const S lg = log(Ic + delta);
  if (STRESS) {
    const S c = mu * (S(1) - S(1) / (Ic + delta));
    P[0] = lam * Jm * F[3] + c * F[0];
    P[1] = -lam * Jm * F[2] + c * F[1];
    P[2] = -lam * Jm * F[1] + c * F[2];
    P[3] = lam * Jm * F[0] + c * F[3];
  }
  scale = S(0.5) * (mu * fabs(Ic - S(2)) + lam * Jm * Jm + mu * fabs(lg)) + fabs(psi0);
  return S(0.5) * (mu * (Ic - S(2)) + lam * Jm * Jm - mu * lg) - psi0;
}

template <typename S, bool STRESS>
__device__ __forceinline__ S linear2_eval(const S* G, S lam, S mu, S* P, S& scale) {
  const S e00 = G[0], e11 = G[3], e01 = S(0.5) * (G[1] + G[2]);
  const S tr = e00 + e11;
  if (STRESS) {
    P[0] = S(2) * mu * e00 + lam * tr;
    P[1] = S(2) * mu * e01;
    P[2] = S(2) * mu * e01;
    P[3] = S(2) * mu * e11 + lam * tr;
  }
  const S psi = mu * (e00 * e00 + e11 * e11 + S(2) * e01 * e01) + S(0.5) * lam * tr * tr;
  scale = psi;
  return psi;
}

// cyclic Jacobi on a symmetric 4x4 (full storage), eigenvectors in the columns of V
template <typename S, int SWEEPS>
__device__ __forceinline__ void jacobi4(S (&A)[16], S (&V)[16]) {
#pragma unroll
  for (int k = 0; k < 16; ++k) V[k] = (k % 5 == 0) ? S(1) : S(0);
#pragma unroll
  for (int sw = 0; sw < SWEEPS; ++sw) {
#pragma unroll
    for (int p = 0; p < 3; ++p) {
#pragma unroll
      for (int q = p + 1; q < 4; ++q) {
        const S apq = A[p * 4 + q];
        const S tiny = S(1e-30) + (sizeof(S) == 4 ? S(1e-7) : S(1e-16)) * (fabs(A[p * 5]) + fabs(A[q * 5]));
        if (fabs(apq) > tiny * S(1e-3)) {
          const S theta = (A[q * 5] - A[p * 5]) / (S(2) * apq);
          const S at = fabs(theta);
          S t = S(1) / (at + sqrt(at * at + S(1)));
          if (theta < S(0)) t = -t;
          const S c = S(1) / sqrt(t * t + S(1)), s = t * c;
          // A' = J^T A J with J the rotation in the (p, q) plane
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const S akp = A[k * 4 + p], akq = A[k * 4 + q];
            A[k * 4 + p] = c * akp - s * akq;
            A[k * 4 + q] = s * akp + c * akq;
          }
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const S apk = A[p * 4 + k], aqk = A[q * 4 + k];
            A[p * 4 + k] = c * apk - s * aqk;
            A[q * 4 + k] = s * apk + c * aqk;
          }
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const S vkp = V[k * 4 + p], vkq = V[k * 4 + q];
            V[k * 4 + p] = c * vkp - s * vkq;
            V[k * 4 + q] = s * vkp + c * vkq;
          }
        }
      }
    }
  }
}

// one element pass: energy (+ scale), and with FORCES the local forces lf[t][3][3]; inertia from the
// consistent P1 mass rho A / 12 (1 + delta_ij) of the triangle
template <typename SD, bool FORCES, bool TRIAL>
__global__ void __launch_bounds__(TB)
    tri_energy_grad_kernel(ElemFP64 el, const double* __restrict__ u, const double* __restrict__ xt,
                           const V4<SD>* __restrict__ d, double alpha, double dt2, double rho, double* __restrict__ lf,
                           Reduce red) {
  __shared__ double shred[TB / 32][2];
  const int e = blockIdx.x * TB + threadIdx.x;
  double energy = 0, escale = 0;
  if (e < el.nt) {
    const int4 c = el.cells[e];
    const int vid[3] = {c.x, c.y, c.z};
    double uu[3][2], dd[3][2];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      V4<SD> dv;
      if (TRIAL) dv = d[vid[i]];
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        double uk = u[vid[i] * 3 + k];
        if (TRIAL) uk += alpha * (double)comp3<SD>(dv, k);
        uu[i][k] = uk;
        dd[i][k] = uk - xt[vid[i] * 3 + k];
      }
    }
    double Dm[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) Dm[k] = el.dminv[(size_t)k * el.nt + e];
    // F = I + [u1-u0, u2-u0] Dm^-1
    double G[4], F[4];
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
      for (int cc = 0; cc < 2; ++cc) {
        G[r * 2 + cc] = (uu[1][r] - uu[0][r]) * Dm[0 * 2 + cc] + (uu[2][r] - uu[0][r]) * Dm[1 * 2 + cc];
        F[r * 2 + cc] = (r == cc ? 1.0 : 0.0) + G[r * 2 + cc];
      }
    const double lam = el.lam[e], mu = el.mu[e], A = el.vol[e];
    double P[4], sc;
    const double psi = el.model == 1
                           ? linear2_eval<double, FORCES>(G, lam, mu, P, sc)
                           : snh2_eval<double, FORCES>(F, lam, mu, el.alpha[e], el.delta[e], el.psi0[e], P, sc);
    const double m = rho * A * (1.0 / 12.0);
    double sd[2] = {dd[0][0] + dd[1][0] + dd[2][0], dd[0][1] + dd[1][1] + dd[2][1]};
    double q = sd[0] * sd[0] + sd[1] * sd[1];
#pragma unroll
    for (int i = 0; i < 3; ++i) q += dd[i][0] * dd[i][0] + dd[i][1] * dd[i][1];
    if (FORCES) {
      const double s = dt2 * A;
      double out[9];
      double tot[2] = {0, 0};
#pragma unroll
      for (int i = 1; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          const double h = P[j * 2 + 0] * Dm[(i - 1) * 2 + 0] + P[j * 2 + 1] * Dm[(i - 1) * 2 + 1];
          tot[j] += h;
          out[i * 3 + j] = s * h + m * (dd[i][j] + sd[j]);
        }
#pragma unroll
      for (int j = 0; j < 2; ++j) out[j] = -s * tot[j] + m * (dd[0][j] + sd[j]);
      out[2] = out[5] = out[8] = 0.0;
      double* dst = lf + (size_t)e * 9;
#pragma unroll
      for (int k = 0; k < 9; ++k) dst[k] = out[k];
    }
    energy = dt2 * A * psi + 0.5 * m * q;
    escale = dt2 * A * sc + 0.5 * m * q;
  }
  double v2[2] = {energy, escale};
  block_sum<2, TB>(v2, shred);
  double tot[2];
  if (grid_sum_last<2, TB>(v2, red.partials, red.counter, tot)) {
    if (TRIAL) {
      red.sc->trial_energy = tot[0];
      red.sc->trial_energy_scale = tot[1];
    } else {
      red.sc->energy = tot[0];
      red.sc->energy_scale = tot[1];
    }
  }
}

// element Hessian dt^2 A pfpx^T H pfpx (projected when spsd), the 6 upper 3x3 vertex blocks per triangle
template <typename S>
__global__ void __launch_bounds__(TB)
    tri_hessian_kernel(ElemFP64 el, const double* __restrict__ u, double dt2, int spsd, S* __restrict__ Kbuf) {
  const int e = blockIdx.x * TB + threadIdx.x;
  if (e >= el.nt) return;
  const int4 c = el.cells[e];
  const int vid[3] = {c.x, c.y, c.z};
  double du[2][2];  // u_{1,2} - u_0
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int k = 0; k < 2; ++k) du[i][k] = u[vid[i + 1] * 3 + k] - u[vid[0] * 3 + k];
  double Dm[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) Dm[k] = el.dminv[(size_t)k * el.nt + e];
  S F[4];
#pragma unroll
  for (int r = 0; r < 2; ++r)
#pragma unroll
    for (int cc = 0; cc < 2; ++cc)
      F[r * 2 + cc] = (S)((r == cc ? 1.0 : 0.0) + du[0][r] * Dm[0 * 2 + cc] + du[1][r] * Dm[1 * 2 + cc]);
  const S lam = (S)el.lam[e], mu = (S)el.mu[e];
  S H[16];
  if (el.model == 1) {
#pragma unroll
    for (int k = 0; k < 16; ++k) H[k] = (k % 5 == 0) ? mu : S(0);
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        H[(i * 2 + j) * 4 + (j * 2 + i)] += mu;
        H[(i * 2 + i) * 4 + (j * 2 + j)] += lam;
      }
  } else {
    const S delta = (S)el.delta[e], alpha = (S)el.alpha[e];
    const S Ic = F[0] * F[0] + F[1] * F[1] + F[2] * F[2] + F[3] * F[3];
    const S J = F[0] * F[3] - F[1] * F[2];
    const S g[4] = {F[3], -F[2], -F[1], F[0]};
    const S a = mu * (S(1) - S(1) / (Ic + delta)), b = mu * S(2) / ((Ic + delta) * (Ic + delta));
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) H[i * 4 + j] = (i == j ? a : S(0)) + b * F[i] * F[j] + lam * g[i] * g[j];
    const S s = lam * (J - alpha);
    H[3] += s;
    H[12] += s;
    H[6] -= s;
    H[9] -= s;
  }
  if (spsd) {
    S A[16], V[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) A[k] = H[k];
    jacobi4<S, sizeof(S) == 4 ? 5 : 6>(A, V);
    S w[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) w[k] = fmax(A[k * 5], S(1e-3));
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j)
        H[i * 4 + j] = V[i * 4 + 0] * w[0] * V[j * 4 + 0] + V[i * 4 + 1] * w[1] * V[j * 4 + 1] +
                       V[i * 4 + 2] * w[2] * V[j * 4 + 2] + V[i * 4 + 3] * w[3] * V[j * 4 + 3];
  }
  // B[v][c] = dF(a, c)/dx_{v, a}
  S B[3][2];
#pragma unroll
  for (int cc = 0; cc < 2; ++cc) {
    B[1][cc] = (S)Dm[0 * 2 + cc];
    B[2][cc] = (S)Dm[1 * 2 + cc];
    B[0][cc] = -(B[1][cc] + B[2][cc]);
  }
  const S sc = (S)(dt2 * el.vol[e]);
  S* out = Kbuf + (size_t)e * 54;
  int blk = 0;
#pragma unroll
  for (int v = 0; v < 3; ++v)
#pragma unroll
    for (int w = v; w < 3; ++w) {
      S K[9];
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
          S t = S(0);
          if (a < 2 && b < 2) {
#pragma unroll
            for (int c1 = 0; c1 < 2; ++c1)
#pragma unroll
              for (int c2 = 0; c2 < 2; ++c2) t += B[v][c1] * H[(a * 2 + c1) * 4 + b * 2 + c2] * B[w][c2];
          }
          K[a * 3 + b] = sc * t;
        }
#pragma unroll
      for (int k = 0; k < 9; ++k) out[blk * 9 + k] = K[k];
      ++blk;
    }
}

// FP32 element pass of the mixed path (the triangle analogue of elem_energy_grad32_kernel): displacement
// differences from the per-vertex FP32 split ((hi_j - hi_i) + (lo_j - lo_i) + alpha (d_j - d_i)), inertia
// offsets from w = u - x~ rounded once per vertex, the strain-relative 2D stable Neo-Hookean
// (snh2_eval_small) or the linear model, FP32 forces lf32[t][3][3] (z = 0) for vertex_gather32; energy
// and its magnitude sum summed in FP64 across warps, blocks and the grid.
template <bool FORCES, bool TRIAL>
__global__ void __launch_bounds__(TB)
    tri_energy_grad32_kernel(ElemFP64 el, ElemFP32 ef, const float* __restrict__ delta32, Split32 sp,
                             const float4* __restrict__ d, float alpha, float dt2, float rho, float* __restrict__ lf32,
                             Reduce red) {
  __shared__ double shred[TB / 32][2];
  const int e = blockIdx.x * TB + threadIdx.x;
  float part[2] = {0.f, 0.f};
  if (e < el.nt) {
    const int4 c = el.cells[e];
    const int vid[3] = {c.x, c.y, c.z};
    float4 hv[3], lv[3], dv[3];
    float dd[3][2];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      hv[i] = sp.uh[vid[i]];
      lv[i] = sp.ul[vid[i]];
      const float4 wv = sp.w[vid[i]];
      if (TRIAL) dv[i] = d[vid[i]];
      dd[i][0] = TRIAL ? wv.x + alpha * dv[i].x : wv.x;
      dd[i][1] = TRIAL ? wv.y + alpha * dv[i].y : wv.y;
    }
    float Dm[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) Dm[k] = ef.dminv[(size_t)k * el.nt + e];
    // Du(r, k) = (x_{k+1} - x_0)_r from the split, G = Du Dm^-1
    float Du[4];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      float a0 = (hv[k + 1].x - hv[0].x) + (lv[k + 1].x - lv[0].x);
      float a1 = (hv[k + 1].y - hv[0].y) + (lv[k + 1].y - lv[0].y);
      if (TRIAL) {
        a0 += alpha * (dv[k + 1].x - dv[0].x);
        a1 += alpha * (dv[k + 1].y - dv[0].y);
      }
      Du[0 * 2 + k] = a0;
      Du[1 * 2 + k] = a1;
    }
    float G[4];
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
      for (int cc = 0; cc < 2; ++cc) G[r * 2 + cc] = Du[r * 2 + 0] * Dm[0 * 2 + cc] + Du[r * 2 + 1] * Dm[1 * 2 + cc];
    const float lam = ef.lam[e], mu = ef.mu[e], A = ef.vol[e];
    float P[4], sc;
    const float psi = el.model == 1 ? linear2_eval<float, FORCES>(G, lam, mu, P, sc)
                                    : snh2_eval_small<float, FORCES>(G, lam, mu, delta32[e], P, sc);
    const float m = rho * A * (1.0f / 12.0f);
    const float sd[2] = {dd[0][0] + dd[1][0] + dd[2][0], dd[0][1] + dd[1][1] + dd[2][1]};
    float q = sd[0] * sd[0] + sd[1] * sd[1];
#pragma unroll
    for (int i = 0; i < 3; ++i) q += dd[i][0] * dd[i][0] + dd[i][1] * dd[i][1];
    if (FORCES) {
      const float sA = dt2 * A;
      float out[9];
      float tot[2] = {0.f, 0.f};
#pragma unroll
      for (int i = 1; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          const float h = P[j * 2 + 0] * Dm[(i - 1) * 2 + 0] + P[j * 2 + 1] * Dm[(i - 1) * 2 + 1];
          tot[j] += h;
          out[i * 3 + j] = sA * h + m * (dd[i][j] + sd[j]);
        }
#pragma unroll
      for (int j = 0; j < 2; ++j) out[j] = -sA * tot[j] + m * (dd[0][j] + sd[j]);
      out[2] = out[5] = out[8] = 0.f;
      float* dst = lf32 + (size_t)e * 9;
#pragma unroll
      for (int k = 0; k < 9; ++k) dst[k] = out[k];
    }
    part[0] = dt2 * A * psi + 0.5f * m * q;
    part[1] = dt2 * A * sc + 0.5f * m * q;
  }
  double v2[2];
  block_sum_s<2, TB, float>(part, v2, shred);
  double tot[2];
  if (grid_sum_last<2, TB>(v2, red.partials, red.counter, tot)) {
    if (TRIAL) {
      red.sc->trial_energy = tot[0];
      red.sc->trial_energy_scale = tot[1];
    } else {
      red.sc->energy = tot[0];
      red.sc->energy_scale = tot[1];
    }
  }
}

}  // namespace

template <typename SD>
void launch_tri_energy_grad(const ElemFP64& el, const double* u, const double* xt, const V4<SD>* d, double alpha,
                            double dt2, double rho, double* lf, bool with_forces, bool trial, const Reduce& red,
                            cudaStream_t st) {
  const int grid = div_up(el.nt, TB);
  if (trial && with_forces)
    tri_energy_grad_kernel<SD, true, true><<<grid, TB, 0, st>>>(el, u, xt, d, alpha, dt2, rho, lf, red);
  else if (trial)
    tri_energy_grad_kernel<SD, false, true><<<grid, TB, 0, st>>>(el, u, xt, d, alpha, dt2, rho, lf, red);
  else if (with_forces)
    tri_energy_grad_kernel<SD, true, false><<<grid, TB, 0, st>>>(el, u, xt, d, alpha, dt2, rho, lf, red);
  else
    tri_energy_grad_kernel<SD, false, false><<<grid, TB, 0, st>>>(el, u, xt, d, alpha, dt2, rho, lf, red);
  after_launch("tri_energy_grad");
}

void launch_tri_energy_grad32(const ElemFP64& el, const ElemFP32& ef, const float* delta32, const Split32& sp,
                              const float4* d, double alpha, double dt2, double rho, float* lf32, bool with_forces,
                              bool trial, const Reduce& red, cudaStream_t st) {
  if (el.nt <= 0) return;
  const int grid = div_up(el.nt, TB);
  const float a = (float)alpha, f_dt2 = (float)dt2, f_rho = (float)rho;
  if (trial && with_forces)
    tri_energy_grad32_kernel<true, true><<<grid, TB, 0, st>>>(el, ef, delta32, sp, d, a, f_dt2, f_rho, lf32, red);
  else if (trial)
    tri_energy_grad32_kernel<false, true><<<grid, TB, 0, st>>>(el, ef, delta32, sp, d, a, f_dt2, f_rho, lf32, red);
  else if (with_forces)
    tri_energy_grad32_kernel<true, false><<<grid, TB, 0, st>>>(el, ef, delta32, sp, d, a, f_dt2, f_rho, lf32, red);
  else
    tri_energy_grad32_kernel<false, false><<<grid, TB, 0, st>>>(el, ef, delta32, sp, d, a, f_dt2, f_rho, lf32, red);
  after_launch("tri_energy_grad32");
}

template <typename S>
void launch_tri_hessian(const ElemFP64& el, const double* u, double dt2, bool spsd, S* Kbuf, cudaStream_t st) {
  tri_hessian_kernel<S><<<div_up(el.nt, TB), TB, 0, st>>>(el, u, dt2, spsd ? 1 : 0, Kbuf);
  after_launch("tri_hessian");
}

template void launch_tri_energy_grad<float>(const ElemFP64&, const double*, const double*, const float4*, double,
                                            double, double, double*, bool, bool, const Reduce&, cudaStream_t);
template void launch_tri_energy_grad<double>(const ElemFP64&, const double*, const double*, const double4_32a*,
                                             double, double, double, double*, bool, bool, const Reduce&,
                                             cudaStream_t);
template void launch_tri_hessian<float>(const ElemFP64&, const double*, double, bool, float*, cudaStream_t);
template void launch_tri_hessian<double>(const ElemFP64&, const double*, double, bool, double*, cudaStream_t);

}  // namespace ssim_gb
