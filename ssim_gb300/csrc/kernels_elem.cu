// kernels_elem.cu -- element-parallel kernels: FP64 energy / gradient (update_energy_and_gradients,
// time_step.hpp:577-624), the vertex gather of element forces (global_composer.hpp:36-66 +
// time_step.hpp:608-617) and the element Hessian (wrapped_pfpx, time_step.hpp:23-60, 626-651).
#include <cfloat>

#include <cuda_fp16.h>

#include "hessian_elem.cuh"

namespace ssim_gb {

std::atomic<uint64_t> g_launches{0};

namespace {

constexpr int EB = 128;  // element block (energy / gradient)
constexpr int HB = 64;   // element block (Hessian): 64 x 90 x sizeof(S) bytes of staging

template <typename S>
__device__ __forceinline__ S comp(const V4<S>& v, int k) {
  return k == 0 ? v.x : (k == 1 ? v.y : v.z);
}

// One thread per tet.  x = X + u (+ alpha d), F = Ds Dminv (def_grad.hpp:108-126), PK1 and energy
// (stable_neohookean.hpp:38-62), local forces P Dminv^T with row 0 = -sum (time_step.hpp:62-90), scaled
// by dt^2 V_e (the composer's weight, global_composer.hpp:233-240, times alpha = dt^2), plus the
// element's share of the consistent-mass inertia term: with M_e(i, j) = rho V_e / 20 (1 + delta_ij)
// (bilinears.hpp:140-148), (M_e d)_i = rho V_e / 20 (d_i + sum_j d_j) and
// 1/2 d^T M_e d = rho V_e / 40 (sum_i |d_i|^2 + |sum_i d_i|^2).  Summed over tets this is exactly the
// unfiltered mass matrix product of time_step.hpp:589-592.
template <typename SD, bool FORCES, bool TRIAL>
__global__ void __launch_bounds__(EB)
    elem_energy_grad_kernel(ElemFP64 el, const double* __restrict__ X, const double* __restrict__ u,
                            const double* __restrict__ xt, const V4<SD>* __restrict__ d, double alpha, double dt2,
                            double rho, double* __restrict__ lf, Reduce red) {
  __shared__ double stage[FORCES ? EB * 12 : 1];
  __shared__ double shred[EB / 32][2];
  const int e0 = blockIdx.x * EB;
  const int e = e0 + threadIdx.x;
  double energy = 0, escale = 0;
  double lfv[12];
  if (e < el.nt) {
    const int4 c = el.cells[e];
    const int vid[4] = {c.x, c.y, c.z, c.w};
    double uu[4][3], dd[4][3];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      V4<SD> dv;
      if (TRIAL) dv = d[vid[i]];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        double uk = u[vid[i] * 3 + k];
        if (TRIAL) uk += alpha * (double)comp<SD>(dv, k);
        uu[i][k] = uk;
        dd[i][k] = uk - xt[vid[i] * 3 + k];
      }
    }
    double Dm[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) Dm[k] = el.dminv[(size_t)k * el.nt + e];
    // F = Ds Dm^-1 with Ds = [x1-x0, x2-x0, x3-x0] (def_grad.hpp:108-126); the rest edges times Dm^-1 are
    // the identity, so F = I + [u1-u0, u2-u0, u3-u0] Dm^-1, which keeps the displacement's digits
    double Du[9];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int k = 0; k < 3; ++k) Du[r * 3 + k] = uu[k + 1][r] - uu[0][r];
    double G[9], F[9];  // displacement gradient and F = I + G
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int cc = 0; cc < 3; ++cc) {
        G[r * 3 + cc] = Du[r * 3 + 0] * Dm[0 * 3 + cc] + Du[r * 3 + 1] * Dm[1 * 3 + cc] + Du[r * 3 + 2] * Dm[2 * 3 + cc];
        F[r * 3 + cc] = (r == cc ? 1.0 : 0.0) + G[r * 3 + cc];
      }
    const double lam = el.lam[e], mu = el.mu[e], V = el.vol[e];
    const double m = rho * V * (1.0 / 20.0);
    double sd[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) sd[k] = dd[0][k] + dd[1][k] + dd[2][k] + dd[3][k];
    double q = sd[0] * sd[0] + sd[1] * sd[1] + sd[2] * sd[2];
#pragma unroll
    for (int i = 0; i < 4; ++i) q += dd[i][0] * dd[i][0] + dd[i][1] * dd[i][1] + dd[i][2] * dd[i][2];
    double P[9], sc;
    const double psi = el.model == 1 ? linear_eval<double, FORCES>(G, lam, mu, P, sc)
                                     : snh_eval<double, FORCES>(F, lam, mu, el.alpha[e], el.psi0[e], P, sc);
    if (FORCES) {
      const double s = dt2 * V;
      double tot[3] = {0, 0, 0};
#pragma unroll
      for (int i = 1; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const double h = P[j * 3 + 0] * Dm[(i - 1) * 3 + 0] + P[j * 3 + 1] * Dm[(i - 1) * 3 + 1] +
                           P[j * 3 + 2] * Dm[(i - 1) * 3 + 2];
          tot[j] += h;
          lfv[i * 3 + j] = s * h + m * (dd[i][j] + sd[j]);
        }
#pragma unroll
      for (int j = 0; j < 3; ++j) lfv[j] = -s * tot[j] + m * (dd[0][j] + sd[j]);
    }
    energy = dt2 * V * psi + 0.5 * m * q;
    escale = dt2 * V * sc + 0.5 * m * q;
  }
  if (FORCES) {
    if (e < el.nt) {
#pragma unroll
      for (int k = 0; k < 12; ++k) stage[threadIdx.x * 12 + k] = lfv[k];
    }
    __syncthreads();
    const int nvalid = min(EB, el.nt - e0);
    double* dst = lf + (size_t)e0 * 12;
    for (int i = threadIdx.x; i < nvalid * 12; i += EB) dst[i] = stage[i];
  }
  double v2[2] = {energy, escale};
  block_sum<2, EB>(v2, shred);
  double tot[2];
  if (grid_sum_last<2, EB>(v2, red.partials, red.counter, tot)) {
    if (TRIAL) {
      red.sc->trial_energy = tot[0];
      red.sc->trial_energy_scale = tot[1];
    } else {
      red.sc->energy = tot[0];
      red.sc->energy_scale = tot[1];
    }
  }
}

// The same pass with the element arithmetic in FP32 (the mixed steppers' early iterations).  Per vertex,
// u is split into FP32 (hi, lo) with hi + lo = u to ~2^-48 and the inertia offset w = u - x~ is rounded
// once (split32_kernel, once per base point), so the element forms its displacement differences
// (hi_j - hi_i) + (lo_j - lo_i) (+ alpha (d_j - d_i)) in FP32 with rounding relative to the difference:
// no FP64 arithmetic per element (GB300's FP64 pipe bound the earlier version).  Energy and stress use
// the small-strain forms (snh_eval_small / linear_eval); energies are summed in FP32 within a warp and in
// FP64 across warps and blocks; forces go to lf32[t][4][3] (FP32).
__global__ void __launch_bounds__(256)
    split32_kernel(int nv, const double* __restrict__ u, const double* __restrict__ xt, float4* __restrict__ uh,
                   float4* __restrict__ ul, float4* __restrict__ w) {
  const int v = blockIdx.x * 256 + threadIdx.x;
  if (v >= nv) return;
  float h[3], l[3], o[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double x = u[3 * v + k];
    h[k] = (float)x;
    l[k] = (float)(x - (double)h[k]);
    o[k] = xt != nullptr ? (float)(x - xt[3 * v + k]) : 0.f;
  }
  uh[v] = make_float4(h[0], h[1], h[2], 0.f);
  ul[v] = make_float4(l[0], l[1], l[2], 0.f);
  if (w != nullptr) w[v] = make_float4(o[0], o[1], o[2], 0.f);
}

template <bool FORCES, bool TRIAL, int EB, int MINB = 1>
__global__ void __launch_bounds__(EB, MINB)
    elem_energy_grad32_kernel(ElemFP64 el, ElemFP32 ef, Split32 sp, const float4* __restrict__ d, float alpha,
                              float dt2, float rho, float* __restrict__ lf32, Reduce red) {
  __shared__ float stage[FORCES ? EB * 12 : 1];
  __shared__ double shred[EB / 32][2];
  const int e0 = blockIdx.x * EB;
  const int e = e0 + threadIdx.x;
  float part[2] = {0.f, 0.f};
  float lfv[12];
  if (e < el.nt) {
    const int4 c = el.cells[e];
    const int vid[4] = {c.x, c.y, c.z, c.w};
    float4 hv[4], lv[4], dv[4];
    float dd[4][3];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      hv[i] = sp.uh[vid[i]];
      lv[i] = sp.ul[vid[i]];
      const float4 wv = sp.w[vid[i]];
      if (TRIAL) dv[i] = d[vid[i]];
      dd[i][0] = TRIAL ? wv.x + alpha * dv[i].x : wv.x;
      dd[i][1] = TRIAL ? wv.y + alpha * dv[i].y : wv.y;
      dd[i][2] = TRIAL ? wv.z + alpha * dv[i].z : wv.z;
    }
    float Dm[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) Dm[k] = ef.dminv[(size_t)k * el.nt + e];
    float Du[9];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      float a0 = (hv[k + 1].x - hv[0].x) + (lv[k + 1].x - lv[0].x);
      float a1 = (hv[k + 1].y - hv[0].y) + (lv[k + 1].y - lv[0].y);
      float a2 = (hv[k + 1].z - hv[0].z) + (lv[k + 1].z - lv[0].z);
      if (TRIAL) {
        a0 += alpha * (dv[k + 1].x - dv[0].x);
        a1 += alpha * (dv[k + 1].y - dv[0].y);
        a2 += alpha * (dv[k + 1].z - dv[0].z);
      }
      Du[0 * 3 + k] = a0;
      Du[1 * 3 + k] = a1;
      Du[2 * 3 + k] = a2;
    }
    float G[9];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int cc = 0; cc < 3; ++cc)
        G[r * 3 + cc] = Du[r * 3 + 0] * Dm[0 * 3 + cc] + Du[r * 3 + 1] * Dm[1 * 3 + cc] + Du[r * 3 + 2] * Dm[2 * 3 + cc];
    const float lam = ef.lam[e], mu = ef.mu[e], V = ef.vol[e];
    const float m = rho * V * (1.0f / 20.0f);
    float sd[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) sd[k] = dd[0][k] + dd[1][k] + dd[2][k] + dd[3][k];
    float q = sd[0] * sd[0] + sd[1] * sd[1] + sd[2] * sd[2];
#pragma unroll
    for (int i = 0; i < 4; ++i) q += dd[i][0] * dd[i][0] + dd[i][1] * dd[i][1] + dd[i][2] * dd[i][2];
    float P[9], sc;
    const float psi = el.model == 1 ? linear_eval<float, FORCES>(G, lam, mu, P, sc)
                                    : snh_eval_small<float, FORCES>(G, lam, mu, P, sc);
    if (FORCES) {
      const float sV = dt2 * V;
      float tot[3] = {0, 0, 0};
#pragma unroll
      for (int i = 1; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const float h = P[j * 3 + 0] * Dm[(i - 1) * 3 + 0] + P[j * 3 + 1] * Dm[(i - 1) * 3 + 1] +
                          P[j * 3 + 2] * Dm[(i - 1) * 3 + 2];
          tot[j] += h;
          lfv[i * 3 + j] = sV * h + m * (dd[i][j] + sd[j]);
        }
#pragma unroll
      for (int j = 0; j < 3; ++j) lfv[j] = -sV * tot[j] + m * (dd[0][j] + sd[j]);
    }
    part[0] = dt2 * V * psi + 0.5f * m * q;
    part[1] = dt2 * V * sc + 0.5f * m * q;
  }
  if (FORCES) {
    if (e < el.nt) {
#pragma unroll
      for (int k = 0; k < 12; ++k) stage[threadIdx.x * 12 + k] = lfv[k];
    }
    __syncthreads();
    const int nvalid = min(EB, el.nt - e0);
    float* dst = lf32 + (size_t)e0 * 12;
    for (int i = threadIdx.x; i < nvalid * 12; i += EB) dst[i] = stage[i];
  }
  double v2[2];
  block_sum_s<2, EB, float>(part, v2, shred);
  double tot[2];
  if (grid_sum_last<2, EB>(v2, red.partials, red.counter, tot)) {
    if (TRIAL) {
      red.sc->trial_energy = tot[0];
      red.sc->trial_energy_scale = tot[1];
    } else {
      red.sc->energy = tot[0];
      red.sc->energy_scale = tot[1];
    }
  }
}

// The mixed Newton's iterations after the switch from the FP32 pass: energy and forces as increments from a
// reference state u_r evaluated once in FP64 (its energy e_ref and forces, which the gather adds back).  Per
// element the stable Neo-Hookean increment between G_r and G_r + dG in FP32 (snh_increment: rounding
// relative to the increment, not to the stress), the consistent-mass inertia increment
// (M_e (d_r + x))^T-terms with d_r = u_r - x~ and x = u - u_r, and the local force increments.  Vertex data:
// ref = the FP32 split (hi, lo) of u_r and w = u_r - x~ (split32_kernel at u_r); db = u_b - u_r at the line
// search's base point; the trial point is u_b + alpha d.
template <bool FORCES, bool TRIAL, int EB>
__global__ void __launch_bounds__(EB)
    elem_delta32_kernel(ElemFP64 el, ElemFP32 ef, Split32 ref, const float4* __restrict__ db,
                        const float4* __restrict__ d, float alpha, float dt2, float rho, double e_ref,
                        double escale_ref, float* __restrict__ lf32, Reduce red) {
  __shared__ float stage[FORCES ? EB * 12 : 1];
  __shared__ double shred[EB / 32][1];
  const int e0 = blockIdx.x * EB;
  const int e = e0 + threadIdx.x;
  float part[1] = {0.f};
  float lfv[12];
  if (e < el.nt) {
    const int4 c = el.cells[e];
    const int vid[4] = {c.x, c.y, c.z, c.w};
    float4 hv[4], lv[4], wv[4];
    float x[4][3];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      hv[i] = ref.uh[vid[i]];
      lv[i] = ref.ul[vid[i]];
      wv[i] = ref.w[vid[i]];
      const float4 b = db[vid[i]];
      x[i][0] = b.x;
      x[i][1] = b.y;
      x[i][2] = b.z;
      if (TRIAL) {
        const float4 dv = d[vid[i]];
        x[i][0] += alpha * dv.x;
        x[i][1] += alpha * dv.y;
        x[i][2] += alpha * dv.z;
      }
    }
    float Dm[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) Dm[k] = ef.dminv[(size_t)k * el.nt + e];
    float Gr[9], dG[9];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      const float hr[3] = {comp<float>(hv[1], r) - comp<float>(hv[0], r) + (comp<float>(lv[1], r) - comp<float>(lv[0], r)),
                           comp<float>(hv[2], r) - comp<float>(hv[0], r) + (comp<float>(lv[2], r) - comp<float>(lv[0], r)),
                           comp<float>(hv[3], r) - comp<float>(hv[0], r) + (comp<float>(lv[3], r) - comp<float>(lv[0], r))};
      const float xr[3] = {x[1][r] - x[0][r], x[2][r] - x[0][r], x[3][r] - x[0][r]};
#pragma unroll
      for (int cc = 0; cc < 3; ++cc) {
        Gr[r * 3 + cc] = hr[0] * Dm[0 * 3 + cc] + hr[1] * Dm[1 * 3 + cc] + hr[2] * Dm[2 * 3 + cc];
        dG[r * 3 + cc] = xr[0] * Dm[0 * 3 + cc] + xr[1] * Dm[1 * 3 + cc] + xr[2] * Dm[2 * 3 + cc];
      }
    }
    const float lam = ef.lam[e], mu = ef.mu[e], V = ef.vol[e];
    const float m = rho * V * (1.0f / 20.0f);
    float dP[9];
    const float dpsi = snh_increment<float>(Gr, dG, lam, mu, FORCES ? dP : nullptr);
    // inertia: 1/2 (d_r + x)^T M_e (d_r + x) - 1/2 d_r^T M_e d_r with M_e(i, j) = m (1 + delta_ij)
    float sw[3], sx[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      sw[k] = comp<float>(wv[0], k) + comp<float>(wv[1], k) + comp<float>(wv[2], k) + comp<float>(wv[3], k);
      sx[k] = x[0][k] + x[1][k] + x[2][k] + x[3][k];
    }
    float cross = sw[0] * sx[0] + sw[1] * sx[1] + sw[2] * sx[2];
    float quad = sx[0] * sx[0] + sx[1] * sx[1] + sx[2] * sx[2];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        cross += comp<float>(wv[i], k) * x[i][k];
        quad += x[i][k] * x[i][k];
      }
    if (FORCES) {
      const float sV = dt2 * V;
      float tot[3] = {0, 0, 0};
#pragma unroll
      for (int i = 1; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const float h = dP[j * 3 + 0] * Dm[(i - 1) * 3 + 0] + dP[j * 3 + 1] * Dm[(i - 1) * 3 + 1] +
                          dP[j * 3 + 2] * Dm[(i - 1) * 3 + 2];
          tot[j] += h;
          lfv[i * 3 + j] = sV * h + m * (x[i][j] + sx[j]);
        }
#pragma unroll
      for (int j = 0; j < 3; ++j) lfv[j] = -sV * tot[j] + m * (x[0][j] + sx[j]);
    }
    part[0] = dt2 * V * dpsi + m * cross + 0.5f * m * quad;
  }
  if (FORCES) {
    if (e < el.nt) {
#pragma unroll
      for (int k = 0; k < 12; ++k) stage[threadIdx.x * 12 + k] = lfv[k];
    }
    __syncthreads();
    const int nvalid = min(EB, el.nt - e0);
    float* dst = lf32 + (size_t)e0 * 12;
    for (int i = threadIdx.x; i < nvalid * 12; i += EB) dst[i] = stage[i];
  }
  double v1[1];
  block_sum_s<1, EB, float>(part, v1, shred);
  double tot[1];
  if (grid_sum_last<1, EB>(v1, red.partials, red.counter, tot)) {
    if (TRIAL) {
      red.sc->trial_energy = e_ref + tot[0];
      red.sc->trial_energy_scale = escale_ref;
    } else {
      red.sc->energy = e_ref + tot[0];
      red.sc->energy_scale = escale_ref;
    }
  }
}

// forces as the reference's FP64 forces plus the FP32 local force increments lf32[(e, i)][3] summed per
// vertex, Dirichlet dofs zeroed; |g|^2 in FP64
template <int B>
__global__ void __launch_bounds__(B)
    vertex_gather_delta32_kernel(int nv, const int* __restrict__ vptr, const int* __restrict__ vinc,
                                 const float* __restrict__ lf32, const uint8_t* __restrict__ mask,
                                 const double* __restrict__ gref, double* __restrict__ g, Reduce red) {
  __shared__ double shred[B / 32][1];
  const int v = blockIdx.x * B + threadIdx.x;
  double part[1] = {0.0};
  if (v < nv) {
    float a0 = 0.f, a1 = 0.f, a2 = 0.f;
    const int k1 = vptr[v + 1];
    for (int k = vptr[v]; k < k1; ++k) {
      const float* s = lf32 + (size_t)vinc[k] * 3;
      a0 += s[0];
      a1 += s[1];
      a2 += s[2];
    }
    const uint8_t mk = mask[v];
    const double g0 = (mk & 1) ? 0.0 : gref[3 * v] + (double)a0;
    const double g1 = (mk & 2) ? 0.0 : gref[3 * v + 1] + (double)a1;
    const double g2 = (mk & 4) ? 0.0 : gref[3 * v + 2] + (double)a2;
    g[3 * v] = g0;
    g[3 * v + 1] = g1;
    g[3 * v + 2] = g2;
    part[0] = g0 * g0 + g1 * g1 + g2 * g2;
  }
  block_sum<1, B>(part, shred);
  double tot[1];
  if (grid_sum_last<1, B>(part, red.partials, red.counter, tot)) red.sc->gnorm2 = tot[0];
}

// x_b = u - u_ref per vertex, rounded once to FP32 (the base point of the increment evaluations)
__global__ void __launch_bounds__(256)
    delta_base_kernel(int nv, const double* __restrict__ u, const double* __restrict__ uref, float4* __restrict__ db) {
  const int v = blockIdx.x * 256 + threadIdx.x;
  if (v >= nv) return;
  db[v] = make_float4((float)(u[3 * v] - uref[3 * v]), (float)(u[3 * v + 1] - uref[3 * v + 1]),
                      (float)(u[3 * v + 2] - uref[3 * v + 2]), 0.f);
}

// forces from FP32 local forces lf32[(e, i)][3], summed per vertex in FP32, Dirichlet dofs zeroed; |g|^2
template <int B>
__global__ void __launch_bounds__(B)
    vertex_gather32_kernel(int nv, const int* __restrict__ vptr, const int* __restrict__ vinc,
                           const float* __restrict__ lf32, const uint8_t* __restrict__ mask, double* __restrict__ g,
                           Reduce red) {
  __shared__ double shred[B / 32][1];
  const int v = blockIdx.x * B + threadIdx.x;
  float part[1] = {0.f};
  if (v < nv) {
    float a0 = 0.f, a1 = 0.f, a2 = 0.f;
    const int k1 = vptr[v + 1];
    for (int k = vptr[v]; k < k1; ++k) {
      const float* s = lf32 + (size_t)vinc[k] * 3;
      a0 += s[0];
      a1 += s[1];
      a2 += s[2];
    }
    const uint8_t mk = mask[v];
    if (mk & 1) a0 = 0.f;
    if (mk & 2) a1 = 0.f;
    if (mk & 4) a2 = 0.f;
    g[3 * v] = a0;
    g[3 * v + 1] = a1;
    g[3 * v + 2] = a2;
    part[0] = a0 * a0 + a1 * a1 + a2 * a2;
  }
  double v1[1];
  block_sum_s<1, B, float>(part, v1, shred);
  double tot[1];
  if (grid_sum_last<1, B>(v1, red.partials, red.counter, tot)) red.sc->gnorm2 = tot[0];
}

constexpr int GB = 256;

__global__ void __launch_bounds__(GB)
    vertex_gather_kernel(int nv, const int* __restrict__ vptr, const int* __restrict__ vinc,
                         const double* __restrict__ lf, const uint8_t* __restrict__ mask, double* __restrict__ g,
                         Reduce red) {
  __shared__ double shred[GB / 32][1];
  const int v = blockIdx.x * GB + threadIdx.x;
  double part = 0;
  if (v < nv) {
    double a0 = 0, a1 = 0, a2 = 0;
    const int k1 = vptr[v + 1];
    for (int k = vptr[v]; k < k1; ++k) {
      const double* s = lf + (size_t)vinc[k] * 3;
      a0 += s[0];
      a1 += s[1];
      a2 += s[2];
    }
    const uint8_t m = mask[v];  // boundary_condition::grads (boundary.hpp:45-51)
    if (m & 1) a0 = 0;
    if (m & 2) a1 = 0;
    if (m & 4) a2 = 0;
    g[v * 3 + 0] = a0;
    g[v * 3 + 1] = a1;
    g[v * 3 + 2] = a2;
    part = a0 * a0 + a1 * a1 + a2 * a2;
  }
  double v1[1] = {part};
  block_sum<1, GB>(v1, shred);
  double tot[1];
  if (grid_sum_last<1, GB>(v1, red.partials, red.counter, tot)) red.sc->gnorm2 = tot[0];
}

// ------------------------------------------------------------------ element Hessian
// One thread per tet: K_e = dt^2 V_e pfpx^T H+ pfpx (the gather weight V_e and alpha = dt^2 of
// time_step.hpp:646-651 folded in), written as the 10 upper 3x3 vertex blocks, staged through shared
// memory so the global writes are contiguous.  Launch bounds of 8 blocks per SM (128 registers, a few
// spills) beat the unconstrained 168 registers: 168 against 192 us per launch at 1.02M tets.
// H16 (FP32 arithmetic only): each block written as twelve FP16 words, the nine values scaled by 2^-k and
// k (the power of two that puts the block's largest magnitude in [2^14, 2^15)) in word 9: 24 bytes a block
// instead of 36, read back with three 8-byte loads (kernels_sparse.cu assemble_kernel).
__device__ __forceinline__ void pack_block16(const float* v, uint2* out) {
  float m = 0.f;
#pragma unroll
  for (int i = 0; i < 9; ++i) m = fmaxf(m, fabsf(v[i]));
  int k = 0;
  if (m > 0.f && m <= FLT_MAX) k = ((__float_as_int(m) >> 23) & 0xff) - 127 - 14;  // floor(log2 m) - 14
  k = max(-100, min(100, k));
  const float inv = __int_as_float((127 - k) << 23);  // 2^-k, exact
  unsigned short h[12];
#pragma unroll
  for (int i = 0; i < 9; ++i) h[i] = __half_as_ushort(__float2half_rn(v[i] * inv));
  h[9] = (unsigned short)(short)k;
  h[10] = h[11] = 0;
#pragma unroll
  for (int j = 0; j < 3; ++j)
    out[j] = make_uint2((unsigned int)h[4 * j] | ((unsigned int)h[4 * j + 1] << 16),
                        (unsigned int)h[4 * j + 2] | ((unsigned int)h[4 * j + 3] << 16));
}

template <typename S, bool XF, int HB, bool H16 = false>
__global__ void __launch_bounds__(HB, 512 / HB)
    elem_hessian_kernel(ElemFP64 e64, ElemFP32 e32, const double* __restrict__ X, const double* __restrict__ u,
                        const float4* __restrict__ xf, S dt2, int spsd, S* __restrict__ Kbuf) {
  __shared__ S stage[HB * 90];
  const int nt = e64.nt;
  const int e0 = blockIdx.x * HB;
  const int e = e0 + threadIdx.x;
  if (e < nt) {
    S K[78];
    element_hessian_at<S, XF>(e64, e32, X, u, xf, dt2, spsd, e, K);
    int blk = 0;
#pragma unroll
    for (int v = 0; v < 4; ++v)
#pragma unroll
      for (int w = v; w < 4; ++w) {
        S bv[9];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
          for (int b = 0; b < 3; ++b) {
            const int i = v * 3 + a, j = w * 3 + b;
            bv[a * 3 + b] = (i <= j) ? K[kup(i, j)] : K[kup(j, i)];
          }
        if constexpr (H16) {
          // packed straight from registers: thread t's 30 words at 30 t (the element's global order)
          pack_block16(bv, reinterpret_cast<uint2*>(stage) + threadIdx.x * 30 + 3 * blk);
        } else {
#pragma unroll
          for (int c = 0; c < 9; ++c) stage[threadIdx.x * 90 + blk * 9 + c] = bv[c];
        }
        ++blk;
      }
  }
  __syncthreads();
  const int nvalid = min(HB, nt - e0);
  if constexpr (H16) {
    const uint2* src = reinterpret_cast<const uint2*>(stage);
    uint2* dst = reinterpret_cast<uint2*>(Kbuf) + (size_t)e0 * 30;
    for (int i = threadIdx.x; i < nvalid * 30; i += HB) dst[i] = src[i];
  } else {
    S* dst = Kbuf + (size_t)e0 * 90;
    for (int i = threadIdx.x; i < nvalid * 90; i += HB) dst[i] = stage[i];
  }
}

}  // namespace

template <typename SD>
void launch_elem_energy_grad(const ElemFP64& el, const double* X, const double* u, const double* xt,
                             const V4<SD>* d, double alpha, double dt2, double rho, double* lf, bool with_forces,
                             bool trial, const Reduce& red, cudaStream_t st) {
  if (el.nt <= 0) return;
  const int grid = div_up(el.nt, EB);
  if (trial && with_forces) {
    elem_energy_grad_kernel<SD, true, true><<<grid, EB, 0, st>>>(el, X, u, xt, d, alpha, dt2, rho, lf, red);
  } else if (trial) {
    elem_energy_grad_kernel<SD, false, true><<<grid, EB, 0, st>>>(el, X, u, xt, d, alpha, dt2, rho, lf, red);
  } else if (with_forces) {
    elem_energy_grad_kernel<SD, true, false><<<grid, EB, 0, st>>>(el, X, u, xt, d, alpha, dt2, rho, lf, red);
  } else {
    elem_energy_grad_kernel<SD, false, false><<<grid, EB, 0, st>>>(el, X, u, xt, d, alpha, dt2, rho, lf, red);
  }
  after_launch("elem_energy_grad");
}
template void launch_elem_energy_grad<float>(const ElemFP64&, const double*, const double*, const double*,
                                             const float4*, double, double, double, double*, bool, bool,
                                             const Reduce&, cudaStream_t);
template void launch_elem_energy_grad<double>(const ElemFP64&, const double*, const double*, const double*,
                                              const double4_32a*, double, double, double, double*, bool, bool,
                                              const Reduce&, cudaStream_t);

void launch_split32(int nv, const double* u, const double* xt, float4* uh, float4* ul, float4* w, cudaStream_t st) {
  if (nv <= 0) return;
  split32_kernel<<<div_up(nv, 256), 256, 0, st>>>(nv, u, xt, uh, ul, w);
  after_launch("split32");
}

void launch_elem_energy_grad32(const ElemFP64& el, const ElemFP32& ef, const Split32& sp, const float4* d,
                               double alpha, double dt2, double rho, float* lf32, bool with_forces, bool trial,
                               const Reduce& red, cudaStream_t st, int block, int regcap) {
  if (el.nt <= 0) return;
  const float f_dt2 = (float)dt2, f_rho = (float)rho, a = (float)alpha;
  // regcap: the variant compiled for 1024 / b resident blocks per SM (at most 64 registers a thread: more warps
  // in flight for the dependent vertex gathers, a few bytes of spill)
  auto launch = [&](auto B, auto M) {
    constexpr int b = decltype(B)::value, m = decltype(M)::value;
    const int grid = div_up(el.nt, b);
    if (trial && with_forces)
      elem_energy_grad32_kernel<true, true, b, m><<<grid, b, 0, st>>>(el, ef, sp, d, a, f_dt2, f_rho, lf32, red);
    else if (trial)
      elem_energy_grad32_kernel<false, true, b, m><<<grid, b, 0, st>>>(el, ef, sp, d, a, f_dt2, f_rho, lf32, red);
    else if (with_forces)
      elem_energy_grad32_kernel<true, false, b, m><<<grid, b, 0, st>>>(el, ef, sp, d, a, f_dt2, f_rho, lf32, red);
    else
      elem_energy_grad32_kernel<false, false, b, m><<<grid, b, 0, st>>>(el, ef, sp, d, a, f_dt2, f_rho, lf32, red);
  };
  auto go = [&](auto B) {
    constexpr int b = decltype(B)::value;
    if (regcap)
      launch(B, std::integral_constant<int, 1024 / b>{});
    else
      launch(B, std::integral_constant<int, 1>{});
  };
  dispatch_block<64, 128, 256>(block == 0 ? EB : block, go);
  after_launch("elem_energy_grad32");
}
void launch_elem_delta32(const ElemFP64& el, const ElemFP32& ef, const Split32& ref, const float4* db, const float4* d,
                         double alpha, double dt2, double rho, double e_ref, double escale_ref, float* lf32,
                         bool with_forces, bool trial, const Reduce& red, cudaStream_t st, int block) {
  if (el.nt <= 0) return;
  const float f_dt2 = (float)dt2, f_rho = (float)rho, a = (float)alpha;
  auto go = [&](auto B) {
    constexpr int b = decltype(B)::value;
    const int grid = div_up(el.nt, b);
    if (trial && with_forces)
      elem_delta32_kernel<true, true, b><<<grid, b, 0, st>>>(el, ef, ref, db, d, a, f_dt2, f_rho, e_ref, escale_ref, lf32, red);
    else if (trial)
      elem_delta32_kernel<false, true, b><<<grid, b, 0, st>>>(el, ef, ref, db, d, a, f_dt2, f_rho, e_ref, escale_ref, lf32, red);
    else if (with_forces)
      elem_delta32_kernel<true, false, b><<<grid, b, 0, st>>>(el, ef, ref, db, d, a, f_dt2, f_rho, e_ref, escale_ref, lf32, red);
    else
      elem_delta32_kernel<false, false, b><<<grid, b, 0, st>>>(el, ef, ref, db, d, a, f_dt2, f_rho, e_ref, escale_ref, lf32, red);
  };
  dispatch_block<64, 128, 256>(block == 0 ? EB : block, go);
  after_launch("elem_delta32");
}
void launch_vertex_gather_delta32(int nv, const int* vptr, const int* vinc, const float* lf32, const uint8_t* mask,
                                  const double* gref, double* g, const Reduce& red, cudaStream_t st, int block) {
  if (nv <= 0) return;
  auto go = [&](auto B) {
    constexpr int b = decltype(B)::value;
    vertex_gather_delta32_kernel<b><<<div_up(nv, b), b, 0, st>>>(nv, vptr, vinc, lf32, mask, gref, g, red);
  };
  dispatch_block<128, 256, 512>(block == 0 ? 256 : block, go);
  after_launch("vertex_gather_delta32");
}
void launch_delta_base(int nv, const double* u, const double* uref, float4* db, cudaStream_t st) {
  if (nv <= 0) return;
  delta_base_kernel<<<div_up(nv, 256), 256, 0, st>>>(nv, u, uref, db);
  after_launch("delta_base");
}

void launch_vertex_gather32(int nv, const int* vptr, const int* vinc, const float* lf32, const uint8_t* mask,
                            double* g, const Reduce& red, cudaStream_t st, int block) {
  if (nv <= 0) return;
  auto go = [&](auto B) {
    constexpr int b = decltype(B)::value;
    vertex_gather32_kernel<b><<<div_up(nv, b), b, 0, st>>>(nv, vptr, vinc, lf32, mask, g, red);
  };
  dispatch_block<128, 256, 512>(block == 0 ? 256 : block, go);
  after_launch("vertex_gather32");
}
void launch_vertex_gather(int nv, const int* vptr, const int* vinc, const double* lf, const uint8_t* mask,
                          double* g, const Reduce& red, cudaStream_t st) {
  if (nv <= 0) return;
  vertex_gather_kernel<<<div_up(nv, GB), GB, 0, st>>>(nv, vptr, vinc, lf, mask, g, red);
  after_launch("vertex_gather");
}

template <typename S>
void launch_elem_hessian(const ElemFP64& e64, const ElemFP32& e32, const double* X, const double* u,
                         const float4* xf, double dt2, bool spsd, S* Kbuf, cudaStream_t st, int block) {
  if (e64.nt <= 0) return;
  auto go = [&](auto B) {
    constexpr int b = decltype(B)::value;
    const int grid = div_up(e64.nt, b);
    if (xf != nullptr)
      elem_hessian_kernel<S, true, b><<<grid, b, 0, st>>>(e64, e32, X, u, xf, (S)dt2, spsd ? 1 : 0, Kbuf);
    else
      elem_hessian_kernel<S, false, b><<<grid, b, 0, st>>>(e64, e32, X, u, xf, (S)dt2, spsd ? 1 : 0, Kbuf);
  };
  dispatch_block<32, 64, 128>(block == 0 ? HB : block, go);
  after_launch("elem_hessian");
}
void launch_elem_hessian16(const ElemFP64& e64, const ElemFP32& e32, const double* X, const double* u,
                           const float4* xf, double dt2, bool spsd, uint2* K16, cudaStream_t st, int block) {
  if (e64.nt <= 0) return;
  float* kb = reinterpret_cast<float*>(K16);
  auto go = [&](auto B) {
    constexpr int b = decltype(B)::value;
    const int grid = div_up(e64.nt, b);
    if (xf != nullptr)
      elem_hessian_kernel<float, true, b, true><<<grid, b, 0, st>>>(e64, e32, X, u, xf, (float)dt2, spsd ? 1 : 0, kb);
    else
      elem_hessian_kernel<float, false, b, true><<<grid, b, 0, st>>>(e64, e32, X, u, xf, (float)dt2, spsd ? 1 : 0, kb);
  };
  dispatch_block<32, 64, 128>(block == 0 ? HB : block, go);
  after_launch("elem_hessian16");
}template void launch_elem_hessian<float>(const ElemFP64&, const ElemFP32&, const double*, const double*,
                                         const float4*, double, bool, float*, cudaStream_t, int);
template void launch_elem_hessian<double>(const ElemFP64&, const ElemFP32&, const double*, const double*,
                                          const float4*, double, bool, double*, cudaStream_t, int);

}  // namespace ssim_gb
