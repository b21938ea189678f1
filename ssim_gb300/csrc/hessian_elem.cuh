// hessian_elem.cuh -- the element Hessian of one tet, shared by the two-kernel path (elem_hessian_kernel +
// assemble_kernel) and the fused element-Hessian + assembly kernel.
#pragma once
#include "elem_math.cuh"
#include "kernels.cuh"

namespace ssim_gb {

// the element constants in the arithmetic type of the Hessian: FP32 copies on the mixed path
template <typename S>
struct ElemSel;
template <>
struct ElemSel<float> {
  __device__ static const float* dminv(const ElemFP64&, const ElemFP32& b) { return b.dminv; }
  __device__ static float vol(const ElemFP64&, const ElemFP32& b, int e) { return b.vol[e]; }
  __device__ static float lam(const ElemFP64&, const ElemFP32& b, int e) { return b.lam[e]; }
  __device__ static float mu(const ElemFP64&, const ElemFP32& b, int e) { return b.mu[e]; }
};
template <>
struct ElemSel<double> {
  __device__ static const double* dminv(const ElemFP64& a, const ElemFP32&) { return a.dminv; }
  __device__ static double vol(const ElemFP64& a, const ElemFP32&, int e) { return a.vol[e]; }
  __device__ static double lam(const ElemFP64& a, const ElemFP32&, int e) { return a.lam[e]; }
  __device__ static double mu(const ElemFP64& a, const ElemFP32&, int e) { return a.mu[e]; }
};

// K_e = dt^2 V_e pfpx^T H(+) pfpx of tet e (wrapped_pfpx, time_step.hpp:23-60, with the gather weight V_e
// and alpha = dt^2 of time_step.hpp:646-651 folded in) as the packed upper triangle of the 12 x 12 matrix
// (row = vertex * 3 + dof).  Positions: X + u in FP64 rounded to S, or the FP32 positions xf (XF).
template <typename S, bool XF>
__device__ __forceinline__ void element_hessian_at(const ElemFP64& e64, const ElemFP32& e32,
                                                   const double* __restrict__ X, const double* __restrict__ u,
                                                   const float4* __restrict__ xf, S dt2, int spsd, int e,
                                                   S (&K)[78]) {
  const int nt = e64.nt;
  const int4 c = e64.cells[e];
  const int vid[4] = {c.x, c.y, c.z, c.w};
  S x[4][3];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    if (XF) {
      const float4 p = xf[vid[i]];
      x[i][0] = (S)p.x;
      x[i][1] = (S)p.y;
      x[i][2] = (S)p.z;
    } else {
#pragma unroll
      for (int k = 0; k < 3; ++k) x[i][k] = (S)(X[vid[i] * 3 + k] + u[vid[i] * 3 + k]);
    }
  }
  const S* dm = ElemSel<S>::dminv(e64, e32);
  S Dm[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) Dm[k] = dm[(size_t)k * nt + e];
  S F[9];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int cc = 0; cc < 3; ++cc)
      F[r * 3 + cc] = (x[1][r] - x[0][r]) * Dm[0 * 3 + cc] + (x[2][r] - x[0][r]) * Dm[1 * 3 + cc] +
                      (x[3][r] - x[0][r]) * Dm[2 * 3 + cc];
  S D[4][3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    D[1][j] = Dm[0 * 3 + j];
    D[2][j] = Dm[1 * 3 + j];
    D[3][j] = Dm[2 * 3 + j];
    D[0][j] = -(Dm[0 * 3 + j] + Dm[1 * 3 + j] + Dm[2 * 3 + j]);
  }
  if (e64.model == 1)
    linear_stiffness<S>(D, ElemSel<S>::lam(e64, e32, e), ElemSel<S>::mu(e64, e32, e), spsd != 0,
                        dt2 * ElemSel<S>::vol(e64, e32, e), K);
  else
    element_stiffness<S>(F, D, ElemSel<S>::lam(e64, e32, e), ElemSel<S>::mu(e64, e32, e), spsd != 0,
                         dt2 * ElemSel<S>::vol(e64, e32, e), K);
}

}  // namespace ssim_gb
