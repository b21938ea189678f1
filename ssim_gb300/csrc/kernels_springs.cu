// kernels_springs.cu -- mass-spring systems (cloth) through the same time-step machinery as the tets:
// energy 1/2 |x - x~|^2_M + dt^2 sum_s k_s / 2 (|x_i - x_j| - L_s)^2 with a lumped (diagonal) mass.  There
// is no spring model in the reference; this is the classic mass-spring energy the projective-dynamics
// literature uses (Liu et al., "Fast Simulation of Mass-Spring Systems", SIGGRAPH Asia 2013).
//
// Springs are 2-vertex cells: the vertex gather, the block pattern, the atomic-free assembly and the
// PCG are the tet ones; the spring forces go to lf[s][2][3], the Hessian blocks to Kbuf[s][3][9] (upper
// vertex blocks (0,0), (0,1), (1,1)).
#include "kernels.cuh"

namespace ssim_gb {
namespace {

constexpr int PB = 256;

template <typename S>
__device__ __forceinline__ S comp4(const V4<S>& v, int k) {
  return k == 0 ? v.x : (k == 1 ? v.y : v.z);
}

// edge vector x_i - x_j = (X_i - X_j) + (u_i - u_j) (+ alpha (d_i - d_j)), from differences so a short
// spring keeps its digits
template <typename SD, bool TRIAL>
__device__ __forceinline__ void edge_vec(const SpringData& sp, const double* __restrict__ u, const V4<SD>* d,
                                         double alpha, int s, int& i, int& j, double (&e)[3]) {
  const int2 c = sp.ends[s];
  i = c.x;
  j = c.y;
  V4<SD> di, dj;
  if (TRIAL) {
    di = d[i];
    dj = d[j];
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    double v = (sp.X[3 * i + k] - sp.X[3 * j + k]) + (u[3 * i + k] - u[3 * j + k]);
    if (TRIAL) v += alpha * ((double)comp4<SD>(di, k) - (double)comp4<SD>(dj, k));
    e[k] = v;
  }
}

// FP64 spring pass.  FP64 arithmetic is scarce on GB300, so the pass spends it where the digits matter:
// the edge vector, |e|, l - L, the energy and the forces (one rsqrt gives both l = |e|^2 rsqrt and the
// force factor's 1/l); the trial direction's difference d_i - d_j is formed in the direction's own type,
// and the energy's term magnitude (used only as the round-off scale of the line search) in FP32.
template <typename SD, bool FORCES, bool TRIAL>
__global__ void __launch_bounds__(PB)
    spring_energy_grad_kernel(SpringData sp, const double* __restrict__ u, const V4<SD>* __restrict__ d,
                              double alpha, double dt2, double* __restrict__ lf, Reduce red) {
  __shared__ double shred[PB / 32][1];
  __shared__ double shred2[PB / 32][1];
  const int s = blockIdx.x * PB + threadIdx.x;
  double energy[1] = {0.0};
  float escale[1] = {0.f};
  if (s < sp.ns) {
    const int2 c = sp.ends[s];
    const int i = c.x, j = c.y;
    double e[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) e[k] = (sp.X[3 * i + k] - sp.X[3 * j + k]) + (u[3 * i + k] - u[3 * j + k]);
    if (TRIAL) {
      const V4<SD> di = d[i], dj = d[j];
      e[0] += alpha * (double)(di.x - dj.x);
      e[1] += alpha * (double)(di.y - dj.y);
      e[2] += alpha * (double)(di.z - dj.z);
    }
    const double l2 = e[0] * e[0] + e[1] * e[1] + e[2] * e[2];
    const double rl = l2 > 0.0 ? rsqrt(l2) : 0.0;
    const double l = l2 * rl;
    const double L = sp.rest[s], kk = dt2 * sp.k[s];
    const double dl = l - L;
    energy[0] = 0.5 * kk * dl * dl;
    escale[0] = 0.5f * (float)kk * ((float)l2 + (float)L * (float)L);
    if (FORCES) {
      const double cf = kk * dl * rl;
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        lf[(size_t)s * 6 + q] = cf * e[q];
        lf[(size_t)s * 6 + 3 + q] = -cf * e[q];
      }
    }
  }
  block_sum<1, PB>(energy, shred);
  double sc1[1];
  block_sum_s<1, PB, float>(escale, sc1, shred2);
  double v2[2] = {energy[0], sc1[0]};
  double tot[2];
  if (grid_sum_last<2, PB>(v2, red.partials, red.counter, tot)) {
    if (TRIAL) {
      red.sc->trial_energy = tot[0];
      red.sc->trial_energy_scale = tot[1];
    } else {
      red.sc->energy = tot[0];
      red.sc->energy_scale = tot[1];
    }
  }
}

// FP32 spring pass.  The displacement difference D = (u_i - u_j) (+ alpha (d_i - d_j)) is formed in FP32
// from the per-vertex split u = hi + lo as (hi_i - hi_j) + (lo_i - lo_j), rounding relative to D itself;
// with E0 the rest edge, e = E0 + D and l^2 - L^2 = 2 E0.D + D.D, so l - L = (l^2 - L^2) / (l + L)
// carries FP32 rounding relative to the stretch itself rather than to the length (a direct FP32 |e| - L
// would lose the stretch of a stiff spring to cancellation).  Forces f_s = dt^2 k (l - L) / l e go to
// lf32[s] (vertex i gets +f_s, vertex j -f_s).
template <typename SD, bool FORCES, bool TRIAL>
__global__ void __launch_bounds__(PB)
    spring_energy_grad32_kernel(SpringData sp, Split32 s3, const V4<SD>* __restrict__ d, double alpha, float dt2,
                                float4* __restrict__ lf32, Reduce red) {
  __shared__ double shred[PB / 32][2];
  const int s = blockIdx.x * PB + threadIdx.x;
  float part[2] = {0.f, 0.f};
  if (s < sp.ns) {
    const int2 c = sp.ends[s];
    const float4 e0 = sp.e0[s];
    const float4 hi = s3.uh[c.x], hj = s3.uh[c.y], li = s3.ul[c.x], lj = s3.ul[c.y];
    float D[3] = {(hi.x - hj.x) + (li.x - lj.x), (hi.y - hj.y) + (li.y - lj.y), (hi.z - hj.z) + (li.z - lj.z)};
    if (TRIAL) {
      const V4<SD> di = d[c.x], dj = d[c.y];
      const float a = (float)alpha;
      D[0] += a * (float)(di.x - dj.x);
      D[1] += a * (float)(di.y - dj.y);
      D[2] += a * (float)(di.z - dj.z);
    }
    const float ex = e0.x + D[0], ey = e0.y + D[1], ez = e0.z + D[2];
    const float L = e0.w, l2 = ex * ex + ey * ey + ez * ez;
    const float l = sqrtf(l2);
    const float dl2 = 2.f * (e0.x * D[0] + e0.y * D[1] + e0.z * D[2]) + (D[0] * D[0] + D[1] * D[1] + D[2] * D[2]);
    const float dl = dl2 / (l + L);
    const float kk = dt2 * sp.k32[s];
    part[0] = 0.5f * kk * dl * dl;
    part[1] = 0.5f * kk * (l2 + L * L);
    if (FORCES) {
      const float cf = l > 0.f ? kk * dl / l : 0.f;
      lf32[s] = make_float4(cf * ex, cf * ey, cf * ez, 0.f);
    }
  }
  double v2[2];
  block_sum_s<2, PB, float>(part, v2, shred);
  double tot[2];
  if (grid_sum_last<2, PB>(v2, red.partials, red.counter, tot)) {
    if (TRIAL) {
      red.sc->trial_energy = tot[0];
      red.sc->trial_energy_scale = tot[1];
    } else {
      red.sc->energy = tot[0];
      red.sc->energy_scale = tot[1];
    }
  }
}

// g_v from the FP32 spring forces (summed in FP32 over the incident springs) + m_v (u_v (+ alpha d_v) - x~_v)
// in FP64, Dirichlet dofs zeroed; |g|^2
template <typename SD>
__global__ void __launch_bounds__(PB)
    spring_gather32_kernel(int nv, const int* __restrict__ vptr, const int* __restrict__ vinc,
                           const float4* __restrict__ lf32, const double* __restrict__ m, const double* __restrict__ u,
                           const V4<SD>* __restrict__ d, double alpha, const double* __restrict__ xt,
                           const uint8_t* __restrict__ mask, double* __restrict__ g, Reduce red) {
  __shared__ double shred[PB / 32][1];
  const int v = blockIdx.x * PB + threadIdx.x;
  double part = 0;
  if (v < nv) {
    float a[3] = {0.f, 0.f, 0.f};
    const int k1 = vptr[v + 1];
    for (int k = vptr[v]; k < k1; ++k) {
      const int code = vinc[k];
      const float4 f = lf32[code >> 1];
      const float sg = (code & 1) ? -1.f : 1.f;
      a[0] += sg * f.x;
      a[1] += sg * f.y;
      a[2] += sg * f.z;
    }
    double dv[3] = {0, 0, 0};
    if (d != nullptr) {
      const V4<SD> t = d[v];
      dv[0] = alpha * (double)t.x;
      dv[1] = alpha * (double)t.y;
      dv[2] = alpha * (double)t.z;
    }
    const uint8_t mk = mask[v];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      double gq = (double)a[q] + m[v] * ((u[3 * v + q] - xt[3 * v + q]) + dv[q]);
      if ((mk >> q) & 1) gq = 0;
      g[3 * v + q] = gq;
      part += gq * gq;
    }
  }
  double v1[1] = {part};
  block_sum<1, PB>(v1, shred);
  double tot[1];
  if (grid_sum_last<1, PB>(v1, red.partials, red.counter, tot)) red.sc->gnorm2 = tot[0];
}

// lumped inertia 1/2 sum_v m_v |u_v (+ alpha d_v) - x~_v|^2, added to the (trial) energy and its scale
template <typename SD, bool TRIAL>
__global__ void __launch_bounds__(PB)
    lumped_inertia_energy_kernel(int nv, const double* __restrict__ m, const double* __restrict__ u,
                                 const double* __restrict__ xt, const V4<SD>* __restrict__ d, double alpha,
                                 Reduce red) {
  __shared__ double shred[PB / 32][1];
  const int v = blockIdx.x * PB + threadIdx.x;
  double part = 0;
  if (v < nv) {
    V4<SD> dv;
    if (TRIAL) dv = d[v];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      double w = u[3 * v + k] - xt[3 * v + k];
      if (TRIAL) w += alpha * (double)comp4<SD>(dv, k);
      part += w * w;
    }
    part *= 0.5 * m[v];
  }
  double v1[1] = {part};
  block_sum<1, PB>(v1, shred);
  double tot[1];
  if (grid_sum_last<1, PB>(v1, red.partials, red.counter, tot)) {
    if (TRIAL) {
      red.sc->trial_energy += tot[0];
      red.sc->trial_energy_scale += tot[0];
    } else {
      red.sc->energy += tot[0];
      red.sc->energy_scale += tot[0];
    }
  }
}

// g_v = sum of the incident spring forces + m_v (u_v (+ alpha d_v) - x~_v), Dirichlet dofs zeroed; |g|^2.
// With d the springs' forces must be those of the same trial point u + alpha d.
template <typename SD>
__global__ void __launch_bounds__(PB)
    spring_gather_kernel(int nv, const int* __restrict__ vptr, const int* __restrict__ vinc,
                         const double* __restrict__ lf, const double* __restrict__ m, const double* __restrict__ u,
                         const V4<SD>* __restrict__ d, double alpha, const double* __restrict__ xt,
                         const uint8_t* __restrict__ mask, double* __restrict__ g, Reduce red) {
  __shared__ double shred[PB / 32][1];
  const int v = blockIdx.x * PB + threadIdx.x;
  double part = 0;
  if (v < nv) {
    double a[3] = {0, 0, 0};
    const int k1 = vptr[v + 1];
    for (int k = vptr[v]; k < k1; ++k) {
      const double* s = lf + (size_t)vinc[k] * 3;
      a[0] += s[0];
      a[1] += s[1];
      a[2] += s[2];
    }
    const uint8_t mk = mask[v];
    double dv[3] = {0, 0, 0};
    if (d != nullptr) {
      const V4<SD> t = d[v];
      dv[0] = alpha * (double)t.x;
      dv[1] = alpha * (double)t.y;
      dv[2] = alpha * (double)t.z;
    }
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      a[q] += m[v] * ((u[3 * v + q] - xt[3 * v + q]) + dv[q]);
      if ((mk >> q) & 1) a[q] = 0;
      g[3 * v + q] = a[q];
      part += a[q] * a[q];
    }
  }
  double v1[1] = {part};
  block_sum<1, PB>(v1, shred);
  double tot[1];
  if (grid_sum_last<1, PB>(v1, red.partials, red.counter, tot)) red.sc->gnorm2 = tot[0];
}

// Hessian blocks of a spring: K = dt^2 k [n n^T + c (I - n n^T)], c = 1 - L / l, with c clamped to >= 0
// when make_spsd (the compressed spring's negative transverse stiffness removed, the standard projection of
// a spring Hessian); upper vertex blocks (0,0) = K, (0,1) = -K, (1,1) = K.
template <typename S>
__global__ void __launch_bounds__(PB)
    spring_hessian_kernel(SpringData sp, const double* __restrict__ u, double dt2, int spsd, S* __restrict__ Kbuf) {
  const int s = blockIdx.x * PB + threadIdx.x;
  if (s >= sp.ns) return;
  int i, j;
  double e[3];
  edge_vec<S, false>(sp, u, nullptr, 0.0, s, i, j, e);
  const double l = sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
  const double L = sp.rest[s], k = sp.k[s];
  double c = l > 0 ? 1.0 - L / l : 0.0;
  if (spsd) c = fmax(c, 0.0);
  double n[3] = {0, 0, 0};
  if (l > 0)
#pragma unroll
    for (int q = 0; q < 3; ++q) n[q] = e[q] / l;
  S K[9];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b)
      K[a * 3 + b] = (S)(dt2 * k * ((1.0 - c) * n[a] * n[b] + (a == b ? c : 0.0)));
  S* o = Kbuf + (size_t)s * 27;
#pragma unroll
  for (int q = 0; q < 9; ++q) {
    o[q] = K[q];
    o[9 + q] = -K[q];
    o[18 + q] = K[q];
  }
}

}  // namespace

template <typename SD>
void launch_spring_energy_grad(const SpringData& sp, const double* u, const double* xt, const double* m, int nv,
                               const V4<SD>* d, double alpha, double dt2, double* lf, bool with_forces, bool trial,
                               const Reduce& red, cudaStream_t st) {
  if (sp.ns > 0) {
    const int grid = div_up(sp.ns, PB);
    if (trial && with_forces)
      spring_energy_grad_kernel<SD, true, true><<<grid, PB, 0, st>>>(sp, u, d, alpha, dt2, lf, red);
    else if (trial)
      spring_energy_grad_kernel<SD, false, true><<<grid, PB, 0, st>>>(sp, u, d, alpha, dt2, lf, red);
    else if (with_forces)
      spring_energy_grad_kernel<SD, true, false><<<grid, PB, 0, st>>>(sp, u, d, alpha, dt2, lf, red);
    else
      spring_energy_grad_kernel<SD, false, false><<<grid, PB, 0, st>>>(sp, u, d, alpha, dt2, lf, red);
    after_launch("spring_energy_grad");
  }
  if (trial)
    lumped_inertia_energy_kernel<SD, true><<<div_up(nv, PB), PB, 0, st>>>(nv, m, u, xt, d, alpha, red);
  else
    lumped_inertia_energy_kernel<SD, false><<<div_up(nv, PB), PB, 0, st>>>(nv, m, u, xt, d, alpha, red);
  after_launch("lumped_inertia_energy");
}

template <typename SD>
void launch_spring_gather(int nv, const int* vptr, const int* vinc, const double* lf, const double* m,
                          const double* u, const V4<SD>* d, double alpha, const double* xt, const uint8_t* mask,
                          double* g, const Reduce& red, cudaStream_t st) {
  spring_gather_kernel<SD><<<div_up(nv, PB), PB, 0, st>>>(nv, vptr, vinc, lf, m, u, d, alpha, xt, mask, g, red);
  after_launch("spring_gather");
}

template <typename SD>
void launch_spring_energy_grad32(const SpringData& sp, const Split32& s3, const double* u, const double* xt,
                                 const double* m, int nv, const V4<SD>* d, double alpha, double dt2, float4* lf32,
                                 bool with_forces, bool trial, const Reduce& red, cudaStream_t st) {
  if (sp.ns > 0) {
    const int grid = div_up(sp.ns, PB);
    const float f2 = (float)dt2;
    if (trial && with_forces)
      spring_energy_grad32_kernel<SD, true, true><<<grid, PB, 0, st>>>(sp, s3, d, alpha, f2, lf32, red);
    else if (trial)
      spring_energy_grad32_kernel<SD, false, true><<<grid, PB, 0, st>>>(sp, s3, d, alpha, f2, lf32, red);
    else if (with_forces)
      spring_energy_grad32_kernel<SD, true, false><<<grid, PB, 0, st>>>(sp, s3, d, alpha, f2, lf32, red);
    else
      spring_energy_grad32_kernel<SD, false, false><<<grid, PB, 0, st>>>(sp, s3, d, alpha, f2, lf32, red);
    after_launch("spring_energy_grad32");
  }
  if (trial)
    lumped_inertia_energy_kernel<SD, true><<<div_up(nv, PB), PB, 0, st>>>(nv, m, u, xt, d, alpha, red);
  else
    lumped_inertia_energy_kernel<SD, false><<<div_up(nv, PB), PB, 0, st>>>(nv, m, u, xt, d, alpha, red);
  after_launch("lumped_inertia_energy");
}

template <typename SD>
void launch_spring_gather32(int nv, const int* vptr, const int* vinc, const float4* lf32, const double* m,
                            const double* u, const V4<SD>* d, double alpha, const double* xt, const uint8_t* mask,
                            double* g, const Reduce& red, cudaStream_t st) {
  spring_gather32_kernel<SD><<<div_up(nv, PB), PB, 0, st>>>(nv, vptr, vinc, lf32, m, u, d, alpha, xt, mask, g, red);
  after_launch("spring_gather32");
}

template <typename S>
void launch_spring_hessian(const SpringData& sp, const double* u, double dt2, bool spsd, S* Kbuf, cudaStream_t st) {
  if (sp.ns <= 0) return;
  spring_hessian_kernel<S><<<div_up(sp.ns, PB), PB, 0, st>>>(sp, u, dt2, spsd ? 1 : 0, Kbuf);
  after_launch("spring_hessian");
}

template void launch_spring_energy_grad<float>(const SpringData&, const double*, const double*, const double*, int,
                                               const float4*, double, double, double*, bool, bool, const Reduce&,
                                               cudaStream_t);
template void launch_spring_energy_grad<double>(const SpringData&, const double*, const double*, const double*, int,
                                                const double4_32a*, double, double, double*, bool, bool,
                                                const Reduce&, cudaStream_t);
template void launch_spring_gather<float>(int, const int*, const int*, const double*, const double*, const double*,
                                          const float4*, double, const double*, const uint8_t*, double*,
                                          const Reduce&, cudaStream_t);
template void launch_spring_gather<double>(int, const int*, const int*, const double*, const double*, const double*,
                                           const double4_32a*, double, const double*, const uint8_t*, double*,
                                           const Reduce&, cudaStream_t);
template void launch_spring_energy_grad32<float>(const SpringData&, const Split32&, const double*, const double*,
                                                 const double*, int, const float4*, double, double, float4*, bool,
                                                 bool, const Reduce&, cudaStream_t);
template void launch_spring_gather32<float>(int, const int*, const int*, const float4*, const double*,
                                            const double*, const float4*, double, const double*, const uint8_t*,
                                            double*, const Reduce&, cudaStream_t);
template void launch_spring_hessian<float>(const SpringData&, const double*, double, bool, float*, cudaStream_t);
template void launch_spring_hessian<double>(const SpringData&, const double*, double, bool, double*, cudaStream_t);

}  // namespace ssim_gb
