// kernels_lbfgs.cu -- the L-BFGS two-loop recursion and curvature pair with every coefficient kept in device
// memory, so an L-BFGS iteration needs no host round trip until its line-search trial has been evaluated.
//
// The recursion is the textbook one (Nocedal & Wright, Algorithm 7.4): first loop a_i = rho_i s_i.q,
// q -= a_i y_i (newest pair first); z = H0 q; second loop b_i = rho_i y_i.z, z += (a_i - b_i) s_i (oldest
// first); d = -z.  Each pass kernel applies the previous step's update and forms the next step's dot in one
// sweep over the vectors; the last block to finish writes the coefficient, which the next launch reads.
#include "kernels.cuh"

namespace ssim_gb {
namespace {

constexpr int LB = 256;

// Per-vertex arithmetic is in S (FP32 in mixed precision: GB300's FP64 pipe is narrow, and a float<->double
// conversion costs an FP64 slot); partial sums go to FP64 at the warp level and the grid sums are FP64.
template <typename S>
__device__ __forceinline__ S dot3(const V4<S>& a, const V4<S>& b) {
  return a.x * b.x + a.y * b.y + a.z * b.z;
}

// vout = scale * (vin + c w), c = csign (cA - cB) read from device memory (w == null: no update; vin == null:
// the FP64 gradient g is the input); then out = rho * (a . vout) when a != null
template <typename S>
__global__ void __launch_bounds__(LB)
    lbfgs_pass_kernel(int nv, const V4<S>* vin, const double* __restrict__ g, V4<S>* vout, const V4<S>* __restrict__ w,
                      const double* __restrict__ cA, const double* __restrict__ cB, double csign,
                      const double* __restrict__ scale_ptr, double scale, const V4<S>* __restrict__ a, double rho,
                      double* __restrict__ out, Reduce red) {
  __shared__ double shred[LB / 32][1];
  const int u = blockIdx.x * LB + threadIdx.x;
  S part[1] = {S(0)};
  if (u < nv) {
    V4<S> x;
    if (vin != nullptr)
      x = vin[u];
    else
      x = mk4<S>((S)g[3 * u], (S)g[3 * u + 1], (S)g[3 * u + 2]);
    if (w != nullptr) {
      const S c = (S)(csign * (cA[0] - (cB != nullptr ? cB[0] : 0.0)));
      const V4<S> wv = w[u];
      x.x += c * wv.x;
      x.y += c * wv.y;
      x.z += c * wv.z;
    }
    const S sc = (S)(scale_ptr != nullptr ? scale_ptr[0] : scale);
    const V4<S> r = mk4<S>(sc * x.x, sc * x.y, sc * x.z);
    vout[u] = r;
    if (a != nullptr) part[0] = dot3<S>(a[u], r);
  }
  if (a == nullptr) return;
  double v1[1];
  block_sum_s<1, LB, S>(part, v1, shred);
  double tot[1];
  if (grid_sum_last<1, LB>(v1, red.partials, red.counter, tot)) out[0] = rho * tot[0];
}

// d = -(z + c w), g . d and |d|^2 into the scalars (c = cA - cB; w == null: none); d may be z
template <typename S>
__global__ void __launch_bounds__(LB)
    lbfgs_final_kernel(int nv, const V4<S>* z, const V4<S>* __restrict__ w, const double* __restrict__ cA,
                       const double* __restrict__ cB, const double* __restrict__ g, V4<S>* d, Reduce red) {
  __shared__ double shred[LB / 32][2];
  const int u = blockIdx.x * LB + threadIdx.x;
  S part[2] = {S(0), S(0)};
  if (u < nv) {
    V4<S> x = z[u];
    if (w != nullptr) {
      const S c = (S)(cA[0] - (cB != nullptr ? cB[0] : 0.0));
      const V4<S> wv = w[u];
      x.x += c * wv.x;
      x.y += c * wv.y;
      x.z += c * wv.z;
    }
    const V4<S> dv = mk4<S>(-x.x, -x.y, -x.z);
    d[u] = dv;
    const V4<S> gv = mk4<S>((S)g[3 * u], (S)g[3 * u + 1], (S)g[3 * u + 2]);
    part[0] = dot3<S>(gv, dv);
    part[1] = dot3<S>(dv, dv);
  }
  double v2[2];
  block_sum_s<2, LB, S>(part, v2, shred);
  double tot[2];
  if (grid_sum_last<2, LB>(v2, red.partials, red.counter, tot)) {
    red.sc->gd = tot[0];
    red.sc->dnorm2 = tot[1];
  }
}

// the curvature pair of a trial point: s = alpha d, y = g_new - g_old (differenced in FP64, then rounded);
// s . y and y . y into the scalars
template <typename S>
__global__ void __launch_bounds__(LB)
    lbfgs_pair_kernel(int nv, double alpha, const V4<S>* __restrict__ d, const double* __restrict__ gnew,
                      const double* __restrict__ gold, V4<S>* __restrict__ sv, V4<S>* __restrict__ yv, Reduce red) {
  __shared__ double shred[LB / 32][2];
  const int u = blockIdx.x * LB + threadIdx.x;
  S part[2] = {S(0), S(0)};
  if (u < nv) {
    const V4<S> dv = d[u];
    const S a = (S)alpha;
    const V4<S> s = mk4<S>(a * dv.x, a * dv.y, a * dv.z);
    const V4<S> y = mk4<S>((S)(gnew[3 * u] - gold[3 * u]), (S)(gnew[3 * u + 1] - gold[3 * u + 1]),
                           (S)(gnew[3 * u + 2] - gold[3 * u + 2]));
    sv[u] = s;
    yv[u] = y;
    part[0] = dot3<S>(s, y);
    part[1] = dot3<S>(y, y);
  }
  double v2[2];
  block_sum_s<2, LB, S>(part, v2, shred);
  double tot[2];
  if (grid_sum_last<2, LB>(v2, red.partials, red.counter, tot)) {
    red.sc->pair_sy = tot[0];
    red.sc->pair_yy = tot[1];
  }
}

// accept a step: u += alpha d (FP64 state), g_old = g_new
template <typename S>
__global__ void __launch_bounds__(LB)
    lbfgs_accept_kernel(int nv, double alpha, const V4<S>* __restrict__ d, double* __restrict__ u,
                        const double* __restrict__ gnew, double* __restrict__ gold) {
  const int v = blockIdx.x * LB + threadIdx.x;
  if (v >= nv) return;
  const V4<S> dv = d[v];
  u[3 * v] += alpha * (double)dv.x;
  u[3 * v + 1] += alpha * (double)dv.y;
  u[3 * v + 2] += alpha * (double)dv.z;
  gold[3 * v] = gnew[3 * v];
  gold[3 * v + 1] = gnew[3 * v + 1];
  gold[3 * v + 2] = gnew[3 * v + 2];
}

// ---------------------------------------------------------------- compact form
// The same L-BFGS matrix in the compact representation of Byrd, Nocedal & Schnabel (Math. Prog. 63, 1994;
// Nocedal & Wright eq. 7.24): H g = gamma g + S p - gamma Y q with q = R^-1 (S^T g) and
// p = R^-T ((D + gamma Y^T Y) q - gamma Y^T g), R the upper triangle of S^T Y in age order, D its diagonal.
// One pass forms S^T g, Y^T g and the newest pair's column of S^T Y and Y^T Y (all vectors read once); the
// last block solves the small triangular systems; a second pass forms d = -H g.

// per vertex: a_j = s_j.g, b_j = y_j.g, c_j = s_j.y_new, e_j = y_j.y_new (j in age order, oldest first);
// the last block keeps the new column in the slot-indexed S^T Y / Y^T Y tables and writes the coefficients
template <typename S>
__global__ void __launch_bounds__(LB)
    lbfgs_multidot_kernel(int nv, const double* __restrict__ g, LbfgsHist<S> h, double* __restrict__ partials,
                          double* __restrict__ tab, unsigned int* counter) {
  constexpr int NV = 4 * kLbfgsMaxCompact;
  static_assert(LB % NV == 0 && LB / NV <= LB / 32, "the last block's group sums reuse the warp-sum table");
  __shared__ double shred[LB / 32][NV];
  __shared__ double tot[NV];
  __shared__ bool am_last;
  S acc[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) acc[k] = S(0);
  // a grid of a few blocks per SM striding over the vertices: the block sums and the last block's sum
  // over the grid (NV values per block) stay short
  for (int u = blockIdx.x * LB + threadIdx.x; u < nv; u += gridDim.x * LB) {
    const V4<S> gv = mk4<S>((S)g[3 * u], (S)g[3 * u + 1], (S)g[3 * u + 2]);
    const V4<S> yn = h.y[h.n - 1][u];
#pragma unroll
    for (int j = 0; j < kLbfgsMaxCompact; ++j) {
      if (j < h.n) {
        const V4<S> sv = h.s[j][u], yv = h.y[j][u];
        acc[4 * j + 0] += dot3<S>(sv, gv);
        acc[4 * j + 1] += dot3<S>(yv, gv);
        acc[4 * j + 2] += dot3<S>(sv, yn);
        acc[4 * j + 3] += dot3<S>(yv, yn);
      }
    }
  }
  // block sums (FP32 within a warp, FP64 across warps), then the grid sum in FP64 by the last block
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    S x = acc[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) shred[warp][k] = (double)x;
  }
  __syncthreads();
  if (threadIdx.x < NV) {
    double b = 0;
#pragma unroll
    for (int w = 0; w < LB / 32; ++w) b += shred[w][threadIdx.x];
    partials[(size_t)blockIdx.x * NV + threadIdx.x] = b;
  }
  __syncthreads();  // orders the partials before thread 0's release
  if (threadIdx.x == 0) am_last = (atom_inc_acq_rel_gpu(counter) == gridDim.x - 1);
  __syncthreads();
  if (!am_last) return;
  {  // LB / NV groups of threads each sum every (LB / NV)-th block's partials, then the groups in order
    constexpr int G = LB / NV;
    const int k = threadIdx.x % NV, grp = threadIdx.x / NV;
    double t = 0;
    for (int b = grp; b < (int)gridDim.x; b += G) t += __ldcg(partials + (size_t)b * NV + k);
    shred[grp][k] = t;
    __syncthreads();
    if (threadIdx.x < NV) {
      double a = 0;
#pragma unroll
      for (int q = 0; q < G; ++q) a += shred[q][threadIdx.x];
      tot[threadIdx.x] = a;
    }
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  *counter = 0;
  // tables: tab[0 .. M*M) = S^T Y by slot (row s-slot, column y-slot), tab[M*M .. 2 M*M) = Y^T Y by slot;
  // coefficients written to tab[2 M*M ..): p (age order), q (age order), gamma
  constexpr int M = kLbfgsMaxCompact;
  double* SY = tab;
  double* YY = tab + M * M;
  double* out = tab + 2 * M * M;
  const int n = h.n, sn = h.slot[n - 1];
  for (int j = 0; j < n; ++j) {
    SY[h.slot[j] * M + sn] = tot[4 * j + 2];
    YY[h.slot[j] * M + sn] = tot[4 * j + 3];
    YY[sn * M + h.slot[j]] = tot[4 * j + 3];
  }
  const double gamma = SY[sn * M + sn] / YY[sn * M + sn];
  double q[M], p[M];
  for (int j = n - 1; j >= 0; --j) {  // R q = a, R[j][k] = s_j.y_k (k >= j)
    double r = tot[4 * j + 0];
    for (int k = j + 1; k < n; ++k) r -= SY[h.slot[j] * M + h.slot[k]] * q[k];
    q[j] = r / SY[h.slot[j] * M + h.slot[j]];
  }
  for (int j = 0; j < n; ++j) {  // t = (D + gamma Y^T Y) q - gamma b, then R^T p = t
    double t = SY[h.slot[j] * M + h.slot[j]] * q[j] - gamma * tot[4 * j + 1];
    for (int k = 0; k < n; ++k) t += gamma * YY[h.slot[j] * M + h.slot[k]] * q[k];
    for (int k = 0; k < j; ++k) t -= SY[h.slot[k] * M + h.slot[j]] * p[k];
    p[j] = t / SY[h.slot[j] * M + h.slot[j]];
  }
  for (int j = 0; j < n; ++j) {
    out[j] = p[j];
    out[M + j] = -gamma * q[j];
  }
  out[2 * M] = gamma;
}

// d = -(gamma g + sum_j p_j s_j + sum_j q'_j y_j) (coefficients from the multidot pass; gamma_host when
// h.n == 0), g . d and |d|^2 into the scalars
template <typename S>
__global__ void __launch_bounds__(LB)
    lbfgs_combine_kernel(int nv, const double* __restrict__ g, LbfgsHist<S> h, const double* __restrict__ coef,
                         double gamma_host, V4<S>* __restrict__ d, Reduce red) {
  constexpr int M = kLbfgsMaxCompact;
  __shared__ double shred[LB / 32][2];
  __shared__ S cs[2 * M + 1];
  if (threadIdx.x < 2 * M + 1) {
    const int k = threadIdx.x;
    const bool used = k == 2 * M || (k < M ? k < h.n : k - M < h.n);
    cs[k] = used ? (S)(k == 2 * M && h.n == 0 ? gamma_host : coef[k]) : S(0);
  }
  __syncthreads();
  const int u = blockIdx.x * LB + threadIdx.x;
  S part[2] = {S(0), S(0)};
  if (u < nv) {
    const V4<S> gv = mk4<S>((S)g[3 * u], (S)g[3 * u + 1], (S)g[3 * u + 2]);
    const S gm = cs[2 * M];
    S x = gm * gv.x, y = gm * gv.y, z = gm * gv.z;
#pragma unroll
    for (int j = 0; j < M; ++j) {
      if (j < h.n) {
        const V4<S> sv = h.s[j][u], yv = h.y[j][u];
        const S a = cs[j], b = cs[M + j];
        x += a * sv.x + b * yv.x;
        y += a * sv.y + b * yv.y;
        z += a * sv.z + b * yv.z;
      }
    }
    const V4<S> dv = mk4<S>(-x, -y, -z);
    d[u] = dv;
    part[0] = dot3<S>(gv, dv);
    part[1] = dot3<S>(dv, dv);
  }
  double v2[2];
  block_sum_s<2, LB, S>(part, v2, shred);
  double tot[2];
  if (grid_sum_last<2, LB>(v2, red.partials, red.counter, tot)) {
    red.sc->gd = tot[0];
    red.sc->dnorm2 = tot[1];
  }
}

}  // namespace

// 2 blocks per SM (each thread then sums several vertices in FP32 before the block sums)
int multidot_grid(int nv) {
  int dev = 0, nsm = 0;
  SSIM_CUDA(cudaGetDevice(&dev));
  SSIM_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  return std::max(1, std::min(div_up(nv, LB), 2 * std::max(nsm, 1)));
}

template <typename S>
void launch_lbfgs_multidot(int nv, const double* g, const LbfgsHist<S>& h, double* partials, double* tab,
                           unsigned int* counter, cudaStream_t st) {
  lbfgs_multidot_kernel<S><<<multidot_grid(nv), LB, 0, st>>>(nv, g, h, partials, tab, counter);
  after_launch("lbfgs_multidot");
}

template <typename S>
void launch_lbfgs_combine(int nv, const double* g, const LbfgsHist<S>& h, const double* coef, double gamma_host,
                          V4<S>* d, const Reduce& red, cudaStream_t st) {
  lbfgs_combine_kernel<S><<<div_up(nv, LB), LB, 0, st>>>(nv, g, h, coef, gamma_host, d, red);
  after_launch("lbfgs_combine");
}

int lbfgs_multidot_partials(int nv) { return div_up(nv, LB) * 4 * kLbfgsMaxCompact; }

template <typename S>
void launch_lbfgs_pass(int nv, const V4<S>* vin, const double* g, V4<S>* vout, const V4<S>* w, const double* cA,
                       const double* cB, double csign, const double* scale_ptr, double scale, const V4<S>* a,
                       double rho, double* out, const Reduce& red, cudaStream_t st) {
  lbfgs_pass_kernel<S><<<div_up(nv, LB), LB, 0, st>>>(nv, vin, g, vout, w, cA, cB, csign, scale_ptr, scale, a, rho,
                                                      out, red);
  after_launch("lbfgs_pass");
}

template <typename S>
void launch_lbfgs_final(int nv, const V4<S>* z, const V4<S>* w, const double* cA, const double* cB, const double* g,
                        V4<S>* d, const Reduce& red, cudaStream_t st) {
  lbfgs_final_kernel<S><<<div_up(nv, LB), LB, 0, st>>>(nv, z, w, cA, cB, g, d, red);
  after_launch("lbfgs_final");
}

template <typename S>
void launch_lbfgs_pair(int nv, double alpha, const V4<S>* d, const double* gnew, const double* gold, V4<S>* sv,
                       V4<S>* yv, const Reduce& red, cudaStream_t st) {
  lbfgs_pair_kernel<S><<<div_up(nv, LB), LB, 0, st>>>(nv, alpha, d, gnew, gold, sv, yv, red);
  after_launch("lbfgs_pair");
}

template <typename S>
void launch_lbfgs_accept(int nv, double alpha, const V4<S>* d, double* u, const double* gnew, double* gold,
                         cudaStream_t st) {
  lbfgs_accept_kernel<S><<<div_up(nv, LB), LB, 0, st>>>(nv, alpha, d, u, gnew, gold);
  after_launch("lbfgs_accept");
}

#define SSIM_LBFGS_INST(S)                                                                                         \
  template void launch_lbfgs_multidot<S>(int, const double*, const LbfgsHist<S>&, double*, double*, unsigned int*, \
                                         cudaStream_t);                                                           \
  template void launch_lbfgs_combine<S>(int, const double*, const LbfgsHist<S>&, const double*, double, V4<S>*,   \
                                        const Reduce&, cudaStream_t);                                             \
  template void launch_lbfgs_pass<S>(int, const V4<S>*, const double*, V4<S>*, const V4<S>*, const double*,       \
                                     const double*, double, const double*, double, const V4<S>*, double, double*, \
                                     const Reduce&, cudaStream_t);                                                \
  template void launch_lbfgs_final<S>(int, const V4<S>*, const V4<S>*, const double*, const double*,             \
                                      const double*, V4<S>*, const Reduce&, cudaStream_t);                        \
  template void launch_lbfgs_pair<S>(int, double, const V4<S>*, const double*, const double*, V4<S>*, V4<S>*,     \
                                     const Reduce&, cudaStream_t);                                                \
  template void launch_lbfgs_accept<S>(int, double, const V4<S>*, double*, const double*, double*, cudaStream_t);

SSIM_LBFGS_INST(float)
SSIM_LBFGS_INST(double)

}  // namespace ssim_gb
