// common.cuh -- shared device/host helpers of the GB300 FEM library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <stdexcept>
#include <string>

#include "errors.h"

namespace ssim_gb {

#define SSIM_CUDA(expr)                                                                             \
  do {                                                                                              \
    cudaError_t _e = (expr);                                                                        \
    if (_e != cudaSuccess) {                                                                        \
      if (_e == cudaErrorMemoryAllocation) throw std::bad_alloc();                                  \
      throw ::ssim_gb::cuda_error(std::string(#expr) + ": " + cudaGetErrorString(_e) + " at " +     \
                                  __FILE__ + ":" + std::to_string(__LINE__));                       \
    }                                                                                               \
  } while (0)

// every launch site calls this right after the <<<>>> so a launch error surfaces immediately and the
// process-wide launch counter stays exact
extern std::atomic<uint64_t> g_launches;
inline void after_launch(const char* what) {
  g_launches.fetch_add(1, std::memory_order_relaxed);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) throw cuda_error(std::string("launch of ") + what + ": " + cudaGetErrorString(e));
}

// ---------------------------------------------------------------- device vectors
template <typename T>
struct vec4 {};
template <>
struct vec4<float> {
  using type = float4;
};
template <>
struct vec4<double> {
  using type = double4_32a;  // 32-byte aligned: one 256-bit load per vertex
};

inline int div_up(long long a, long long b) { return (int)((a + b - 1) / b); }

// scalars shared by the reductions of one handle (device memory, one block per handle)
struct DevScalars {
  // gradient / energy
  double energy_elastic;  // dt^2 * sum V_e Psi_e  (+ inertia, see kernels)
  double energy;          // total incremental potential of the last evaluation
  double gnorm2;          // |g|^2 (Dirichlet dofs zeroed)
  double trial_energy;    // energy at u + alpha * d
  double energy_scale;    // sum of |energy terms| of the last evaluation (round-off scale)
  double trial_energy_scale;
  double gd;              // g . d
  double dnorm2;          // |d|^2
  double pair_sy, pair_yy;  // s . y and y . y of the L-BFGS pair formed at the last trial point
  // PCG
  double rz, rz_old, pq, rr, rr0, tol2;
  double alpha, beta;  // rz / pq and rz / rz_old, formed once by the reducing block
  double inv_rz, inv_alpha;  // 1 / rz and 1 / alpha of the last Chronopoulos-Gear step
  int32_t iters;
  int32_t done;
  int32_t status;  // 0 ok, 1 breakdown (pq <= 0), 2 non-finite residual
  int32_t wait_failed;  // set by a persistent kernel whose grid-barrier wait gave up
  double true_rr, true_bb;  // |b - K x|^2 on the FP32 values and |b|^2 after a solve on the FP16 copy
};

// Deterministic grid reduction: every block writes its partial sums, the last block to finish (found
// with a device-scope counter, the "threadFenceReduction" pattern of the CUDA samples) adds the
// partials in block order and calls the epilogue.  No floating-point atomics: bitwise reproducible.
template <int NV>
struct BlockPartials {
  double v[NV];
};

template <int NV, int BLOCK>
__device__ __forceinline__ void block_sum(double (&vals)[NV], double (*sh)[NV]) {
  // warp reduce then shared reduce; result valid in thread 0
  // the NV sums advance level by level together, so their FP64 latency chains overlap (FP64 latency is
  // long on GB300); each sum's order of additions is that of a per-value tree
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int k = 0; k < NV; ++k) vals[k] += __shfl_down_sync(0xffffffffu, vals[k], o);
  }
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) sh[warp][k] = vals[k];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) s[k] = 0;
#pragma unroll
    for (int w = 0; w < BLOCK / 32; ++w) {
#pragma unroll
      for (int k = 0; k < NV; ++k) s[k] += sh[w][k];
    }
#pragma unroll
    for (int k = 0; k < NV; ++k) vals[k] = s[k];
  }
}

// Block sum of per-thread values of type S: the warp-level tree runs in S (FP32 on the mixed path, so the
// scarce FP64 pipe is not used per element), each warp's sum is widened to FP64 and the warps are added in
// FP64 in a fixed order.  Result (FP64) valid in thread 0.
template <int NV, int BLOCK, typename S>
__device__ __forceinline__ void block_sum_s(const S (&vals)[NV], double (&out)[NV], double (*sh)[NV]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  S x[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) x[k] = vals[k];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int k = 0; k < NV; ++k) x[k] += __shfl_down_sync(0xffffffffu, x[k], o);
  }
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) sh[warp][k] = (double)x[k];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) s[k] = 0;
#pragma unroll
    for (int w = 0; w < BLOCK / 32; ++w) {
#pragma unroll
      for (int k = 0; k < NV; ++k) s[k] += sh[w][k];
    }
#pragma unroll
    for (int k = 0; k < NV; ++k) out[k] = s[k];
  }
}

// Fixed-order tree sums of per-256-row partials (the PCG dots): partials are grouped 32 at a time (group g =
// parts 32g..32g+31); a group is summed by one warp's shuffle tree, and the group sums by the same tree in
// chunks of 32, chunks added in order.  The order depends only on the number of parts, so the distributed
// version in the persistent PCG (each group summed by whichever block completes it) and the single-block
// version below give identical bits.  Results in lane 0.
template <int NV>
__device__ __forceinline__ void warp_group_sum(const double* parts, int base, int count, double (&v)[NV]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int k = 0; k < NV; ++k) v[k] = lane < count ? __ldcg(parts + (size_t)(base + lane) * NV + k) : 0.0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
  }
}

template <int NV>
__device__ __forceinline__ void warp_top_sum(const double* gsums, int ngroups, double (&tot)[NV]) {
#pragma unroll
  for (int k = 0; k < NV; ++k) tot[k] = 0.0;
  for (int c0 = 0; c0 < ngroups; c0 += 32) {
    double v[NV];
    warp_group_sum<NV>(gsums, c0, min(32, ngroups - c0), v);
#pragma unroll
    for (int k = 0; k < NV; ++k) tot[k] += v[k];
  }
}

// one block's arrival at the end-of-kernel reductions: an acquire-release atomic at GPU scope publishes the
// block's partials (release) and lets the last arrival see every earlier block's (acquire; the atomics on
// the counter chain them), with no separate fences
__device__ __forceinline__ unsigned int atom_inc_acq_rel_gpu(unsigned int* p) {
  unsigned int old;
  asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], 1;" : "=r"(old) : "l"(p) : "memory");
  return old;
}

// grid_sum_last with the tree order above: the last block's warps sum the groups (group sums in gscratch,
// ceil(grid / 32) * NV doubles), then warp 0 the group sums.  true in thread 0 of the last block.
template <int NV, int BLOCK>
__device__ __forceinline__ bool grid_sum_last_tree(const double (&blockval)[NV], double* partials, double* gscratch,
                                                   unsigned int* counter, double (&tot)[NV]) {
  __shared__ bool am_last;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) partials[blockIdx.x * NV + k] = blockval[k];
    am_last = (atom_inc_acq_rel_gpu(counter) == gridDim.x - 1);
  }
  __syncthreads();
  if (!am_last) return false;
  const int nparts = (int)gridDim.x, ngroups = (nparts + 31) / 32, warp = threadIdx.x >> 5;
  for (int g = warp; g < ngroups; g += BLOCK / 32) {
    double v[NV];
    warp_group_sum<NV>(partials, 32 * g, min(32, nparts - 32 * g), v);
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
      for (int k = 0; k < NV; ++k) gscratch[g * NV + k] = v[k];
    }
  }
  __syncthreads();
  if (warp == 0) {
    warp_top_sum<NV>(gscratch, ngroups, tot);
    if (threadIdx.x == 0) {
      *counter = 0;  // ready for the next launch on this stream
      __threadfence();
      return true;
    }
  }
  return false;
}

// returns true in exactly one thread (thread 0 of the last block), with tot[] = sum of all partials.
// The last block reads the partials with every thread at once (L2-coherent loads) and combines them in a
// fixed order, so the result depends only on the grid and block sizes.
template <int NV, int BLOCK>
__device__ __forceinline__ bool grid_sum_last(const double (&blockval)[NV], double* partials, unsigned int* counter,
                                              double (&tot)[NV]) {
  __shared__ bool am_last;
  __shared__ double sh[BLOCK / 32][NV];
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) partials[blockIdx.x * NV + k] = blockval[k];
    am_last = (atom_inc_acq_rel_gpu(counter) == gridDim.x - 1);
  }
  __syncthreads();
  if (!am_last) return false;
  double acc[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) acc[k] = 0;
  // four partials per value in flight at once, added in the same order as one at a time
  const int nparts = (int)gridDim.x;
  for (int b0 = threadIdx.x; b0 < nparts; b0 += 4 * BLOCK) {
    double v[4][NV];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int b = b0 + j * BLOCK;
#pragma unroll
      for (int k = 0; k < NV; ++k) v[j][k] = b < nparts ? __ldcg(partials + b * NV + k) : 0.0;
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if (b0 + j * BLOCK < nparts) {
#pragma unroll
        for (int k = 0; k < NV; ++k) acc[k] += v[j][k];
      }
    }
  }
  block_sum<NV, BLOCK>(acc, sh);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) tot[k] = acc[k];
    *counter = 0;  // ready for the next launch on this stream
    __threadfence();
    return true;
  }
  return false;
}

}  // namespace ssim_gb
