// noalloc.cu -- an entry point that allocates no device memory: the incremental-potential value of a tet
// mesh from caller-owned device arrays, with the scratch of its grid reduction in a fixed device array of
// this library.
//
// Who needs it: callers that cannot call cudaMalloc -- code running under an allocator that owns all of the
// device memory it is given (a framework's caching allocator or a fixed memory budget set at start-up), or a
// loop that must not pay an allocation's latency or risk its failure once it is running.  They hand in
// every input and the output; this file brings the rest with it.
#include <cuda.h>  // CUcontext / CUresult types only: cuCtxGetCurrent is fetched through the runtime
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "../../include/ssim_gb.h"
#include "common.cuh"
#include "elem_math.cuh"

namespace ssim_gb {
namespace {

constexpr int NB = 128;  // threads per block, one tet per thread

// Scratch of the deterministic grid reduction: one partial sum per block, then the arrival counter.
// Every GPU that loads the library holds these 64 KiB until the process exits.
constexpr int kMaxBlocks = SSIM_GB_NOALLOC_MAX_CELLS / NB;
static __device__ __align__(256) double g_noalloc_scratch[kMaxBlocks + 32];

// Address of g_noalloc_scratch per device, with the CUDA context it was looked up in: a symbol's device
// address belongs to a context, so a call made in another context (a non-primary context, or the primary
// context re-created after cudaDeviceReset) looks it up again.
std::mutex g_mutex;
double* g_scratch_ptr[64] = {nullptr};
CUcontext g_scratch_ctx[64] = {nullptr};

typedef CUresult (*CtxGetCurrentFn)(CUcontext*);

// the calling thread's current context, or nullptr if the driver entry point is not available
CUcontext current_context() {
  static CtxGetCurrentFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      p = nullptr;
    }
    return reinterpret_cast<CtxGetCurrentFn>(p);
  }();
  CUcontext c = nullptr;
  if (fn == nullptr || fn(&c) != CUDA_SUCCESS) return nullptr;
  return c;
}

// The value-only variant of the element energy kernel (kernels_elem.cu, elem_energy_grad_kernel): same
// per-tet terms, the reference's AoS [T,3,3] Dm^-1 layout, and the reduction's partials and counter in the
// library's fixed scratch instead of memory of the time-step object.
__global__ void __launch_bounds__(NB)
    energy_noalloc_kernel(const double* __restrict__ X, const double* __restrict__ u, const double* __restrict__ xt,
                          const int4* __restrict__ cells, const double* __restrict__ dminv,
                          const double* __restrict__ vol, const double* __restrict__ lam_e,
                          const double* __restrict__ mu_e, int nt, double dt2, double rho, double* scratch,
                          double* out) {
  __shared__ double shred[NB / 32][1];
  const int e = blockIdx.x * NB + threadIdx.x;
  double energy = 0;
  if (e < nt) {
    const int4 c = cells[e];
    const int vid[4] = {c.x, c.y, c.z, c.w};
    double x[4][3], dd[4][3];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const double uk = u[vid[i] * 3 + k];
        x[i][k] = X[vid[i] * 3 + k] + uk;
        dd[i][k] = uk - xt[vid[i] * 3 + k];
      }
    double Dm[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) Dm[k] = dminv[9 * (size_t)e + k];
    double F[9];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int cc = 0; cc < 3; ++cc)
        F[r * 3 + cc] = (x[1][r] - x[0][r]) * Dm[0 * 3 + cc] + (x[2][r] - x[0][r]) * Dm[1 * 3 + cc] +
                        (x[3][r] - x[0][r]) * Dm[2 * 3 + cc];
    const double V = vol[e], lam = lam_e[e], mu = mu_e[e];
    const double m = rho * V * (1.0 / 20.0);
    double sd[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) sd[k] = dd[0][k] + dd[1][k] + dd[2][k] + dd[3][k];
    double q = sd[0] * sd[0] + sd[1] * sd[1] + sd[2] * sd[2];
#pragma unroll
    for (int i = 0; i < 4; ++i) q += dd[i][0] * dd[i][0] + dd[i][1] * dd[i][1] + dd[i][2] * dd[i][2];
    energy = dt2 * V * snh_energy<double>(F, lam, mu) + 0.5 * m * q;
  }
  double v1[1] = {energy};
  block_sum<1, NB>(v1, shred);
  double tot[1];
  unsigned int* counter = reinterpret_cast<unsigned int*>(scratch + kMaxBlocks);
  if (grid_sum_last<1, NB>(v1, scratch, counter, tot)) *out = tot[0];
}

}  // namespace
}  // namespace ssim_gb

extern "C" SSIM_GB_API ssim_gb_status ssim_gb_energy_noalloc(const double* X, const double* u, const double* x_tilde,
                                                            const int32_t* cells, const double* dminv,
                                                            const double* rest_volume, const double* lambda_,
                                                            const double* mu, int32_t num_cells, double time_step,
                                                            double density, void* stream, double* energy_out) {
  using namespace ssim_gb;
  auto fail = [](ssim_gb_status s, const std::string& msg) {
    set_global_error("ssim_gb_energy_noalloc: " + msg);
    return s;
  };
  if (!X || !u || !x_tilde || !cells || !dminv || !rest_volume || !lambda_ || !mu || !energy_out)
    return fail(SSIM_GB_ERR_INVALID_ARGUMENT, "null pointer");
  if (num_cells <= 0 || num_cells > SSIM_GB_NOALLOC_MAX_CELLS)
    return fail(SSIM_GB_ERR_INVALID_ARGUMENT, "num_cells = " + std::to_string(num_cells) +
                                                  " is outside 1.." + std::to_string(SSIM_GB_NOALLOC_MAX_CELLS) +
                                                  ", the size its fixed scratch serves");
  if (((uintptr_t)cells & 15) != 0) return fail(SSIM_GB_ERR_INVALID_ARGUMENT, "cells must be 16-byte aligned");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    cudaGetLastError();
    return fail(SSIM_GB_ERR_CUDA, "no usable CUDA device");
  }
  double* scratch = nullptr;
  {
    const CUcontext ctx = current_context();
    std::lock_guard<std::mutex> lock(g_mutex);
    if (g_scratch_ptr[dev] == nullptr || ctx == nullptr || ctx != g_scratch_ctx[dev]) {
      // first call on this device (or in this context): the device address of the fixed scratch array (host
      // code cannot use the symbol itself, which names a host-side stand-in).  Without the driver's context
      // query the lookup runs on every call.
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || p == nullptr) {
        cudaGetLastError();
        return fail(SSIM_GB_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      }
      g_scratch_ptr[dev] = static_cast<double*>(p);
      g_scratch_ctx[dev] = ctx;
    }
    scratch = g_scratch_ptr[dev];
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // the arrival counter must start at zero (each completed call leaves it at zero; clearing it here also
  // recovers from a call that did not complete)
  unsigned int* counter = reinterpret_cast<unsigned int*>(scratch + kMaxBlocks);
  const cudaError_t me = cudaMemsetAsync(counter, 0, sizeof(unsigned int), st);
  if (me != cudaSuccess) {
    cudaGetLastError();
    return fail(SSIM_GB_ERR_CUDA, std::string("clearing the scratch counter: ") + cudaGetErrorString(me));
  }
  const int grid = (num_cells + NB - 1) / NB;
  energy_noalloc_kernel<<<grid, NB, 0, st>>>(X, u, x_tilde, reinterpret_cast<const int4*>(cells), dminv, rest_volume,
                                             lambda_, mu, num_cells, time_step * time_step, density, scratch,
                                             energy_out);
  g_launches.fetch_add(1, std::memory_order_relaxed);
  const cudaError_t le = cudaGetLastError();
  if (le != cudaSuccess) return fail(SSIM_GB_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(le));
  return SSIM_GB_OK;
}
