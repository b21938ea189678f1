// kernels_fused.cu -- element Hessian and assembly in one pass (update_hessian, time_step.hpp:626-658): the
// element blocks are summed into the system matrix inside the CTA that owns their rows, so the per-element
// 12 x 12 blocks never go to memory.
#include "hessian_elem.cuh"

namespace ssim_gb {
namespace {

constexpr int FH = 128;          // threads per CTA = entries per chunk of a CTA's element list
constexpr int kMaxLocalSlots = 1024;

__device__ __forceinline__ size_t fused_sell_base(int q) { return (size_t)9 * (size_t)(q & ~31) + (size_t)(q & 31); }

// CTA b owns the block rows of slices [spc b, spc (b + 1)) and their upper slots [q0, q1).  It walks its
// element list (every element with an upper block in its rows; see FusedLists) in chunks of FH: each thread
// evaluates one element's K_e in registers, then the chunk adds its blocks to the CTA's slot accumulators in
// shared memory rank by rank (the rank of a block is the number of earlier entries of the chunk adding to
// the same slot, so no two threads write one slot in the same round and every slot sums its contributions
// in list order: deterministic, no atomics).  After the last chunk each slot adds the consistent mass,
// applies the Dirichlet identity filter (boundary.hpp:53-67) and is written once; the diagonal slots also
// write the block-Jacobi preconditioner rows.  Elements whose blocks fall in several CTAs' rows are
// evaluated by each of those CTAs.
// launch bounds: 4 CTAs per SM in FP32 (128 registers, 72 bytes of spills against 168 registers and 3 CTAs
// unconstrained), 2 in FP64
template <typename S, bool XF>
__global__ void __launch_bounds__(FH, sizeof(S) == 4 ? 4 : 2)
    fused_hessian_kernel(ElemFP64 e64, ElemFP32 e32, const double* __restrict__ X, const double* __restrict__ u,
                         const float4* __restrict__ xf, S dt2, int spsd, SellMatrix A, int nslices, int spc,
                         const int* __restrict__ fptr, const int* __restrict__ felem,
                         const uint16_t* __restrict__ fcode, const S* __restrict__ slot_mass,
                         const uint8_t* __restrict__ mask, int filter, S* __restrict__ vals,
                         V4<S>* __restrict__ dinv, int precond) {
  extern __shared__ __align__(16) unsigned char fused_smem[];
  S* acc = reinterpret_cast<S*>(fused_smem);  // [local slot][9]
  __shared__ int s_wmax[FH / 32];
  const int b = blockIdx.x;
  const int s0 = b * spc, s1 = min(nslices, s0 + spc);
  const int q0 = A.sl_off[s0], nloc = A.sl_off[s1] - q0;
  for (int i = threadIdx.x; i < 9 * nloc; i += FH) acc[i] = S(0);
  const int p0 = fptr[b], p1 = fptr[b + 1];
  __syncthreads();
  for (int c0 = p0; c0 < p1; c0 += FH) {
    const int idx = c0 + threadIdx.x;
    const bool active = idx < p1;
    S K[78];
    uint32_t code[10];
    int rounds = 0;
    if (active) {
      element_hessian_at<S, XF>(e64, e32, X, u, xf, dt2, spsd, felem[idx], K);
      // the ten 16-bit codes of the entry: five aligned 32-bit words
      const uint32_t* cw = reinterpret_cast<const uint32_t*>(fcode + 10 * (size_t)idx);
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        const uint32_t wd = cw[k];
        code[2 * k] = wd & 0xffffu;
        code[2 * k + 1] = wd >> 16;
      }
#pragma unroll
      for (int k = 0; k < 10; ++k)
        if (code[k] != 0xffffu) rounds = max(rounds, (int)(code[k] >> 11) + 1);
    }
    // rounds of this chunk: the block-wide maximum (the same in every thread)
    rounds = __reduce_max_sync(0xffffffffu, rounds);
    if ((threadIdx.x & 31) == 0) s_wmax[threadIdx.x >> 5] = rounds;
    __syncthreads();
#pragma unroll
    for (int w = 0; w < FH / 32; ++w) rounds = max(rounds, s_wmax[w]);
    for (int r = 0; r < rounds; ++r) {
      if (active) {
        int blk = 0;
#pragma unroll
        for (int v = 0; v < 4; ++v)
#pragma unroll
          for (int w = v; w < 4; ++w, ++blk) {
            const uint32_t cd = code[blk];
            if (cd != 0xffffu && (int)(cd >> 11) == r) {
              S* a = acc + 9 * (cd & 1023u);
              const bool tr = (cd >> 10) & 1u;
#pragma unroll
              for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) {
                  // block (v, w) entry (i, j) = K[3v + i][3w + j]; transposed: entry (i, j) = K[3v + j][3w + i]
                  // (both indices compile-time constants, so K stays in registers)
                  const int i0 = 3 * v + i, j0 = 3 * w + j, i1 = 3 * v + j, j1 = 3 * w + i;
                  const S vn = i0 <= j0 ? K[kup(i0, j0)] : K[kup(j0, i0)];
                  const S vt = i1 <= j1 ? K[kup(i1, j1)] : K[kup(j1, i1)];
                  a[3 * i + j] += tr ? vt : vn;
                }
            }
          }
      }
      __syncthreads();
    }
    __syncthreads();  // s_wmax is rewritten by the next chunk
  }
  for (int l = threadIdx.x; l < nloc; l += FH) {
    const int q = q0 + l;
    S m[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) m[k] = acc[9 * l + k];
    const int ur = A.slot_row[q];
    if (ur >= 0) {
      const S ms = slot_mass[q];
      m[0] += ms;
      m[4] += ms;
      m[8] += ms;
      const int wc = A.sl_col[q];
      if (filter) {
        const int mu_ = mask[ur], mw = mask[wc];
        if (mu_ | mw) {
#pragma unroll
          for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j)
              if (((mu_ >> i) & 1) || ((mw >> j) & 1)) m[i * 3 + j] = (ur == wc && i == j) ? S(1) : S(0);
        }
      }
      if (dinv != nullptr && ur == wc) precond_rows<S>(m, precond, dinv + 3 * (size_t)ur);
    }
    const size_t base = fused_sell_base(q);
#pragma unroll
    for (int k = 0; k < 9; ++k) vals[base + 32 * k] = m[k];
  }
}

}  // namespace

template <typename S>
void launch_fused_hessian(const ElemFP64& e64, const ElemFP32& e32, const double* X, const double* u,
                          const float4* xf, double dt2, bool spsd, const SellMatrix& A, int nslices, int spc,
                          int ncta, const int* fptr, const int* felem, const uint16_t* fcode, const S* slot_mass,
                          const uint8_t* mask, bool filter, S* vals, V4<S>* dinv, int precond, cudaStream_t st) {
  if (ncta <= 0) return;
  const size_t smem = (size_t)9 * kMaxLocalSlots * sizeof(S);
  const void* fn = xf != nullptr ? (const void*)fused_hessian_kernel<S, true> : (const void*)fused_hessian_kernel<S, false>;
  SSIM_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  if (xf != nullptr)
    fused_hessian_kernel<S, true><<<ncta, FH, smem, st>>>(e64, e32, X, u, xf, (S)dt2, spsd ? 1 : 0, A, nslices, spc,
                                                          fptr, felem, fcode, slot_mass, mask, filter ? 1 : 0, vals,
                                                          dinv, precond);
  else
    fused_hessian_kernel<S, false><<<ncta, FH, smem, st>>>(e64, e32, X, u, xf, (S)dt2, spsd ? 1 : 0, A, nslices, spc,
                                                           fptr, felem, fcode, slot_mass, mask, filter ? 1 : 0, vals,
                                                           dinv, precond);
  after_launch("fused_hessian");
}
template void launch_fused_hessian<float>(const ElemFP64&, const ElemFP32&, const double*, const double*,
                                          const float4*, double, bool, const SellMatrix&, int, int, int, const int*,
                                          const int*, const uint16_t*, const float*, const uint8_t*, bool, float*,
                                          float4*, int, cudaStream_t);
template void launch_fused_hessian<double>(const ElemFP64&, const ElemFP32&, const double*, const double*,
                                           const float4*, double, bool, const SellMatrix&, int, int, int, const int*,
                                           const int*, const uint16_t*, const double*, const uint8_t*, bool, double*,
                                           double4_32a*, int, cudaStream_t);

int fused_chunk() { return FH; }

}  // namespace ssim_gb
