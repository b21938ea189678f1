// kernels_sparse.cu -- CSR/SELL assembly, SpMV, the fused Jacobi-PCG and the state-update vector kernels.
#include <algorithm>

#include <cuda_fp16.h>

#include "kernels.cuh"

namespace ssim_gb {
namespace {

constexpr int SB = 256;  // block of the slot / row / dof kernels (a multiple of the 32-row slice)


__device__ __forceinline__ size_t sell_base(int q) { return (size_t)9 * (size_t)(q & ~31) + (size_t)(q & 31); }

// Assembly (update_hessian, time_step.hpp:631-657): each upper slot (one 3x3 vertex-pair block of the
// symmetric matrix) adds its precomputed list of element blocks (global_composer.hpp:103-119 builds the
// same map entry by entry) to the consistent-mass block, then applies the Dirichlet identity filter
// (boundary.hpp:53-67).  One thread per slot, no atomics: deterministic.
// one element block in the FP16 form of launch_elem_hessian16: three 8-byte words, nine FP16 values and the
// power-of-two exponent k in word 9; value = half * 2^k (exact in FP32)
__device__ __forceinline__ void load_block16(const uint2* __restrict__ K16, int blk, float (&kv)[9]) {
  const uint2* p = K16 + 3 * (size_t)blk;
  const uint2 w0 = p[0], w1 = p[1], w2 = p[2];
  const unsigned int u[6] = {w0.x, w0.y, w1.x, w1.y, w2.x, w2.y};
  const int k = (int)(short)(unsigned short)(u[4] >> 16);
  const float sc = __int_as_float((127 + k) << 23);
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    const unsigned short h = (unsigned short)((u[i >> 1] >> (16 * (i & 1))) & 0xffffu);
    kv[i] = __half2float(__ushort_as_half(h)) * sc;
  }
}

template <typename S, int B, bool H16 = false>
__global__ void __launch_bounds__(B)
    assemble_kernel(SellMatrix A, const int* __restrict__ cptr, const int* __restrict__ csrc,
                    const S* __restrict__ Kbuf, const S* __restrict__ slot_mass, const uint8_t* __restrict__ mask,
                    int filter, S* __restrict__ vals, V4<S>* __restrict__ dinv, int precond) {
  const int q = blockIdx.x * B + threadIdx.x;
  if (q >= A.nslots) return;
  S acc[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) acc[i] = S(0);
  if constexpr (H16) {
    const uint2* K16 = reinterpret_cast<const uint2*>(Kbuf);
    const int c1 = cptr[q + 1];
    int c = cptr[q];
    auto add16 = [&](int code, const float (&kv)[9]) {
      if (code >= 0) {
#pragma unroll
        for (int i = 0; i < 9; ++i) acc[i] += kv[i];
      } else {
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
          for (int b = 0; b < 3; ++b) acc[a * 3 + b] += kv[b * 3 + a];
      }
    };
    for (; c + 2 <= c1; c += 2) {
      const int code0 = csrc[c], code1 = csrc[c + 1];
      float kv0[9], kv1[9];
      load_block16(K16, code0 & 0x7fffffff, kv0);
      load_block16(K16, code1 & 0x7fffffff, kv1);
      add16(code0, kv0);
      add16(code1, kv1);
    }
    if (c < c1) {
      const int code = csrc[c];
      float kv[9];
      load_block16(K16, code & 0x7fffffff, kv);
      add16(code, kv);
    }
  } else if (Kbuf != nullptr) {
    // contributions in pairs: 18 independent block loads in flight per thread (the gathers are latency-bound)
    auto add = [&](int code, const S (&kv)[9]) {
      if (code >= 0) {
#pragma unroll
        for (int i = 0; i < 9; ++i) acc[i] += kv[i];
      } else {
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
          for (int b = 0; b < 3; ++b) acc[a * 3 + b] += kv[b * 3 + a];
      }
    };
    const int c1 = cptr[q + 1];
    int c = cptr[q];
    for (; c + 2 <= c1; c += 2) {
      const int code0 = csrc[c], code1 = csrc[c + 1];
      const S* k0 = Kbuf + (size_t)(code0 & 0x7fffffff) * 9;
      const S* k1 = Kbuf + (size_t)(code1 & 0x7fffffff) * 9;
      S kv0[9], kv1[9];
#pragma unroll
      for (int i = 0; i < 9; ++i) {
        kv0[i] = k0[i];
        kv1[i] = k1[i];
      }
      add(code0, kv0);
      add(code1, kv1);
    }
    if (c < c1) {
      const int code = csrc[c];
      const S* k = Kbuf + (size_t)(code & 0x7fffffff) * 9;
      S kv[9];
#pragma unroll
      for (int i = 0; i < 9; ++i) kv[i] = k[i];
      add(code, kv);
    }
  }
  const int u = A.slot_row[q];
  if (u >= 0) {
    const S m = slot_mass[q];
    acc[0] += m;
    acc[4] += m;
    acc[8] += m;
    const int w = A.sl_col[q];
    if (filter) {
      const int mu = mask[u], mw = mask[w];
      if (mu | mw) {
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
          for (int b = 0; b < 3; ++b)
            if (((mu >> a) & 1) || ((mw >> b) & 1)) acc[a * 3 + b] = (u == w && a == b) ? S(1) : S(0);
      }
    }
    if (dinv != nullptr && u == w) precond_rows<S>(acc, precond, dinv + 3 * (size_t)u);
  }
  const size_t base = sell_base(q);
#pragma unroll
  for (int c = 0; c < 9; ++c) vals[base + 32 * c] = acc[c];
}

// Symmetric SELL-32 3x3-block SpMV, one thread per block row; a warp walks one slice in lockstep so every
// upper value load is one contiguous line.  The lower blocks are the transposed upper slots of earlier
// rows; for meshes numbered along a grid the slots read by neighbouring lanes are neighbours too.
template <typename S>
__device__ __forceinline__ V4<S> load_x(const V4<S>* x0, const V4<S>* x1, S beta, int col) {
  V4<S> xv = x0[col];
  if (x1 != nullptr) {
    const V4<S> pv = x1[col];
    xv.x += beta * pv.x;
    xv.y += beta * pv.y;
    xv.z += beta * pv.z;
  }
  return xv;
}

// y_u = sum over the upper slots of A_uw x_w + sum over the lower slots of (A_wu)^T x_w, accumulated slot
// by slot in chunks of two (indices first, then the two slots' x gathers and 18 values, then the FMAs);
// lower padding entries point at an all-zero slot, so no branch stops the loads from being hoisted.
// KRON: a matrix (scalar) (x) I3 stored with one value per block (the 3x3 block is v I3); vb then walks
// one value per slot (stride 32 per slot row of the slice)
template <typename S, int U, bool KRON = false>
__device__ __forceinline__ void upper_chunk(const S* __restrict__ vb, const int (&c)[U], const V4<S>* x0,
                                            const V4<S>* x1, S beta, int k, S& a0, S& a1, S& a2) {
  if constexpr (KRON) {
    S v[U];
#pragma unroll
    for (int j = 0; j < U; ++j) v[j] = vb[(size_t)(k + j) * 32];
    V4<S> xv[U];
#pragma unroll
    for (int j = 0; j < U; ++j) xv[j] = load_x<S>(x0, x1, beta, c[j]);
#pragma unroll
    for (int j = 0; j < U; ++j) {
      a0 += v[j] * xv[j].x;
      a1 += v[j] * xv[j].y;
      a2 += v[j] * xv[j].z;
    }
  } else {
    S v[U][9];
#pragma unroll
    for (int j = 0; j < U; ++j)
#pragma unroll
      for (int m = 0; m < 9; ++m) v[j][m] = vb[(size_t)(k + j) * 288 + 32 * m];
    V4<S> xv[U];
#pragma unroll
    for (int j = 0; j < U; ++j) xv[j] = load_x<S>(x0, x1, beta, c[j]);
#pragma unroll
    for (int j = 0; j < U; ++j) {
      a0 += v[j][0] * xv[j].x + v[j][1] * xv[j].y + v[j][2] * xv[j].z;
      a1 += v[j][3] * xv[j].x + v[j][4] * xv[j].y + v[j][5] * xv[j].z;
      a2 += v[j][6] * xv[j].x + v[j][7] * xv[j].y + v[j][8] * xv[j].z;
    }
  }
}

template <typename S, int U, bool KRON = false>
__device__ __forceinline__ void lower_chunk(const S* __restrict__ vals, const int (&q)[U], const int (&c)[U],
                                            const V4<S>* x0, const V4<S>* x1, S beta, S& a0, S& a1, S& a2) {
  if constexpr (KRON) {  // v I3 is its own transpose
    S v[U];
#pragma unroll
    for (int j = 0; j < U; ++j) v[j] = vals[q[j]];
    V4<S> xv[U];
#pragma unroll
    for (int j = 0; j < U; ++j) xv[j] = load_x<S>(x0, x1, beta, c[j]);
#pragma unroll
    for (int j = 0; j < U; ++j) {
      a0 += v[j] * xv[j].x;
      a1 += v[j] * xv[j].y;
      a2 += v[j] * xv[j].z;
    }
  } else {
    S v[U][9];
#pragma unroll
    for (int j = 0; j < U; ++j) {
      const S* p = vals + sell_base(q[j]);
#pragma unroll
      for (int m = 0; m < 9; ++m) v[j][m] = p[32 * m];
    }
    V4<S> xv[U];
#pragma unroll
    for (int j = 0; j < U; ++j) xv[j] = load_x<S>(x0, x1, beta, c[j]);
    // (A_wu)^T x_w: column a of the stored block times x
#pragma unroll
    for (int j = 0; j < U; ++j) {
      a0 += v[j][0] * xv[j].x + v[j][3] * xv[j].y + v[j][6] * xv[j].z;
      a1 += v[j][1] * xv[j].x + v[j][4] * xv[j].y + v[j][7] * xv[j].z;
      a2 += v[j][2] * xv[j].x + v[j][5] * xv[j].y + v[j][8] * xv[j].z;
    }
  }
}

// Index source of one row: straight from global memory, or from a per-warp shared-memory copy of the
// slice's first ST_UP upper columns and ST_LO lower (slot, column) pairs, filled with cp.async in one
// round trip so the value and x loads of every chunk depend only on fast shared loads.
constexpr int ST_UP = 12, ST_LO = 10, ST_K = ST_UP + 2 * ST_LO;

__device__ __forceinline__ void cp_async4(int* dst, const int* src) {
  const unsigned int d = (unsigned int)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

template <typename S, bool STAGED, bool KRON = false>
__device__ __forceinline__ void row_product_t(const SellMatrix& A, const S* __restrict__ vals, int u, const V4<S>* x0,
                                              const V4<S>* x1, S beta, int (*sidx)[32], S& a0, S& a1, S& a2) {
  const int lane = u & 31, s = u >> 5;
  const int ub = A.sl_off[s], Wu = (A.sl_off[s + 1] - ub) >> 5;
  const int lb = A.lo_off[s], Wl = (A.lo_off[s + 1] - lb) >> 5;
  const int* cb = A.sl_col + ub + lane;
  const int* sb = A.lo_src + lb + lane;
  const int* lcb = A.lo_col + lb + lane;
  if (STAGED) {
    const int nu = min(Wu, ST_UP), nl = min(Wl, ST_LO);
    for (int k = 0; k < nu; ++k) cp_async4(&sidx[k][lane], cb + k * 32);
    for (int k = 0; k < nl; ++k) {
      cp_async4(&sidx[ST_UP + 2 * k][lane], sb + k * 32);
      cp_async4(&sidx[ST_UP + 2 * k + 1][lane], lcb + k * 32);
    }
    cp_async_wait_all();
  }
  auto ucol = [&](int k) { return (STAGED && k < ST_UP) ? sidx[k][lane] : cb[k * 32]; };
  auto lsrc = [&](int k) { return (STAGED && k < ST_LO) ? sidx[ST_UP + 2 * k][lane] : sb[k * 32]; };
  auto lcol = [&](int k) { return (STAGED && k < ST_LO) ? sidx[ST_UP + 2 * k + 1][lane] : lcb[k * 32]; };
  a0 = a1 = a2 = S(0);
  const S* vb = vals + (size_t)(KRON ? 1 : 9) * ub + lane;
  int k = 0;
  for (; k + 2 <= Wu; k += 2) {
    const int c[2] = {ucol(k), ucol(k + 1)};
    upper_chunk<S, 2, KRON>(vb, c, x0, x1, beta, k, a0, a1, a2);
  }
  if (k < Wu) {
    const int c[1] = {ucol(k)};
    upper_chunk<S, 1, KRON>(vb, c, x0, x1, beta, k, a0, a1, a2);
  }
  k = 0;
  for (; k + 2 <= Wl; k += 2) {
    const int qq[2] = {lsrc(k), lsrc(k + 1)}, c[2] = {lcol(k), lcol(k + 1)};
    lower_chunk<S, 2, KRON>(vals, qq, c, x0, x1, beta, a0, a1, a2);
  }
  if (k < Wl) {
    const int qq[1] = {lsrc(k)}, c[1] = {lcol(k)};
    lower_chunk<S, 1, KRON>(vals, qq, c, x0, x1, beta, a0, a1, a2);
  }
}

template <typename S>
__device__ __forceinline__ void row_product(const SellMatrix& A, const S* __restrict__ vals, int u, const V4<S>* x0,
                                            const V4<S>* x1, S beta, S& a0, S& a1, S& a2) {
  row_product_t<S, false>(A, vals, u, x0, x1, beta, nullptr, a0, a1, a2);
}

template <typename S>
__global__ void __launch_bounds__(SB)
    spmv_kernel(SellMatrix A, const S* __restrict__ vals, const V4<S>* __restrict__ x, V4<S>* __restrict__ y) {
  const int u = blockIdx.x * SB + threadIdx.x;
  if (u >= A.nv) return;
  S a0, a1, a2;
  row_product<S>(A, vals, u, x, nullptr, S(0), a0, a1, a2);
  y[u] = mk4<S>(a0, a1, a2);
}

// Symmetric storage -> the reference's full CSR: each upper slot writes its block into row u (position
// slot_k) and, off the diagonal, its transpose into row w (position slot_kt).
template <typename S>
__global__ void __launch_bounds__(SB)
    export_csr_kernel(SellMatrix A, const int* __restrict__ bptr, const int* __restrict__ slot_k,
                      const int* __restrict__ slot_kt, const S* __restrict__ vals, double* __restrict__ out) {
  const int q = blockIdx.x * SB + threadIdx.x;
  if (q >= A.nslots) return;
  const int u = A.slot_row[q];
  if (u < 0) return;
  const int w = A.sl_col[q];
  const size_t base = sell_base(q);
  {
    const long long b0 = bptr[u];
    const int deg = bptr[u + 1] - bptr[u], k = slot_k[q];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) out[9 * b0 + 3LL * deg * a + 3 * k + b] = (double)vals[base + 32 * (a * 3 + b)];
  }
  if (w != u) {
    const long long b0 = bptr[w];
    const int deg = bptr[w + 1] - bptr[w], k = slot_kt[q];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) out[9 * b0 + 3LL * deg * a + 3 * k + b] = (double)vals[base + 32 * (b * 3 + a)];
  }
}

// ------------------------------------------------------------------ PCG
// Jacobi-PCG (the mathprim cg + diagonal_preconditioner the reference's Newton uses, fem_cu/main.cu:52-54),
// two fused kernels per iteration.  Vectors in S; dot products summed in S within a warp (32 rows) and in
// FP64 across warps, blocks and the grid.  The search direction is
// double-buffered: the SpMV kernel forms p_new = z + beta p_old on the fly for every neighbour it reads,
// so the update of p needs no kernel of its own.
template <typename S>
__global__ void __launch_bounds__(SB)
    pcg_setup_kernel(int nv, const double* __restrict__ g, const V4<S>* __restrict__ dinv, V4<S>* __restrict__ x,
                     V4<S>* __restrict__ r, V4<S>* __restrict__ z, V4<S>* __restrict__ p0, double rtol, int max_iters,
                     int negate, Reduce red) {
  __shared__ double shred[SB / 32][2];
  const int u = blockIdx.x * SB + threadIdx.x;
  S part[2] = {S(0), S(0)};
  if (u < nv) {
    const double sg = negate ? -1.0 : 1.0;
    const S r0 = (S)(sg * g[u * 3 + 0]), r1 = (S)(sg * g[u * 3 + 1]), r2 = (S)(sg * g[u * 3 + 2]);
    const V4<S> d0 = dinv[3 * u], d1 = dinv[3 * u + 1], d2 = dinv[3 * u + 2];
    const S z0 = d0.x * r0 + d0.y * r1 + d0.z * r2;
    const S z1 = d1.x * r0 + d1.y * r1 + d1.z * r2;
    const S z2 = d2.x * r0 + d2.y * r1 + d2.z * r2;
    x[u] = mk4<S>(0, 0, 0);
    r[u] = mk4<S>(r0, r1, r2);
    z[u] = mk4<S>(z0, z1, z2);
    p0[u] = mk4<S>(0, 0, 0);
    part[0] = r0 * z0 + r1 * z1 + r2 * z2;
    part[1] = r0 * r0 + r1 * r1 + r2 * r2;
  }
  double bs[2];
  block_sum_s<2, SB, S>(part, bs, shred);
  double tot[2];
  if (grid_sum_last<2, SB>(bs, red.partials, red.counter, tot)) {
    DevScalars* sc = red.sc;
    sc->rz = tot[0];
    sc->rz_old = 1.0;
    sc->rr = tot[1];
    sc->rr0 = tot[1];
    sc->tol2 = rtol * rtol * tot[1];
    sc->iters = 0;
    sc->status = 0;
    sc->done = (tot[1] <= sc->tol2 || tot[1] == 0.0 || max_iters <= 0) ? 1 : 0;
  }
}

// One row of the fused PCG SpMV: p_new = z + beta p_old (formed on the fly for the gathered columns),
// q = A p_new; returns the row's share of p_new . q.
template <typename S, bool KRON = false>
__device__ __forceinline__ S pcg_spmv_row(const SellMatrix& A, const S* __restrict__ vals, const V4<S>* z,
                                          const V4<S>* p_old, V4<S>* p_new, V4<S>* q, S beta, int u,
                                          int (*sidx)[32]) {
  if (u >= A.nv) return S(0);
  S a0, a1, a2;
  row_product_t<S, true, KRON>(A, vals, u, z, p_old, beta, sidx, a0, a1, a2);
  const V4<S> zu = z[u], pu = p_old[u];
  const V4<S> pn = mk4<S>(zu.x + beta * pu.x, zu.y + beta * pu.y, zu.z + beta * pu.z);
  p_new[u] = pn;
  q[u] = mk4<S>(a0, a1, a2);
  return pn.x * a0 + pn.y * a1 + pn.z * a2;
}

// One row of the PCG update: x += alpha p, r -= alpha q, z = D^-1 r; shares of r.z and r.r in part.
template <typename S>
__device__ __forceinline__ void pcg_update_row(int nv, const V4<S>* p, const V4<S>* q, const V4<S>* __restrict__ dinv,
                                               V4<S>* x, V4<S>* r, V4<S>* z, S alpha, int u, S (&part)[2]) {
  part[0] = part[1] = S(0);
  if (u >= nv) return;
  const V4<S> pu = p[u], qu = q[u];
  const V4<S> d0 = dinv[3 * u], d1 = dinv[3 * u + 1], d2 = dinv[3 * u + 2];
  V4<S> xu = x[u], ru = r[u];
  xu.x += alpha * pu.x;
  xu.y += alpha * pu.y;
  xu.z += alpha * pu.z;
  ru.x -= alpha * qu.x;
  ru.y -= alpha * qu.y;
  ru.z -= alpha * qu.z;
  const V4<S> zu = mk4<S>(d0.x * ru.x + d0.y * ru.y + d0.z * ru.z, d1.x * ru.x + d1.y * ru.y + d1.z * ru.z,
                          d2.x * ru.x + d2.y * ru.y + d2.z * ru.z);
  x[u] = xu;
  r[u] = ru;
  z[u] = zu;
  part[0] = ru.x * zu.x + ru.y * zu.y + ru.z * zu.z;
  part[1] = ru.x * ru.x + ru.y * ru.y + ru.z * ru.z;
}

// the scalar epilogues shared by the two-launch and the persistent PCG
__device__ __forceinline__ void pcg_after_pq(DevScalars* sc, double pq) {
  sc->pq = pq;
  sc->alpha = sc->rz / pq;
  if (!(pq > 0.0)) {  // breakdown: not SPD along p (or non-finite)
    sc->done = 1;
    sc->status = 1;
  }
}

__device__ __forceinline__ void pcg_after_rz(DevScalars* sc, double rz, double rr, int max_iters) {
  sc->rz_old = sc->rz;
  sc->rz = rz;
  sc->beta = rz / sc->rz_old;
  sc->rr = rr;
  sc->iters += 1;
  if (!isfinite(rr)) {
    sc->done = 1;
    sc->status = 2;
  } else if (rr <= sc->tol2 || sc->iters >= max_iters || rz == 0.0) {
    sc->done = 1;
  }
}

template <typename S, bool KRON>
__global__ void __launch_bounds__(SB)
    pcg_spmv_kernel(SellMatrix A, const S* __restrict__ vals, const V4<S>* __restrict__ z,
                    const V4<S>* __restrict__ p_old, V4<S>* __restrict__ p_new, V4<S>* __restrict__ q, int first,
                    Reduce red) {
  if (*(volatile int*)&red.sc->done) return;
  __shared__ double shred[SB / 32][1];
  __shared__ int sidx[SB / 32][ST_K][32];
  const S beta = first ? S(0) : (S)red.sc->beta;
  S part[1] = {pcg_spmv_row<S, KRON>(A, vals, z, p_old, p_new, q, beta, blockIdx.x * SB + threadIdx.x,
                                     sidx[threadIdx.x >> 5])};
  double v1[1];
  block_sum_s<1, SB, S>(part, v1, shred);
  double tot[1];
  if (grid_sum_last_tree<1, SB>(v1, red.partials, red.partials + 2 * (size_t)gridDim.x, red.counter, tot))
    pcg_after_pq(red.sc, tot[0]);
}

template <typename S>
__global__ void __launch_bounds__(SB)
    pcg_update_kernel(int nv, const V4<S>* __restrict__ p, const V4<S>* __restrict__ q,
                      const V4<S>* __restrict__ dinv, V4<S>* __restrict__ x, V4<S>* __restrict__ r,
                      V4<S>* __restrict__ z, int max_iters, Reduce red) {
  if (*(volatile int*)&red.sc->done) return;
  __shared__ double shred[SB / 32][2];
  const S alpha = (S)red.sc->alpha;
  S part[2];
  pcg_update_row<S>(nv, p, q, dinv, x, r, z, alpha, blockIdx.x * SB + threadIdx.x, part);
  double bs[2];
  block_sum_s<2, SB, S>(part, bs, shred);
  double tot[2];
  if (grid_sum_last_tree<2, SB>(bs, red.partials, red.partials + 2 * (size_t)gridDim.x, red.counter, tot))
    pcg_after_rz(red.sc, tot[0], tot[1], max_iters);
}

// ------------------------------------------------------------------ persistent PCG
// The whole PCG loop in one cooperative launch (every block resident).  Work is split into 256-row
// "virtual blocks", each block taking virtual blocks blockIdx.x, blockIdx.x + gridDim.x, ...; every virtual
// block writes its partial sums, and at the reducing grid barrier the LAST block to arrive adds them in
// grid_sum_last's order and runs the scalar epilogue into the device scalars before it releases the
// others, who then read alpha / beta / done from there.  The result does not depend on the grid size, and
// the FP64 reduction runs once per barrier (the FP64 pipe is narrow on GB300).  Arrays written inside the
// loop are read with plain loads only after a barrier, whose acquire side orders them after the writers'
// release (the cooperative-groups grid sync pattern); the scalars are read with L2 loads.
// Every counter and release word sits on its own 128-byte line (kSyncStride words apart): the waiting
// blocks poll release words that no atomic touches, and the atomics of one counter do not share a line
// with another's.
constexpr int kSyncStride = 16;
struct GridSync {
  unsigned long long* arrive;  // plain-barrier arrivals since the launch (never reset within it)
  unsigned long long* top;     // arrivals of completed groups at the reducing barriers
  unsigned long long* release; // reducing barriers completed (written by the one that completes each)
  unsigned long long* group;   // [ngroups] arrivals of each group's virtual blocks, kSyncStride apart
  int ngroups;
  unsigned int extra;  // arrivals beyond the grid / the groups (test hook; 0 in normal use)
  long long spin_limit;
  unsigned long long* prelease;  // plain barriers completed (written by the last arrival of each)
};

__device__ __forceinline__ unsigned long long ld_acquire_gpu(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_gpu(unsigned long long* p, unsigned long long v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
// The barriers' ordering: every arrival is one acquire-release atomic at GPU scope (its release half
// publishes the block's writes and partials, its acquire half lets the arrival that completes a count see
// every earlier arrival's writes: the atomics on one counter chain them in observation order), the
// completion is one release store and the waiters poll with acquire loads.  No separate fences: 6.3 against
// 8.1 us per reducing barrier on 705 blocks of a GB300 with fence.acq_rel around relaxed atomics, and 7.3
// with release atomics plus a fence in the completing arrival (micro-benchmark; each fence waits for a
// round trip to L2)
__device__ __forceinline__ unsigned long long atom_add_acq_rel_gpu(unsigned long long* p, unsigned long long v) {
  unsigned long long old;
  asm volatile("atom.add.acq_rel.gpu.global.u64 %0, [%1], %2;" : "=l"(old) : "l"(p), "l"(v) : "memory");
  return old;
}

// thread 0 polls *p until it reaches target (at most spin_limit polls); true if it did
__device__ __forceinline__ bool wait_at_least(const unsigned long long* p, unsigned long long target,
                                              long long spin_limit) {
  long long n = 0;
  while (ld_acquire_gpu(p) < target) {
    if (++n > spin_limit) return false;
    __nanosleep(32);
  }
  return true;
}

// Barrier number k (0-based within the launch) without a reduction: the arrival counter only grows; the
// block whose arrival completes the (k + 1)-th round publishes k + 1 in the release word the others poll.
__device__ __forceinline__ bool plain_barrier(const GridSync& gs, unsigned long long k) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned long long target = (k + 1) * (unsigned long long)(gridDim.x + gs.extra);
    if (atom_add_acq_rel_gpu(gs.arrive, 1ull) == target - 1) st_release_gpu(gs.prelease, k + 1);
    ok = wait_at_least(gs.prelease, k + 1, gs.spin_limit);
  }
  __syncthreads();
  return ok != 0;
}

// Reducing barrier number kr: every block has written the partials of its virtual blocks (NV doubles each,
// part[NV * vb]); warp 0 of each block marks them arrived in their groups of 32; the block completing a
// group sums it (warp_group_sum) into gsum[g], and the block completing the last group sums the group
// sums (warp_top_sum, the order of grid_sum_last_tree), runs epi(tot) in its lane 0 and releases everyone.
// Returns false in every thread of a block whose wait gave up.
template <int NV, typename EPI>
__device__ __forceinline__ bool reduce_barrier(const GridSync& gs, unsigned long long kr, const double* part,
                                               double* gsum, int nvb, EPI&& epi) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    for (int vb = blockIdx.x; vb < nvb; vb += gridDim.x) {
      const int g = vb >> 5, gsize = min(32, nvb - 32 * g);
      int last = 0;
      if (lane == 0)
        last = atom_add_acq_rel_gpu(gs.group + (size_t)g * kSyncStride, 1ull) ==
               (kr + 1) * (unsigned long long)gsize - 1;
      last = __shfl_sync(0xffffffffu, last, 0);
      __syncwarp();
      if (!last) continue;
      double v[NV];
      warp_group_sum<NV>(part, 32 * g, gsize, v);
      int top = 0;
      if (lane == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) gsum[g * NV + k] = v[k];
        top = atom_add_acq_rel_gpu(gs.top, 1ull) == (kr + 1) * (unsigned long long)(gs.ngroups + gs.extra) - 1;
      }
      top = __shfl_sync(0xffffffffu, top, 0);
      __syncwarp();
      if (!top) continue;
      double tot[NV];
      warp_top_sum<NV>(gsum, gs.ngroups, tot);
      if (lane == 0) {
        epi(tot);
        st_release_gpu(gs.release, kr + 1);
      }
    }
  }
  if (threadIdx.x == 0) ok = wait_at_least(gs.release, kr + 1, gs.spin_limit);
  __syncthreads();
  return ok != 0;
}

// Chronopoulos-Gear PCG (Chronopoulos & Gear, J. Comput. Appl. Math. 25, 1989): the same iterates as
// PCG in exact arithmetic, with s = A p carried by its own recurrence so one reduction per iteration
// gives all scalars.  With u = M r and w = A u:
//   phase A:  w = A u;  gamma = (r, u), delta = (w, u), rr = (r, r)          -> one grid reduction
//   scalars:  beta = gamma / gamma_old, alpha = gamma / (delta - beta gamma / alpha_old)  (first: 0, gamma/delta)
//   phase B:  p = u + beta p, s = w + beta s, x += alpha p, r -= alpha s, u = M r   (per vertex)
// The SpMV gathers one vector (u) instead of forming z + beta p for every neighbour; the barrier after
// phase B only orders u's writes before the next gathers.  Vectors: u = z, w = q, p = p0, s = p1.
template <typename S, bool KRON = false>
__device__ __forceinline__ void cgcg_spmv_row(const SellMatrix& A, const S* __restrict__ vals, const V4<S>* z,
                                              const V4<S>* r, V4<S>* q, int u, int (*sidx)[32], S (&part)[3]) {
  part[0] = part[1] = part[2] = S(0);
  if (u >= A.nv) return;
  S a0, a1, a2;
  row_product_t<S, true, KRON>(A, vals, u, z, nullptr, S(0), sidx, a0, a1, a2);
  q[u] = mk4<S>(a0, a1, a2);
  const V4<S> uu = z[u], ru = r[u];
  part[0] = ru.x * uu.x + ru.y * uu.y + ru.z * uu.z;
  part[1] = a0 * uu.x + a1 * uu.y + a2 * uu.z;
  part[2] = ru.x * ru.x + ru.y * ru.y + ru.z * ru.z;
}

template <typename S>
__device__ __forceinline__ void cgcg_update_row(int nv, bool first, S alpha, S beta, const V4<S>* __restrict__ dinv,
                                                V4<S>* z, const V4<S>* q, V4<S>* p, V4<S>* sv, V4<S>* x, V4<S>* r,
                                                int u) {
  if (u >= nv) return;
  const V4<S> uu = z[u], ww = q[u];
  V4<S> pu = uu, su = ww;
  if (!first) {
    const V4<S> po = p[u], so = sv[u];
    pu = mk4<S>(uu.x + beta * po.x, uu.y + beta * po.y, uu.z + beta * po.z);
    su = mk4<S>(ww.x + beta * so.x, ww.y + beta * so.y, ww.z + beta * so.z);
  }
  const V4<S> d0 = dinv[3 * u], d1 = dinv[3 * u + 1], d2 = dinv[3 * u + 2];
  V4<S> xu = x[u], ru = r[u];
  xu.x += alpha * pu.x;
  xu.y += alpha * pu.y;
  xu.z += alpha * pu.z;
  ru.x -= alpha * su.x;
  ru.y -= alpha * su.y;
  ru.z -= alpha * su.z;
  p[u] = pu;
  sv[u] = su;
  x[u] = xu;
  r[u] = ru;
  z[u] = mk4<S>(d0.x * ru.x + d0.y * ru.y + d0.z * ru.z, d1.x * ru.x + d1.y * ru.y + d1.z * ru.z,
                d2.x * ru.x + d2.y * ru.y + d2.z * ru.z);
}

// scalar epilogue after phase A (one thread): stop tests on the residual of the current x, then the
// step lengths.  iters counts the x updates; rr is |r|^2 of the current x.
__device__ __forceinline__ void cgcg_after(DevScalars* sc, double g, double d, double rr, int max_iters) {
  sc->rr = rr;
  if (!isfinite(rr)) {
    sc->done = 1;
    sc->status = 2;
    return;
  }
  if (rr <= sc->tol2 || g == 0.0 || sc->iters >= max_iters) {
    sc->done = 1;
    return;
  }
  // beta = g / g_old and den = d - beta g / alpha_old from the reciprocals kept by the previous step, so
  // only two independent divisions remain on this serial path (FP64 divisions are slow on GB300)
  double beta = 0.0, den = d;
  if (sc->iters > 0) {
    beta = g * sc->inv_rz;
    den = d - beta * g * sc->inv_alpha;
  }
  if (!(den > 0.0)) {  // breakdown: not SPD along p (or non-finite)
    sc->done = 1;
    sc->status = 1;
    return;
  }
  const double inv_den = 1.0 / den, inv_g = 1.0 / g;
  sc->rz_old = sc->rz;
  sc->rz = g;
  sc->pq = den;
  sc->beta = beta;
  sc->alpha = g * inv_den;
  sc->inv_rz = inv_g;
  sc->inv_alpha = den * inv_g;
  sc->iters += 1;
}

template <typename S, bool KRON>
__global__ void __launch_bounds__(SB, sizeof(S) == 4 ? 5 : 4)
    cgcg_persistent_kernel(SellMatrix A, const S* __restrict__ vals, const V4<S>* __restrict__ dinv, V4<S>* x,
                           V4<S>* r, V4<S>* z, V4<S>* p0, V4<S>* p1, V4<S>* q, int max_iters, Reduce red,
                           GridSync gs) {
  __shared__ double shred[SB / 32][3];
  __shared__ int sidx[SB / 32][ST_K][32];
  __shared__ double s_alpha, s_beta;
  __shared__ int s_done;
  DevScalars* sc = red.sc;
  if (threadIdx.x == 0) s_done = *(volatile int*)&sc->done;
  __syncthreads();
  if (s_done) return;
  const int nvb = (A.nv + SB - 1) / SB;
  double* part = red.partials;
  double* gsum = red.partials + 3 * (size_t)nvb;
  bool ok = true;
  for (int k = 0;; ++k) {
    for (int vb = blockIdx.x; vb < nvb; vb += gridDim.x) {
      S pr[3];
      cgcg_spmv_row<S, KRON>(A, vals, z, r, q, vb * SB + threadIdx.x, sidx[threadIdx.x >> 5], pr);
      double bs[3];
      block_sum_s<3, SB, S>(pr, bs, shred);
      if (threadIdx.x == 0) {
        part[3 * vb] = bs[0];
        part[3 * vb + 1] = bs[1];
        part[3 * vb + 2] = bs[2];
      }
      __syncthreads();
    }
    ok = reduce_barrier<3>(gs, (unsigned long long)k, part, gsum, nvb,
                           [&](const double (&t)[3]) { cgcg_after(sc, t[0], t[1], t[2], max_iters); });
    if (!ok) break;
    if (threadIdx.x == 0) {
      s_done = __ldcg(&sc->done);
      s_alpha = __ldcg(&sc->alpha);
      s_beta = __ldcg(&sc->beta);
    }
    __syncthreads();
    if (s_done) break;
    const S alpha = (S)s_alpha, beta = (S)s_beta;
    for (int vb = blockIdx.x; vb < nvb; vb += gridDim.x)
      cgcg_update_row<S>(A.nv, k == 0, alpha, beta, dinv, z, q, p0, p1, x, r, vb * SB + threadIdx.x);
    ok = plain_barrier(gs, (unsigned long long)k);
    if (!ok) break;
  }
  // a barrier wait gave up: flag it (the host clears the flag before the launch) and leave
  if (!ok && threadIdx.x == 0) atomicExch(&sc->wait_failed, 1);
}

// ------------------------------------------------------------------ FP16 copy of the scaled matrix
// (kernels.cuh, HalfMatrix).  The diagonal block of row u is its first upper slot.
__global__ void __launch_bounds__(SB)
    half_prepare_kernel(SellMatrix A, const float* __restrict__ vals, int precond, float4* __restrict__ scale,
                        float4* __restrict__ iscale, float4* __restrict__ dinv16) {
  const int u = blockIdx.x * SB + threadIdx.x;
  if (u >= A.nv) return;
  const int q = A.sl_off[u >> 5] + (u & 31);
  const bool own = A.slot_row[q] == u;  // false only for a vertex that no cell uses (all-zero row)
  const size_t base = sell_base(q);
  float b[9];
#pragma unroll
  for (int c = 0; c < 9; ++c) b[c] = own ? vals[base + 32 * c] : 0.f;
  float sc[3], isc[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float d = b[4 * a];
    if (d > 0.f && isfinite(d)) {
      isc[a] = sqrtf(d);
      sc[a] = 1.f / isc[a];
    } else {
      sc[a] = isc[a] = 1.f;
    }
  }
  float bt[9];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int c = 0; c < 3; ++c) bt[3 * a + c] = b[3 * a + c] * sc[a] * sc[c];
  precond_rows<float>(bt, precond, dinv16 + 3 * (size_t)u);
  scale[u] = make_float4(sc[0], sc[1], sc[2], 0.f);
  iscale[u] = make_float4(isc[0], isc[1], isc[2], 0.f);
}

__device__ __forceinline__ unsigned int pack_half2(float lo, float hi) {
  return (unsigned int)__half_as_ushort(__float2half_rn(lo)) | ((unsigned int)__half_as_ushort(__float2half_rn(hi)) << 16);
}

// one thread per block row, its entries in slot order (stores coalesced across the slice's lanes)
__global__ void __launch_bounds__(SB)
    half_convert_kernel(int nv, const int* __restrict__ off, const int* __restrict__ col, const int* __restrict__ src,
                        const float* __restrict__ vals, const float4* __restrict__ scale, uint4* __restrict__ v8,
                        uint16_t* __restrict__ v1) {
  const int u = blockIdx.x * SB + threadIdx.x;
  if (u >= nv) return;
  const int lane = u & 31, sl = u >> 5;
  const int b = off[sl], W = (off[sl + 1] - b) >> 5;
  const float4 su = scale[u];
  const float sa[3] = {su.x, su.y, su.z};
  for (int k = 0; k < W; ++k) {
    const int e = b + 32 * k + lane;
    const unsigned int code = (unsigned int)src[e];
    const bool tr = (code >> 31) != 0u;
    const size_t base = sell_base((int)(code & 0x7fffffffu));
    const float4 sw4 = scale[col[e]];
    const float sw[3] = {sw4.x, sw4.y, sw4.z};
    float v[9];
#pragma unroll
    for (int c = 0; c < 9; ++c) v[c] = vals[base + 32 * c];
    float h[9];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int c = 0; c < 3; ++c) h[3 * a + c] = (tr ? v[3 * c + a] : v[3 * a + c]) * sa[a] * sw[c];
    v8[e] = make_uint4(pack_half2(h[0], h[1]), pack_half2(h[2], h[3]), pack_half2(h[4], h[5]),
                       pack_half2(h[6], h[7]));
    v1[e] = __half_as_ushort(__float2half_rn(h[8]));
  }
}

__device__ __forceinline__ float2 unpack_half2(unsigned int w) {
  return __half22float2(__halves2half2(__ushort_as_half((unsigned short)(w & 0xffffu)),
                                       __ushort_as_half((unsigned short)(w >> 16))));
}

// y~_u = sum_k K~_{u,w_k} x_{w_k}: column indices staged per warp (cp.async, up to ST_K per row), then two
// entries at a time: one 16-byte and one 2-byte value load and one x gather each
__device__ __forceinline__ void half_row_product(const HalfMatrix& H, int u, const float4* x, int (*sidx)[32],
                                                 float& a0, float& a1, float& a2) {
  const int lane = u & 31, sl = u >> 5;
  const int b = H.off[sl], W = (H.off[sl + 1] - b) >> 5;
  const int* cb = H.col + b + lane;
  const int ns = min(W, ST_K);
  for (int k = 0; k < ns; ++k) cp_async4(&sidx[k][lane], cb + k * 32);
  cp_async_wait_all();
  auto col = [&](int k) { return k < ST_K ? sidx[k][lane] : cb[k * 32]; };
  a0 = a1 = a2 = 0.f;
  auto fma_block = [&](const uint4& p, uint16_t h8, const float4& xv) {
    const float2 f01 = unpack_half2(p.x), f23 = unpack_half2(p.y), f45 = unpack_half2(p.z), f67 = unpack_half2(p.w);
    const float f8 = __half2float(__ushort_as_half(h8));
    a0 += f01.x * xv.x + f01.y * xv.y + f23.x * xv.z;
    a1 += f23.y * xv.x + f45.x * xv.y + f45.y * xv.z;
    a2 += f67.x * xv.x + f67.y * xv.y + f8 * xv.z;
  };
  const size_t e0 = (size_t)b + lane;
  int k = 0;
  for (; k + 2 <= W; k += 2) {
    const uint4 p0 = H.v8[e0 + 32 * (size_t)k], p1 = H.v8[e0 + 32 * (size_t)(k + 1)];
    const uint16_t h0 = H.v1[e0 + 32 * (size_t)k], h1 = H.v1[e0 + 32 * (size_t)(k + 1)];
    const float4 x0 = x[col(k)], x1 = x[col(k + 1)];
    fma_block(p0, h0, x0);
    fma_block(p1, h1, x1);
  }
  if (k < W) fma_block(H.v8[e0 + 32 * (size_t)k], H.v1[e0 + 32 * (size_t)k], x[col(k)]);
}

__global__ void __launch_bounds__(SB)
    half_spmv_kernel(HalfMatrix H, const float4* __restrict__ x, float4* __restrict__ xs, float4* __restrict__ y,
                     int phase) {
  __shared__ int sidx[SB / 32][ST_K][32];
  const int u = blockIdx.x * SB + threadIdx.x;
  if (u >= H.nv) return;
  if (phase == 0) {  // xs = S^-1 x
    const float4 xv = x[u], is = H.iscale[u];
    xs[u] = make_float4(xv.x * is.x, xv.y * is.y, xv.z * is.z, 0.f);
    return;
  }
  float a0, a1, a2;
  half_row_product(H, u, xs, sidx[threadIdx.x >> 5], a0, a1, a2);
  const float4 is = H.iscale[u];
  y[u] = make_float4(a0 * is.x, a1 * is.y, a2 * is.z, 0.f);
}

__global__ void __launch_bounds__(SB)
    pcg_setup_half_kernel(HalfMatrix H, const double* __restrict__ g, const float4* __restrict__ dinv16,
                          float4* __restrict__ x, float4* __restrict__ r, float4* __restrict__ z,
                          float4* __restrict__ p0, double rtol, int max_iters, int negate, Reduce red) {
  __shared__ double shred[SB / 32][2];
  const int u = blockIdx.x * SB + threadIdx.x;
  float part[2] = {0.f, 0.f};
  if (u < H.nv) {
    const double sg = negate ? -1.0 : 1.0;
    const float r0 = (float)(sg * g[u * 3 + 0]), r1 = (float)(sg * g[u * 3 + 1]), r2 = (float)(sg * g[u * 3 + 2]);
    const float4 sc = H.scale[u];
    const float t0 = r0 * sc.x, t1 = r1 * sc.y, t2 = r2 * sc.z;
    const float4 d0 = dinv16[3 * u], d1 = dinv16[3 * u + 1], d2 = dinv16[3 * u + 2];
    const float z0 = d0.x * t0 + d0.y * t1 + d0.z * t2;
    const float z1 = d1.x * t0 + d1.y * t1 + d1.z * t2;
    const float z2 = d2.x * t0 + d2.y * t1 + d2.z * t2;
    x[u] = make_float4(0.f, 0.f, 0.f, 0.f);
    r[u] = make_float4(t0, t1, t2, 0.f);
    z[u] = make_float4(z0, z1, z2, 0.f);
    p0[u] = make_float4(0.f, 0.f, 0.f, 0.f);
    part[0] = t0 * z0 + t1 * z1 + t2 * z2;
    part[1] = r0 * r0 + r1 * r1 + r2 * r2;
  }
  double bs[2];
  block_sum_s<2, SB, float>(part, bs, shred);
  double tot[2];
  if (grid_sum_last<2, SB>(bs, red.partials, red.counter, tot)) {
    DevScalars* sc = red.sc;
    sc->rz = tot[0];
    sc->rz_old = 1.0;
    sc->rr = tot[1];
    sc->rr0 = tot[1];
    sc->tol2 = rtol * rtol * tot[1];
    sc->iters = 0;
    sc->status = 0;
    sc->done = (tot[1] <= sc->tol2 || tot[1] == 0.0 || max_iters <= 0) ? 1 : 0;
  }
}

// Chronopoulos-Gear PCG (cgcg_persistent_kernel) in the scaled space of the FP16 copy: the SpMV reads the
// full entries, the third dot is (r, r) of the unscaled residual r = S^-1 r~, and every block unscales its
// own rows of x after the last iteration.
__global__ void __launch_bounds__(SB, 5)
    cgcg_half_kernel(HalfMatrix H, const float4* __restrict__ dinv16, float4* x, float4* r, float4* z, float4* p0,
                     float4* p1, float4* q, int max_iters, Reduce red, GridSync gs) {
  __shared__ double shred[SB / 32][3];
  __shared__ int sidx[SB / 32][ST_K][32];
  __shared__ double s_alpha, s_beta;
  __shared__ int s_done;
  DevScalars* sc = red.sc;
  if (threadIdx.x == 0) s_done = *(volatile int*)&sc->done;
  __syncthreads();
  if (s_done) return;
  const int nvb = (H.nv + SB - 1) / SB;
  double* part = red.partials;
  double* gsum = red.partials + 3 * (size_t)nvb;
  bool ok = true;
  for (int k = 0;; ++k) {
    for (int vb = blockIdx.x; vb < nvb; vb += gridDim.x) {
      const int u = vb * SB + threadIdx.x;
      float pr[3] = {0.f, 0.f, 0.f};
      if (u < H.nv) {
        float a0, a1, a2;
        half_row_product(H, u, z, sidx[threadIdx.x >> 5], a0, a1, a2);
        q[u] = make_float4(a0, a1, a2, 0.f);
        const float4 uu = z[u], ru = r[u], is = H.iscale[u];
        pr[0] = ru.x * uu.x + ru.y * uu.y + ru.z * uu.z;
        pr[1] = a0 * uu.x + a1 * uu.y + a2 * uu.z;
        const float t0 = ru.x * is.x, t1 = ru.y * is.y, t2 = ru.z * is.z;
        pr[2] = t0 * t0 + t1 * t1 + t2 * t2;
      }
      double bs[3];
      block_sum_s<3, SB, float>(pr, bs, shred);
      if (threadIdx.x == 0) {
        part[3 * vb] = bs[0];
        part[3 * vb + 1] = bs[1];
        part[3 * vb + 2] = bs[2];
      }
      __syncthreads();
    }
    ok = reduce_barrier<3>(gs, (unsigned long long)k, part, gsum, nvb,
                           [&](const double (&t)[3]) { cgcg_after(sc, t[0], t[1], t[2], max_iters); });
    if (!ok) break;
    if (threadIdx.x == 0) {
      s_done = __ldcg(&sc->done);
      s_alpha = __ldcg(&sc->alpha);
      s_beta = __ldcg(&sc->beta);
    }
    __syncthreads();
    if (s_done) break;
    const float alpha = (float)s_alpha, beta = (float)s_beta;
    for (int vb = blockIdx.x; vb < nvb; vb += gridDim.x)
      cgcg_update_row<float>(H.nv, k == 0, alpha, beta, dinv16, z, q, p0, p1, x, r, vb * SB + threadIdx.x);
    ok = plain_barrier(gs, (unsigned long long)k);
    if (!ok) break;
  }
  // x = S x~ (rows of this block only: no other block reads x)
  for (int vb = blockIdx.x; vb < nvb; vb += gridDim.x) {
    const int u = vb * SB + threadIdx.x;
    if (u < H.nv) {
      const float4 xv = x[u], s4 = H.scale[u];
      x[u] = make_float4(xv.x * s4.x, xv.y * s4.y, xv.z * s4.z, 0.f);
    }
  }
  if (!ok && threadIdx.x == 0) atomicExch(&sc->wait_failed, 1);
}

// Pipelined PCG (Ghysels & Vanroose, "Hiding global synchronization latency in the preconditioned
// Conjugate Gradient algorithm", Parallel Computing 40(7), 2014): the Chronopoulos-Gear scalars with the
// SpMV applied to m = M w instead of u, so a vector phase reads nothing that another block writes in the
// same phase except m, and ONE reducing grid barrier per iteration both sums the dots and orders m's
// writes (Chronopoulos-Gear needs a second, plain barrier for u).  Invariants in exact arithmetic:
// u = M r, w = A u, m = M w, s = A p, z = A M s.  M is the per-vertex block-Jacobi inverse, so u = M r
// and M s are formed from r and s where needed instead of carried by recurrences (equal in exact
// arithmetic), which leaves x, r, w, p, s, z and a double-buffered m:
//   prologue:  w = A u0, m_0 = M w;     partials (r, u), (w, u), (r, r)          -> reduction 0
//   phase k:   n = A m_k;  z = n + beta z,  s = w + beta s,  p = M r + beta p;
//              x += alpha p,  r -= alpha s,  w -= alpha z;  m_{k+1} = M w;
//              partials of the new r, u = M r, w                                -> reduction k + 1
// The scalars (cgcg_after) and the stop rule are those of the Chronopoulos-Gear kernel.  The gap between
// the recursive and the true residual grows with the iterations and with the condition number (in FP32
// it reaches the tolerance of long, ill-conditioned solves), so after pipe_iters iterations the solve
// continues as Chronopoulos-Gear PCG from the same state (x, r, p, s, w; u = M r), whose SpMV recomputes
// w = A u every iteration.
template <typename S>
__device__ __forceinline__ V4<S> block_jacobi(const V4<S>* __restrict__ dinv, int u, S a0, S a1, S a2) {
  const V4<S> d0 = dinv[3 * u], d1 = dinv[3 * u + 1], d2 = dinv[3 * u + 2];
  return mk4<S>(d0.x * a0 + d0.y * a1 + d0.z * a2, d1.x * a0 + d1.y * a1 + d1.z * a2,
                d2.x * a0 + d2.y * a1 + d2.z * a2);
}

template <typename S, bool KRON>
__device__ __forceinline__ void pipe_first_row(const SellMatrix& A, const S* __restrict__ vals,
                                               const V4<S>* __restrict__ dinv, const V4<S>* u0, const V4<S>* r,
                                               V4<S>* w, V4<S>* m, int u, int (*sidx)[32], S (&part)[3]) {
  part[0] = part[1] = part[2] = S(0);
  if (u >= A.nv) return;
  S a0, a1, a2;
  row_product_t<S, true, KRON>(A, vals, u, u0, nullptr, S(0), sidx, a0, a1, a2);
  w[u] = mk4<S>(a0, a1, a2);
  m[u] = block_jacobi<S>(dinv, u, a0, a1, a2);
  const V4<S> uu = u0[u], ru = r[u];
  part[0] = ru.x * uu.x + ru.y * uu.y + ru.z * uu.z;
  part[1] = a0 * uu.x + a1 * uu.y + a2 * uu.z;
  part[2] = ru.x * ru.x + ru.y * ru.y + ru.z * ru.z;
}

template <typename S, bool KRON>
__device__ __forceinline__ void pipe_row(const SellMatrix& A, const S* __restrict__ vals, const V4<S>* __restrict__ dinv,
                                         bool first, S alpha, S beta, const V4<S>* mk, V4<S>* mn, V4<S>* x,
                                         V4<S>* r, V4<S>* z, V4<S>* p, V4<S>* sv, V4<S>* w, int u,
                                         int (*sidx)[32], S (&part)[3]) {
  part[0] = part[1] = part[2] = S(0);
  if (u >= A.nv) return;
  S n0, n1, n2;
  row_product_t<S, true, KRON>(A, vals, u, mk, nullptr, S(0), sidx, n0, n1, n2);
  V4<S> ru = r[u], wu = w[u];
  const V4<S> uu = block_jacobi<S>(dinv, u, ru.x, ru.y, ru.z);
  V4<S> zu = mk4<S>(n0, n1, n2), su = wu, pu = uu;
  if (!first) {
    const V4<S> zo = z[u], so = sv[u], po = p[u];
    zu = mk4<S>(n0 + beta * zo.x, n1 + beta * zo.y, n2 + beta * zo.z);
    su = mk4<S>(wu.x + beta * so.x, wu.y + beta * so.y, wu.z + beta * so.z);
    pu = mk4<S>(uu.x + beta * po.x, uu.y + beta * po.y, uu.z + beta * po.z);
  }
  V4<S> xu = x[u];
  xu.x += alpha * pu.x;
  xu.y += alpha * pu.y;
  xu.z += alpha * pu.z;
  ru.x -= alpha * su.x;
  ru.y -= alpha * su.y;
  ru.z -= alpha * su.z;
  wu.x -= alpha * zu.x;
  wu.y -= alpha * zu.y;
  wu.z -= alpha * zu.z;
  z[u] = zu;
  sv[u] = su;
  p[u] = pu;
  x[u] = xu;
  r[u] = ru;
  w[u] = wu;
  mn[u] = block_jacobi<S>(dinv, u, wu.x, wu.y, wu.z);
  const V4<S> un = block_jacobi<S>(dinv, u, ru.x, ru.y, ru.z);
  part[0] = ru.x * un.x + ru.y * un.y + ru.z * un.z;
  part[1] = wu.x * un.x + wu.y * un.y + wu.z * un.z;
  part[2] = ru.x * ru.x + ru.y * ru.y + ru.z * ru.z;
}

// One solve of pipelined PCG.  On entry (pcg_setup): x = 0, r = b, z = M r.  z is read as u0 by the
// prologue only and then holds A M s (u = M r again after the switch to Chronopoulos-Gear); m has room
// for 2 nv vectors.
template <typename S, bool KRON>
__global__ void __launch_bounds__(SB, sizeof(S) == 4 ? 5 : 4)
    pipe_persistent_kernel(SellMatrix A, const S* __restrict__ vals, const V4<S>* __restrict__ dinv, V4<S>* x,
                           V4<S>* r, V4<S>* z, V4<S>* p, V4<S>* sv, V4<S>* w, V4<S>* m, int max_iters, Reduce red,
                           GridSync gs, int pipe_iters) {
  __shared__ double shred[SB / 32][3];
  __shared__ int sidx[SB / 32][ST_K][32];
  __shared__ double s_alpha, s_beta;
  __shared__ int s_done;
  DevScalars* sc = red.sc;
  if (threadIdx.x == 0) s_done = *(volatile int*)&sc->done;
  __syncthreads();
  if (s_done) return;
  const int nv = A.nv;
  const int nvb = (nv + SB - 1) / SB;
  double* part = red.partials;
  double* gsum = red.partials + 3 * (size_t)nvb;
  auto publish = [&](int vb, S (&pr)[3]) {
    double bs[3];
    block_sum_s<3, SB, S>(pr, bs, shred);
    if (threadIdx.x == 0) {
      part[3 * vb] = bs[0];
      part[3 * vb + 1] = bs[1];
      part[3 * vb + 2] = bs[2];
    }
    __syncthreads();
  };
  for (int vb = blockIdx.x; vb < nvb; vb += gridDim.x) {
    S pr[3];
    pipe_first_row<S, KRON>(A, vals, dinv, z, r, w, m, vb * SB + threadIdx.x, sidx[threadIdx.x >> 5], pr);
    publish(vb, pr);
  }
  bool ok = true;
  for (int k = 0;; ++k) {
    ok = reduce_barrier<3>(gs, (unsigned long long)k, part, gsum, nvb,
                           [&](const double (&t)[3]) { cgcg_after(sc, t[0], t[1], t[2], max_iters); });
    if (!ok) break;
    if (threadIdx.x == 0) {
      s_done = __ldcg(&sc->done);
      s_alpha = __ldcg(&sc->alpha);
      s_beta = __ldcg(&sc->beta);
    }
    __syncthreads();
    if (s_done) break;
    const S alpha = (S)s_alpha, beta = (S)s_beta;
    if (k < pipe_iters) {
      const V4<S>* mk = m + (size_t)(k & 1) * nv;
      V4<S>* mn = m + (size_t)((k + 1) & 1) * nv;
      for (int vb = blockIdx.x; vb < nvb; vb += gridDim.x) {
        S pr[3];
        pipe_row<S, KRON>(A, vals, dinv, k == 0, alpha, beta, mk, mn, x, r, z, p, sv, w, vb * SB + threadIdx.x,
                          sidx[threadIdx.x >> 5], pr);
        publish(vb, pr);
      }
      continue;
    }
    // Chronopoulos-Gear from here on: its phase B (u = M r, w the current A u), a plain barrier for u, its
    // phase A (w = A u and the dots)
    for (int vb = blockIdx.x; vb < nvb; vb += gridDim.x) {
      const int u = vb * SB + threadIdx.x;
      if (k == pipe_iters && u < nv) {
        const V4<S> ru = r[u];
        z[u] = block_jacobi<S>(dinv, u, ru.x, ru.y, ru.z);
      }
      cgcg_update_row<S>(nv, k == 0, alpha, beta, dinv, z, w, p, sv, x, r, u);
    }
    ok = plain_barrier(gs, (unsigned long long)(k - pipe_iters));
    if (!ok) break;
    for (int vb = blockIdx.x; vb < nvb; vb += gridDim.x) {
      S pr[3];
      cgcg_spmv_row<S, KRON>(A, vals, z, r, w, vb * SB + threadIdx.x, sidx[threadIdx.x >> 5], pr);
      publish(vb, pr);
    }
  }
  // a barrier wait gave up: flag it (the host clears the flag before the launch) and leave
  if (!ok && threadIdx.x == 0) atomicExch(&sc->wait_failed, 1);
}

// Pipelined PCG (pipe_persistent_kernel) on the FP16 copy, in its scaled space: the SpMV of m = M w reads the
// full FP16 entries, the third dot is (r, r) of the unscaled residual, and every block unscales its own rows
// of x after the last iteration.  After pipe_iters iterations it continues as Chronopoulos-Gear.
__device__ __forceinline__ void pipe_half_row(const HalfMatrix& H, const float4* __restrict__ dinv, bool first,
                                              float alpha, float beta, const float4* mk, float4* mn, float4* x,
                                              float4* r, float4* z, float4* p, float4* sv, float4* w, int u,
                                              int (*sidx)[32], float (&part)[3]) {
  part[0] = part[1] = part[2] = 0.f;
  if (u >= H.nv) return;
  float n0, n1, n2;
  half_row_product(H, u, mk, sidx, n0, n1, n2);
  float4 ru = r[u], wu = w[u];
  const float4 uu = block_jacobi<float>(dinv, u, ru.x, ru.y, ru.z);
  float4 zu = make_float4(n0, n1, n2, 0.f), su = wu, pu = uu;
  if (!first) {
    const float4 zo = z[u], so = sv[u], po = p[u];
    zu = make_float4(n0 + beta * zo.x, n1 + beta * zo.y, n2 + beta * zo.z, 0.f);
    su = make_float4(wu.x + beta * so.x, wu.y + beta * so.y, wu.z + beta * so.z, 0.f);
    pu = make_float4(uu.x + beta * po.x, uu.y + beta * po.y, uu.z + beta * po.z, 0.f);
  }
  float4 xu = x[u];
  xu.x += alpha * pu.x;
  xu.y += alpha * pu.y;
  xu.z += alpha * pu.z;
  ru.x -= alpha * su.x;
  ru.y -= alpha * su.y;
  ru.z -= alpha * su.z;
  wu.x -= alpha * zu.x;
  wu.y -= alpha * zu.y;
  wu.z -= alpha * zu.z;
  z[u] = zu;
  sv[u] = su;
  p[u] = pu;
  x[u] = xu;
  r[u] = ru;
  w[u] = wu;
  mn[u] = block_jacobi<float>(dinv, u, wu.x, wu.y, wu.z);
  const float4 un = block_jacobi<float>(dinv, u, ru.x, ru.y, ru.z);
  const float4 is = H.iscale[u];
  const float t0 = ru.x * is.x, t1 = ru.y * is.y, t2 = ru.z * is.z;
  part[0] = ru.x * un.x + ru.y * un.y + ru.z * un.z;
  part[1] = wu.x * un.x + wu.y * un.y + wu.z * un.z;
  part[2] = t0 * t0 + t1 * t1 + t2 * t2;
}

// The whole solve on the copy in one launch: the set-up (x = 0, r~ = S (sign b), u0 = M r~; a plain
// barrier orders u0 before the prologue's SpMV), the pipelined iterations (Chronopoulos-Gear after
// pipe_iters), x unscaled, and, when a.check is set, the solve's check on the FP32 symmetric store: g . x,
// |x|^2, |sign b - K x|^2 and |b|^2 (b = the Newton gradient g, sign = -1) into sc->gd, dnorm2, true_rr,
// true_bb.  Barriers are numbered by their own counters (the plain ones, the reducing ones) in the order
// every block meets them.
__global__ void __launch_bounds__(SB, 5)
    pipe_half_kernel(HalfMatrix H, const float4* __restrict__ dinv, float4* x, float4* r, float4* z, float4* p,
                     float4* sv, float4* w, float4* m, HalfSolveArgs a, Reduce red, GridSync gs) {
  __shared__ double shred[SB / 32][3];
  __shared__ double shred4[SB / 32][4];
  __shared__ int sidx[SB / 32][ST_K][32];
  __shared__ double s_alpha, s_beta;
  __shared__ int s_done;
  DevScalars* sc = red.sc;
  const int nv = H.nv;
  const int nvb = (nv + SB - 1) / SB;
  double* part = red.partials;
  double* gsum = red.partials + 3 * (size_t)nvb;
  double* gsum4 = red.partials + 4 * (size_t)nvb;
  auto publish = [&](int vb, float (&pr)[3]) {
    double bs[3];
    block_sum_s<3, SB, float>(pr, bs, shred);
    if (threadIdx.x == 0) {
      part[3 * vb] = bs[0];
      part[3 * vb + 1] = bs[1];
      part[3 * vb + 2] = bs[2];
    }
    __syncthreads();
  };
  const double sg = a.negate ? -1.0 : 1.0;
  unsigned long long npb = 0, nrb = 0;
  // set-up (pcg_setup_half_kernel's per-row work)
  for (int vb = blockIdx.x; vb < nvb; vb += gridDim.x) {
    const int u = vb * SB + threadIdx.x;
    if (u < nv) {
      const float r0 = (float)(sg * a.b[u * 3 + 0]), r1 = (float)(sg * a.b[u * 3 + 1]),
                  r2 = (float)(sg * a.b[u * 3 + 2]);
      const float4 s4 = H.scale[u];
      const float t0 = r0 * s4.x, t1 = r1 * s4.y, t2 = r2 * s4.z;
      x[u] = make_float4(0.f, 0.f, 0.f, 0.f);
      r[u] = make_float4(t0, t1, t2, 0.f);
      z[u] = block_jacobi<float>(dinv, u, t0, t1, t2);
      p[u] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
  }
  bool ok = plain_barrier(gs, npb++);
  // prologue: w = A u0, m_0 = M w, the first dots
  if (ok) {
    for (int vb = blockIdx.x; vb < nvb; vb += gridDim.x) {
      const int u = vb * SB + threadIdx.x;
      float pr[3] = {0.f, 0.f, 0.f};
      if (u < nv) {
        float a0, a1, a2;
        half_row_product(H, u, z, sidx[threadIdx.x >> 5], a0, a1, a2);
        w[u] = make_float4(a0, a1, a2, 0.f);
        m[u] = block_jacobi<float>(dinv, u, a0, a1, a2);
        const float4 uu = z[u], ru = r[u], is = H.iscale[u];
        const float t0 = ru.x * is.x, t1 = ru.y * is.y, t2 = ru.z * is.z;
        pr[0] = ru.x * uu.x + ru.y * uu.y + ru.z * uu.z;
        pr[1] = a0 * uu.x + a1 * uu.y + a2 * uu.z;
        pr[2] = t0 * t0 + t1 * t1 + t2 * t2;
      }
      publish(vb, pr);
    }
  }
  for (int k = 0; ok; ++k) {
    const bool first = k == 0;
    ok = reduce_barrier<3>(gs, nrb++, part, gsum, nvb, [&](const double (&t)[3]) {
      if (first) {  // the set-up's scalars: the stop test is relative to this residual
        sc->done = 0;
        sc->rz_old = 1.0;
        sc->rr0 = t[2];
        sc->tol2 = a.rtol * a.rtol * t[2];
        sc->iters = 0;
        sc->status = 0;
      }
      cgcg_after(sc, t[0], t[1], t[2], a.max_iters);
    });
    if (!ok) break;
    if (threadIdx.x == 0) {
      s_done = __ldcg(&sc->done);
      s_alpha = __ldcg(&sc->alpha);
      s_beta = __ldcg(&sc->beta);
    }
    __syncthreads();
    if (s_done) break;
    const float alpha = (float)s_alpha, beta = (float)s_beta;
    if (k < a.pipe_iters) {
      const float4* mk = m + (size_t)(k & 1) * nv;
      float4* mn = m + (size_t)((k + 1) & 1) * nv;
      for (int vb = blockIdx.x; vb < nvb; vb += gridDim.x) {
        float pr[3];
        pipe_half_row(H, dinv, k == 0, alpha, beta, mk, mn, x, r, z, p, sv, w, vb * SB + threadIdx.x,
                      sidx[threadIdx.x >> 5], pr);
        publish(vb, pr);
      }
      continue;
    }
    // Chronopoulos-Gear from here on (as pipe_persistent_kernel)
    for (int vb = blockIdx.x; vb < nvb; vb += gridDim.x) {
      const int u = vb * SB + threadIdx.x;
      if (k == a.pipe_iters && u < nv) {
        const float4 ru = r[u];
        z[u] = block_jacobi<float>(dinv, u, ru.x, ru.y, ru.z);
      }
      cgcg_update_row<float>(nv, k == 0, alpha, beta, dinv, z, w, p, sv, x, r, u);
    }
    ok = plain_barrier(gs, npb++);
    if (!ok) break;
    for (int vb = blockIdx.x; vb < nvb; vb += gridDim.x) {
      const int u = vb * SB + threadIdx.x;
      float pr[3] = {0.f, 0.f, 0.f};
      if (u < nv) {
        float a0, a1, a2;
        half_row_product(H, u, z, sidx[threadIdx.x >> 5], a0, a1, a2);
        w[u] = make_float4(a0, a1, a2, 0.f);
        const float4 uu = z[u], ru = r[u], is = H.iscale[u];
        const float t0 = ru.x * is.x, t1 = ru.y * is.y, t2 = ru.z * is.z;
        pr[0] = ru.x * uu.x + ru.y * uu.y + ru.z * uu.z;
        pr[1] = a0 * uu.x + a1 * uu.y + a2 * uu.z;
        pr[2] = t0 * t0 + t1 * t1 + t2 * t2;
      }
      publish(vb, pr);
    }
  }
  // x = S x~ (rows of this block only)
  for (int vb = blockIdx.x; vb < nvb; vb += gridDim.x) {
    const int u = vb * SB + threadIdx.x;
    if (u < nv) {
      const float4 xv = x[u], s4 = H.scale[u];
      x[u] = make_float4(xv.x * s4.x, xv.y * s4.y, xv.z * s4.z, 0.f);
    }
  }
  // the check on the FP32 values: every block's x is final after a plain barrier
  if (ok && a.check) ok = plain_barrier(gs, npb++);
  if (ok && a.check) {
    for (int vb = blockIdx.x; vb < nvb; vb += gridDim.x) {
      const int u = vb * SB + threadIdx.x;
      double pr[4] = {0, 0, 0, 0};
      if (u < nv) {
        float a0, a1, a2;
        row_product_t<float, true>(a.A32, a.vals32, u, x, nullptr, 0.f, sidx[threadIdx.x >> 5], a0, a1, a2);
        const float4 dv = x[u];
        const double g0 = a.b[u * 3 + 0], g1 = a.b[u * 3 + 1], g2 = a.b[u * 3 + 2];
        pr[0] = g0 * (double)dv.x + g1 * (double)dv.y + g2 * (double)dv.z;
        pr[1] = (double)dv.x * dv.x + (double)dv.y * dv.y + (double)dv.z * dv.z;
        const double q0 = sg * g0 - (double)a0, q1 = sg * g1 - (double)a1, q2 = sg * g2 - (double)a2;
        pr[2] = q0 * q0 + q1 * q1 + q2 * q2;
        pr[3] = g0 * g0 + g1 * g1 + g2 * g2;
      }
      block_sum<4, SB>(pr, shred4);
      if (threadIdx.x == 0) {
#pragma unroll
        for (int c = 0; c < 4; ++c) part[4 * vb + c] = pr[c];
      }
      __syncthreads();
    }
    ok = reduce_barrier<4>(gs, nrb++, part, gsum4, nvb, [&](const double (&t)[4]) {
      sc->gd = t[0];
      sc->dnorm2 = t[1];
      sc->true_rr = t[2];
      sc->true_bb = t[3];
    });
  }
  if (!ok && threadIdx.x == 0) atomicExch(&sc->wait_failed, 1);
}

// Standard PCG in one launch: the two-launch loop's phases (SpMV forming p = z + beta p_old, then the
// update) separated by reducing grid barriers; the last block runs the same reductions and epilogues as
// the two-launch kernels, so the iterates are bitwise theirs.
template <typename S, bool KRON>
__global__ void __launch_bounds__(SB, sizeof(S) == 4 ? 5 : 4)
    pcg_persistent_kernel(SellMatrix A, const S* __restrict__ vals, const V4<S>* __restrict__ dinv, V4<S>* x,
                          V4<S>* r, V4<S>* z, V4<S>* p0, V4<S>* p1, V4<S>* q, int max_iters, Reduce red,
                          GridSync gs) {
  __shared__ double shred[SB / 32][2];
  __shared__ int sidx[SB / 32][ST_K][32];
  __shared__ double s_coef;  // beta for the SpMV phase, alpha for the update phase
  __shared__ int s_done;
  DevScalars* sc = red.sc;
  if (threadIdx.x == 0) s_done = *(volatile int*)&sc->done;
  __syncthreads();
  if (s_done) return;
  const int nvb = (A.nv + SB - 1) / SB;
  double* part_pq = red.partials;
  double* part_rz = red.partials + 2 * (size_t)nvb;
  double* gsum = red.partials + 4 * (size_t)nvb;
  bool ok = true;
  for (int k = 0;; ++k) {
    V4<S>* pold = (k & 1) ? p1 : p0;
    V4<S>* pnew = (k & 1) ? p0 : p1;
    const S beta = k == 0 ? S(0) : (S)s_coef;
    for (int vb = blockIdx.x; vb < nvb; vb += gridDim.x) {
      S part[1] = {pcg_spmv_row<S, KRON>(A, vals, z, pold, pnew, q, beta, vb * SB + threadIdx.x,
                                         sidx[threadIdx.x >> 5])};
      double v1[1];
      block_sum_s<1, SB, S>(part, v1, reinterpret_cast<double(*)[1]>(shred));
      if (threadIdx.x == 0) part_pq[vb] = v1[0];
      __syncthreads();
    }
    ok = reduce_barrier<1>(gs, 2ull * k, part_pq, gsum, nvb, [&](const double (&t)[1]) { pcg_after_pq(sc, t[0]); });
    if (!ok) break;
    if (threadIdx.x == 0) {
      s_done = __ldcg(&sc->done);
      s_coef = __ldcg(&sc->alpha);
    }
    __syncthreads();
    if (s_done) break;
    const S alpha = (S)s_coef;
    for (int vb = blockIdx.x; vb < nvb; vb += gridDim.x) {
      S part[2];
      pcg_update_row<S>(A.nv, pnew, q, dinv, x, r, z, alpha, vb * SB + threadIdx.x, part);
      double bs[2];
      block_sum_s<2, SB, S>(part, bs, shred);
      if (threadIdx.x == 0) {
        part_rz[2 * vb] = bs[0];
        part_rz[2 * vb + 1] = bs[1];
      }
      __syncthreads();
    }
    ok = reduce_barrier<2>(gs, 2ull * k + 1, part_rz, gsum, nvb,
                           [&](const double (&t)[2]) { pcg_after_rz(sc, t[0], t[1], max_iters); });
    if (!ok) break;
    if (threadIdx.x == 0) {
      s_done = __ldcg(&sc->done);
      s_coef = __ldcg(&sc->beta);
    }
    __syncthreads();
    if (s_done) break;
  }
  // a barrier wait gave up: flag it (the host clears the flag before the launch) and leave
  if (!ok && threadIdx.x == 0) atomicExch(&sc->wait_failed, 1);
}

// ------------------------------------------------------------------ scalar CSR on 4-wide vectors
// y = A x for a scalar CSR matrix over dofs (row / column i = vertex i / 3, component i % 3), x and y in the
// solver's 4-wide vertex layout; one thread per row, entries in CSR order (the NCG preconditioner factor).
template <typename S>
__global__ void __launch_bounds__(SB)
    csr_dof_spmv_kernel(int n, const int* __restrict__ rp, const int* __restrict__ ci, const S* __restrict__ vals,
                        const V4<S>* __restrict__ x, V4<S>* __restrict__ y) {
  const int r = blockIdx.x * SB + threadIdx.x;
  if (r >= n) return;
  const S* xs = reinterpret_cast<const S*>(x);
  S acc = S(0);
  const int k1 = rp[r + 1];
  for (int k = rp[r]; k < k1; ++k) {
    const int c = ci[k];
    acc += vals[k] * xs[4 * (c / 3) + c % 3];
  }
  reinterpret_cast<S*>(y)[4 * (r / 3) + r % 3] = acc;
}

// ------------------------------------------------------------------ vectors
template <typename S>
__global__ void __launch_bounds__(SB)
    dot_gd_kernel(int nv, const double* __restrict__ g, const V4<S>* __restrict__ d, Reduce red) {
  __shared__ double shred[SB / 32][2];
  const int u = blockIdx.x * SB + threadIdx.x;
  double part[2] = {0, 0};
  if (u < nv) {
    const V4<S> dv = d[u];
    part[0] = g[u * 3 + 0] * (double)dv.x + g[u * 3 + 1] * (double)dv.y + g[u * 3 + 2] * (double)dv.z;
    part[1] = (double)dv.x * dv.x + (double)dv.y * dv.y + (double)dv.z * dv.z;
  }
  block_sum<2, SB>(part, shred);
  double tot[2];
  if (grid_sum_last<2, SB>(part, red.partials, red.counter, tot)) {
    red.sc->gd = tot[0];
    red.sc->dnorm2 = tot[1];
  }
}

// g . d and |d|^2 as dot_gd_kernel, with the solve's TRUE residual on the FP32 values: |-g - K d|^2 and |g|^2
// (the check of a solve that ran on the FP16 copy of the scaled matrix)
__global__ void __launch_bounds__(SB)
    dot_gd_check_kernel(SellMatrix A, const float* __restrict__ vals, const double* __restrict__ g,
                        const float4* __restrict__ d, Reduce red) {
  __shared__ double shred[SB / 32][4];
  __shared__ int sidx[SB / 32][ST_K][32];
  const int u = blockIdx.x * SB + threadIdx.x;
  double part[4] = {0, 0, 0, 0};
  if (u < A.nv) {
    float a0, a1, a2;
    row_product_t<float, true>(A, vals, u, d, nullptr, 0.f, sidx[threadIdx.x >> 5], a0, a1, a2);
    const float4 dv = d[u];
    const double g0 = g[u * 3 + 0], g1 = g[u * 3 + 1], g2 = g[u * 3 + 2];
    part[0] = g0 * (double)dv.x + g1 * (double)dv.y + g2 * (double)dv.z;
    part[1] = (double)dv.x * dv.x + (double)dv.y * dv.y + (double)dv.z * dv.z;
    const double r0 = -g0 - (double)a0, r1 = -g1 - (double)a1, r2 = -g2 - (double)a2;
    part[2] = r0 * r0 + r1 * r1 + r2 * r2;
    part[3] = g0 * g0 + g1 * g1 + g2 * g2;
  }
  block_sum<4, SB>(part, shred);
  double tot[4];
  if (grid_sum_last<4, SB>(part, red.partials, red.counter, tot)) {
    red.sc->gd = tot[0];
    red.sc->dnorm2 = tot[1];
    red.sc->true_rr = tot[2];
    red.sc->true_bb = tot[3];
  }
}

// the FP32 positions of u + d: what axpy_update_kernel (alpha = 1) and refresh_xf_kernel make after a full
// step, bit for bit (u + 1.0 d rounds once, as the fused multiply-add there does)
template <typename S>
__global__ void full_step_xf_kernel(int nv, const V4<S>* __restrict__ d, const double* __restrict__ X,
                                    const double* __restrict__ u, float4* __restrict__ xf) {
  const int v = blockIdx.x * SB + threadIdx.x;
  if (v >= nv) return;
  const V4<S> dv = d[v];
  const double u0 = u[v * 3 + 0] + (double)dv.x;
  const double u1 = u[v * 3 + 1] + (double)dv.y;
  const double u2 = u[v * 3 + 2] + (double)dv.z;
  xf[v] = make_float4((float)(X[v * 3 + 0] + u0), (float)(X[v * 3 + 1] + u1), (float)(X[v * 3 + 2] + u2), 0.f);
}

template <typename S>
__global__ void axpy_update_kernel(int nv, double alpha, const V4<S>* __restrict__ d, const double* __restrict__ X,
                                   double* __restrict__ u, float4* __restrict__ xf) {
  const int v = blockIdx.x * SB + threadIdx.x;
  if (v >= nv) return;
  const V4<S> dv = d[v];
  const double u0 = u[v * 3 + 0] + alpha * (double)dv.x;
  const double u1 = u[v * 3 + 1] + alpha * (double)dv.y;
  const double u2 = u[v * 3 + 2] + alpha * (double)dv.z;
  u[v * 3 + 0] = u0;
  u[v * 3 + 1] = u1;
  u[v * 3 + 2] = u2;
  if (xf != nullptr)
    xf[v] = make_float4((float)(X[v * 3 + 0] + u0), (float)(X[v * 3 + 1] + u1), (float)(X[v * 3 + 2] + u2), 0.f);
}

__global__ void refresh_xf_kernel(int nv, const double* __restrict__ X, const double* __restrict__ u,
                                  float4* __restrict__ xf) {
  const int v = blockIdx.x * SB + threadIdx.x;
  if (v >= nv) return;
  xf[v] = make_float4((float)(X[v * 3 + 0] + u[v * 3 + 0]), (float)(X[v * 3 + 1] + u[v * 3 + 1]),
                      (float)(X[v * 3 + 2] + u[v * 3 + 2]), 0.f);
}

// prepare_step (time_step.hpp:499-518): x~ = u + dt v + dt^2 a, Dirichlet values, next = x~
__global__ void prepare_step_kernel(int n, double dt, const double* __restrict__ u, const double* __restrict__ v,
                                    const double* __restrict__ a, const int8_t* __restrict__ dof_type,
                                    const double* __restrict__ dbc, double* __restrict__ xt,
                                    double* __restrict__ next) {
  const int i = blockIdx.x * SB + threadIdx.x;
  if (i >= n) return;
  double x = u[i] + dt * v[i];
  x = x + (dt * dt) * a[i];
  if (dof_type[i] == 1) x = dbc[i];
  xt[i] = x;
  next[i] = x;
}

// step_next (time_step.hpp:530-543)
__global__ void step_next_kernel(int n, double inv_dt, double keep, double* __restrict__ prev,
                                 double* __restrict__ u, const double* __restrict__ next, double* __restrict__ v) {
  const int i = blockIdx.x * SB + threadIdx.x;
  if (i >= n) return;
  const double uo = u[i], un = next[i];
  prev[i] = uo;
  u[i] = un;
  v[i] = ((un - uo) * inv_dt) * keep;
}

// restore (time_step.hpp:560-569)
__global__ void restore_kernel(int n, double inv_dt, const int8_t* __restrict__ dof_type,
                               const double* __restrict__ dbc, double* __restrict__ prev, double* __restrict__ u,
                               double* __restrict__ v) {
  const int i = blockIdx.x * SB + threadIdx.x;
  if (i >= n) return;
  if (dof_type[i] == 1) {
    prev[i] = dbc[i];
    u[i] = dbc[i];
  }
  v[i] = (u[i] - prev[i]) * inv_dt;
}

__global__ void axpy_d_kernel(int n, double a, const double* __restrict__ x, double* __restrict__ y) {
  const int i = blockIdx.x * SB + threadIdx.x;
  if (i < n) y[i] += a * x[i];
}

__global__ void add_ext_kernel(int nv, int dof, double val, double* __restrict__ a) {
  const int v = blockIdx.x * SB + threadIdx.x;
  if (v < nv) a[v * 3 + dof] += val;
}

// mark_dirichlet_batched / mark_general_batched (fem_cuda.cu:115-150)
__global__ void mark_dofs_kernel(int n, const int* __restrict__ verts, const double* __restrict__ targ, int dirichlet,
                                 int8_t* __restrict__ dof_type, double* __restrict__ dbc) {
  const int i = blockIdx.x * SB + threadIdx.x;
  if (i >= n) return;
  const int v = verts[i];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    dof_type[v * 3 + k] = dirichlet ? 1 : 0;
    dbc[v * 3 + k] = dirichlet ? targ[i * 3 + k] : 0.0;
  }
}

__global__ void build_mask_kernel(int nv, const int8_t* __restrict__ dof_type, uint8_t* __restrict__ mask) {
  const int v = blockIdx.x * SB + threadIdx.x;
  if (v >= nv) return;
  mask[v] = (uint8_t)((dof_type[v * 3 + 0] == 1 ? 1 : 0) | (dof_type[v * 3 + 1] == 1 ? 2 : 0) |
                      (dof_type[v * 3 + 2] == 1 ? 4 : 0));
}

template <typename S>
__global__ void __launch_bounds__(SB)
    vdot_kernel(int nv, const V4<S>* __restrict__ a, const V4<S>* __restrict__ b, double* out, Reduce red) {
  __shared__ double shred[SB / 32][1];
  const int u = blockIdx.x * SB + threadIdx.x;
  S part[1] = {S(0)};
  if (u < nv) {
    const V4<S> x = a[u], y = b[u];
    part[0] = x.x * y.x + x.y * y.y + x.z * y.z;
  }
  double v1[1];
  block_sum_s<1, SB, S>(part, v1, shred);
  double tot[1];
  if (grid_sum_last<1, SB>(v1, red.partials, red.counter, tot)) *out = tot[0];
}

template <typename S>
__global__ void vaxpby_kernel(int nv, S alpha, V4<S>* __restrict__ y, S beta, const V4<S>* __restrict__ x) {
  const int u = blockIdx.x * SB + threadIdx.x;
  if (u >= nv) return;
  const V4<S> xv = x[u];
  V4<S> yv = y[u];
  yv.x = alpha * yv.x + beta * xv.x;
  yv.y = alpha * yv.y + beta * xv.y;
  yv.z = alpha * yv.z + beta * xv.z;
  y[u] = yv;
}

template <typename S>
__global__ void vdiff_kernel(int nv, const double* __restrict__ a, const double* __restrict__ b, V4<S>* __restrict__ y) {
  const int u = blockIdx.x * SB + threadIdx.x;
  if (u >= nv) return;
  y[u] = mk4<S>((S)(a[3 * u] - b[3 * u]), (S)(a[3 * u + 1] - b[3 * u + 1]), (S)(a[3 * u + 2] - b[3 * u + 2]));
}

template <typename S>
__global__ void __launch_bounds__(SB)
    pcg_setup_v_kernel(int nv, const V4<S>* __restrict__ bv, const V4<S>* __restrict__ dinv, V4<S>* __restrict__ x,
                       V4<S>* __restrict__ r, V4<S>* __restrict__ z, V4<S>* __restrict__ p0, double rtol,
                       int max_iters, Reduce red) {
  __shared__ double shred[SB / 32][2];
  const int u = blockIdx.x * SB + threadIdx.x;
  S part[2] = {S(0), S(0)};
  if (u < nv) {
    const V4<S> rb = bv[u];
    const V4<S> d0 = dinv[3 * u], d1 = dinv[3 * u + 1], d2 = dinv[3 * u + 2];
    const S z0 = d0.x * rb.x + d0.y * rb.y + d0.z * rb.z;
    const S z1 = d1.x * rb.x + d1.y * rb.y + d1.z * rb.z;
    const S z2 = d2.x * rb.x + d2.y * rb.y + d2.z * rb.z;
    x[u] = mk4<S>(0, 0, 0);
    r[u] = mk4<S>(rb.x, rb.y, rb.z);
    z[u] = mk4<S>(z0, z1, z2);
    p0[u] = mk4<S>(0, 0, 0);
    part[0] = rb.x * z0 + rb.y * z1 + rb.z * z2;
    part[1] = rb.x * rb.x + rb.y * rb.y + rb.z * rb.z;
  }
  double bs[2];
  block_sum_s<2, SB, S>(part, bs, shred);
  double tot[2];
  if (grid_sum_last<2, SB>(bs, red.partials, red.counter, tot)) {
    DevScalars* sc = red.sc;
    sc->rz = tot[0];
    sc->rz_old = 1.0;
    sc->rr = tot[1];
    sc->rr0 = tot[1];
    sc->tol2 = rtol * rtol * tot[1];
    sc->iters = 0;
    sc->status = 0;
    sc->done = (tot[1] <= sc->tol2 || tot[1] == 0.0 || max_iters <= 0) ? 1 : 0;
  }
}

__global__ void __launch_bounds__(SB)
    instance_norms_kernel(const int* __restrict__ voff, const double* __restrict__ g, double* __restrict__ out) {
  __shared__ double shred[SB / 32][1];
  const int i = blockIdx.x;
  const long long a = 3LL * voff[i], b = 3LL * voff[i + 1];
  double part = 0;
  for (long long k = a + threadIdx.x; k < b; k += SB) part += g[k] * g[k];
  double v1[1] = {part};
  block_sum<1, SB>(v1, shred);
  if (threadIdx.x == 0) out[i] = v1[0];
}

template <typename S>
__global__ void to_vec4_kernel(int nv, const double* __restrict__ in, V4<S>* __restrict__ out, int negate) {
  const int v = blockIdx.x * SB + threadIdx.x;
  if (v >= nv) return;
  const double s = negate ? -1.0 : 1.0;
  out[v] = mk4<S>((S)(s * in[v * 3 + 0]), (S)(s * in[v * 3 + 1]), (S)(s * in[v * 3 + 2]));
}

template <typename S>
__global__ void from_vec4_kernel(int nv, const V4<S>* __restrict__ in, double* __restrict__ out) {
  const int v = blockIdx.x * SB + threadIdx.x;
  if (v >= nv) return;
  const V4<S> x = in[v];
  out[v * 3 + 0] = (double)x.x;
  out[v * 3 + 1] = (double)x.y;
  out[v * 3 + 2] = (double)x.z;
}

}  // namespace

// one value per slot for a matrix whose blocks are all multiples of I3 (the projective-dynamics matrix
// (M + dt^2 kappa L) (x) I3, Dirichlet rows included): the SpMV then reads 4 bytes per block instead of 36
template <typename S>
__global__ void __launch_bounds__(SB)
    kron_extract_kernel(int nslots, const S* __restrict__ vals, S* __restrict__ svals, int* not_kron) {
  const int q = blockIdx.x * SB + threadIdx.x;
  if (q >= nslots) return;
  const size_t b = sell_base(q);
  S v[9];
#pragma unroll
  for (int c = 0; c < 9; ++c) v[c] = vals[b + 32 * c];
  svals[q] = v[0];
  if (v[1] != S(0) || v[2] != S(0) || v[3] != S(0) || v[5] != S(0) || v[6] != S(0) || v[7] != S(0) ||
      v[4] != v[0] || v[8] != v[0])
    atomicOr(not_kron, 1);
}

// ------------------------------------------------------------------ launchers
template <typename S>
void launch_kron_extract(const SellMatrix& A, const S* vals, S* svals, int* not_kron, cudaStream_t st) {
  if (A.nslots <= 0) return;
  kron_extract_kernel<S><<<div_up(A.nslots, SB), SB, 0, st>>>(A.nslots, vals, svals, not_kron);
  after_launch("kron_extract");
}

template <typename S>
void launch_assemble(const SellMatrix& A, const int* cptr, const int* csrc, const S* Kbuf, const S* slot_mass,
                     const uint8_t* mask, bool filter, S* vals, V4<S>* dinv, int precond, cudaStream_t st,
                     int block) {
  if (A.nslots <= 0) return;
  auto go = [&](auto Bc) {
    constexpr int b = decltype(Bc)::value;
    assemble_kernel<S, b><<<div_up(A.nslots, b), b, 0, st>>>(A, cptr, csrc, Kbuf, slot_mass, mask, filter ? 1 : 0,
                                                             vals, dinv, precond);
  };
  dispatch_block<128, 256, 512>(block == 0 ? SB : block, go);
  after_launch("assemble");
}

void launch_assemble16(const SellMatrix& A, const int* cptr, const int* csrc, const uint2* K16, const float* slot_mass,
                       const uint8_t* mask, bool filter, float* vals, float4* dinv, int precond, cudaStream_t st,
                       int block) {
  if (A.nslots <= 0) return;
  const float* kb = reinterpret_cast<const float*>(K16);
  auto go = [&](auto Bc) {
    constexpr int b = decltype(Bc)::value;
    assemble_kernel<float, b, true><<<div_up(A.nslots, b), b, 0, st>>>(A, cptr, csrc, kb, slot_mass, mask,
                                                                        filter ? 1 : 0, vals, dinv, precond);
  };
  dispatch_block<128, 256, 512>(block == 0 ? SB : block, go);
  after_launch("assemble16");
}

template <typename S>
void launch_spmv(const SellMatrix& A, const S* vals, const V4<S>* x, V4<S>* y, cudaStream_t st) {
  if (A.nv <= 0) return;
  spmv_kernel<S><<<div_up(A.nv, SB), SB, 0, st>>>(A, vals, x, y);
  after_launch("spmv");
}

template <typename S>
void launch_export_csr(const SellMatrix& A, const int* bptr, const int* slot_k, const int* slot_kt, const S* vals,
                       double* csr_vals, cudaStream_t st) {
  if (A.nslots <= 0) return;
  export_csr_kernel<S><<<div_up(A.nslots, SB), SB, 0, st>>>(A, bptr, slot_k, slot_kt, vals, csr_vals);
  after_launch("export_csr");
}

template <typename S>
void launch_pcg_setup(int nv, const double* g, const V4<S>* dinv, V4<S>* x, V4<S>* r, V4<S>* z, V4<S>* p0,
                      double rtol, int max_iters, bool rhs_negate, const Reduce& red, cudaStream_t st) {
  pcg_setup_kernel<S><<<div_up(nv, SB), SB, 0, st>>>(nv, g, dinv, x, r, z, p0, rtol, max_iters, rhs_negate ? 1 : 0,
                                                     red);
  after_launch("pcg_setup");
}

template <typename S>
void launch_pcg_spmv(const SellMatrix& A, const S* vals, const V4<S>* z, const V4<S>* p_old, V4<S>* p_new,
                     V4<S>* q, bool first, const Reduce& red, cudaStream_t st, bool kron) {
  if (kron)
    pcg_spmv_kernel<S, true><<<div_up(A.nv, SB), SB, 0, st>>>(A, vals, z, p_old, p_new, q, first ? 1 : 0, red);
  else
    pcg_spmv_kernel<S, false><<<div_up(A.nv, SB), SB, 0, st>>>(A, vals, z, p_old, p_new, q, first ? 1 : 0, red);
  after_launch("pcg_spmv");
}

size_t grid_sync_words(int nv) { return (size_t)kSyncStride * (4 + ((size_t)div_up(nv, SB) + 31) / 32); }

template <typename S>
bool launch_pcg_persistent(const SellMatrix& A, const S* vals, const V4<S>* dinv, V4<S>* x, V4<S>* r, V4<S>* z,
                           V4<S>* p0, V4<S>* p1, V4<S>* q, int max_iters, const Reduce& red, unsigned long long* gsync,
                           long long spin_limit, int extra, int max_blocks, int variant, cudaStream_t st, bool kron,
                           V4<S>* pm, int pipe_iters) {
  int dev = 0, coop = 0, nsm = 0, per_sm = 0;
  SSIM_CUDA(cudaGetDevice(&dev));
  SSIM_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
  if (!coop) return false;
  if (variant == 4 && pm == nullptr) return false;
  SSIM_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const void* fn = variant == 4   ? (kron ? (const void*)pipe_persistent_kernel<S, true>
                                          : (const void*)pipe_persistent_kernel<S, false>)
                   : variant == 2 ? (kron ? (const void*)cgcg_persistent_kernel<S, true>
                                          : (const void*)cgcg_persistent_kernel<S, false>)
                                  : (kron ? (const void*)pcg_persistent_kernel<S, true>
                                          : (const void*)pcg_persistent_kernel<S, false>);
  SSIM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, SB, 0));
  if (per_sm < 1) return false;
  int grid = std::min(div_up(A.nv, SB), per_sm * nsm);
  if (max_blocks > 0) grid = std::min(grid, max_blocks);
  if (grid < 1) return true;
  const int ngroups = (div_up(A.nv, SB) + 31) / 32;
  SSIM_CUDA(cudaMemsetAsync(gsync, 0, grid_sync_words(A.nv) * sizeof(unsigned long long), st));
  SSIM_CUDA(cudaMemsetAsync(&red.sc->wait_failed, 0, sizeof(int32_t), st));
  GridSync gs{gsync,
              gsync + kSyncStride,
              gsync + 2 * kSyncStride,
              gsync + 4 * kSyncStride,
              ngroups,
              (unsigned int)extra,
              spin_limit > 0 ? spin_limit : (1LL << 25),
              gsync + 3 * kSyncStride};
  SellMatrix a = A;
  Reduce rd = red;
  void* args[] = {(void*)&a,  (void*)&vals, (void*)&dinv, (void*)&x,         (void*)&r,  (void*)&z,
                  (void*)&p0, (void*)&p1,   (void*)&q,    (void*)&max_iters, (void*)&rd, (void*)&gs};
  // pipelined: p = p0, s = p1, w = q, then the two m vectors
  void* pargs[] = {(void*)&a,  (void*)&vals, (void*)&dinv, (void*)&x,         (void*)&r,  (void*)&z,  (void*)&p0,
                   (void*)&p1, (void*)&q,    (void*)&pm,   (void*)&max_iters, (void*)&rd, (void*)&gs, (void*)&pipe_iters};
  SSIM_CUDA(cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(SB), variant == 4 ? pargs : args, 0, st));
  after_launch("pcg_persistent");
  return true;
}

void launch_half_prepare(const SellMatrix& A, const float* vals, int precond, float4* scale, float4* iscale,
                         float4* dinv16, cudaStream_t st) {
  if (A.nv <= 0) return;
  half_prepare_kernel<<<div_up(A.nv, SB), SB, 0, st>>>(A, vals, precond, scale, iscale, dinv16);
  after_launch("half_prepare");
}

void launch_half_convert(const SellMatrix& A, const int* off, const int* col, const int* src, const float* vals,
                         const float4* scale, uint4* v8, uint16_t* v1, cudaStream_t st) {
  if (A.nv <= 0) return;
  half_convert_kernel<<<div_up(A.nv, SB), SB, 0, st>>>(A.nv, off, col, src, vals, scale, v8, v1);
  after_launch("half_convert");
}

void launch_pcg_setup_half(const HalfMatrix& H, const double* b, const float4* dinv16, float4* x, float4* r, float4* z,
                           float4* p0, double rtol, int max_iters, bool negate, const Reduce& red, cudaStream_t st) {
  if (H.nv <= 0) return;
  pcg_setup_half_kernel<<<div_up(H.nv, SB), SB, 0, st>>>(H, b, dinv16, x, r, z, p0, rtol, max_iters, negate ? 1 : 0,
                                                          red);
  after_launch("pcg_setup_half");
}

void launch_half_spmv(const HalfMatrix& H, const float4* x, float4* xs, float4* y, cudaStream_t st) {
  if (H.nv <= 0) return;
  half_spmv_kernel<<<div_up(H.nv, SB), SB, 0, st>>>(H, x, xs, y, 0);
  half_spmv_kernel<<<div_up(H.nv, SB), SB, 0, st>>>(H, x, xs, y, 1);
  after_launch("half_spmv");
}

bool launch_pcg_half(const HalfMatrix& H, const float4* dinv16, float4* x, float4* r, float4* z, float4* p0,
                     float4* p1, float4* q, int max_iters, const Reduce& red, unsigned long long* gsync,
                     long long spin_limit, int extra, int max_blocks, cudaStream_t st, float4* pm,
                     const HalfSolveArgs* pa) {
  int dev = 0, coop = 0, nsm = 0, per_sm = 0;
  SSIM_CUDA(cudaGetDevice(&dev));
  SSIM_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
  if (!coop) return false;
  SSIM_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const bool pipe = pm != nullptr && pa != nullptr;
  const void* fn = pipe ? (const void*)pipe_half_kernel : (const void*)cgcg_half_kernel;
  SSIM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, SB, 0));
  if (per_sm < 1) return false;
  int grid = std::min(div_up(H.nv, SB), per_sm * nsm);
  if (max_blocks > 0) grid = std::min(grid, max_blocks);
  if (grid < 1) return true;
  const int ngroups = (div_up(H.nv, SB) + 31) / 32;
  SSIM_CUDA(cudaMemsetAsync(gsync, 0, grid_sync_words(H.nv) * sizeof(unsigned long long), st));
  SSIM_CUDA(cudaMemsetAsync(&red.sc->wait_failed, 0, sizeof(int32_t), st));
  GridSync gs{gsync,
              gsync + kSyncStride,
              gsync + 2 * kSyncStride,
              gsync + 4 * kSyncStride,
              ngroups,
              (unsigned int)extra,
              spin_limit > 0 ? spin_limit : (1LL << 25),
              gsync + 3 * kSyncStride};
  HalfMatrix h = H;
  Reduce rd = red;
  void* args[] = {(void*)&h,  (void*)&dinv16, (void*)&x, (void*)&r,         (void*)&z,  (void*)&p0,
                  (void*)&p1, (void*)&q,      (void*)&max_iters, (void*)&rd, (void*)&gs};
  // pipelined: p = p0, s = p1, w = q, then the two m vectors
  HalfSolveArgs ha{};
  if (pa) ha = *pa;
  void* pargs[] = {(void*)&h, (void*)&dinv16, (void*)&x,  (void*)&r,  (void*)&z, (void*)&p0,
                   (void*)&p1, (void*)&q,     (void*)&pm, (void*)&ha, (void*)&rd, (void*)&gs};
  SSIM_CUDA(cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(SB), pipe ? pargs : args, 0, st));
  after_launch("pcg_half");
  return true;
}

template <typename S>
void launch_csr_dof_spmv(int n, const int* rp, const int* ci, const S* vals, const V4<S>* x, V4<S>* y,
                         cudaStream_t st) {
  if (n <= 0) return;
  csr_dof_spmv_kernel<S><<<div_up(n, SB), SB, 0, st>>>(n, rp, ci, vals, x, y);
  after_launch("csr_dof_spmv");
}

template <typename S>
void launch_pcg_update(int nv, const V4<S>* p, const V4<S>* q, const V4<S>* dinv, V4<S>* x, V4<S>* r, V4<S>* z,
                       int max_iters, const Reduce& red, cudaStream_t st) {
  pcg_update_kernel<S><<<div_up(nv, SB), SB, 0, st>>>(nv, p, q, dinv, x, r, z, max_iters, red);
  after_launch("pcg_update");
}

template <typename S>
void launch_dot_gd(int nv, const double* g, const V4<S>* d, const Reduce& red, cudaStream_t st) {
  dot_gd_kernel<S><<<div_up(nv, SB), SB, 0, st>>>(nv, g, d, red);
  after_launch("dot_gd");
}

void launch_dot_gd_check(const SellMatrix& A, const float* vals, const double* g, const float4* d, const Reduce& red,
                         cudaStream_t st) {
  if (A.nv <= 0) return;
  dot_gd_check_kernel<<<div_up(A.nv, SB), SB, 0, st>>>(A, vals, g, d, red);
  after_launch("dot_gd_check");
}

template <typename S>
void launch_axpy_update(int nv, double alpha, const V4<S>* d, const double* X, double* u, float4* xf,
                        cudaStream_t st) {
  axpy_update_kernel<S><<<div_up(nv, SB), SB, 0, st>>>(nv, alpha, d, X, u, xf);
  after_launch("axpy_update");
}

template <typename S>
void launch_full_step_xf(int nv, const V4<S>* d, const double* X, const double* u, float4* xf, cudaStream_t st) {
  if (nv <= 0) return;
  full_step_xf_kernel<S><<<div_up(nv, SB), SB, 0, st>>>(nv, d, X, u, xf);
  after_launch("full_step_xf");
}
template void launch_full_step_xf<float>(int, const float4*, const double*, const double*, float4*, cudaStream_t);
template void launch_full_step_xf<double>(int, const double4_32a*, const double*, const double*, float4*,
                                          cudaStream_t);

void launch_refresh_xf(int nv, const double* X, const double* u, float4* xf, cudaStream_t st) {
  if (nv <= 0) return;
  refresh_xf_kernel<<<div_up(nv, SB), SB, 0, st>>>(nv, X, u, xf);
  after_launch("refresh_xf");
}

void launch_prepare_step(int n, double dt, const double* u, const double* v, const double* a,
                         const int8_t* dof_type, const double* dbc, double* xt, double* next, cudaStream_t st) {
  prepare_step_kernel<<<div_up(n, SB), SB, 0, st>>>(n, dt, u, v, a, dof_type, dbc, xt, next);
  after_launch("prepare_step");
}

void launch_step_next(int n, double dt, double damping, double* prev, double* u, const double* next, double* v,
                      cudaStream_t st) {
  step_next_kernel<<<div_up(n, SB), SB, 0, st>>>(n, 1.0 / dt, 1.0 - damping, prev, u, next, v);
  after_launch("step_next");
}

void launch_restore(int n, double dt, const int8_t* dof_type, const double* dbc, double* prev, double* u,
                    double* v, cudaStream_t st) {
  restore_kernel<<<div_up(n, SB), SB, 0, st>>>(n, 1.0 / dt, dof_type, dbc, prev, u, v);
  after_launch("restore");
}

void launch_axpy_d(int n, double a, const double* x, double* y, cudaStream_t st) {
  axpy_d_kernel<<<div_up(n, SB), SB, 0, st>>>(n, a, x, y);
  after_launch("axpy_d");
}

void launch_add_ext(int nv, int dof, double val, double* a, cudaStream_t st) {
  add_ext_kernel<<<div_up(nv, SB), SB, 0, st>>>(nv, dof, val, a);
  after_launch("add_ext");
}

void launch_mark_dofs(int n, const int* verts, const double* targ, int dirichlet, int8_t* dof_type, double* dbc,
                      cudaStream_t st) {
  if (n <= 0) return;
  mark_dofs_kernel<<<div_up(n, SB), SB, 0, st>>>(n, verts, targ, dirichlet, dof_type, dbc);
  after_launch("mark_dofs");
}

void launch_build_mask(int nv, const int8_t* dof_type, uint8_t* mask, cudaStream_t st) {
  build_mask_kernel<<<div_up(nv, SB), SB, 0, st>>>(nv, dof_type, mask);
  after_launch("build_mask");
}

template <typename S>
void launch_to_vec4(int nv, const double* in, V4<S>* out, bool negate, cudaStream_t st) {
  to_vec4_kernel<S><<<div_up(nv, SB), SB, 0, st>>>(nv, in, out, negate ? 1 : 0);
  after_launch("to_vec4");
}

template <typename S>
void launch_from_vec4(int nv, const V4<S>* in, double* out, cudaStream_t st) {
  from_vec4_kernel<S><<<div_up(nv, SB), SB, 0, st>>>(nv, in, out);
  after_launch("from_vec4");
}

template <typename S>
void launch_vdot(int nv, const V4<S>* a, const V4<S>* b, double* out, const Reduce& red, cudaStream_t st) {
  vdot_kernel<S><<<div_up(nv, SB), SB, 0, st>>>(nv, a, b, out, red);
  after_launch("vdot");
}

template <typename S>
void launch_vaxpby(int nv, double alpha, V4<S>* y, double beta, const V4<S>* x, cudaStream_t st) {
  vaxpby_kernel<S><<<div_up(nv, SB), SB, 0, st>>>(nv, (S)alpha, y, (S)beta, x);
  after_launch("vaxpby");
}

template <typename S>
void launch_vdiff(int nv, const double* a, const double* b, V4<S>* y, cudaStream_t st) {
  vdiff_kernel<S><<<div_up(nv, SB), SB, 0, st>>>(nv, a, b, y);
  after_launch("vdiff");
}

template <typename S>
void launch_pcg_setup_v(int nv, const V4<S>* b, const V4<S>* dinv, V4<S>* x, V4<S>* r, V4<S>* z, V4<S>* p0,
                        double rtol, int max_iters, const Reduce& red, cudaStream_t st) {
  pcg_setup_v_kernel<S><<<div_up(nv, SB), SB, 0, st>>>(nv, b, dinv, x, r, z, p0, rtol, max_iters, red);
  after_launch("pcg_setup_v");
}

void launch_instance_norms(int ninst, const int* voff, const double* g, double* out, cudaStream_t st) {
  if (ninst <= 0) return;
  instance_norms_kernel<<<ninst, SB, 0, st>>>(voff, g, out);
  after_launch("instance_norms");
}

#define SSIM_INST(S)                                                                                              \
  template void launch_assemble<S>(const SellMatrix&, const int*, const int*, const S*, const S*, const uint8_t*, \
                                   bool, S*, V4<S>*, int, cudaStream_t, int);                                     \
  template void launch_spmv<S>(const SellMatrix&, const S*, const V4<S>*, V4<S>*, cudaStream_t);                 \
  template void launch_kron_extract<S>(const SellMatrix&, const S*, S*, int*, cudaStream_t);                     \
  template void launch_export_csr<S>(const SellMatrix&, const int*, const int*, const int*, const S*, double*,   \
                                     cudaStream_t);                                                               \
  template void launch_pcg_setup<S>(int, const double*, const V4<S>*, V4<S>*, V4<S>*, V4<S>*, V4<S>*, double,   \
                                    int, bool, const Reduce&, cudaStream_t);                                      \
  template void launch_pcg_spmv<S>(const SellMatrix&, const S*, const V4<S>*, const V4<S>*, V4<S>*, V4<S>*,     \
                                   bool, const Reduce&, cudaStream_t, bool);                                      \
  template void launch_pcg_update<S>(int, const V4<S>*, const V4<S>*, const V4<S>*, V4<S>*, V4<S>*, V4<S>*, int, \
                                     const Reduce&, cudaStream_t);                                                \
  template bool launch_pcg_persistent<S>(const SellMatrix&, const S*, const V4<S>*, V4<S>*, V4<S>*, V4<S>*,       \
                                         V4<S>*, V4<S>*, V4<S>*, int, const Reduce&, unsigned long long*,        \
                                         long long,                                                               \
                                         int, int, int, cudaStream_t, bool, V4<S>*, int);                         \
  template void launch_dot_gd<S>(int, const double*, const V4<S>*, const Reduce&, cudaStream_t);                 \
  template void launch_csr_dof_spmv<S>(int, const int*, const int*, const S*, const V4<S>*, V4<S>*, cudaStream_t); \
  template void launch_axpy_update<S>(int, double, const V4<S>*, const double*, double*, float4*, cudaStream_t); \
  template void launch_to_vec4<S>(int, const double*, V4<S>*, bool, cudaStream_t);                               \
  template void launch_from_vec4<S>(int, const V4<S>*, double*, cudaStream_t);                                  \
  template void launch_vdot<S>(int, const V4<S>*, const V4<S>*, double*, const Reduce&, cudaStream_t);          \
  template void launch_vaxpby<S>(int, double, V4<S>*, double, const V4<S>*, cudaStream_t);                      \
  template void launch_vdiff<S>(int, const double*, const double*, V4<S>*, cudaStream_t);                       \
  template void launch_pcg_setup_v<S>(int, const V4<S>*, const V4<S>*, V4<S>*, V4<S>*, V4<S>*, V4<S>*, double,  \
                                      int, const Reduce&, cudaStream_t);

SSIM_INST(float)
SSIM_INST(double)

}  // namespace ssim_gb
