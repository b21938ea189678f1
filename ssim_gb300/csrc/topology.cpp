// topology.cpp -- host set-up of the CSR pattern, the symmetric SELL-32 slot layout, the assembly lists
// and the vertex incidence.
#include "topology.h"

#include <algorithm>
#include <cmath>
#include <string>

#include "errors.h"

namespace ssim_gb {

namespace {
// local upper block id -> (v, w)
constexpr int kBlkV[10] = {0, 0, 0, 0, 1, 1, 1, 2, 2, 3};
constexpr int kBlkW[10] = {0, 1, 2, 3, 1, 2, 3, 2, 3, 3};
// the same for triangles (3 vertices, 6 upper blocks)
constexpr int kTriV[6] = {0, 0, 0, 1, 1, 2};
constexpr int kTriW[6] = {0, 1, 2, 1, 2, 2};

int find_pos(const Topology& t, int u, int w) {
  const int32_t* nb = t.bcol.data() + t.bptr[u];
  const int deg = t.bptr[u + 1] - t.bptr[u];
  return (int)(std::lower_bound(nb, nb + deg, w) - nb);
}
}  // namespace

void build_topology(int nv, int nt, const int32_t* cells, Topology& t, int cv) {
  if (nv <= 0 || nt <= 0) throw invalid_argument("mesh must have at least one vertex and one cell");
  if (cv != 4 && cv != 3 && cv != 2)
    throw invalid_argument("cells must have 4 (tets), 3 (triangles) or 2 (springs) vertices");
  for (long long i = 0; i < (long long)cv * nt; ++i)
    if (cells[i] < 0 || cells[i] >= nv)
      throw invalid_argument("cell index out of range at cells[" + std::to_string(i) + "] = " +
                             std::to_string(cells[i]));
  const int nb = cv * (cv + 1) / 2;  // upper vertex blocks per cell
  if ((long long)nb * nt >= (1LL << 31)) throw invalid_argument("too many cells for 32-bit assembly codes");
  t.nv = nv;
  t.nt = nt;
  t.cv = cv;
  // neighbour lists (two-pass CSR of the cv x cv vertex pairs of every cell, then sort + unique per row)
  std::vector<int32_t> cnt(nv + 1, 0);
  for (long long i = 0; i < (long long)cv * nt; ++i) cnt[cells[i] + 1] += cv;
  for (int v = 0; v < nv; ++v) cnt[v + 1] += cnt[v];
  std::vector<int32_t> raw(cnt[nv]);
  {
    std::vector<int32_t> fill(cnt.begin(), cnt.end() - 1);
    for (int e = 0; e < nt; ++e)
      for (int i = 0; i < cv; ++i) {
        const int u = cells[cv * e + i];
        for (int j = 0; j < cv; ++j) raw[fill[u]++] = cells[cv * e + j];
      }
  }
  t.bptr.assign(nv + 1, 0);
  t.bcol.clear();
  t.bcol.reserve(raw.size() / 2);
  t.max_deg = 0;
  for (int u = 0; u < nv; ++u) {
    auto b = raw.begin() + cnt[u], e = raw.begin() + cnt[u + 1];
    std::sort(b, e);
    auto last = std::unique(b, e);
    const int deg = (int)(last - b);
    t.bcol.insert(t.bcol.end(), b, last);
    t.bptr[u + 1] = t.bptr[u] + deg;
    t.max_deg = std::max(t.max_deg, deg);
  }
  t.nnzb = t.bptr[nv];
  if (9LL * t.nnzb >= (1LL << 31)) throw invalid_argument("matrix too large for 32-bit CSR indices");
  // lower / upper degree of every row.  Vertices used by no cell have an empty row; they still get one
  // (zero) diagonal slot so every row owns a slot.
  std::vector<int32_t> lo_deg(nv), up_deg(nv);
  for (int u = 0; u < nv; ++u) {
    const int k = find_pos(t, u, u);
    lo_deg[u] = k;
    up_deg[u] = (t.bptr[u + 1] - t.bptr[u]) - k;
  }
  t.nslices = (nv + 31) / 32;
  t.sl_off.assign(t.nslices + 1, 0);
  t.lo_off.assign(t.nslices + 1, 0);
  for (int s = 0; s < t.nslices; ++s) {
    int wu = 1, wl = 0;
    for (int u = 32 * s; u < std::min(nv, 32 * s + 32); ++u) {
      wu = std::max(wu, up_deg[u]);
      wl = std::max(wl, lo_deg[u]);
    }
    t.sl_off[s + 1] = t.sl_off[s] + 32 * wu;
    t.lo_off[s + 1] = t.lo_off[s] + 32 * wl;
  }
  // one slice of padding slots after the last row slice: never assembled into, always zero; the lower
  // index points its padding entries at the first of them, so the SpMV needs no branch on padding
  t.zero_slot = t.sl_off[t.nslices];
  t.nslots = t.sl_off[t.nslices] + 32;
  t.nlslots = t.lo_off[t.nslices];
  t.sl_col.assign(t.nslots, 0);
  t.slot_row.assign(t.nslots, -1);
  t.slot_k.assign(t.nslots, 0);
  t.slot_kt.assign(t.nslots, 0);
  auto slot_of = [&](int u, int kk) { return t.sl_off[u >> 5] + 32 * kk + (u & 31); };
  for (int s = 0; s < t.nslices; ++s) {
    const int W = (t.sl_off[s + 1] - t.sl_off[s]) / 32;
    for (int lane = 0; lane < 32; ++lane) {
      const int u = 32 * s + lane;
      const int k0 = u < nv ? lo_deg[u] : 0;
      const int du = u < nv ? up_deg[u] : 0;
      for (int kk = 0; kk < W; ++kk) {
        const int q = t.sl_off[s] + 32 * kk + lane;
        if (kk < du) {
          const int w = t.bcol[t.bptr[u] + k0 + kk];
          t.sl_col[q] = w;
          t.slot_row[q] = u;
          t.slot_k[q] = k0 + kk;
          t.slot_kt[q] = find_pos(t, w, u);
        } else {
          t.sl_col[q] = u < nv ? u : 0;  // padding: a valid column, zero values
        }
      }
    }
  }
  t.lo_src.assign(t.nlslots, t.zero_slot);
  t.lo_col.assign(t.nlslots, 0);
  for (int s = 0; s < t.nslices; ++s) {
    const int W = (t.lo_off[s + 1] - t.lo_off[s]) / 32;
    for (int lane = 0; lane < 32; ++lane) {
      const int u = 32 * s + lane;
      const int dl = u < nv ? lo_deg[u] : 0;
      for (int kk = 0; kk < W; ++kk) {
        const int q = t.lo_off[s] + 32 * kk + lane;
        if (kk < dl) {
          const int w = t.bcol[t.bptr[u] + kk];  // w < u
          t.lo_src[q] = slot_of(w, find_pos(t, w, u) - lo_deg[w]);
          t.lo_col[q] = w;
        } else {
          t.lo_col[q] = u < nv ? u : 0;
        }
      }
    }
  }
  // assembly lists (global_composer.hpp:103-119 at block granularity, upper blocks only), stable in
  // element order.  A local pair (v, w) lands in global block (cells[v], cells[w]); pairs whose global
  // block is a lower one are the transposes of pairs already counted, except on the diagonal (a cell
  // repeating a vertex) where both orientations add, as they do in the reference's full gather.
  std::vector<int32_t> ccnt(t.nslots + 1, 0);
  auto visit = [&](auto&& fn) {
    for (int e = 0; e < nt; ++e)
      for (int v = 0; v < cv; ++v)
        for (int w = 0; w < cv; ++w) {
          const int gu = cells[cv * e + v], gw = cells[cv * e + w];
          if (gu > gw) continue;
          const int q = slot_of(gu, find_pos(t, gu, gw) - lo_deg[gu]);
          const int lo = std::min(v, w), hi = std::max(v, w);
          int32_t code = (int32_t)(nb * e + (lo * cv - (lo * (lo - 1)) / 2 + (hi - lo)));
          if (v > w) code = (int32_t)((uint32_t)code | 0x80000000u);
          fn(q, code);
        }
  };
  visit([&](int q, int32_t) { ccnt[q + 1]++; });
  for (int q = 0; q < t.nslots; ++q) ccnt[q + 1] += ccnt[q];
  t.cptr = ccnt;
  t.csrc.assign(ccnt[t.nslots], 0);
  {
    std::vector<int32_t> fill(ccnt.begin(), ccnt.end() - 1);
    visit([&](int q, int32_t code) { t.csrc[fill[q]++] = code; });
  }
  // vertex incidence (global_composer.hpp:36-66)
  t.vptr.assign(nv + 1, 0);
  for (long long i = 0; i < (long long)cv * nt; ++i) t.vptr[cells[i] + 1]++;
  for (int v = 0; v < nv; ++v) t.vptr[v + 1] += t.vptr[v];
  t.vinc.assign((long long)cv * nt, 0);
  {
    std::vector<int32_t> fill(t.vptr.begin(), t.vptr.end() - 1);
    for (long long i = 0; i < (long long)cv * nt; ++i) t.vinc[fill[cells[i]]++] = (int32_t)i;
  }
}

int upper_slot(const Topology& t, int u, int w) {
  const int lo = find_pos(t, u, u);
  return t.sl_off[u >> 5] + 32 * (find_pos(t, u, w) - lo) + (u & 31);
}

bool build_full_sell(const Topology& t, std::vector<int32_t>& off, std::vector<int32_t>& col,
                     std::vector<int32_t>& src) {
  off.assign(t.nslices + 1, 0);
  long long total = 0;
  for (int s = 0; s < t.nslices; ++s) {
    int w = 0;
    for (int u = 32 * s; u < std::min(t.nv, 32 * s + 32); ++u) w = std::max(w, t.bptr[u + 1] - t.bptr[u]);
    total += 32LL * w;
    if (total >= (1LL << 31)) return false;
    off[s + 1] = (int32_t)total;
  }
  col.assign(total, 0);
  src.assign(total, t.zero_slot);
  for (int s = 0; s < t.nslices; ++s) {
    const int W = (off[s + 1] - off[s]) / 32;
    for (int lane = 0; lane < 32; ++lane) {
      const int u = 32 * s + lane;
      const int deg = u < t.nv ? t.bptr[u + 1] - t.bptr[u] : 0;
      for (int k = 0; k < W; ++k) {
        const int e = off[s] + 32 * k + lane;
        if (k < deg) {
          const int w = t.bcol[t.bptr[u] + k];
          col[e] = w;
          src[e] = w >= u ? upper_slot(t, u, w) : (int32_t)(0x80000000u | (uint32_t)upper_slot(t, w, u));
        } else {
          col[e] = u < t.nv ? u : 0;
        }
      }
    }
  }
  return true;
}

void csr_pattern(const Topology& t, int32_t* row_ptr, int32_t* col_idx) {
  row_ptr[0] = 0;
  for (int u = 0; u < t.nv; ++u) {
    const int deg = t.bptr[u + 1] - t.bptr[u];
    for (int a = 0; a < 3; ++a) {
      const long long r = 3LL * u + a;
      const long long o = 9LL * t.bptr[u] + 3LL * deg * a;
      row_ptr[r + 1] = (int32_t)(o + 3LL * deg);
      for (int k = 0; k < deg; ++k)
        for (int b = 0; b < 3; ++b) col_idx[o + 3 * k + b] = 3 * t.bcol[t.bptr[u] + k] + b;
    }
  }
}

void slot_masses(const Topology& t, const std::vector<double>& detJ, double rho, std::vector<double>& out) {
  out.assign(t.nslots, 0.0);
  for (int q = 0; q < t.nslots; ++q) {
    double m = 0;
    for (int c = t.cptr[q]; c < t.cptr[q + 1]; ++c) {
      const uint32_t code = (uint32_t)t.csrc[c];
      const int eb = (int)(code & 0x7fffffffu);
      const int e = eb / 10, blk = eb % 10;
      const bool diag = kBlkV[blk] == kBlkW[blk];
      m += (detJ[e] * (diag ? 1.0 / 60 : 1.0 / 120)) * rho;  // (|det J| p_ij) * alpha as bilinears.hpp:236,249
    }
    out[q] = m;
  }
}

void slot_pd_values(const Topology& t, const int32_t* cells, const double* X, const std::vector<double>& detJ,
                    double rho, double alpha, std::vector<double>& out, const std::vector<double>* alpha_e) {
  // per element: grad phi_i from the inverse Jacobian (bilinears.hpp:158-167 summed over k = l)
  std::vector<double> lap(10 * (size_t)t.nt);
  for (int e = 0; e < t.nt; ++e) {
    const double* x0 = X + 3 * (size_t)cells[4 * e];
    double J[9];
    for (int k = 0; k < 3; ++k) {
      const double* xk = X + 3 * (size_t)cells[4 * e + k + 1];
      for (int r = 0; r < 3; ++r) J[r * 3 + k] = xk[r] - x0[r];
    }
    const double d = J[0] * (J[4] * J[8] - J[5] * J[7]) - J[1] * (J[3] * J[8] - J[5] * J[6]) +
                     J[2] * (J[3] * J[7] - J[4] * J[6]);
    const double id = 1.0 / d;
    const double B[9] = {(J[4] * J[8] - J[5] * J[7]) * id, (J[2] * J[7] - J[1] * J[8]) * id,
                         (J[1] * J[5] - J[2] * J[4]) * id, (J[5] * J[6] - J[3] * J[8]) * id,
                         (J[0] * J[8] - J[2] * J[6]) * id, (J[2] * J[3] - J[0] * J[5]) * id,
                         (J[3] * J[7] - J[4] * J[6]) * id, (J[1] * J[6] - J[0] * J[7]) * id,
                         (J[0] * J[4] - J[1] * J[3]) * id};
    double g[4][3];
    for (int k = 0; k < 3; ++k) {
      g[1][k] = B[0 * 3 + k];
      g[2][k] = B[1 * 3 + k];
      g[3][k] = B[2 * 3 + k];
      g[0][k] = -(g[1][k] + g[2][k] + g[3][k]);
    }
    for (int b = 0; b < 10; ++b) {
      const int v = kBlkV[b], w = kBlkW[b];
      lap[10 * (size_t)e + b] =
          (detJ[e] / 6.0 * (g[v][0] * g[w][0] + g[v][1] * g[w][1] + g[v][2] * g[w][2])) *
          (alpha_e ? (*alpha_e)[e] : alpha);
    }
  }
  out.assign(t.nslots, 0.0);
  for (int q = 0; q < t.nslots; ++q) {
    double m = 0;
    for (int c = t.cptr[q]; c < t.cptr[q + 1]; ++c) {
      const uint32_t code = (uint32_t)t.csrc[c];
      const int eb = (int)(code & 0x7fffffffu);
      const int e = eb / 10, blk = eb % 10;
      const bool diag = kBlkV[blk] == kBlkW[blk];
      m += (detJ[e] * (diag ? 1.0 / 60 : 1.0 / 120)) * rho + lap[eb];
    }
    out[q] = m;
  }
}

void slot_masses_2d(const Topology& t, const std::vector<double>& detJ, double rho, std::vector<double>& out) {
  out.assign(t.nslots, 0.0);
  for (int q = 0; q < t.nslots; ++q) {
    double m = 0;
    for (int c = t.cptr[q]; c < t.cptr[q + 1]; ++c) {
      const int eb = (int)((uint32_t)t.csrc[c] & 0x7fffffffu);
      const int e = eb / 6, blk = eb % 6;
      m += (detJ[e] * (kTriV[blk] == kTriW[blk] ? 1.0 / 12 : 1.0 / 24)) * rho;  // p12_element_f_f
    }
    out[q] = m;
  }
}

void slot_pd_values_2d(const Topology& t, const int32_t* cells, const double* X, const std::vector<double>& detJ,
                       double rho, double alpha, std::vector<double>& out, const std::vector<double>* alpha_e) {
  // per triangle: grad phi_i from the inverse 2x2 Jacobian; integral = |det J| / 2 * grad phi_v . grad phi_w
  std::vector<double> lap(6 * (size_t)t.nt);
  for (int e = 0; e < t.nt; ++e) {
    const double* x0 = X + 3 * (size_t)cells[3 * e];
    const double* x1 = X + 3 * (size_t)cells[3 * e + 1];
    const double* x2 = X + 3 * (size_t)cells[3 * e + 2];
    const double J[4] = {x1[0] - x0[0], x2[0] - x0[0], x1[1] - x0[1], x2[1] - x0[1]};
    const double d = J[0] * J[3] - J[1] * J[2];
    const double B[4] = {J[3] / d, -J[1] / d, -J[2] / d, J[0] / d};
    double g[3][2];
    for (int k = 0; k < 2; ++k) {
      g[1][k] = B[0 * 2 + k];
      g[2][k] = B[1 * 2 + k];
      g[0][k] = -(g[1][k] + g[2][k]);
    }
    for (int b = 0; b < 6; ++b) {
      const int v = kTriV[b], w = kTriW[b];
      lap[6 * (size_t)e + b] =
          (detJ[e] / 2.0 * (g[v][0] * g[w][0] + g[v][1] * g[w][1])) * (alpha_e ? (*alpha_e)[e] : alpha);
    }
  }
  out.assign(t.nslots, 0.0);
  for (int q = 0; q < t.nslots; ++q) {
    double m = 0;
    for (int c = t.cptr[q]; c < t.cptr[q + 1]; ++c) {
      const int eb = (int)((uint32_t)t.csrc[c] & 0x7fffffffu);
      const int e = eb / 6, blk = eb % 6;
      m += (detJ[e] * (kTriV[blk] == kTriW[blk] ? 1.0 / 12 : 1.0 / 24)) * rho + lap[eb];
    }
    out[q] = m;
  }
}

void build_fused_lists(const Topology& t, const int32_t* cells, int slices_per_cta, int chunk, FusedLists& f) {
  f = FusedLists();
  if (t.cv != 4 || slices_per_cta <= 0 || chunk <= 0) return;
  const int rows = 32 * slices_per_cta;
  const int ncta = (t.nslices + slices_per_cta - 1) / slices_per_cta;
  f.slices_per_cta = slices_per_cta;
  f.chunk = chunk;
  f.ncta = ncta;
  for (int b = 0; b < ncta; ++b) {
    const int s0 = b * slices_per_cta, s1 = std::min(t.nslices, s0 + slices_per_cta);
    if (t.sl_off[s1] - t.sl_off[s0] > 1024) return;  // local slots need more than 10 bits
  }
  // the CTAs whose rows hold a block of element e, each once, ascending
  auto ctas_of = [&](int e, int (&out)[10]) {
    const int32_t* c = cells + 4 * (size_t)e;
    int n = 0;
    for (int v = 0; v < 4; ++v)
      for (int w = v; w < 4; ++w) {
        const int b = std::min(c[v], c[w]) / rows;
        bool seen = false;
        for (int k = 0; k < n; ++k) seen |= out[k] == b;
        if (!seen) out[n++] = b;
      }
    std::sort(out, out + n);
    return n;
  };
  f.ptr.assign(ncta + 1, 0);
  for (int e = 0; e < t.nt; ++e) {
    int cs[10];
    const int n = ctas_of(e, cs);
    for (int k = 0; k < n; ++k) f.ptr[cs[k] + 1]++;
  }
  for (int b = 0; b < ncta; ++b) f.ptr[b + 1] += f.ptr[b];
  f.elem.assign(f.ptr[ncta], 0);
  {
    std::vector<int32_t> cur(f.ptr.begin(), f.ptr.end() - 1);
    for (int e = 0; e < t.nt; ++e) {
      int cs[10];
      const int n = ctas_of(e, cs);
      for (int k = 0; k < n; ++k) f.elem[cur[cs[k]]++] = e;
    }
  }
  f.code.assign(10 * (size_t)f.ptr[ncta], kFusedSkip);
  std::vector<int32_t> stamp(1024), count(1024);
  for (int b = 0; b < ncta; ++b) {
    const int q0 = t.sl_off[b * slices_per_cta];
    std::fill(stamp.begin(), stamp.end(), -1);
    for (int p = f.ptr[b]; p < f.ptr[b + 1]; ++p) {
      const int e = f.elem[p], ch = (p - f.ptr[b]) / chunk;
      const int32_t* c = cells + 4 * (size_t)e;
      for (int v = 0; v < 4; ++v)
        for (int w = v; w < 4; ++w) {
          const int a = c[v], d = c[w], u = std::min(a, d);
          if (u / rows != b) continue;
          const int ls = upper_slot(t, u, std::max(a, d)) - q0;
          if (stamp[ls] != ch) {
            stamp[ls] = ch;
            count[ls] = 0;
          }
          const int rank = count[ls]++;
          if (rank > 31) return;  // ok stays false
          f.code[10 * (size_t)p + upper_block_id(v, w)] = (uint16_t)(ls | ((a > d) ? 1 << 10 : 0) | (rank << 11));
        }
    }
  }
  f.ok = true;
}

}  // namespace ssim_gb
