// topology.cpp -- host set-up of the CSR pattern, SELL-32 slot layout, assembly lists and incidence.
#include "topology.h"

#include <algorithm>
#include <string>

#include "errors.h"

namespace ssim_gb {

void build_topology(int nv, int nt, const int32_t* cells, Topology& t) {
  if (nv <= 0 || nt <= 0) throw invalid_argument("mesh must have at least one vertex and one cell");
  for (long long i = 0; i < 4LL * nt; ++i)
    if (cells[i] < 0 || cells[i] >= nv)
      throw invalid_argument("cell index out of range at cells[" + std::to_string(i) + "] = " +
                             std::to_string(cells[i]));
  if (10LL * nt >= (1LL << 31)) throw invalid_argument("too many cells for 32-bit assembly codes");
  t.nv = nv;
  t.nt = nt;
  // neighbour lists (two-pass CSR of the 4x4 vertex pairs of every tet, then sort + unique per row)
  std::vector<int32_t> cnt(nv + 1, 0);
  for (long long i = 0; i < 4LL * nt; ++i) cnt[cells[i] + 1] += 4;
  for (int v = 0; v < nv; ++v) cnt[v + 1] += cnt[v];
  std::vector<int32_t> raw(cnt[nv]);
  {
    std::vector<int32_t> fill(cnt.begin(), cnt.end() - 1);
    for (int e = 0; e < nt; ++e)
      for (int i = 0; i < 4; ++i) {
        const int u = cells[4 * e + i];
        for (int j = 0; j < 4; ++j) raw[fill[u]++] = cells[4 * e + j];
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
  // SELL-32
  t.nslices = (nv + 31) / 32;
  t.sl_off.assign(t.nslices + 1, 0);
  for (int s = 0; s < t.nslices; ++s) {
    int w = 0;
    for (int u = 32 * s; u < std::min(nv, 32 * s + 32); ++u) w = std::max(w, t.bptr[u + 1] - t.bptr[u]);
    t.sl_off[s + 1] = t.sl_off[s] + 32 * w;
  }
  t.nslots = t.sl_off[t.nslices];
  t.sl_col.assign(t.nslots, 0);
  t.slot_row.assign(t.nslots, -1);
  for (int s = 0; s < t.nslices; ++s) {
    const int W = (t.sl_off[s + 1] - t.sl_off[s]) / 32;
    for (int lane = 0; lane < 32; ++lane) {
      const int u = 32 * s + lane;
      const int deg = u < nv ? t.bptr[u + 1] - t.bptr[u] : 0;
      for (int k = 0; k < W; ++k) {
        const int q = t.sl_off[s] + 32 * k + lane;
        if (k < deg) {
          t.sl_col[q] = t.bcol[t.bptr[u] + k];
          t.slot_row[q] = u;
        } else {
          t.sl_col[q] = u < nv ? u : 0;  // padding: a valid column, zero values
          t.slot_row[q] = -1;
        }
      }
    }
  }
  // assembly lists (global_composer.hpp:103-119 at block granularity), stable in element order
  std::vector<int32_t> slot_of(16LL * nt);
  std::vector<int32_t> ccnt(t.nslots + 1, 0);
  for (int e = 0; e < nt; ++e)
    for (int v = 0; v < 4; ++v) {
      const int u = cells[4 * e + v];
      const int32_t* nb = t.bcol.data() + t.bptr[u];
      const int deg = t.bptr[u + 1] - t.bptr[u];
      for (int w = 0; w < 4; ++w) {
        const int x = cells[4 * e + w];
        const int k = (int)(std::lower_bound(nb, nb + deg, x) - nb);
        const int q = t.sl_off[u >> 5] + 32 * k + (u & 31);
        slot_of[16LL * e + 4 * v + w] = q;
        ccnt[q + 1]++;
      }
    }
  for (int q = 0; q < t.nslots; ++q) ccnt[q + 1] += ccnt[q];
  t.cptr = ccnt;
  t.csrc.assign(16LL * nt, 0);
  {
    std::vector<int32_t> fill(ccnt.begin(), ccnt.end() - 1);
    for (int e = 0; e < nt; ++e)
      for (int v = 0; v < 4; ++v)
        for (int w = 0; w < 4; ++w) {
          const int q = slot_of[16LL * e + 4 * v + w];
          const int lo = std::min(v, w), hi = std::max(v, w);
          int32_t code = (int32_t)(10 * e + upper_block_id(lo, hi));
          if (v > w) code = (int32_t)((uint32_t)code | 0x80000000u);
          t.csrc[fill[q]++] = code;
        }
  }
  // vertex incidence (global_composer.hpp:36-66)
  t.vptr.assign(nv + 1, 0);
  for (long long i = 0; i < 4LL * nt; ++i) t.vptr[cells[i] + 1]++;
  for (int v = 0; v < nv; ++v) t.vptr[v + 1] += t.vptr[v];
  t.vinc.assign(4LL * nt, 0);
  {
    std::vector<int32_t> fill(t.vptr.begin(), t.vptr.end() - 1);
    for (long long i = 0; i < 4LL * nt; ++i) t.vinc[fill[cells[i]]++] = (int32_t)i;
  }
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
      const bool diag = (blk == 0 || blk == 4 || blk == 7 || blk == 9);
      m += (detJ[e] * (diag ? 1.0 / 60 : 1.0 / 120)) * rho;  // (|det J| p_ij) * alpha as bilinears.hpp:236,249
    }
    out[q] = m;
  }
}

}  // namespace ssim_gb
