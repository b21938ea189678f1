// topology.h -- one-time host set-up of the sparse structures of a tet mesh.
#pragma once
#include <stdint.h>

#include <vector>

namespace ssim_gb {

struct Topology {
  int nv = 0, nt = 0;
  // block CSR: block row u holds its sorted neighbour vertices (self included).  The scalar CSR of the
  // reference (global_composer.hpp:68-100) follows: row 3u+a has columns {3w+b : w in bcol[u], b<3}, so
  // row_ptr[3u+a] = 9*bptr[u] + 3*deg(u)*a.
  std::vector<int32_t> bptr, bcol;
  long long nnzb = 0;
  // SELL-32 slots: slice s = rows 32s..32s+31, width W_s = max degree in the slice
  int nslices = 0, nslots = 0;
  std::vector<int32_t> sl_off;    // [nslices+1], multiples of 32
  std::vector<int32_t> sl_col;    // [nslots] block column (own row for padding)
  std::vector<int32_t> slot_row;  // [nslots] block row or -1
  // assembly lists: per slot, codes (e*10 + upper block id) | (bit 31 if the element block is transposed)
  std::vector<int32_t> cptr, csrc;
  // vertex incidence for the force gather: per vertex, the (e*4 + i) with cells[e][i] == vertex
  std::vector<int32_t> vptr, vinc;
  int max_deg = 0;
};

// validates the cell indices (throws ssim_gb::invalid_argument) and builds everything above
void build_topology(int nv, int nt, const int32_t* cells, Topology& t);

// the upper-triangular block id of the local vertex pair (v <= w) used by the element Hessian kernel
inline int upper_block_id(int v, int w) { return v * 4 - (v * (v - 1)) / 2 + (w - v); }

// scalar CSR pattern (row_ptr [3nv+1], col_idx [9*nnzb])
void csr_pattern(const Topology& t, int32_t* row_ptr, int32_t* col_idx);

// consistent mass per slot, sum over the slot's element blocks of rho |det Dm| (1/60 diagonal, 1/120
// off-diagonal) (bilinears.hpp:140-148, time_step.hpp:437-454), in element order
void slot_masses(const Topology& t, const std::vector<double>& detJ, double rho, std::vector<double>& out);

}  // namespace ssim_gb
