// topology.h -- one-time host set-up of the sparse structures of a tet mesh.
#pragma once
#include <stdint.h>

#include <vector>

namespace ssim_gb {

struct Topology {
  int nv = 0, nt = 0;
  int cv = 4;  // vertices per cell: 4 (tets), 3 (triangles) or 2 (springs)
  // block CSR of the full pattern: block row u holds its sorted neighbour vertices (self included).  The
  // scalar CSR of the reference (global_composer.hpp:68-100) follows: row 3u+a has columns
  // {3w+b : w in bcol[u], b<3}, so row_ptr[3u+a] = 9*bptr[u] + 3*deg(u)*a.
  std::vector<int32_t> bptr, bcol;
  long long nnzb = 0;
  int max_deg = 0;
  // The matrix is symmetric; only the upper blocks (w >= u) are stored, in SELL-32: slice s = block rows
  // 32s..32s+31, width = the slice's largest upper degree.
  int nslices = 0, nslots = 0;  // nslots = sl_off[nslices] + 32 (a trailing all-padding slice)
  int zero_slot = 0;             // first slot of the trailing slice: values always zero
  std::vector<int32_t> sl_off;    // [nslices+1] multiples of 32
  std::vector<int32_t> sl_col;    // [nslots] block column w (own row for padding)
  std::vector<int32_t> slot_row;  // [nslots] block row u, -1 for padding
  std::vector<int32_t> slot_k;    // [nslots] position of w in bcol of row u
  std::vector<int32_t> slot_kt;   // [nslots] position of u in bcol of row w
  // lower blocks of row u are the transposes of upper slots of other rows, listed in SELL-32 too
  int nlslots = 0;
  std::vector<int32_t> lo_off;  // [nslices+1]
  std::vector<int32_t> lo_src;  // [nlslots] upper slot holding block (w, u), zero_slot for padding
  std::vector<int32_t> lo_col;  // [nlslots] w (own row for padding)
  // assembly lists: per upper slot, codes (e*nb + local upper block id) | (bit 31 if that element block
  // enters transposed), nb = cv (cv + 1) / 2 upper vertex blocks per cell (10 for tets, 3 for springs)
  std::vector<int32_t> cptr, csrc;
  // vertex incidence for the force gather: per vertex, the (e*cv + i) with cells[e][i] == vertex
  std::vector<int32_t> vptr, vinc;
};

// Lists of the fused element-Hessian + assembly kernel (tets).  CTA b owns the block rows of slices
// [spc b, spc (b + 1)) (spc = slices per CTA, 32 rows each), i.e. the upper slots
// [sl_off[spc b], sl_off[spc (b + 1)]), and computes the Hessian of every element that has an upper block
// (a vertex pair v <= w of the element, row min(cell[v], cell[w])) in one of its rows; an element whose
// blocks fall in several CTAs' rows is computed by each of them.  ptr / elem: per CTA its elements,
// ascending.  code: per entry, one 16-bit code per upper block in upper_block_id order: 0xffff when the
// block's row belongs to another CTA, else the local slot (bits 0-9, relative to the CTA's first slot), the
// transposed flag (bit 10: the block enters its slot transposed, cell[v] > cell[w]) and the rank (bits
// 11-15): how many earlier entries of the same chunk (chunk consecutive entries of the CTA's list) add to
// that slot.  The kernel adds the blocks of a chunk rank by rank, so every slot sums its contributions in
// the list's order (deterministic, no atomics).  ok is false when a CTA has more than 1024 local slots or
// a rank exceeds 31; the mesh then keeps the two-kernel path.
struct FusedLists {
  int slices_per_cta = 0, chunk = 0, ncta = 0;
  bool ok = false;
  std::vector<int32_t> ptr, elem;
  std::vector<uint16_t> code;
};
constexpr uint16_t kFusedSkip = 0xffff;
void build_fused_lists(const Topology& t, const int32_t* cells, int slices_per_cta, int chunk, FusedLists& f);

// validates the cell indices (throws ssim_gb::invalid_argument) and builds everything above; cells are
// [nt][cv] with cv = 4 (tets), 3 (triangles) or 2 (springs)
void build_topology(int nv, int nt, const int32_t* cells, Topology& t, int cv = 4);

// Both triangles of the block pattern in SELL-32 (the FP16 copy of the system matrix that the mixed Newton's
// loose PCG solves read): slice s = block rows 32s..32s+31, width = the slice's largest degree; entry
// off[s] + 32k + lane holds row u = 32s + lane's k-th neighbour w (ascending) in col and, in src, the upper slot
// holding block (min(u, w), max(u, w)) with bit 31 set when the entry is that slot's transpose (w < u).
// Padding entries: column u (0 past the last row) and the all-zero slot.  false if the entries do not fit
// 31-bit indices.
bool build_full_sell(const Topology& t, std::vector<int32_t>& off, std::vector<int32_t>& col,
                     std::vector<int32_t>& src);

// the upper-triangular block id of the local vertex pair (v <= w) used by the element Hessian kernel
inline int upper_block_id(int v, int w) { return v * 4 - (v * (v - 1)) / 2 + (w - v); }

// SELL slot of the upper block (u, w), u <= w, w a neighbour of u
int upper_slot(const Topology& t, int u, int w);

// scalar CSR pattern (row_ptr [3nv+1], col_idx [9*nnzb])
void csr_pattern(const Topology& t, int32_t* row_ptr, int32_t* col_idx);

// consistent mass per upper slot, the sum over its element blocks of (|det Dm| p_ij) rho with p = 1/60 on
// the element diagonal and 1/120 off it (bilinears.hpp:140-148, time_step.hpp:437-454), element order
void slot_masses(const Topology& t, const std::vector<double>& detJ, double rho, std::vector<double>& out);

// PD matrix scalar per upper slot: mass(rho) + laplace(alpha) element integrals (projective_dynamics.hpp:62-82)
// alpha_e (optional): per-element Laplacian weights replacing the uniform alpha
void slot_pd_values(const Topology& t, const int32_t* cells, const double* X, const std::vector<double>& detJ,
                    double rho, double alpha, std::vector<double>& out,
                    const std::vector<double>* alpha_e = nullptr);

// the 2D (triangle) versions: p12_element_f_f masses |det J| {1/12, 1/24} rho and the 2D Laplacian
// (bilinears.hpp:45-96); detJ = |det Dm| = twice the area
void slot_masses_2d(const Topology& t, const std::vector<double>& detJ, double rho, std::vector<double>& out);
void slot_pd_values_2d(const Topology& t, const int32_t* cells, const double* X, const std::vector<double>& detJ,
                       double rho, double alpha, std::vector<double>& out,
                       const std::vector<double>* alpha_e = nullptr);

}  // namespace ssim_gb
