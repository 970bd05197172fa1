// Nested-dissection multifrontal factorization of the Newton Jacobian.
//
// Two uses: (1) monolithic — all four fields, with the zero (p,p) and (φ,φ)
// diagonal blocks replaced by −ε·diag(mass) so that the matrix is
// quasi-definite and factorizable without pivoting (the direct-solve semantics of
// GridapMHD's :julia solver, src/main.jl:181-186, as an FP32 or FP64
// preconditioner); (2) the (u,j) block of the Badia2024 block preconditioner
// (src/Solvers/badia2024.jl:22-40 uses an LU for that block).
//
// Symbolic phase (host): geometric nested dissection of the cells; every
// (u,j) dof is eliminated at the highest separator that contains it; the
// front of a node is [eliminated dofs ; boundary dofs], where the boundary is
// the set of dofs of the node's cells not eliminated inside its subtree.
// Fronts of one tree level are padded to a common size and stored as dense
// column-major matrices.
//
// Numeric phase (device): per level, fronts are gathered from the CSR values
// (arrowheads), children's Schur complements are extend-added, and the eliminated
// pivots are removed by a blocked right-looking LU whose diagonal NB-pivot blocks are
// inverted with partial pivoting inside the block (panel and trailing updates are
// strided-batched GEMMs).  After it a front holds
//   [ D⁻¹ \ L11    U11 ]      D⁻¹: the inverses of the NB x NB diagonal blocks,
//   [ L21          S   ]      L unit block-lower, U block-upper, S = F22 − L21 U12
// (U12 is the upper-right block).  A solve is a forward substitution with L and a backward
// one with U, per super-block of rows: a short chain of NB-block steps, then a dense GEMV.
// Keeping the factors in LU form (rather than the explicit inverse of the eliminated block)
// keeps FP32 rounding from being amplified by the conditioning of the whole block.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "internal.h"

namespace gbmhd {

struct MFLevel {
  int32_t E = 0, B = 0, n = 0;   // padded eliminated / boundary / front sizes
  int64_t first = 0, count = 0;  // fronts [first, first+count) of this level
  int64_t off = 0;               // element offset of the first front
  int64_t ah_begin = 0, ah_end = 0;       // arrowhead entries of the level
  int64_t ch_begin = 0, ch_end = 0;       // children (index into child list) extend-added here
};

struct MFSymbolic {
  bool monolithic = false;
  int64_t nuj = 0;                        // dofs in the factorized system
  int64_t storage = 0;                    // elements of all fronts
  std::vector<MFLevel> levels;
  std::vector<int32_t> f_ne, f_nb, f_level, f_parent;
  std::vector<int64_t> f_off;
  std::vector<int64_t> elim_ptr, bnd_ptr; // per front, into elim / bnd (global dof ids)
  std::vector<int32_t> elim, bnd;
  std::vector<int32_t> ah_src;            // CSR value index
  std::vector<int64_t> ah_dst;            // element offset in the front storage
  std::vector<int32_t> child_list;        // fronts ordered by the level of their parent
  std::vector<int64_t> ea_ptr;            // per front: positions of its boundary in the parent front
  std::vector<int32_t> ea_pos;
  double flops = 0.0;                     // Gauss-Jordan flops of a factorization
  std::vector<int64_t> reg_dst;           // monolithic: diagonal positions of the p and φ pivots
  std::vector<int32_t> reg_dof;           //             and their global dof ids
};

// cell_row: [ncells][129] global free ids (-1 Dirichlet); uj_slot(a) selects the
// local slots of u and j.  rowptr/col: CSR pattern of the full Jacobian.  order: the field
// order of elimination inside each front, letters u, p, j, f (φ) (null: "jufp").
std::string mf_analyse(int64_t ncells, const double* cell_coords, const int32_t* cell_row, int64_t ndofs,
                       const int64_t* rowptr, const int32_t* col, bool monolithic, MFSymbolic& S,
                       int leaf_cells = 8, const char* order = nullptr);

}  // namespace gbmhd

struct MFNumeric;
int mf_create(gbmhd_ctx* ctx, const gbmhd::MFSymbolic& S, MFNumeric** out);
// Factor from the Jacobian values of the given precision (GBMHD_FP64 / GBMHD_MIXED);
// d_reg (monolithic only): value added to the diagonal of each p and φ dof.
// values: precision of the Jacobian values read (the FP32 factors may read FP64 values).
int mf_factor(gbmhd_ctx* ctx, MFNumeric* M, int precision, int values, const double* d_reg);
// x[sys] = A⁻¹ b[sys] (or A⁻ᵀ b[sys] when transpose) on the factorized dofs;
// b is overwritten in those entries.
int mf_solve(gbmhd_ctx* ctx, MFNumeric* M, double* d_b, double* d_x, bool transpose);
void mf_destroy(MFNumeric* M);
// Waits for the context stream and returns -3 (with the message) if a solve sweep since the
// last factorization gave up waiting for its TMA copies, 0 otherwise.
int mf_check_sweeps(gbmhd_ctx* ctx, MFNumeric* M);
// Solves timed since the last call (CUDA events on the context stream), their total
// device time, and the factor bytes one solve reads; resets the counters.
void mf_sweep_stats(MFNumeric* M, int64_t* applies, double* seconds, double* bytes_per_apply);
int mf_precision(const MFNumeric* M);
