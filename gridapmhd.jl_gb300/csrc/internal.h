// Internal declarations shared by the host and device parts of libgbmhd.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/gbmhd.h"

namespace gbmhd {

constexpr int NQ = 27;        // 3x3x3 Gauss points (quadrature degree 5)
constexpr int NQF = 9;        // 3x3 Gauss points on a face
constexpr int NU = 81, NP = 4, NJ = 36, NPHI = 8, ND = 129;
constexpr int OU = 0, OP = 81, OJ = 85, OPHI = 121;

// Reference-element tables at the quadrature points (FP64 master copy; the
// kernels stage an FP32 or FP64 copy in shared memory).
struct RefTables {
  double w[NQ];                 // Gauss weights on [0,1]^3
  double gq1[NQ][8][3];         // Q1 geometry gradients
  double n2[NQ][27];            // Q2 values
  double g2[NQ][27][3];         // Q2 reference gradients
  double p1[NQ][4];             // P1 values
  double q1[NQ][8];             // Q1 values (φ)
  double rt[NQ][36];            // value of the single nonzero component of each RT function
  double rtdiv[NQ][36];         // reference divergence
  // faces: local face f, face point t
  double fw[NQF];                 // face weights on [0,1]^2
  double fgq1[6][NQF][8][3];      // Q1 geometry gradients at face points
  double frt[6][NQF][36];         // RT component value at face points
  double frtg[6][NQF][36][3];     // reference gradient of that component
};
void build_ref_tables(RefTables& T);

// Post-processing rule: degree 2(order+1) = 6, i.e. 4 Gauss-Legendre points per direction
// (src/Applications/hunt.jl:247), with the bases the error integrals need.
constexpr int NQP = 64;
struct PostTables {
  double w[NQP];                // weights on [0,1]^3
  double q1[NQP][8];            // Q1 values (the geometry map)
  double gq1[NQP][8][3];        // Q1 gradients
  double n2[NQP][27];           // Q2 values
  double g2[NQP][27][3];        // Q2 reference gradients
  double rt[NQP][36];           // value of the single nonzero component of each RT function
};
void build_post_tables(PostTables& T);
inline int rt_axis(int b) { return b / 12; }

// Device-side float copy layouts are the same struct with float/double.
template <typename T>
struct DevTables {
  T w[NQ];
  T gq1[NQ][8][3];
  T n2[NQ][27];
  T g2[NQ][27][3];
  T p1[NQ][4];
  T q1[NQ][8];
  T rt[NQ][36];
  T rtdiv[NQ][36];
};

struct FacetTables {
  double fw[NQF];
  double fgq1[6][NQF][8][3];
  double frt[6][NQF][36];
  double frtg[6][NQF][36][3];
};

struct DevParams {
  double alpha, beta, gamma, sigma;
  double B[3], f[3], g[3];
  double zeta_u, zeta_j;
  int convection;
  int has_fcell;
};

// CSR pattern + cell -> nnz map, built on the host.
struct Pattern {
  int64_t n = 0, nnz = 0;
  std::vector<int64_t> rowptr;
  std::vector<int32_t> col;
  int32_t nclass = 0;
  std::vector<int32_t> cell_class;     // [ncells]
  std::vector<uint16_t> offtab;        // [nclass][ND*ND], offset of (a,b) inside row a's columns
};
// cell_row: [ncells][ND] global free row id or -1.  Returns "" or an error text.
std::string build_pattern(int64_t ncells, int64_t ndofs, const int32_t* cell_row, Pattern& P);
bool touched(int a, int b);

// Launch accounting (reported by gbmhd_counters).
void count_launch(int64_t n = 1);
int64_t launch_count();
void count_gemm(int64_t n = 1);

}  // namespace gbmhd

// Library context.
struct gbmhd_ctx {
  std::string err;
  int device = 0;
  cudaStream_t stream = nullptr;
  int num_sms = 0;
  int64_t ncells = 0, ndofs = 0, nnz = 0;
  int64_t nfree[4] = {0, 0, 0, 0}, offs[4] = {0, 0, 0, 0}, ndir[4] = {0, 0, 0, 0};
  int64_t nfull = 0;                   // ndofs + Dirichlet values
  // host copies needed later
  std::vector<int32_t> h_cell_row;
  std::vector<int64_t> h_rowptr;       // host copy of the CSR pattern (solver set-up)
  std::vector<int32_t> h_col;
  std::vector<double> h_cellX;
  gbmhd::DevParams prm{};
  // device buffers
  double* d_cellX = nullptr;           // [ncells][24]
  int32_t* d_gidx = nullptr;           // [ncells][129] index into d_xfull
  int32_t* d_row = nullptr;            // [ncells][129] global free id or -1
  uint64_t* d_sign = nullptr;          // [ncells] bit b set = RT dof b has sign -1 (or null)
  double* d_xfull = nullptr;           // [nfull]
  double* d_fcell = nullptr;           // [ncells][3] or null
  int64_t nfacets = 0;
  int32_t* d_fcellid = nullptr;
  int8_t* d_flface = nullptr;
  double* d_fprm = nullptr;            // [nfacets][4] tau, cw, jw, phi0
  void* d_tab64 = nullptr;             // DevTables<double>
  void* d_tab32 = nullptr;             // DevTables<float>
  void* d_ftab = nullptr;              // FacetTables
  void* d_posttab = nullptr;           // PostTables (built on first use)
  int64_t* d_rowptr = nullptr;
  int32_t* d_col = nullptr;
  int32_t* d_class = nullptr;
  uint16_t* d_offtab = nullptr;
  int32_t nclass = 0;
  double* d_val64 = nullptr;
  float* d_val32 = nullptr;
  // the state-independent terms of the FP64 Jacobian (all but convection), assembled once per
  // parameter set; an FP64 Jacobian is then this copy plus the convection terms at the state
  double* d_val64s = nullptr;
  int64_t val64s_gen = -1;             // params_gen of d_val64s (-1: not assembled)
  bool val64s_off = false;             // no room for it: FP64 Jacobians assembled whole
  int jac_precision = -1;              // precision of the last assembled Jacobian
  double* d_r = nullptr;               // [ndofs] residual work vector
  double* d_xtmp = nullptr;            // [ndofs]
  struct Solver* solver = nullptr;     // linear-solver workspace (solver.cu)
  int64_t params_gen = 0;              // incremented by every gbmhd_set_params
};

// assemble.cu
int gb_assemble_device(gbmhd_ctx* ctx, const double* d_x, double* d_r, int want_jac, int precision);
int gb_upload_tables(gbmhd_ctx* ctx);
// param derivatives used by the adjoint: dR/dγ, dR/dcw, f_z moments, dR/dα, dR/dβ (all on
// device; a NULL output is skipped)
int gb_param_derivs(gbmhd_ctx* ctx, const double* d_x, double* d_dr_dgamma, double* d_dr_dcw,
                    double* d_fz /*[ncells][27]*/, double* d_dr_dalpha = nullptr, double* d_dr_dbeta = nullptr);

#define GB_CUDA(call)                                                           \
  do {                                                                          \
    cudaError_t e_ = (call);                                                    \
    if (e_ != cudaSuccess) {                                                    \
      ctx->err = std::string(#call) + ": " + cudaGetErrorString(e_);            \
      return -2;                                                                \
    }                                                                           \
  } while (0)
