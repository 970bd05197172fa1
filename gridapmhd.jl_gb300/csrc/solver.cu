// Newton driver, FGMRES and the Badia2024 block preconditioner.
//
// Reference structure (GridapMHD):
//   src/main.jl:181-186          Newton with an LU linear solver (:julia)
//   src/Solvers/badia2024.jl:2-48 Newton ∘ FGMRES(m) ∘ upper block-triangular P with
//                                blocks [(u,j) | p | φ], coefficients [1 1 1; 0 1 0; 0 0 1],
//                                p block  α_p M_p, α_p = −1/(β+ζᵤ)
//                                φ block  α_φ M_φ, α_φ = −1/(1+ζⱼ)
//                                (u,j) block solved by an LU (here: multifrontal, mf_*.cu)
// Vectors, Gram-Schmidt (classical, re-orthogonalised), the Newton residual and
// update are FP64.  The operator and the (u,j) factors are FP32 in the mixed
// path and FP64 in the plain path.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "mf.h"
#include "solver.h"

using namespace gbmhd;

struct Solver {
  MFNumeric* mf = nullptr;
  int pc_kind = -1;             // GBMHD_PC_MONOLITHIC or GBMHD_PC_BADIA2024
  std::string mf_order;         // field order of elimination of the current symbolic analysis
  double* reg = nullptr;        // [ndofs] diagonal regularisation of the p and φ pivots
  double reg_eps = -1.0;
  bool have_mass = false;
  double mass_beta = 0, mass_zu = 0, mass_zj = 0;
  double* Mp_inv = nullptr;     // [ncells][16]  (α_p M_p)⁻¹
  double* Mf_inv = nullptr;     // [ncells][64]  (α_φ M_φ)⁻¹
  int32_t* seg = nullptr;       // [ndofs][2] p/φ column segment (offsets inside the row)
  // FGMRES workspace
  int m = 0;
  double* V = nullptr;          // (m+1) x n
  double* Z = nullptr;          // m x n
  double* w = nullptr;
  double* t1 = nullptr;
  double* t2 = nullptr;
  float* x32 = nullptr;         // [ndofs] SpMV input rounded to FP32 (FP32 Jacobian)
  double* part = nullptr;       // partial dot products
  double* hdev = nullptr;       // [kHcol] device: two CGS passes' coefficients + the norm²
  double* hhost = nullptr;      // [kHcol] pinned host copy of hdev
  int64_t part_len = 0;
  // transposed pattern for the adjoint
  // transposed Jacobian for the adjoint: the pattern is structurally symmetric, so Aᵀ
  // shares rowptr/col and only the values move: valT[t] = val[permT[t]]
  int64_t* permT = nullptr;
  double* valT = nullptr;
  int64_t factor_gen = -1;      // ctx->params_gen when the factors were computed
  // constant-pressure mode: 1 when the all-ones vector on the p dofs is a null vector of the
  // Jacobian (velocity fixed on every wall), checked once per parameter set
  int p_null = -1;
  int64_t p_null_gen = -1;
  double* gsum = nullptr;       // [2] device scratch of the check and the projection
};

#define S_CUDA GB_CUDA

// Layout of Solver::hdev / hhost: [0, 256) first Gram–Schmidt pass, [256, 512) second
// pass, [512] squared norm of the new direction.
constexpr int kHB = 256, kHN = 512, kHcol = 513;

// ---- the constant-pressure mode
// max over rows of |Σ_c J[r, c]| and of Σ_c |J[r, c]| over the columns c in [cb, ce) (the p
// dofs), as the bit patterns of non-negative doubles (which order like the values)
__global__ void k_const_mode(int64_t n, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                             const double* __restrict__ val, int32_t cb, int32_t ce, unsigned long long* out) {
  double sm = 0.0, am = 0.0;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0, a = 0.0;
    for (int64_t e = rowptr[r]; e < rowptr[r + 1]; ++e)
      if (col[e] >= cb && col[e] < ce) {
        s += val[e];
        a += fabs(val[e]);
      }
    sm = fmax(sm, fabs(s));
    am = fmax(am, a);
  }
  for (int o = 16; o > 0; o >>= 1) {
    sm = fmax(sm, __shfl_xor_sync(0xffffffffu, sm, o));
    am = fmax(am, __shfl_xor_sync(0xffffffffu, am, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(&out[0], (unsigned long long)__double_as_longlong(sm));
    atomicMax(&out[1], (unsigned long long)__double_as_longlong(am));
  }
}

// out[0] += Σ_{i in [a, b)} v[i]
__global__ void k_range_sum(const double* __restrict__ v, int64_t a, int64_t b, double* out) {
  double s = 0.0;
  for (int64_t i = a + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < b; i += (int64_t)gridDim.x * blockDim.x)
    s += v[i];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, s);
}

// v[i] −= sum / (b − a), i in [a, b)
__global__ void k_range_shift(double* __restrict__ v, int64_t a, int64_t b, const double* __restrict__ sum) {
  const double m = *sum / (double)(b - a);
  for (int64_t i = a + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < b; i += (int64_t)gridDim.x * blockDim.x)
    v[i] -= m;
}

// ------------------------------------------------------------------ kernels
// y = A x for the FP32 Jacobian: x arrives rounded to FP32 and the products accumulate in
// FP32 (per lane, then a warp-shuffle reduction); one conversion per row to the FP64 y.
// The rounding is of the order of the FP32 matrix values' own.  GB300 issues FP64 at a
// small fraction of its FP32 rate, and a per-nonzero FP64 convert + FMA made this kernel
// FP64-bound rather than HBM-bound.
__global__ void k_spmv_f32(int64_t n, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                           const float* __restrict__ val, const float* __restrict__ x, double* __restrict__ y) {
  const int lane = threadIdx.x & 31;
  for (int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; row < n;
       row += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    float acc = 0.0f;
    const int64_t t1 = rowptr[row + 1];
    for (int64_t t = rowptr[row] + lane; t < t1; t += 32) acc = fmaf(val[t], x[col[t]], acc);
    for (int s = 16; s > 0; s >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, s);
    if (lane == 0) y[row] = (double)acc;
  }
}

// y = A x for the FP64 Jacobian: 8 lanes per row, so a row's reduction takes 3 shuffle
// steps over 8 lanes instead of 5 over 32 (FP64 issue slots are the scarce resource).
__global__ void k_spmv_f64(int64_t r0, int64_t n, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                           const double* __restrict__ val, const double* __restrict__ x, double* __restrict__ y) {
  const int sub = threadIdx.x & 7;
  for (int64_t row = r0 + ((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 3); row - ((threadIdx.x & 31) >> 3) < n;
       row += ((int64_t)gridDim.x * blockDim.x) >> 3) {
    double acc = 0.0;
    if (row < n) {
      // four nonzeros per lane in flight (column and value loads first, then the gathers);
      // the matrix streams past L2 (evict-first), the vector stays resident
      const int64_t t1 = rowptr[row + 1];
      int64_t t = rowptr[row] + sub;
      for (; t + 24 < t1; t += 32) {
        const int32_t c0 = __ldcs(col + t), c1 = __ldcs(col + t + 8), c2 = __ldcs(col + t + 16), c3 = __ldcs(col + t + 24);
        const double v0 = __ldcs(val + t), v1 = __ldcs(val + t + 8), v2 = __ldcs(val + t + 16), v3 = __ldcs(val + t + 24);
        acc = fma(v0, x[c0], acc);
        acc = fma(v1, x[c1], acc);
        acc = fma(v2, x[c2], acc);
        acc = fma(v3, x[c3], acc);
      }
      for (; t < t1; t += 8) acc = fma(__ldcs(val + t), x[__ldcs(col + t)], acc);
    }
    for (int s = 4; s > 0; s >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, s, 8);
    if (sub == 0 && row < n) y[row] = acc;
  }
}

__global__ void k_to_f32(int64_t n, const double* __restrict__ x, float* __restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = (float)x[i];
}

// permT[t] = position of the entry (col[t], row(t)) in row col[t] (binary search in the
// sorted row); err = 1 if the pattern is not structurally symmetric.
__global__ void k_transpose_map(int64_t n, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                                int64_t* __restrict__ permT, int32_t* err) {
  const int lane = threadIdx.x & 31;
  for (int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; r < n;
       r += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    for (int64_t t = rowptr[r] + lane; t < rowptr[r + 1]; t += 32) {
      const int32_t c = col[t];
      int64_t lo = rowptr[c], hi = rowptr[c + 1];
      while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (col[mid] < r) lo = mid + 1;
        else hi = mid;
      }
      if (lo < rowptr[c + 1] && col[lo] == r) permT[t] = lo;
      else { permT[t] = t; atomicExch(err, 1); }
    }
  }
}

__global__ void k_gather_vals(int64_t nnz, const double* __restrict__ val, const int64_t* __restrict__ perm,
                              double* __restrict__ out) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nnz; t += (int64_t)gridDim.x * blockDim.x)
    out[t] = val[perm[t]];
}

template <typename V>
__global__ void k_coupling(int64_t n, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                           const V* __restrict__ val, const int32_t* __restrict__ seg, const double* __restrict__ z,
                           double* __restrict__ y) {
  for (int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; row < n; row += (int64_t)gridDim.x * blockDim.x) {
    const int32_t lo = seg[2 * row], hi = seg[2 * row + 1];
    if (lo >= hi) continue;
    double acc = 0.0;
    const int64_t b = rowptr[row];
    for (int32_t t = lo; t < hi; ++t) acc += (double)val[b + t] * z[col[b + t]];
    y[row] -= acc;
  }
}

__global__ void k_mass_apply(int64_t ncells, const int32_t* __restrict__ row, const double* __restrict__ Mp,
                             const double* __restrict__ Mf, const double* __restrict__ v, double* __restrict__ z,
                             bool only_p_phi_from_v) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncells; c += (int64_t)gridDim.x * blockDim.x) {
    const int32_t* r = row + c * ND;
    double vp[4], vf[8];
    for (int k = 0; k < 4; ++k) vp[k] = r[OP + k] >= 0 ? v[r[OP + k]] : 0.0;
    for (int k = 0; k < 8; ++k) vf[k] = r[OPHI + k] >= 0 ? v[r[OPHI + k]] : 0.0;
    for (int k = 0; k < 4; ++k) {
      double s = 0.0;
      for (int l = 0; l < 4; ++l) s += Mp[c * 16 + k * 4 + l] * vp[l];
      if (r[OP + k] >= 0) z[r[OP + k]] = s;
    }
    for (int k = 0; k < 8; ++k) {
      double s = 0.0;
      for (int l = 0; l < 8; ++l) s += Mf[c * 64 + k * 8 + l] * vf[l];
      if (r[OPHI + k] >= 0) z[r[OPHI + k]] = s;
    }
  }
}

// (α M)⁻¹ of the p (4x4) and φ (8x8) cell mass matrices (FP64 geometry).
__global__ void k_mass_inverse(int64_t ncells, const double* __restrict__ cellX, const double* __restrict__ w27,
                               const double* __restrict__ gq1, const double* __restrict__ p1,
                               const double* __restrict__ q1, double ap, double af, double* Mp, double* Mf) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncells; c += (int64_t)gridDim.x * blockDim.x) {
    const double* X = cellX + 24 * c;
    double A[4][8], Bm[8][16];
    for (int i = 0; i < 4; ++i) for (int j = 0; j < 8; ++j) A[i][j] = (j - 4 == i) ? 1.0 : 0.0;
    for (int i = 0; i < 8; ++i) for (int j = 0; j < 16; ++j) Bm[i][j] = (j - 8 == i) ? 1.0 : 0.0;
    for (int q = 0; q < NQ; ++q) {
      double J[3][3];
      for (int i = 0; i < 3; ++i)
        for (int a = 0; a < 3; ++a) {
          double s = 0.0;
          for (int v = 0; v < 8; ++v) s += X[3 * v + i] * gq1[(q * 8 + v) * 3 + a];
          J[i][a] = s;
        }
      const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                         J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                         J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
      const double wd = w27[q] * det;
      for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) A[i][j] += ap * wd * p1[q * 4 + i] * p1[q * 4 + j];
      for (int i = 0; i < 8; ++i)
        for (int j = 0; j < 8; ++j) Bm[i][j] += af * wd * q1[q * 8 + i] * q1[q * 8 + j];
    }
    // Gauss-Jordan (symmetric definite up to sign: no pivoting needed)
    for (int i = 0; i < 4; ++i) {
      const double d = 1.0 / A[i][i];
      for (int j = 0; j < 8; ++j) A[i][j] *= d;
      for (int k = 0; k < 4; ++k)
        if (k != i) {
          const double m = A[k][i];
          for (int j = 0; j < 8; ++j) A[k][j] -= m * A[i][j];
        }
    }
    for (int i = 0; i < 8; ++i) {
      const double d = 1.0 / Bm[i][i];
      for (int j = 0; j < 16; ++j) Bm[i][j] *= d;
      for (int k = 0; k < 8; ++k)
        if (k != i) {
          const double m = Bm[k][i];
          for (int j = 0; j < 16; ++j) Bm[k][j] -= m * Bm[i][j];
        }
    }
    for (int i = 0; i < 4; ++i) for (int j = 0; j < 4; ++j) Mp[c * 16 + i * 4 + j] = A[i][4 + j];
    for (int i = 0; i < 8; ++i) for (int j = 0; j < 8; ++j) Mf[c * 64 + i * 8 + j] = Bm[i][8 + j];
  }
}

// reg[p dof] = −ε_p ∫ψ_k², reg[φ dof] = −ε_φ ∫χ_k² (diagonals of the cell mass matrices).
__global__ void k_reg_diag(int64_t ncells, const double* __restrict__ cellX, const int32_t* __restrict__ row,
                           const double* __restrict__ w27, const double* __restrict__ gq1,
                           const double* __restrict__ p1, const double* __restrict__ q1, double ep, double ef,
                           double* reg) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncells; c += (int64_t)gridDim.x * blockDim.x) {
    const double* X = cellX + 24 * c;
    double dp[4] = {0, 0, 0, 0}, df[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int q = 0; q < NQ; ++q) {
      double J[3][3];
      for (int i = 0; i < 3; ++i)
        for (int a = 0; a < 3; ++a) {
          double s = 0.0;
          for (int v = 0; v < 8; ++v) s += X[3 * v + i] * gq1[(q * 8 + v) * 3 + a];
          J[i][a] = s;
        }
      const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                         J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                         J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
      const double wd = fabs(w27[q] * det);
      for (int k = 0; k < 4; ++k) dp[k] += wd * p1[q * 4 + k] * p1[q * 4 + k];
      for (int k = 0; k < 8; ++k) df[k] += wd * q1[q * 8 + k] * q1[q * 8 + k];
    }
    for (int k = 0; k < 4; ++k)
      if (row[c * ND + OP + k] >= 0) reg[row[c * ND + OP + k]] = -ep * dp[k];
    for (int k = 0; k < 8; ++k)
      if (row[c * ND + OPHI + k] >= 0) reg[row[c * ND + OPHI + k]] = -ef * df[k];
  }
}

// h[i] partials: part[i*nb + block] = Σ_chunk V_i·w
__global__ void k_mdot_partial(int64_t n, int k1, const double* __restrict__ V, const double* __restrict__ w,
                               double* __restrict__ part) {
  __shared__ double red[32];
  const int i = blockIdx.y;
  const double* vi = V + (int64_t)i * n;
  double acc = 0.0;
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x)
    acc += vi[j] * w[j];
  for (int s = 16; s > 0; s >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    acc = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int s = 16; s > 0; s >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, s);
    if (threadIdx.x == 0) part[(int64_t)i * gridDim.x + blockIdx.x] = acc;
  }
}

__global__ void k_mdot_final(int k1, int nb, const double* __restrict__ part, double* __restrict__ h) {
  __shared__ double red[32];
  const int i = blockIdx.x;
  double acc = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) acc += part[(int64_t)i * nb + b];
  for (int s = 16; s > 0; s >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    acc = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int s = 16; s > 0; s >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, s);
    if (threadIdx.x == 0) h[i] = acc;
  }
}

// w -= Σ_i h_i V_i
__global__ void k_mgs_update(int64_t n, int k1, const double* __restrict__ V, const double* __restrict__ h,
                             double* __restrict__ w) {
  __shared__ double hs[256];
  for (int i = threadIdx.x; i < k1; i += blockDim.x) hs[i] = h[i];
  __syncthreads();
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
    double s = w[j];
    for (int i = 0; i < k1; ++i) s -= hs[i] * V[(int64_t)i * n + j];
    w[j] = s;
  }
}

// x += Σ_i y_i Z_i
__global__ void k_combine(int64_t n, int k1, const double* __restrict__ Z, const double* __restrict__ y,
                          double* __restrict__ x) {
  __shared__ double ys[256];
  for (int i = threadIdx.x; i < k1; i += blockDim.x) ys[i] = y[i];
  __syncthreads();
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
    double s = x[j];
    for (int i = 0; i < k1; ++i) s += ys[i] * Z[(int64_t)i * n + j];
    x[j] = s;
  }
}

__global__ void k_axpby(int64_t n, double a, const double* __restrict__ x, double b, double* __restrict__ y) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x)
    y[j] = a * x[j] + b * y[j];
}

__global__ void k_scale_copy(int64_t n, double a, const double* __restrict__ x, double* __restrict__ y) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x)
    y[j] = a * x[j];
}

// y = x / sqrt(*nrm2) when *nrm2 > 0 (the norm stays on the device)
__global__ void k_scale_rsqrt(int64_t n, const double* __restrict__ nrm2, const double* __restrict__ x,
                              double* __restrict__ y) {
  const double q = *nrm2;
  if (!(q > 0.0)) return;
  const double a = 1.0 / sqrt(q);
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x)
    y[j] = a * x[j];
}

__global__ void k_fz_grad(int64_t ncells, const int32_t* __restrict__ row, const double* __restrict__ lam,
                          const double* __restrict__ fz, double* __restrict__ out) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncells; c += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int n = 0; n < 27; ++n) {
      const int32_t r = row[c * ND + OU + 2 * 27 + n];
      if (r >= 0) s += lam[r] * fz[c * 27 + n];
    }
    out[c] = s;  // dJ/df_z(c) = −λᵀ ∂R/∂f_z(c) = +Σ λ ∫ v_z
  }
}

// ------------------------------------------------------------------ helpers
static int grid_for(gbmhd_ctx* ctx, int64_t n, int threads = 256) {
  int64_t g = (n + threads - 1) / threads;
  return (int)std::max<int64_t>(1, std::min<int64_t>(g, (int64_t)ctx->num_sms * 8));
}

static int dot(gbmhd_ctx* ctx, Solver* s, const double* V, int k1, const double* w, double* hhost) {
  const int64_t n = ctx->ndofs;
  const int nb = (int)std::min<int64_t>(std::max<int64_t>(1, (n + 255) / 256), (int64_t)ctx->num_sms * 2);
  dim3 g(nb, k1);
  { k_mdot_partial<<<g, 256, 0, ctx->stream>>>(n, k1, V, w, s->part); gbmhd::count_launch(); }
  { k_mdot_final<<<k1, 256, 0, ctx->stream>>>(k1, nb, s->part, s->hdev); gbmhd::count_launch(); }
  S_CUDA(cudaGetLastError());
  S_CUDA(cudaMemcpyAsync(hhost, s->hdev, sizeof(double) * k1, cudaMemcpyDeviceToHost, ctx->stream));
  S_CUDA(cudaStreamSynchronize(ctx->stream));
  return 0;
}

// h_dev[i] = V_iᵀ w, i < k1, left on the device (no host round trip).
static int dot_dev(gbmhd_ctx* ctx, Solver* s, const double* V, int k1, const double* w, double* h_dev) {
  const int64_t n = ctx->ndofs;
  const int nb = (int)std::min<int64_t>(std::max<int64_t>(1, (n + 255) / 256), (int64_t)ctx->num_sms * 2);
  dim3 g(nb, k1);
  { k_mdot_partial<<<g, 256, 0, ctx->stream>>>(n, k1, V, w, s->part); gbmhd::count_launch(); }
  { k_mdot_final<<<k1, 256, 0, ctx->stream>>>(k1, nb, s->part, h_dev); gbmhd::count_launch(); }
  S_CUDA(cudaGetLastError());
  return 0;
}

static int spmv(gbmhd_ctx* ctx, int precision, const double* x, double* y) {
  const int64_t n = ctx->ndofs;
  Solver* s = ctx->solver;
  if (precision == GBMHD_MIXED) {
    { k_to_f32<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(n, x, s->x32); gbmhd::count_launch(); }
    { k_spmv_f32<<<grid_for(ctx, n * 32), 256, 0, ctx->stream>>>(n, ctx->d_rowptr, ctx->d_col, ctx->d_val32, s->x32, y); gbmhd::count_launch(); }
  } else {
    { k_spmv_f64<<<grid_for(ctx, n * 8), 256, 0, ctx->stream>>>(0, n, ctx->d_rowptr, ctx->d_col, ctx->d_val64, x, y); gbmhd::count_launch(); }
  }
  S_CUDA(cudaGetLastError());
  return 0;
}

// y[r0:r1) = (Aᵀ x)[r0:r1) with the FP64 transposed values (built by prepare_transpose).
static int spmv_t(gbmhd_ctx* ctx, Solver* s, int64_t r0, int64_t r1, const double* x, double* y) {
  if (r1 <= r0) return 0;
  if (!s->valT) { ctx->err = "transposed operator not prepared"; return -1; }
  { k_spmv_f64<<<grid_for(ctx, (r1 - r0) * 8), 256, 0, ctx->stream>>>(r0, r1, ctx->d_rowptr, ctx->d_col, s->valT, x, y); gbmhd::count_launch(); }
  S_CUDA(cudaGetLastError());
  return 0;
}

static int ensure_workspace(gbmhd_ctx* ctx, int m) {
  Solver* s = ctx->solver;
  const int64_t n = ctx->ndofs;
  if (s->m < m) {
    if (s->V) cudaFree(s->V);
    if (s->Z) cudaFree(s->Z);
    s->V = s->Z = nullptr;
    S_CUDA(cudaMalloc(&s->V, sizeof(double) * n * (m + 1)));
    S_CUDA(cudaMalloc(&s->Z, sizeof(double) * n * m));
    s->m = m;
  }
  if (!s->w) {
    S_CUDA(cudaMalloc(&s->w, sizeof(double) * n));
    S_CUDA(cudaMalloc(&s->t1, sizeof(double) * n));
    S_CUDA(cudaMalloc(&s->t2, sizeof(double) * n));
    S_CUDA(cudaMalloc(&s->x32, sizeof(float) * std::max<int64_t>(n, 1)));
    s->part_len = (int64_t)ctx->num_sms * 2 * 257;
    S_CUDA(cudaMalloc(&s->part, sizeof(double) * s->part_len));
    S_CUDA(cudaMalloc(&s->hdev, sizeof(double) * kHcol));
    S_CUDA(cudaMallocHost(&s->hhost, sizeof(double) * kHcol));
  }
  return 0;
}

// Scale of the root regularisation −ε·diag(mass) of the global p/φ representatives for FP32
// factors (FP64: 1).  Measured at 64×64×4, Ha = 500 (FGMRES iterations per Newton solve, order
// u, j, φ, p): ε = 1: ~29; 1e-2: 25–28; 1e-3: 15–17; 1e-4: 15–16; 1e-5: a singular pivot block.
constexpr double kEps32 = 1e-3;

// Removes the constant-pressure component from a preconditioned FGMRES direction z (z_p −= mean
// z_p) when the all-ones vector on the p dofs is a null vector of the Jacobian (velocity fixed
// on every wall; then also of its transpose).  The pressure is then defined up to a constant
// that the Krylov relation cannot see, and the preconditioner (whose root carries −ε·mass on
// the global p representatives) puts a large, arbitrary amount of that mode into every z.
// Summed into the update, it lets the pressure level drift by O(100) per Newton step, and the
// FP64 residual's rounding, which grows with |p|, stalls Newton above its tolerance.  Removing
// it from each z before J·z is formed keeps the Arnoldi relation exact for the vectors the
// update is built from (removing it from the update afterwards would not: J·1_p vanishes only
// to rounding, and times an O(100) constant that is already the size of the last steps'
// residuals).  The null test uses the FP64 Jacobian:
// max_r |Σ_p J[r, p]| ≤ 1e-10 · max_r Σ_p |J[r, p]|.
static int project_pressure_gauge(gbmhd_ctx* ctx, double* z) {
  Solver* s = ctx->solver;
  const int64_t pb = ctx->offs[1], pe = ctx->offs[2];
  if (pe <= pb || !ctx->d_val64) return 0;
  if (const char* g = std::getenv("GBMHD_GAUGE_PROJECTION"))
    if (std::atoi(g) == 0) return 0;
  if (!s->gsum) S_CUDA(cudaMalloc(&s->gsum, 2 * sizeof(double)));
  if (s->p_null < 0 || s->p_null_gen != ctx->params_gen) {
    S_CUDA(cudaMemsetAsync(s->gsum, 0, 2 * sizeof(double), ctx->stream));
    { k_const_mode<<<grid_for(ctx, ctx->ndofs), 256, 0, ctx->stream>>>(ctx->ndofs, ctx->d_rowptr, ctx->d_col, ctx->d_val64, (int32_t)pb, (int32_t)pe, reinterpret_cast<unsigned long long*>(s->gsum)); gbmhd::count_launch(); }
    double h[2] = {0.0, 0.0};
    S_CUDA(cudaMemcpyAsync(h, s->gsum, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    S_CUDA(cudaStreamSynchronize(ctx->stream));
    s->p_null = h[1] > 0.0 && h[0] <= 1e-10 * h[1];
    s->p_null_gen = ctx->params_gen;
  }
  if (!s->p_null) return 0;
  S_CUDA(cudaMemsetAsync(s->gsum, 0, sizeof(double), ctx->stream));
  { k_range_sum<<<grid_for(ctx, pe - pb), 256, 0, ctx->stream>>>(z, pb, pe, s->gsum); gbmhd::count_launch(); }
  { k_range_shift<<<grid_for(ctx, pe - pb), 256, 0, ctx->stream>>>(z, pb, pe, s->gsum); gbmhd::count_launch(); }
  S_CUDA(cudaGetLastError());
  return 0;
}

// Preconditioner set-up: (u,j) factorization + mass blocks.
static int setup_pc(gbmhd_ctx* ctx, int precision, int kind, double* t_setup) {
  auto t0 = std::chrono::steady_clock::now();
  Solver* s = ctx->solver;
  // Field order of elimination inside a front, per factor precision (measured at 64×64×4,
  // Ha = 500, with the root regularisation below): FP32 factors precondition best with the
  // velocities first (u, j, φ, p: 15–17 FGMRES iterations per Newton solve, against 80–87 for
  // j, u, φ, p with ε = 1 and 27 with ε = 1e-3); with FP64 factors that order let the Newton
  // residual drift up from its floor at the third step, so they keep j, u, φ, p.
  const char* order = precision == GBMHD_FP64 ? "jufp" : "ujfp";
  if (s->mf && (s->pc_kind != kind || s->mf_order != order)) {
    mf_destroy(s->mf);
    s->mf = nullptr;
  }
  s->pc_kind = kind;
  if (!s->mf) {
    MFSymbolic S;
    std::string e = mf_analyse(ctx->ncells, ctx->h_cellX.data(), ctx->h_cell_row.data(), ctx->ndofs,
                               ctx->h_rowptr.data(), ctx->h_col.data(), kind == GBMHD_PC_MONOLITHIC, S, 8, order);
    s->mf_order = order;
    if (!e.empty()) { ctx->err = e; return -1; }
    int rc = mf_create(ctx, S, &s->mf);
    if (rc) return rc;
    // p/φ column segments of the (u,j) rows
    std::vector<int32_t> seg(2 * ctx->ndofs, 0);
    const int64_t pb = ctx->offs[1], pe = ctx->offs[2], fb = ctx->offs[3];
    for (int64_t r = 0; r < ctx->ndofs; ++r) {
      const bool urow = r < pb, jrow = r >= pe && r < fb;
      if (!urow && !jrow) continue;
      const int64_t lo = urow ? pb : fb, hi = urow ? pe : ctx->ndofs;
      const int32_t* cb = ctx->h_col.data() + ctx->h_rowptr[r];
      const int64_t len = ctx->h_rowptr[r + 1] - ctx->h_rowptr[r];
      int64_t a = std::lower_bound(cb, cb + len, (int32_t)lo) - cb;
      int64_t b = std::lower_bound(cb, cb + len, (int32_t)hi) - cb;
      seg[2 * r] = (int32_t)a;
      seg[2 * r + 1] = (int32_t)b;
    }
    S_CUDA(cudaMalloc(&s->seg, sizeof(int32_t) * 2 * ctx->ndofs));
    S_CUDA(cudaMemcpy(s->seg, seg.data(), sizeof(int32_t) * 2 * ctx->ndofs, cudaMemcpyHostToDevice));
  }
  const double want_eps = precision == GBMHD_MIXED ? (std::getenv("GBMHD_PC_EPS32") ? std::atof(std::getenv("GBMHD_PC_EPS32")) : kEps32)
                                                   : (std::getenv("GBMHD_PC_EPS64") ? std::atof(std::getenv("GBMHD_PC_EPS64")) : 1.0);
  if (!s->have_mass || s->mass_beta != ctx->prm.beta || s->mass_zu != ctx->prm.zeta_u ||
      s->mass_zj != ctx->prm.zeta_j || s->reg_eps != want_eps) {
    if (!s->Mp_inv) {
      S_CUDA(cudaMalloc(&s->Mp_inv, sizeof(double) * 16 * ctx->ncells));
      S_CUDA(cudaMalloc(&s->Mf_inv, sizeof(double) * 64 * ctx->ncells));
    }
    RefTables R;
    build_ref_tables(R);
    std::vector<double> w(NQ), gq(NQ * 24), p1(NQ * 4), q1(NQ * 8);
    for (int q = 0; q < NQ; ++q) {
      w[q] = R.w[q];
      for (int v = 0; v < 8; ++v)
        for (int a = 0; a < 3; ++a) gq[(q * 8 + v) * 3 + a] = R.gq1[q][v][a];
      for (int k = 0; k < 4; ++k) p1[q * 4 + k] = R.p1[q][k];
      for (int k = 0; k < 8; ++k) q1[q * 8 + k] = R.q1[q][k];
    }
    double *dw, *dg, *dp, *dq;
    S_CUDA(cudaMalloc(&dw, sizeof(double) * w.size()));
    S_CUDA(cudaMalloc(&dg, sizeof(double) * gq.size()));
    S_CUDA(cudaMalloc(&dp, sizeof(double) * p1.size()));
    S_CUDA(cudaMalloc(&dq, sizeof(double) * q1.size()));
    S_CUDA(cudaMemcpy(dw, w.data(), sizeof(double) * w.size(), cudaMemcpyHostToDevice));
    S_CUDA(cudaMemcpy(dg, gq.data(), sizeof(double) * gq.size(), cudaMemcpyHostToDevice));
    S_CUDA(cudaMemcpy(dp, p1.data(), sizeof(double) * p1.size(), cudaMemcpyHostToDevice));
    S_CUDA(cudaMemcpy(dq, q1.data(), sizeof(double) * q1.size(), cudaMemcpyHostToDevice));
    const double ap = -1.0 / (ctx->prm.beta + ctx->prm.zeta_u);
    const double af = -1.0 / (1.0 + ctx->prm.zeta_j);
    // monolithic: the root's global p/φ representatives get −ε·diag(mass) scaled like the
    // Schur complements (only those pivots are singular when the walls fix u and j·n everywhere)
    double eps = precision == GBMHD_MIXED ? kEps32 : 1.0;
    if (const char* ev = std::getenv(precision == GBMHD_MIXED ? "GBMHD_PC_EPS32" : "GBMHD_PC_EPS64")) eps = std::atof(ev);
    if (!s->reg) S_CUDA(cudaMalloc(&s->reg, sizeof(double) * ctx->ndofs));
    S_CUDA(cudaMemsetAsync(s->reg, 0, sizeof(double) * ctx->ndofs, ctx->stream));
    { k_reg_diag<<<grid_for(ctx, ctx->ncells, 128), 128, 0, ctx->stream>>>(ctx->ncells, ctx->d_cellX, ctx->d_row, dw, dg, dp, dq, -eps * ap, -eps * af, s->reg); gbmhd::count_launch(); }
    s->reg_eps = eps;
    { k_mass_inverse<<<grid_for(ctx, ctx->ncells, 128), 128, 0, ctx->stream>>>(ctx->ncells, ctx->d_cellX, dw, dg, dp,
                                                                             dq, ap, af, s->Mp_inv, s->Mf_inv); gbmhd::count_launch(); }
    S_CUDA(cudaGetLastError());
    S_CUDA(cudaStreamSynchronize(ctx->stream));
    cudaFree(dw); cudaFree(dg); cudaFree(dp); cudaFree(dq);
    s->have_mass = true;
    s->mass_beta = ctx->prm.beta; s->mass_zu = ctx->prm.zeta_u; s->mass_zj = ctx->prm.zeta_j;
  }
  int rc = mf_factor(ctx, s->mf, precision, ctx->jac_precision, kind == GBMHD_PC_MONOLITHIC ? s->reg : nullptr);
  if (rc) return rc;
  s->factor_gen = ctx->params_gen;
  if (t_setup) *t_setup += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return 0;
}

// z = P⁻¹ v (or P⁻ᵀ v).  v is not modified.
static int apply_pc(gbmhd_ctx* ctx, int precision, const double* v, double* z, bool transpose) {
  Solver* s = ctx->solver;
  const int64_t n = ctx->ndofs;
  double* b = s->t2;
  if (s->pc_kind == GBMHD_PC_MONOLITHIC) {
    S_CUDA(cudaMemcpyAsync(b, v, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream));
    return mf_solve(ctx, s->mf, b, z, transpose);
  }
  if (!transpose) {
    // p and φ blocks, then the (u,j) block with the coupling moved to the right-hand side
    { k_mass_apply<<<grid_for(ctx, ctx->ncells, 128), 128, 0, ctx->stream>>>(ctx->ncells, ctx->d_row, s->Mp_inv,
                                                                           s->Mf_inv, v, z, true); gbmhd::count_launch(); }
    S_CUDA(cudaMemcpyAsync(b, v, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream));
    const int g = grid_for(ctx, n);
    if (precision == GBMHD_MIXED)
      { k_coupling<float><<<g, 256, 0, ctx->stream>>>(n, ctx->d_rowptr, ctx->d_col, ctx->d_val32, s->seg, z, b); gbmhd::count_launch(); }
    else
      { k_coupling<double><<<g, 256, 0, ctx->stream>>>(n, ctx->d_rowptr, ctx->d_col, ctx->d_val64, s->seg, z, b); gbmhd::count_launch(); }
    S_CUDA(cudaGetLastError());
    return mf_solve(ctx, s->mf, b, z, false);
  }
  // transpose: (u,j) block first, then p and φ with the coupling Aᵀ z_uj removed
  S_CUDA(cudaMemcpyAsync(b, v, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream));
  int rc = mf_solve(ctx, s->mf, b, z, true);
  if (rc) return rc;
  // t1 = z restricted to (u,j); rows p, φ of Aᵀ t1
  double* t1 = s->t1;
  S_CUDA(cudaMemcpyAsync(t1, z, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream));
  S_CUDA(cudaMemsetAsync(t1 + ctx->offs[1], 0, sizeof(double) * ctx->nfree[1], ctx->stream));
  S_CUDA(cudaMemsetAsync(t1 + ctx->offs[3], 0, sizeof(double) * ctx->nfree[3], ctx->stream));
  double* y = s->w;  // scratch (w is not live during apply_pc in the adjoint path)
  if ((rc = spmv_t(ctx, s, ctx->offs[1], ctx->offs[2], t1, y))) return rc;
  if ((rc = spmv_t(ctx, s, ctx->offs[3], n, t1, y))) return rc;
  // b(p,φ) = v − y
  { k_axpby<<<grid_for(ctx, ctx->nfree[1]), 256, 0, ctx->stream>>>(ctx->nfree[1], -1.0, y + ctx->offs[1], 1.0,
                                                                  b + ctx->offs[1]); gbmhd::count_launch(); }
  { k_axpby<<<grid_for(ctx, ctx->nfree[3]), 256, 0, ctx->stream>>>(ctx->nfree[3], -1.0, y + ctx->offs[3], 1.0,
                                                                  b + ctx->offs[3]); gbmhd::count_launch(); }
  { k_mass_apply<<<grid_for(ctx, ctx->ncells, 128), 128, 0, ctx->stream>>>(ctx->ncells, ctx->d_row, s->Mp_inv,
                                                                         s->Mf_inv, b, z, true); gbmhd::count_launch(); }
  S_CUDA(cudaGetLastError());
  return 0;
}

// FGMRES(m), right preconditioned, FP64 vectors.  Solves A x = b from x = 0.
// Returns iterations in *iters; final relative residual in *rel.
// With stagnated non-null, the solve also stops when the residual estimate is still above half
// of |b| after kStagIters iterations (a preconditioner that does not work) and reports it there.
constexpr int kStagIters = 100;
constexpr double kStagRel = 0.5;
// Diagnostic overrides of the stagnation test (GBMHD_STAG_ITERS, GBMHD_STAG_REL), used by a
// test that drives the refactorization and FP64-fallback path on purpose.
static int stag_iters() {
  const char* e = std::getenv("GBMHD_STAG_ITERS");
  return e ? std::max(1, std::atoi(e)) : kStagIters;
}
static double stag_rel() {
  const char* e = std::getenv("GBMHD_STAG_REL");
  return e ? std::atof(e) : kStagRel;
}
static int fgmres(gbmhd_ctx* ctx, int precision, const double* b, double* x, int m, int maxit, double rtol,
                  bool transpose, int* iters, double* rel, int verbose, bool* stagnated = nullptr) {
  if (stagnated) *stagnated = false;
  Solver* s = ctx->solver;
  const int64_t n = ctx->ndofs;
  int rc = ensure_workspace(ctx, m);
  if (rc) return rc;
  auto op = [&](const double* in, double* out) -> int {
    if (!transpose) return spmv(ctx, precision, in, out);
    int r = spmv_t(ctx, s, 0, n, in, out);
    return r;
  };
  S_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * n, ctx->stream));
  const int s_iters = stag_iters();
  const double s_rel = stag_rel();
  std::vector<double> H((m + 1) * m), cs(m), sn(m), g(m + 1), h(m + 2);
  double bnorm = 0.0;
  if ((rc = dot(ctx, s, b, 1, b, &bnorm))) return rc;
  bnorm = std::sqrt(bnorm);
  *iters = 0;
  *rel = 0.0;
  if (bnorm == 0.0) return 0;
  double beta = bnorm;
  // r = b (x = 0)
  double* r = s->V;  // V_0 will hold r / beta
  { k_scale_copy<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(n, 1.0 / beta, b, r); gbmhd::count_launch(); }
  int it = 0;
  const int guard = std::max(1, maxit);
  while (true) {
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = beta;
    int k = 0;
    for (; k < m && it < guard; ++k) {
      double* vk = s->V + (int64_t)k * n;
      double* zk = s->Z + (int64_t)k * n;
      if ((rc = apply_pc(ctx, precision, vk, zk, transpose))) return rc;
      if ((rc = project_pressure_gauge(ctx, zk))) return rc;
      if ((rc = op(zk, s->w))) return rc;
      // CGS2 with the coefficients kept on the device; one host round trip per iteration
      if ((rc = dot_dev(ctx, s, s->V, k + 1, s->w, s->hdev))) return rc;
      { k_mgs_update<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(n, k + 1, s->V, s->hdev, s->w); gbmhd::count_launch(); }
      if ((rc = dot_dev(ctx, s, s->V, k + 1, s->w, s->hdev + kHB))) return rc;
      { k_mgs_update<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(n, k + 1, s->V, s->hdev + kHB, s->w); gbmhd::count_launch(); }
      if ((rc = dot_dev(ctx, s, s->w, 1, s->w, s->hdev + kHN))) return rc;
      { k_scale_rsqrt<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(n, s->hdev + kHN, s->w, s->V + (int64_t)(k + 1) * n); gbmhd::count_launch(); }
      S_CUDA(cudaMemcpyAsync(s->hhost, s->hdev, sizeof(double) * kHcol, cudaMemcpyDeviceToHost, ctx->stream));
      S_CUDA(cudaStreamSynchronize(ctx->stream));
      for (int i = 0; i <= k; ++i) h[i] = s->hhost[i] + s->hhost[kHB + i];
      const double hn = std::sqrt(std::max(0.0, s->hhost[kHN]));
      for (int i = 0; i <= k; ++i) H[i * m + k] = h[i];
      H[(k + 1) * m + k] = hn;
      for (int i = 0; i < k; ++i) {
        const double t = cs[i] * H[i * m + k] + sn[i] * H[(i + 1) * m + k];
        H[(i + 1) * m + k] = -sn[i] * H[i * m + k] + cs[i] * H[(i + 1) * m + k];
        H[i * m + k] = t;
      }
      const double d = std::hypot(H[k * m + k], H[(k + 1) * m + k]);
      cs[k] = d > 0 ? H[k * m + k] / d : 1.0;
      sn[k] = d > 0 ? H[(k + 1) * m + k] / d : 0.0;
      H[k * m + k] = d;
      H[(k + 1) * m + k] = 0.0;
      g[k + 1] = -sn[k] * g[k];
      g[k] = cs[k] * g[k];
      ++it;
      *rel = std::fabs(g[k + 1]) / bnorm;
      if (verbose > 1) std::fprintf(stderr, "  fgmres %d: %.3e\n", it, *rel);
      if (!std::isfinite(*rel)) { ctx->err = "FGMRES produced a non-finite residual"; return -3; }
      if (*rel <= rtol || hn == 0.0) { ++k; break; }
      if (stagnated && it >= s_iters && *rel > s_rel) { *stagnated = true; ++k; break; }
    }
    // x += Z y,  H y = g (upper triangular k x k)
    std::vector<double> y(k, 0.0);
    for (int i = k - 1; i >= 0; --i) {
      double sacc = g[i];
      for (int j = i + 1; j < k; ++j) sacc -= H[i * m + j] * y[j];
      y[i] = H[i * m + i] != 0.0 ? sacc / H[i * m + i] : 0.0;
    }
    S_CUDA(cudaMemcpyAsync(s->hdev, y.data(), sizeof(double) * std::max(k, 1), cudaMemcpyHostToDevice, ctx->stream));
    { k_combine<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(n, k, s->Z, s->hdev, x); gbmhd::count_launch(); }
    S_CUDA(cudaGetLastError());
    if (*rel <= rtol || it >= guard || (stagnated && *stagnated)) break;
    // restart: r = b − A x
    if ((rc = op(x, s->w))) return rc;
    { k_axpby<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(n, 1.0, b, -1.0, s->w); gbmhd::count_launch(); }
    double rr = 0.0;
    if ((rc = dot(ctx, s, s->w, 1, s->w, &rr))) return rc;
    beta = std::sqrt(rr);
    *rel = beta / bnorm;
    if (*rel <= rtol) break;
    { k_scale_copy<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(n, 1.0 / beta, s->w, s->V); gbmhd::count_launch(); }
  }
  *iters = it;
  return 0;
}

void solver_destroy(gbmhd_ctx* ctx) {
  Solver* s = ctx->solver;
  if (!s) return;
  mf_destroy(s->mf);
  void* ptrs[] = {s->reg, s->Mp_inv, s->Mf_inv, s->seg, s->V, s->Z, s->w, s->t1, s->t2, s->x32, s->part,
                  s->hdev, s->permT, s->valT, s->gsum};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (s->hhost) cudaFreeHost(s->hhost);
  delete s;
  ctx->solver = nullptr;
}

static int check_opts(gbmhd_ctx* ctx, const gbmhd_solve_opts* o) {
  if (!o) { ctx->err = "solve options are NULL"; return -1; }
  if (o->precision != GBMHD_FP64 && o->precision != GBMHD_MIXED && o->precision != GBMHD_MIXED_F64OP) {
    ctx->err = "unknown precision";
    return -1;
  }
  if (o->max_newton < 1 || o->max_newton > 60) { ctx->err = "max_newton must be in [1, 60]"; return -1; }
  if (o->restart < 1 || o->restart > 250) { ctx->err = "restart must be in [1, 250]"; return -1; }
  if (o->max_linear < 1) { ctx->err = "max_linear must be >= 1"; return -1; }
  if (o->preconditioner != GBMHD_PC_MONOLITHIC && o->preconditioner != GBMHD_PC_BADIA2024) {
    ctx->err = "unknown preconditioner";
    return -1;
  }
  if (!(o->newton_rtol >= 0.0) || !(o->newton_atol >= 0.0) || !(o->linear_rtol > 0.0)) {
    ctx->err = "tolerances must be non-negative";
    return -1;
  }
  return 0;
}

static double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

extern "C" int gbmhd_newton_solve_device(gbmhd_ctx* ctx, double* d_x, const gbmhd_solve_opts* o, gbmhd_report* rep) {
  if (!ctx) return -1;
  int rc = check_opts(ctx, o);
  if (rc) return rc;
  if (!d_x) { ctx->err = "x is NULL"; return -1; }
  if (!ctx->solver) ctx->solver = new Solver();
  if ((rc = ensure_workspace(ctx, o->restart))) return rc;  // dot() needs the reduction buffers
  gbmhd_report R{};
  const double t_start = now_s();
  const int64_t n = ctx->ndofs;
  // The FGMRES operator is the FP64 Jacobian in every mode.  The factors (the preconditioner)
  // are FP32 in the mixed modes: in GBMHD_MIXED they come from FP32 element matrices, in
  // GBMHD_MIXED_F64OP from the FP64 Jacobian.  (An FP32-Jacobian operator for the first
  // steps, i.e. Newton-level iterative refinement, measured 85–240 FGMRES iterations per
  // solve at Ha = 500 against 79–84 with the FP64 operator from the start.)
  // precision of the factors: FP32 in the mixed modes until the stagnation safeguard moves
  // it to FP64 for the rest of the solve
  int fprec = o->precision == GBMHD_FP64 ? GBMHD_FP64 : GBMHD_MIXED;
  const bool fp32_elements = o->precision == GBMHD_MIXED;
  if (!ctx->d_val64) S_CUDA(cudaMalloc(&ctx->d_val64, sizeof(double) * ctx->nnz));
  if (fp32_elements && !ctx->d_val32) S_CUDA(cudaMalloc(&ctx->d_val32, sizeof(float) * ctx->nnz));
  double* r = ctx->d_r;
  double r0 = 0.0;
  bool factored = false;
  int status = 1;
  for (int it = 0;; ++it) {
    double ta = now_s();
    if ((rc = gb_assemble_device(ctx, d_x, r, 0, GBMHD_FP64))) return rc;
    double rn = 0.0;
    if ((rc = dot(ctx, ctx->solver, r, 1, r, &rn))) return rc;
    rn = std::sqrt(rn);
    R.time_assembly_s += now_s() - ta;
    if (!std::isfinite(rn)) { ctx->err = "non-finite Newton residual"; return -3; }
    if (it == 0) { r0 = rn; R.initial_residual = rn; }
    if (it < 64) R.residual_history[it] = rn;
    R.final_residual = rn;
    R.newton_iters = it;
    if (o->verbose) std::fprintf(stderr, "newton %d: |r| = %.6e\n", it, rn);
    const double target = std::max(o->newton_atol, o->newton_rtol * r0);
    if (rn <= target) { status = 0; break; }
    const double prev = it > 0 ? R.residual_history[std::min(it - 1, 63)] : rn;
    // attainable-accuracy stop: the FP64 residual no longer decreases
    if (it >= 2 && rn > 0.9 * prev && rn <= 1e-9 * r0) { status = 0; break; }
    if (it >= o->max_newton) break;
    ta = now_s();
    if (!factored) {
      // the factors are computed once, from the Jacobian at the initial state, and reused as a
      // lagged preconditioner by the later steps
      if (fp32_elements && (rc = gb_assemble_device(ctx, d_x, nullptr, 1, GBMHD_MIXED))) return rc;
      if (!fp32_elements && (rc = gb_assemble_device(ctx, d_x, nullptr, 1, GBMHD_FP64))) return rc;
      S_CUDA(cudaStreamSynchronize(ctx->stream));
      R.time_assembly_s += now_s() - ta;
      if ((rc = setup_pc(ctx, fprec, o->preconditioner, &R.time_setup_pc_s))) return rc;
      factored = true;
      ta = now_s();
    }
    if (fp32_elements || it > 0)  // the operator: FP64 Jacobian at the current state
      if ((rc = gb_assemble_device(ctx, d_x, nullptr, 1, GBMHD_FP64))) return rc;
    S_CUDA(cudaStreamSynchronize(ctx->stream));
    R.time_assembly_s += now_s() - ta;
    // solve J δ = −r (δ in r); a linear solve on the FP64 operator reduces the Newton residual
    // by about its tolerance, so it asks for just the reduction that reaches the target
    // (never less than linear_rtol, never beyond 1e-10)
    double tl = now_s();
    int iters = 0;
    double rel = 0.0;
    if ((rc = ensure_workspace(ctx, o->restart))) return rc;
    { k_scale_copy<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(n, -1.0, r, ctx->d_xtmp); gbmhd::count_launch(); }
    const double lin_rtol = std::min(o->linear_rtol, std::max(0.5 * target / rn, 1e-10));
    bool stagnated = false;
    if ((rc = fgmres(ctx, GBMHD_FP64, ctx->d_xtmp, r, o->restart, o->max_linear, lin_rtol, false, &iters, &rel,
                     o->verbose, fprec == GBMHD_MIXED ? &stagnated : nullptr)))
      return rc;
    R.linear_iters += iters;
    if (stagnated) {
      // The FP32 factors carry the rounding of the FP32 assembly and extend-add (atomics in
      // arbitrary order), so two factorizations of the same Jacobian differ; a rare one does
      // not precondition at all.  Refactor once, in FP32 from the FP64 Jacobian at the current
      // state, and solve the step again; if that stagnates too, factor in FP64 (the plain
      // path's preconditioner) for the rest of the solve.
      if (o->verbose) std::fprintf(stderr, "  linear solve stagnated (%d iterations, rel %.3e): refactoring\n", iters, rel);
      R.pc_refactorizations += 1;
      S_CUDA(cudaStreamSynchronize(ctx->stream));
      if ((rc = setup_pc(ctx, fprec, o->preconditioner, &R.time_setup_pc_s))) return rc;
      if ((rc = fgmres(ctx, GBMHD_FP64, ctx->d_xtmp, r, o->restart, o->max_linear, lin_rtol, false, &iters, &rel,
                       o->verbose, &stagnated)))
        return rc;
      R.linear_iters += iters;
      if (stagnated) {
        if (o->verbose) std::fprintf(stderr, "  stagnated again: FP64 factors\n");
        R.pc_refactorizations += 1;
        fprec = GBMHD_FP64;  // the later steps keep the FP64 factors and skip the stagnation test
        S_CUDA(cudaStreamSynchronize(ctx->stream));
        if ((rc = setup_pc(ctx, GBMHD_FP64, o->preconditioner, &R.time_setup_pc_s))) return rc;
        if ((rc = fgmres(ctx, GBMHD_FP64, ctx->d_xtmp, r, o->restart, o->max_linear, lin_rtol, false, &iters,
                         &rel, o->verbose)))
          return rc;
        R.linear_iters += iters;
      }
    }
    // a preconditioner application whose TMA copies timed out was cut short: fail this step
    if (ctx->solver->mf && (rc = mf_check_sweeps(ctx, ctx->solver->mf))) return rc;
    { k_axpby<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(n, 1.0, r, 1.0, d_x); gbmhd::count_launch(); }
    S_CUDA(cudaStreamSynchronize(ctx->stream));
    R.time_linear_s += now_s() - tl;
    if (o->verbose) std::fprintf(stderr, "  linear: %d iterations, rel %.3e\n", iters, rel);
  }
  R.converged = status == 0;
  R.time_total_s = now_s() - t_start;
  if (rep) *rep = R;
  return status;
}

extern "C" int gbmhd_newton_solve(gbmhd_ctx* ctx, double* x, const gbmhd_solve_opts* o, gbmhd_report* rep) {
  if (!ctx) return -1;
  if (!x) { ctx->err = "x is NULL"; return -1; }
  double* d_x = nullptr;
  S_CUDA(cudaMalloc(&d_x, sizeof(double) * ctx->ndofs));
  cudaError_t e = cudaMemcpyAsync(d_x, x, sizeof(double) * ctx->ndofs, cudaMemcpyHostToDevice, ctx->stream);
  if (e != cudaSuccess) { cudaFree(d_x); ctx->err = cudaGetErrorString(e); return -2; }
  int rc = gbmhd_newton_solve_device(ctx, d_x, o, rep);
  if (rc >= 0) {
    e = cudaMemcpyAsync(x, d_x, sizeof(double) * ctx->ndofs, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) { ctx->err = cudaGetErrorString(e); rc = -2; }
  }
  cudaFree(d_x);
  return rc;
}

// Transposed FP64 Jacobian values for the adjoint (the map once per context, the values
// after every FP64 assembly).
static int prepare_transpose(gbmhd_ctx* ctx) {
  Solver* s = ctx->solver;
  const int64_t n = ctx->ndofs, nnz = ctx->nnz;
  if (!s->permT) {
    int32_t* d_err = nullptr;
    S_CUDA(cudaMalloc(&s->permT, sizeof(int64_t) * std::max<int64_t>(nnz, 1)));
    S_CUDA(cudaMalloc(&d_err, sizeof(int32_t)));
    S_CUDA(cudaMemsetAsync(d_err, 0, sizeof(int32_t), ctx->stream));
    { k_transpose_map<<<grid_for(ctx, n * 32), 256, 0, ctx->stream>>>(n, ctx->d_rowptr, ctx->d_col, s->permT, d_err); gbmhd::count_launch(); }
    int32_t herr = 0;
    S_CUDA(cudaMemcpyAsync(&herr, d_err, sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
    S_CUDA(cudaStreamSynchronize(ctx->stream));
    cudaFree(d_err);
    if (herr) {
      cudaFree(s->permT);
      s->permT = nullptr;
      ctx->err = "adjoint: the Jacobian pattern is not structurally symmetric";
      return -3;
    }
  }
  if (!s->valT) S_CUDA(cudaMalloc(&s->valT, sizeof(double) * std::max<int64_t>(nnz, 1)));
  { k_gather_vals<<<grid_for(ctx, nnz), 256, 0, ctx->stream>>>(nnz, ctx->d_val64, s->permT, s->valT); gbmhd::count_launch(); }
  S_CUDA(cudaGetLastError());
  return 0;
}

extern "C" int gbmhd_adjoint(gbmhd_ctx* ctx, const double* x, const gbmhd_objective* obj, const gbmhd_solve_opts* o,
                             double* dJ, int64_t ntheta, double* lambda_out, gbmhd_report* rep) {
  if (!ctx) return -1;
  int rc = check_opts(ctx, o);
  if (rc) return rc;
  if (!x || !obj || !obj->dJdx || !dJ) { ctx->err = "adjoint: NULL argument"; return -1; }
  const int64_t need = 4 + (obj->n_theta_cells > 0 ? ctx->ncells : 0);
  if (ntheta < need) { ctx->err = "adjoint: dJ_dtheta too short"; return -1; }
  if (!ctx->solver) ctx->solver = new Solver();
  if ((rc = ensure_workspace(ctx, o->restart))) return rc;
  Solver* s = ctx->solver;
  const double t0 = now_s();
  gbmhd_report R{};
  const int64_t n = ctx->ndofs;
  double *d_x = nullptr, *d_g = nullptr, *d_lam = nullptr, *d_dg = nullptr, *d_dc = nullptr, *d_fz = nullptr,
         *d_out = nullptr, *d_da = nullptr, *d_db = nullptr;
  auto cleanup = [&]() {
    for (double* p : {d_x, d_g, d_lam, d_dg, d_dc, d_fz, d_out, d_da, d_db})
      if (p) cudaFree(p);
  };
  auto fail = [&](int code) { cleanup(); return code; };
  if (cudaMalloc(&d_x, sizeof(double) * n) || cudaMalloc(&d_g, sizeof(double) * n) ||
      cudaMalloc(&d_lam, sizeof(double) * n) || cudaMalloc(&d_dg, sizeof(double) * n) ||
      cudaMalloc(&d_dc, sizeof(double) * n) || cudaMalloc(&d_fz, sizeof(double) * 27 * ctx->ncells) ||
      cudaMalloc(&d_out, sizeof(double) * ctx->ncells) || cudaMalloc(&d_da, sizeof(double) * n) ||
      cudaMalloc(&d_db, sizeof(double) * n)) {
    ctx->err = "adjoint: device allocation failed";
    return fail(-2);
  }
  if (cudaMemcpy(d_x, x, sizeof(double) * n, cudaMemcpyHostToDevice) ||
      cudaMemcpy(d_g, obj->dJdx, sizeof(double) * n, cudaMemcpyHostToDevice)) {
    ctx->err = "adjoint: copy failed";
    return fail(-2);
  }
  // Iterative refinement on the FP64 transposed Jacobian: each correction solves Aᵀδ = r with
  // FGMRES (FP64 operator) preconditioned by the path's factors.  The factors of the last
  // Newton solve on this context are reused when their precision and kind match and the
  // parameters have not changed since: the refinement converges to the FP64 adjoint
  // whatever Jacobian they came from.
  const int fprec = o->precision == GBMHD_FP64 ? GBMHD_FP64 : GBMHD_MIXED;
  if (!ctx->d_val64) {
    if (cudaMalloc(&ctx->d_val64, sizeof(double) * ctx->nnz)) { ctx->err = "adjoint: allocation"; return fail(-2); }
  }
  double ta = now_s();
  if ((rc = gb_assemble_device(ctx, d_x, nullptr, 1, GBMHD_FP64))) return fail(rc);
  const bool reuse = s->mf && mf_precision(s->mf) == fprec && s->pc_kind == o->preconditioner &&
                     s->factor_gen == ctx->params_gen;
  if (!reuse && (rc = setup_pc(ctx, fprec, o->preconditioner, &R.time_setup_pc_s))) return fail(rc);
  if ((rc = prepare_transpose(ctx))) return fail(rc);
  cudaStreamSynchronize(ctx->stream);
  R.time_assembly_s += now_s() - ta;
  double tl = now_s();
  double *d_res = nullptr, *d_del = nullptr;
  if (cudaMalloc(&d_res, sizeof(double) * n) || cudaMalloc(&d_del, sizeof(double) * n)) {
    ctx->err = "adjoint: allocation";
    if (d_res) cudaFree(d_res);
    return fail(-2);
  }
  S_CUDA(cudaMemsetAsync(d_lam, 0, sizeof(double) * n, ctx->stream));
  S_CUDA(cudaMemcpyAsync(d_res, d_g, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream));
  double gn = 0.0, rn = 0.0, rel = 1.0;
  int total = 0;
  if ((rc = dot(ctx, s, d_g, 1, d_g, &gn))) { cudaFree(d_res); cudaFree(d_del); return fail(rc); }
  gn = std::sqrt(gn);
  // Each correction solve only has to reduce the current residual to the target; the loop
  // stops when the true residual no longer halves (the FP64 operator's attainable accuracy).
  double prev = 1.0;
  for (int k = 0; k < 20 && gn > 0.0; ++k) {
    int iters = 0;
    double irel = 0.0;
    const double inner_rtol = std::min(0.5, std::max(o->linear_rtol / rel, 1e-12));
    if ((rc = fgmres(ctx, GBMHD_FP64, d_res, d_del, o->restart, o->max_linear, inner_rtol, true, &iters, &irel,
                     o->verbose))) {
      cudaFree(d_res); cudaFree(d_del);
      return fail(rc);
    }
    total += iters;
    { k_axpby<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(n, 1.0, d_del, 1.0, d_lam); gbmhd::count_launch(); }
    if ((rc = spmv_t(ctx, s, 0, n, d_lam, d_res))) { cudaFree(d_res); cudaFree(d_del); return fail(rc); }
    { k_axpby<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(n, 1.0, d_g, -1.0, d_res); gbmhd::count_launch(); }
    if ((rc = dot(ctx, s, d_res, 1, d_res, &rn))) { cudaFree(d_res); cudaFree(d_del); return fail(rc); }
    rel = std::sqrt(rn) / gn;
    if (o->verbose) std::fprintf(stderr, "adjoint refinement %d: %d iterations, |g - Aᵀλ|/|g| = %.3e\n", k, iters, rel);
    if (rel <= o->linear_rtol || rel > 0.5 * prev) break;
    prev = rel;
  }
  cudaFree(d_res);
  cudaFree(d_del);
  if (s->mf && (rc = mf_check_sweeps(ctx, s->mf))) return fail(rc);
  R.linear_iters = total;
  R.final_residual = rel;
  R.time_linear_s = now_s() - tl;
  if ((rc = gb_param_derivs(ctx, d_x, d_dg, d_dc, d_fz, d_da, d_db))) return fail(rc);
  std::vector<double> tmp(4);
  if ((rc = dot(ctx, s, d_lam, 1, d_dg, &tmp[0]))) return fail(rc);
  if ((rc = dot(ctx, s, d_lam, 1, d_dc, &tmp[1]))) return fail(rc);
  if ((rc = dot(ctx, s, d_lam, 1, d_da, &tmp[2]))) return fail(rc);
  if ((rc = dot(ctx, s, d_lam, 1, d_db, &tmp[3]))) return fail(rc);
  for (int k = 0; k < 4; ++k) dJ[k] = -tmp[k];
  if (obj->n_theta_cells > 0) {
    { k_fz_grad<<<grid_for(ctx, ctx->ncells), 256, 0, ctx->stream>>>(ctx->ncells, ctx->d_row, d_lam, d_fz, d_out); gbmhd::count_launch(); }
    // the context stream is non-blocking: copy on it and wait for it
    if (cudaMemcpyAsync(dJ + 4, d_out, sizeof(double) * ctx->ncells, cudaMemcpyDeviceToHost, ctx->stream) ||
        cudaStreamSynchronize(ctx->stream)) {
      ctx->err = "adjoint: copy failed";
      return fail(-2);
    }
  }
  if (lambda_out) {
    if (cudaMemcpyAsync(lambda_out, d_lam, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream) ||
        cudaStreamSynchronize(ctx->stream)) {
      ctx->err = "adjoint: copy failed";
      return fail(-2);
    }
  }
  R.converged = rel <= o->linear_rtol;
  R.time_total_s = now_s() - t0;
  if (rep) *rep = R;
  cleanup();
  return R.converged ? 0 : 1;
}

// Diagnostic: relative error ‖x − A_uj⁻¹(A_uj x)‖/‖x‖ of the (u,j) block solve for a
// seeded random x, with the factors of the Jacobian assembled at d_state in `precision`.
__global__ void k_rand_uj(int64_t n, int64_t pb, int64_t pe, int64_t fb, uint64_t seed, double* x) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
    const bool uj = j < pb || (j >= pe && j < fb);
    uint64_t z = seed + 0x9E3779B97F4A7C15ull * (uint64_t)(j + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    x[j] = uj ? ((double)(z >> 11) * (1.0 / 9007199254740992.0) - 0.5) : 0.0;
  }
}

__global__ void k_zero_non_uj(int64_t n, int64_t pb, int64_t pe, int64_t fb, double* x) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
    const bool uj = j < pb || (j >= pe && j < fb);
    if (!uj) x[j] = 0.0;
  }
}

extern "C" int gbmhd_sweep_stats(gbmhd_ctx* ctx, int64_t* applies, double* seconds, double* bytes_per_apply) {
  if (!ctx || !applies || !seconds || !bytes_per_apply) return -1;
  *applies = 0;
  *seconds = 0.0;
  *bytes_per_apply = 0.0;
  if (!ctx->solver || !ctx->solver->mf) return 0;
  mf_sweep_stats(ctx->solver->mf, applies, seconds, bytes_per_apply);
  return 0;
}

extern "C" int gbmhd_diag_uj_solve_error(gbmhd_ctx* ctx, const double* d_state, int32_t precision, double* err) {
  if (!ctx || !d_state || !err) return -1;
  if (!ctx->solver) ctx->solver = new Solver();
  int rc = ensure_workspace(ctx, 1);
  if (rc) return rc;
  Solver* s = ctx->solver;
  const int64_t n = ctx->ndofs;
  if (precision == GBMHD_MIXED) {
    if (!ctx->d_val32) S_CUDA(cudaMalloc(&ctx->d_val32, sizeof(float) * ctx->nnz));
  } else {
    if (!ctx->d_val64) S_CUDA(cudaMalloc(&ctx->d_val64, sizeof(double) * ctx->nnz));
  }
  if ((rc = gb_assemble_device(ctx, d_state, nullptr, 1, precision))) return rc;
  if ((rc = setup_pc(ctx, precision, GBMHD_PC_BADIA2024, nullptr))) return rc;
  double* x = s->V;  // V has room for at least two vectors
  double* y = s->V + n;
  const int64_t pb = ctx->offs[1], pe = ctx->offs[2], fb = ctx->offs[3];
  { k_rand_uj<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(n, pb, pe, fb, 12345ull, x); gbmhd::count_launch(); }
  if ((rc = spmv(ctx, precision, x, s->t1))) return rc;
  { k_zero_non_uj<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(n, pb, pe, fb, s->t1); gbmhd::count_launch(); }
  S_CUDA(cudaMemsetAsync(y, 0, sizeof(double) * n, ctx->stream));
  if ((rc = mf_solve(ctx, s->mf, s->t1, y, false))) return rc;
  { k_axpby<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(n, 1.0, x, -1.0, y); gbmhd::count_launch(); }
  double e2 = 0.0, x2 = 0.0;
  if ((rc = dot(ctx, s, y, 1, y, &e2))) return rc;
  if ((rc = dot(ctx, s, x, 1, x, &x2))) return rc;
  *err = std::sqrt(e2 / x2);
  return 0;
}


// Diagnostic: ‖y32 − y64‖/‖y64‖ for y = P⁻¹ b (or P⁻ᵀ b) with the monolithic preconditioner
// factored in FP32 (from the FP32 Jacobian) and in FP64, for a seeded random b, the Jacobian
// assembled at d_state.  Both factorizations are of the same regularised matrix, so the
// difference measures the FP32 factors and sweeps in that direction.
__global__ void k_rand_all(int64_t n, uint64_t seed, double* x) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
    uint64_t z = seed + 0x9E3779B97F4A7C15ull * (uint64_t)(j + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    x[j] = (double)(z >> 11) * (1.0 / 9007199254740992.0) - 0.5;
  }
}

extern "C" int gbmhd_diag_pc_compare(gbmhd_ctx* ctx, const double* d_state, int32_t transpose, double* err) {
  if (!ctx || !d_state || !err) return -1;
  if (!ctx->solver) ctx->solver = new Solver();
  int rc = ensure_workspace(ctx, 4);
  if (rc) return rc;
  Solver* s = ctx->solver;
  const int64_t n = ctx->ndofs;
  if (!ctx->d_val32) S_CUDA(cudaMalloc(&ctx->d_val32, sizeof(float) * ctx->nnz));
  if (!ctx->d_val64) S_CUDA(cudaMalloc(&ctx->d_val64, sizeof(double) * ctx->nnz));
  double* b = s->V;
  double* y32 = s->V + n;
  double* y64 = s->V + 2 * n;
  { k_rand_all<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(n, 4242ull, b); gbmhd::count_launch(); }
  if ((rc = gb_assemble_device(ctx, d_state, nullptr, 1, GBMHD_MIXED))) return rc;
  if ((rc = setup_pc(ctx, GBMHD_MIXED, GBMHD_PC_MONOLITHIC, nullptr))) return rc;
  if ((rc = apply_pc(ctx, GBMHD_MIXED, b, y32, transpose != 0))) return rc;
  if ((rc = gb_assemble_device(ctx, d_state, nullptr, 1, GBMHD_FP64))) return rc;
  if ((rc = setup_pc(ctx, GBMHD_FP64, GBMHD_PC_MONOLITHIC, nullptr))) return rc;
  if ((rc = apply_pc(ctx, GBMHD_FP64, b, y64, transpose != 0))) return rc;
  if ((rc = mf_check_sweeps(ctx, s->mf))) return rc;
  double d2 = 0.0, r2 = 0.0;
  { k_axpby<<<grid_for(ctx, n), 256, 0, ctx->stream>>>(n, -1.0, y64, 1.0, y32); gbmhd::count_launch(); }
  if ((rc = dot(ctx, s, y32, 1, y32, &d2))) return rc;
  if ((rc = dot(ctx, s, y64, 1, y64, &r2))) return rc;
  *err = std::sqrt(d2 / r2);
  return 0;
}
