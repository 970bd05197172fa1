// Cell and facet assembly kernels of the inductionless-MHD Newton system.
//
// Integrands (GridapMHD src/weakforms.jl):
//   residual  :255-281  β∇u:∇v + α v·((∇u)ᵀu) − p div v − γ(j×B)·v − div u q + j·s
//                       − σφ div s − σ(u×B)·s − div j ϕ − f·v − g·s
//                       (+ ζᵤ Πp(div u) div v + ζⱼ div j div s)
//   Jacobian  :283-312  β∇du:∇v + α v·((∇du)ᵀu + (∇u)ᵀdu) − dp div v − γ(dj×B)·v
//                       − div du q + dj·s − σ dφ div s − σ(du×B)·s − div dj ϕ (+ AL)
//   facets    :716-733  τ(s·n)(j·n − jw + cw n·∇j·n) and (s·n)φ0
//
// Design: one persistent CTA per SM slot walks the cells; the reference tables
// are staged once per CTA in shared memory; geometry (J, det J, J⁻¹) is FP64;
// element blocks are formed in T (float for the mixed path, double for the
// FP64 path) and added into the CSR values with fire-and-forget atomics at the
// offsets of the cell's map class.  The residual is always FP64.
#include <algorithm>
#include <cstdio>

#include "internal.h"

namespace gbmhd {

constexpr int CELL_THREADS = 128;  // threads of a cell CTA (single-pass phases need >= 27)
static_assert(CELL_THREADS >= NQ && CELL_THREADS >= 24, "cell kernel phases assume one thread per Gauss point");
constexpr int CELL_MINB = 3;       // resident CTAs per SM the register budget is sized for

template <typename T>
struct CellWork {
  double X[24];
  double val[ND];
  double wdet[NQ];
  double idet[NQ];
  double Jinv[NQ][9];   // [e*3+i] = (J⁻¹)_{e i}
  double Jd[NQ][9];     // [i*3+m] = J_{i m} / det J
  double Mpi[16];
  double pic[4];
  double divmom[4];
  int64_t rbase[ND];
  int32_t row[ND];
  unsigned long long sign;
  int32_t pad;
  T wdT[NQ];            // w det J in the element-matrix precision
  T idetT[NQ];
  T JinvT[NQ][9];
  T JdT[NQ][9];
  T valT[ND];           // local state in the element-matrix precision
  T G[NQ][3][27];       // physical Q2 gradients  [q][i][n]
  T S[NQ][3][36];       // physical RT values     [q][i][b]
  T Sdiv[NQ][36];
  T u[NQ][3];
  T gu[NQ][9];          // [i*3+c] = ∂_i u_c
  T jv[NQ][3];
  T divj[NQ];
  T ph[NQ];
  T pp[NQ];
  T ugb[NQ][27];        // w det Σ_k u_k ∂_k N_b
  T wn2[NQ][27];        // w det N_a
  T Bd[4][81];          // ∫ ψ_k div φ_(c,a)
  T Tm[4][81];          // Mp⁻¹ Bd
};

struct GeoTables {
  double w[NQ];
  double gq1[NQ][8][3];
};

struct KArgs {
  int64_t ncells;
  const double* cellX;
  const int32_t* gidx;
  const int32_t* row;
  const unsigned long long* sign;
  const double* xfull;
  const double* fcell;
  const int64_t* rowptr;
  const int32_t* cls;
  const uint16_t* offtab;
  void* val;          // T*
  double* r;
  DevParams prm;
  int jpart;          // Jacobian terms: 0 all, 1 the state-independent ones, 2 convection only
};

__device__ __forceinline__ void red_add(float* p, float v) { atomicAdd(p, v); }
__device__ __forceinline__ void red_add(double* p, double v) { atomicAdd(p, v); }

template <typename T, bool JAC, bool RES>
__global__ void __launch_bounds__(CELL_THREADS, CELL_MINB) k_cells(KArgs A, const DevTables<T>* __restrict__ gtab,
                                               const GeoTables* __restrict__ ggeo) {
  extern __shared__ __align__(16) unsigned char smem[];
  DevTables<T>& tb = *reinterpret_cast<DevTables<T>*>(smem);
  GeoTables& geo = *reinterpret_cast<GeoTables*>(smem + ((sizeof(DevTables<T>) + 15) & ~size_t(15)));
  CellWork<T>& w = *reinterpret_cast<CellWork<T>*>(
      smem + ((sizeof(DevTables<T>) + 15) & ~size_t(15)) + ((sizeof(GeoTables) + 15) & ~size_t(15)));
  const int tid = threadIdx.x;
  const int nth = blockDim.x;
  {
    const T* src = reinterpret_cast<const T*>(gtab);
    T* dst = reinterpret_cast<T*>(&tb);
    for (int i = tid; i < (int)(sizeof(DevTables<T>) / sizeof(T)); i += nth) dst[i] = src[i];
    const double* s2 = reinterpret_cast<const double*>(ggeo);
    double* d2 = reinterpret_cast<double*>(&geo);
    for (int i = tid; i < (int)(sizeof(GeoTables) / sizeof(double)); i += nth) d2[i] = s2[i];
  }
  const DevParams& P = A.prm;
  T* val = reinterpret_cast<T*>(A.val);
  for (int64_t cell = blockIdx.x; cell < A.ncells; cell += gridDim.x) {
    __syncthreads();
    // ---------------------------------------------------------------- load
    if (tid < 24) w.X[tid] = A.cellX[cell * 24 + tid];
    for (int a = tid; a < ND; a += nth) {  // ND = 129 slots: more than one pass for 128 threads
      w.val[a] = A.xfull[A.gidx[cell * ND + a]];
      w.valT[a] = (T)w.val[a];
      const int32_t rr = A.row[cell * ND + a];
      w.row[a] = rr;
      w.rbase[a] = rr >= 0 ? A.rowptr[rr] : -1;
    }
    if (tid == 0) w.sign = A.sign ? A.sign[cell] : 0ull;
    __syncthreads();
    // ---------------------------------------------------------------- geometry (FP64)
    if (tid < NQ) {
      const int q = tid;
      double J[3][3];
      for (int i = 0; i < 3; ++i)
        for (int a = 0; a < 3; ++a) {
          double s = 0.0;
          for (int v = 0; v < 8; ++v) s += w.X[3 * v + i] * geo.gq1[q][v][a];
          J[i][a] = s;
        }
      double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                   J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                   J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
      double id = 1.0 / det;
      double Ji[3][3];
      Ji[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) * id;
      Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
      Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
      Ji[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) * id;
      Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
      Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
      Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) * id;
      Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
      Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
      w.wdet[q] = geo.w[q] * det;
      // FP64 geometry, rounded once to the element-matrix precision: FP64 converts and FMAs in
      // the per-entry loops bound this kernel on GB300's FP64 issue rate
      w.wdT[q] = (T)w.wdet[q];
      w.idet[q] = id;
      w.idetT[q] = (T)id;
      for (int e = 0; e < 3; ++e)
        for (int i = 0; i < 3; ++i) {
          w.Jinv[q][e * 3 + i] = Ji[e][i];
          w.JinvT[q][e * 3 + i] = (T)Ji[e][i];
        }
      for (int i = 0; i < 3; ++i)
        for (int m = 0; m < 3; ++m) {
          w.Jd[q][i * 3 + m] = J[i][m] * id;
          w.JdT[q][i * 3 + m] = (T)(J[i][m] * id);
        }
    }
    __syncthreads();
    // ---------------------------------------------------------------- physical bases
    for (int idx = tid; idx < NQ * 27; idx += nth) {
      const int q = idx / 27, n = idx % 27;
      const T g0 = tb.g2[q][n][0], g1 = tb.g2[q][n][1], g2 = tb.g2[q][n][2];
      for (int i = 0; i < 3; ++i)
        w.G[q][i][n] = w.JinvT[q][0 * 3 + i] * g0 + w.JinvT[q][1 * 3 + i] * g1 + w.JinvT[q][2 * 3 + i] * g2;
    }
    for (int idx = tid; idx < NQ * 36; idx += nth) {
      const int q = idx / 36, b = idx % 36;
      const int d = b / 12;
      const T sg = ((w.sign >> b) & 1ull) ? (T)-1 : (T)1;
      const T r = tb.rt[q][b] * sg;
      for (int i = 0; i < 3; ++i) w.S[q][i][b] = w.JdT[q][i * 3 + d] * r;
      w.Sdiv[q][b] = tb.rtdiv[q][b] * sg * w.idetT[q];
    }
    __syncthreads();
    // ---------------------------------------------------------------- state at the points
    for (int idx = tid; idx < NQ * 3 + NQ * 3; idx += nth) {
      if (idx < NQ * 3) {
        const int q = idx / 3, c = idx % 3;
        T uc = 0, g0 = 0, g1 = 0, g2 = 0;
        for (int n = 0; n < 27; ++n) {
          const T v = w.valT[OU + c * 27 + n];
          uc += v * tb.n2[q][n];
          g0 += v * w.G[q][0][n];
          g1 += v * w.G[q][1][n];
          g2 += v * w.G[q][2][n];
        }
        w.u[q][c] = uc;
        w.gu[q][0 * 3 + c] = g0;
        w.gu[q][1 * 3 + c] = g1;
        w.gu[q][2 * 3 + c] = g2;
      } else {
        const int k = idx - NQ * 3;
        const int q = k / 3, i = k % 3;
        T s = 0;
        for (int b = 0; b < 36; ++b) s += w.valT[OJ + b] * w.S[q][i][b];
        w.jv[q][i] = s;
        if (i == 0) {
          T dv = 0;
          for (int b = 0; b < 36; ++b) dv += w.valT[OJ + b] * w.Sdiv[q][b];
          w.divj[q] = dv;
          T p = 0;
          for (int m = 0; m < 4; ++m) p += w.valT[OP + m] * tb.p1[q][m];
          w.pp[q] = p;
          T f = 0;
          for (int m = 0; m < 8; ++m) f += w.valT[OPHI + m] * tb.q1[q][m];
          w.ph[q] = f;
        }
      }
    }
    __syncthreads();
    // ---------------------------------------------------------------- AL projection data
    const bool al_u = P.zeta_u != 0.0;
    if (al_u) {
      for (int idx = tid; idx < 4 * 81; idx += nth) {
        const int k = idx / 81, ca = idx % 81, c = ca / 27, a = ca % 27;
        T s = 0;
        for (int q = 0; q < NQ; ++q) s += w.wdT[q] * tb.p1[q][k] * w.G[q][c][a];
        w.Bd[k][ca] = s;
      }
      if (tid == 0) {
        double M[4][8];
        for (int k = 0; k < 4; ++k)
          for (int l = 0; l < 4; ++l) {
            double s = 0.0;
            for (int q = 0; q < NQ; ++q) s += w.wdet[q] * (double)tb.p1[q][k] * (double)tb.p1[q][l];
            M[k][l] = s;
            M[k][4 + l] = (k == l) ? 1.0 : 0.0;
          }
        for (int i = 0; i < 4; ++i) {
          int piv = i;
          for (int k = i + 1; k < 4; ++k)
            if (fabs(M[k][i]) > fabs(M[piv][i])) piv = k;
          for (int j = 0; j < 8; ++j) { double t = M[i][j]; M[i][j] = M[piv][j]; M[piv][j] = t; }
          double d = 1.0 / M[i][i];
          for (int j = 0; j < 8; ++j) M[i][j] *= d;
          for (int k = 0; k < 4; ++k)
            if (k != i) {
              double m = M[k][i];
              for (int j = 0; j < 8; ++j) M[k][j] -= m * M[i][j];
            }
        }
        for (int k = 0; k < 4; ++k)
          for (int l = 0; l < 4; ++l) w.Mpi[k * 4 + l] = M[k][4 + l];
      }
      __syncthreads();
      for (int idx = tid; idx < 4 * 81; idx += nth) {
        const int k = idx / 81, ca = idx % 81;
        T s = 0;
        for (int l = 0; l < 4; ++l) s += (T)w.Mpi[k * 4 + l] * w.Bd[l][ca];
        w.Tm[k][ca] = s;
      }
      if (tid < 4) {
        double s = 0.0;
        for (int ca = 0; ca < 81; ++ca) s += (double)w.Bd[tid][ca] * w.val[OU + ca];
        w.divmom[tid] = s;
      }
      __syncthreads();
      if (tid < 4) {
        double s = 0.0;
        for (int l = 0; l < 4; ++l) s += w.Mpi[tid * 4 + l] * w.divmom[l];
        w.pic[tid] = s;
      }
      __syncthreads();
    }
    // ---------------------------------------------------------------- residual (FP64 path)
    if (RES) {
      const double* fv = P.has_fcell ? A.fcell + 3 * cell : P.f;
      for (int a = tid; a < ND; a += nth) {
        if (w.row[a] < 0) continue;
        double acc = 0.0;
        if (a < OP) {
          const int c = a / 27, n = a % 27;
          for (int q = 0; q < NQ; ++q) {
            const double vv = tb.n2[q][n];
            const double d0 = w.G[q][0][n], d1 = w.G[q][1][n], d2 = w.G[q][2][n];
            const double gterm = w.gu[q][0 * 3 + c] * d0 + w.gu[q][1 * 3 + c] * d1 + w.gu[q][2 * 3 + c] * d2;
            const double divv = c == 0 ? d0 : (c == 1 ? d1 : d2);
            const double j0 = w.jv[q][0], j1 = w.jv[q][1], j2 = w.jv[q][2];
            const double jxB = c == 0 ? (j1 * P.B[2] - j2 * P.B[1])
                                      : (c == 1 ? (j2 * P.B[0] - j0 * P.B[2]) : (j0 * P.B[1] - j1 * P.B[0]));
            double v = P.beta * gterm - (double)w.pp[q] * divv - P.gamma * jxB * vv - fv[c] * vv;
            if (P.convection != 0) {
              const double conv = w.gu[q][0 * 3 + c] * w.u[q][0] + w.gu[q][1 * 3 + c] * w.u[q][1] +
                                  w.gu[q][2 * 3 + c] * w.u[q][2];
              v += P.alpha * vv * conv;
            }
            if (al_u) {
              double pd = 0.0;
              for (int k = 0; k < 4; ++k) pd += w.pic[k] * (double)tb.p1[q][k];
              v += P.zeta_u * pd * divv;
            }
            acc += w.wdet[q] * v;
          }
        } else if (a < OJ) {
          const int k = a - OP;
          for (int q = 0; q < NQ; ++q) {
            const double divu = w.gu[q][0] + w.gu[q][4] + w.gu[q][8];
            acc += w.wdet[q] * (-divu * (double)tb.p1[q][k]);
          }
        } else if (a < OPHI) {
          const int b = a - OJ;
          for (int q = 0; q < NQ; ++q) {
            const double s0 = w.S[q][0][b], s1 = w.S[q][1][b], s2 = w.S[q][2][b];
            const double u0 = w.u[q][0], u1 = w.u[q][1], u2 = w.u[q][2];
            const double uB0 = u1 * P.B[2] - u2 * P.B[1], uB1 = u2 * P.B[0] - u0 * P.B[2],
                         uB2 = u0 * P.B[1] - u1 * P.B[0];
            const double js = w.jv[q][0] * s0 + w.jv[q][1] * s1 + w.jv[q][2] * s2;
            const double ds = w.Sdiv[q][b];
            double v = js - P.sigma * (double)w.ph[q] * ds - P.sigma * (uB0 * s0 + uB1 * s1 + uB2 * s2) -
                       (P.g[0] * s0 + P.g[1] * s1 + P.g[2] * s2);
            if (P.zeta_j != 0.0) v += P.zeta_j * (double)w.divj[q] * ds;
            acc += w.wdet[q] * v;
          }
        } else {
          const int k = a - OPHI;
          for (int q = 0; q < NQ; ++q) acc += w.wdet[q] * (-(double)w.divj[q] * (double)tb.q1[q][k]);
        }
        atomicAdd(&A.r[w.row[a]], acc);
      }
    }
    if (!JAC) continue;
    // ---------------------------------------------------------------- Jacobian
    const uint16_t* ot = A.offtab + (size_t)A.cls[cell] * (ND * ND);
    const bool conv = P.convection != 0, newton = P.convection == 2;
    for (int idx = tid; idx < NQ * 27; idx += nth) {
      const int q = idx / 27, b = idx % 27;
      w.ugb[q][b] = w.wdT[q] * (w.u[q][0] * w.G[q][0][b] + w.u[q][1] * w.G[q][1][b] + w.u[q][2] * w.G[q][2][b]);
      w.wn2[q][b] = w.wdT[q] * tb.n2[q][b];
    }
    __syncthreads();
    const T beta = (T)P.beta, alpha = (T)P.alpha, gam = (T)P.gamma, sig = (T)P.sigma;
    const T zu = (T)P.zeta_u, zj = (T)P.zeta_j;
    const T B0 = (T)P.B[0], B1 = (T)P.B[1], B2 = (T)P.B[2];
    // u-u: 27x27 scalar pairs, 9 component entries each.  K = ∫ w ∇N_a·∇N_b and the Newton
    // part M_cd = ∫ w N_a N_b ∂_d u_c are symmetric in (a, b), so each unordered pair a ≤ b
    // (378 of them) forms them once and writes both (a, b) and (b, a); only the Picard part
    // ∫ N_a (u·∇N_b) and the AL term are formed per ordered pair.
    // jpart 1 keeps the state-independent terms (viscous, AL, and every block but u-u below),
    // jpart 2 the convection terms only (Picard ∫ N_a (u·∇N_b) and Newton ∫ N_a N_b ∂_d u_c)
    const bool part_static = A.jpart != 2, part_conv = A.jpart != 1;
    const bool cconv = conv && part_conv, cnewton = newton && part_conv;
    for (int idx = tid; idx < 27 * 28 / 2; idx += nth) {
      int a = 0, r = idx;
      while (r >= 27 - a) { r -= 27 - a; ++a; }
      const int b = a + r;
      T K = 0, Cab = 0, Cba = 0;
      T Mg[9];  // Σ_q w N_a N_b ∂_d u_c at [d*3+c]
#pragma unroll
      for (int k = 0; k < 9; ++k) Mg[k] = 0;
      for (int q = 0; q < NQ; ++q) {
        const T wd = w.wdT[q];
        if (part_static)
          K += wd * (w.G[q][0][a] * w.G[q][0][b] + w.G[q][1][a] * w.G[q][1][b] + w.G[q][2][a] * w.G[q][2][b]);
        if (cconv) {
          Cab += tb.n2[q][a] * w.ugb[q][b];
          Cba += tb.n2[q][b] * w.ugb[q][a];
        }
        if (cnewton) {
          const T m = w.wn2[q][a] * tb.n2[q][b];
#pragma unroll
          for (int k = 0; k < 9; ++k) Mg[k] += m * w.gu[q][k];
        }
      }
      for (int side = 0; side < (a == b ? 1 : 2); ++side) {
        const int ta = side ? b : a, tb_ = side ? a : b;  // test, trial
        const T diag = beta * K + alpha * (side ? Cba : Cab);
        for (int c = 0; c < 3; ++c) {
          const int ra = OU + c * 27 + ta;
          if (w.row[ra] < 0) continue;
          for (int d = 0; d < 3; ++d) {
            const int cb = OU + d * 27 + tb_;
            if (w.row[cb] < 0) continue;
            if (!part_static && !cnewton && c != d) continue;  // nothing to add
            T v = (c == d) ? diag : (T)0;
            v += alpha * Mg[d * 3 + c];
            if (al_u && part_static) {
              T s2 = 0;
              for (int k = 0; k < 4; ++k) s2 += w.Bd[k][c * 27 + ta] * w.Tm[k][d * 27 + tb_];
              v += zu * s2;
            }
            red_add(&val[w.rbase[ra] + ot[ra * ND + cb]], v);
          }
        }
      }
    }
    if (!part_static) continue;  // the blocks below hold no convection term
    // u-p and p-u
    for (int idx = tid; idx < 81 * 4; idx += nth) {
      const int ca = idx / 4, k = idx % 4, c = ca / 27, a = ca % 27;
      T s = 0;
      for (int q = 0; q < NQ; ++q) s += w.wdT[q] * tb.p1[q][k] * w.G[q][c][a];
      const int ru = OU + ca, rp = OP + k;
      if (w.row[ru] >= 0) {
        red_add(&val[w.rbase[ru] + ot[ru * ND + rp]], -s);
        red_add(&val[w.rbase[rp] + ot[rp * ND + ru]], -s);
      }
    }
    // u-j and j-u: ∫ N_a (S_b × B) = (∫ N_a S_b) × B, the cross product after the sum
    for (int idx = tid; idx < 27 * 36; idx += nth) {
      const int a = idx / 36, b = idx % 36;
      T s0 = 0, s1 = 0, s2 = 0;
      for (int q = 0; q < NQ; ++q) {
        const T m = w.wn2[q][a];
        s0 += m * w.S[q][0][b];
        s1 += m * w.S[q][1][b];
        s2 += m * w.S[q][2][b];
      }
      const T c0 = s1 * B2 - s2 * B1, c1 = s2 * B0 - s0 * B2, c2 = s0 * B1 - s1 * B0;
      const int rj = OJ + b;
      const T cc[3] = {c0, c1, c2};
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const int ru = OU + c * 27 + a;
        if (w.row[ru] < 0 || w.row[rj] < 0) continue;
        red_add(&val[w.rbase[ru] + ot[ru * ND + rj]], -gam * cc[c]);
        red_add(&val[w.rbase[rj] + ot[rj * ND + ru]], sig * cc[c]);
      }
    }
    // j-j: symmetric, one pass per unordered pair a ≤ b (666 of 36x36)
    for (int idx = tid; idx < 36 * 37 / 2; idx += nth) {
      int a = 0, r = idx;
      while (r >= 36 - a) { r -= 36 - a; ++a; }
      const int b = a + r;
      const int ra = OJ + a, rb = OJ + b;
      if (w.row[ra] < 0 || w.row[rb] < 0) continue;
      T s = 0;
      for (int q = 0; q < NQ; ++q) {
        T t = w.S[q][0][a] * w.S[q][0][b] + w.S[q][1][a] * w.S[q][1][b] + w.S[q][2][a] * w.S[q][2][b];
        if (P.zeta_j != 0.0) t += zj * w.Sdiv[q][a] * w.Sdiv[q][b];
        s += w.wdT[q] * t;
      }
      red_add(&val[w.rbase[ra] + ot[ra * ND + rb]], s);
      if (a != b) red_add(&val[w.rbase[rb] + ot[rb * ND + ra]], s);
    }
    // j-φ and φ-j
    for (int idx = tid; idx < 36 * 8; idx += nth) {
      const int b = idx / 8, k = idx % 8;
      const int rj = OJ + b, rf = OPHI + k;
      if (w.row[rj] < 0) continue;
      T s = 0;
      for (int q = 0; q < NQ; ++q) s += w.wdT[q] * tb.q1[q][k] * w.Sdiv[q][b];
      red_add(&val[w.rbase[rj] + ot[rj * ND + rf]], -sig * s);
      red_add(&val[w.rbase[rf] + ot[rf * ND + rj]], -s);
    }
  }
}

// ---------------------------------------------------------------------- residual (flux form)
// One warp per cell.  Lane q < 27 evaluates the state at Gauss point q and the fluxes
// multiplying each test-function quantity, pulled back to the reference cell:
//   u rows: F̂g[e][c] = w det Σ_i (J⁻¹)_{e i} (β ∂_i u_c − p δ_ic),  Fv[c] = w det (α conv_c − γ (j×B)_c − f_c)
//   j rows: F̂s[d]    = w Σ_i J_{i d} (j − σ u×B − g)_i,          F̂d   = w (−σφ + ζⱼ div j)
//   p rows: −w det div u,   φ rows: −w det div j
// then every lane contracts them with the reference tables for its rows (FP64 throughout).
// Used when ζᵤ = 0 (the local pressure projection of the AL term lives in k_cells).
constexpr int RF_WARPS = 8;
constexpr int RF_NF = 18;
struct ResWarp {
  double X[24];
  double val[ND];
  double flux[NQ][RF_NF];
  int32_t row[ND];
  unsigned long long sign;
};

__global__ void __launch_bounds__(RF_WARPS * 32) k_residual_flux(KArgs A, const DevTables<double>* __restrict__ gtab,
                                                                 const GeoTables* __restrict__ ggeo) {
  extern __shared__ __align__(16) unsigned char smem[];
  DevTables<double>& tb = *reinterpret_cast<DevTables<double>*>(smem);
  ResWarp* wsm = reinterpret_cast<ResWarp*>(smem + ((sizeof(DevTables<double>) + 15) & ~size_t(15)));
  {
    const double* src = reinterpret_cast<const double*>(gtab);
    double* dst = reinterpret_cast<double*>(&tb);
    for (int i = threadIdx.x; i < (int)(sizeof(DevTables<double>) / sizeof(double)); i += blockDim.x) dst[i] = src[i];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  ResWarp& w = wsm[wid];
  const DevParams& P = A.prm;
  const int64_t nwarps = (int64_t)gridDim.x * RF_WARPS;
  for (int64_t cell = (int64_t)blockIdx.x * RF_WARPS + wid; cell < A.ncells; cell += nwarps) {
    if (lane < 24) w.X[lane] = A.cellX[cell * 24 + lane];
    for (int a = lane; a < ND; a += 32) {
      w.val[a] = A.xfull[A.gidx[cell * ND + a]];
      w.row[a] = A.row[cell * ND + a];
    }
    if (lane == 0) w.sign = A.sign ? A.sign[cell] : 0ull;
    __syncwarp();
    if (lane < NQ) {
      const int q = lane;
      double J[3][3];
      for (int i = 0; i < 3; ++i)
        for (int a = 0; a < 3; ++a) {
          double s = 0.0;
          for (int v = 0; v < 8; ++v) s += w.X[3 * v + i] * ggeo->gq1[q][v][a];
          J[i][a] = s;
        }
      const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                         J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                         J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
      const double id = 1.0 / det;
      double Ji[3][3];
      Ji[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) * id;
      Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
      Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
      Ji[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) * id;
      Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
      Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
      Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) * id;
      Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
      Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
      const double wq = ggeo->w[q], wd = wq * det;
      // state
      double u[3], gu[3][3];  // gu[i][c] = ∂_i u_c
      for (int c = 0; c < 3; ++c) {
        double uc = 0.0, g0 = 0.0, g1 = 0.0, g2 = 0.0;
        for (int n = 0; n < 27; ++n) {
          const double v = w.val[OU + c * 27 + n];
          uc += v * tb.n2[q][n];
          g0 += v * tb.g2[q][n][0];
          g1 += v * tb.g2[q][n][1];
          g2 += v * tb.g2[q][n][2];
        }
        u[c] = uc;
        for (int i = 0; i < 3; ++i) gu[i][c] = Ji[0][i] * g0 + Ji[1][i] * g1 + Ji[2][i] * g2;
      }
      double p = 0.0;
      for (int k = 0; k < 4; ++k) p += w.val[OP + k] * tb.p1[q][k];
      double jr[3] = {0.0, 0.0, 0.0}, dv = 0.0;
      for (int b = 0; b < 36; ++b) {
        const double sv = (((w.sign >> b) & 1ull) ? -1.0 : 1.0) * w.val[OJ + b];
        jr[b / 12] += sv * tb.rt[q][b];
        dv += sv * tb.rtdiv[q][b];
      }
      double j[3];
      for (int i = 0; i < 3; ++i) j[i] = (J[i][0] * jr[0] + J[i][1] * jr[1] + J[i][2] * jr[2]) * id;
      const double divj = dv * id;
      double phi = 0.0;
      for (int k = 0; k < 8; ++k) phi += w.val[OPHI + k] * tb.q1[q][k];
      const double* fv = P.has_fcell ? A.fcell + 3 * cell : P.f;
      // fluxes
      double Fg[3][3];
      for (int i = 0; i < 3; ++i)
        for (int c = 0; c < 3; ++c) Fg[i][c] = P.beta * gu[i][c] - (i == c ? p : 0.0);
      const double jxB[3] = {j[1] * P.B[2] - j[2] * P.B[1], j[2] * P.B[0] - j[0] * P.B[2], j[0] * P.B[1] - j[1] * P.B[0]};
      const double uxB[3] = {u[1] * P.B[2] - u[2] * P.B[1], u[2] * P.B[0] - u[0] * P.B[2], u[0] * P.B[1] - u[1] * P.B[0]};
      double* F = w.flux[q];
      for (int e = 0; e < 3; ++e)
        for (int c = 0; c < 3; ++c) F[e * 3 + c] = wd * (Ji[e][0] * Fg[0][c] + Ji[e][1] * Fg[1][c] + Ji[e][2] * Fg[2][c]);
      for (int c = 0; c < 3; ++c) {
        double v = -P.gamma * jxB[c] - fv[c];
        if (P.convection != 0) v += P.alpha * (gu[0][c] * u[0] + gu[1][c] * u[1] + gu[2][c] * u[2]);
        F[9 + c] = wd * v;
      }
      double Fs[3];
      for (int i = 0; i < 3; ++i) Fs[i] = j[i] - P.sigma * uxB[i] - P.g[i];
      for (int d = 0; d < 3; ++d) F[12 + d] = wq * (Fs[0] * J[0][d] + Fs[1] * J[1][d] + Fs[2] * J[2][d]);
      F[15] = wq * (-P.sigma * phi + P.zeta_j * divj);
      F[16] = -wd * (gu[0][0] + gu[1][1] + gu[2][2]);
      F[17] = -wd * divj;
    }
    __syncwarp();
    for (int a = lane; a < ND; a += 32) {
      if (w.row[a] < 0) continue;
      double acc = 0.0;
      if (a < OP) {
        const int c = a / 27, n = a % 27;
        for (int q = 0; q < NQ; ++q) {
          const double* F = w.flux[q];
          acc += F[c] * tb.g2[q][n][0] + F[3 + c] * tb.g2[q][n][1] + F[6 + c] * tb.g2[q][n][2] + F[9 + c] * tb.n2[q][n];
        }
      } else if (a < OJ) {
        const int k = a - OP;
        for (int q = 0; q < NQ; ++q) acc += w.flux[q][16] * tb.p1[q][k];
      } else if (a < OPHI) {
        const int b = a - OJ, d = b / 12;
        for (int q = 0; q < NQ; ++q) acc += w.flux[q][12 + d] * tb.rt[q][b] + w.flux[q][15] * tb.rtdiv[q][b];
        if ((w.sign >> b) & 1ull) acc = -acc;
      } else {
        const int k = a - OPHI;
        for (int q = 0; q < NQ; ++q) acc += w.flux[q][17] * tb.q1[q][k];
      }
      atomicAdd(&A.r[w.row[a]], acc);
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------- facets
struct FArgs {
  int64_t nfacets;
  const int32_t* fcell;
  const int8_t* flface;
  const double* fprm;  // [n][4] tau, cw, jw, phi0
  const double* cellX;
  const int32_t* gidx;
  const int32_t* row;
  const unsigned long long* sign;
  const double* xfull;
  const int64_t* rowptr;
  const int32_t* cls;
  const uint16_t* offtab;
  void* val;
  double* r;
  double* dr_dcw;   // optional: accumulate τ∫(s·n) n·∇j·n (derivative w.r.t. cw)
};

template <typename T, bool JAC, bool RES>
__global__ void __launch_bounds__(64) k_facets(FArgs A, const FacetTables* __restrict__ ft) {
  __shared__ double X[24];
  __shared__ double vj[36];
  __shared__ double sn[NQF][36], gnn[NQF][36], dA[NQF];
  __shared__ int32_t rw[36];
  __shared__ int64_t rb[36];
  const int tid = threadIdx.x;
  const int64_t e = blockIdx.x;
  if (e >= A.nfacets) return;
  const int64_t cell = A.fcell[e];
  const int f = A.flface[e];
  const int ax = f / 2, side = f % 2;
  const unsigned long long sgn = A.sign ? A.sign[cell] : 0ull;
  if (tid < 24) X[tid] = A.cellX[cell * 24 + tid];
  if (tid < 36) {
    vj[tid] = A.xfull[A.gidx[cell * ND + OJ + tid]];
    rw[tid] = A.row[cell * ND + OJ + tid];
    rb[tid] = rw[tid] >= 0 ? A.rowptr[rw[tid]] : -1;
  }
  __syncthreads();
  if (tid < NQF) {
    const int t = tid;
    double J[3][3];
    for (int i = 0; i < 3; ++i)
      for (int a = 0; a < 3; ++a) {
        double s = 0.0;
        for (int v = 0; v < 8; ++v) s += X[3 * v + i] * ft->fgq1[f][t][v][a];
        J[i][a] = s;
      }
    double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                 J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                 J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
    double id = 1.0 / det;
    double Ji[3][3];
    Ji[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) * id;
    Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
    Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
    Ji[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) * id;
    Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
    Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
    Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) * id;
    Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
    Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
    double n[3];
    for (int i = 0; i < 3; ++i) n[i] = Ji[ax][i] * (side ? 1.0 : -1.0);
    const double nl = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    for (int i = 0; i < 3; ++i) n[i] /= nl;
    dA[t] = ft->fw[t] * fabs(det) * nl;
    double nJinv[3];  // Σ_i n_i (J⁻¹)_{a i}
    for (int a = 0; a < 3; ++a) nJinv[a] = n[0] * Ji[a][0] + n[1] * Ji[a][1] + n[2] * Ji[a][2];
    for (int b = 0; b < 36; ++b) {
      const int d = b / 12;
      const double sg = ((sgn >> b) & 1ull) ? -1.0 : 1.0;
      const double nJd = n[0] * J[0][d] + n[1] * J[1][d] + n[2] * J[2][d];
      sn[t][b] = sg * nJd * id * ft->frt[f][t][b];
      const double* g = ft->frtg[f][t][b];
      gnn[t][b] = sg * id * (nJinv[0] * g[0] + nJinv[1] * g[1] + nJinv[2] * g[2]) * nJd;
    }
  }
  __syncthreads();
  const double tau = A.fprm[4 * e + 0], cw = A.fprm[4 * e + 1], jw = A.fprm[4 * e + 2], phi0 = A.fprm[4 * e + 3];
  if (RES || A.dr_dcw) {
    if (tid < 36 && rw[tid] >= 0) {
      double acc = 0.0, accw = 0.0;
      for (int t = 0; t < NQF; ++t) {
        double jn = 0.0, jnn = 0.0;
        for (int b = 0; b < 36; ++b) {
          jn += vj[b] * sn[t][b];
          jnn += vj[b] * gnn[t][b];
        }
        acc += dA[t] * (tau * sn[t][tid] * (jn - jw + cw * jnn) + sn[t][tid] * phi0);
        accw += dA[t] * tau * sn[t][tid] * jnn;
      }
      if (RES) atomicAdd(&A.r[rw[tid]], acc);
      if (A.dr_dcw) atomicAdd(&A.dr_dcw[rw[tid]], accw);
    }
  }
  if (JAC && tau != 0.0) {
    T* val = reinterpret_cast<T*>(A.val);
    const uint16_t* ot = A.offtab + (size_t)A.cls[cell] * (ND * ND);
    for (int idx = tid; idx < 36 * 36; idx += blockDim.x) {
      const int a = idx / 36, b = idx % 36;
      if (rw[a] < 0 || rw[b] < 0) continue;
      double s = 0.0;
      for (int t = 0; t < NQF; ++t) s += dA[t] * tau * sn[t][a] * (sn[t][b] + cw * gnn[t][b]);
      red_add(&val[rb[a] + ot[(OJ + a) * ND + OJ + b]], (T)s);
    }
  }
}

// ---------------------------------------------------------------------- dR/dγ and f_z moments
__global__ void __launch_bounds__(128) k_param_derivs(int64_t ncells, const double* __restrict__ cellX,
                                                      const int32_t* __restrict__ gidx,
                                                      const int32_t* __restrict__ row,
                                                      const unsigned long long* __restrict__ sign,
                                                      const double* __restrict__ xfull,
                                                      const DevTables<double>* __restrict__ tb,
                                                      const GeoTables* __restrict__ geo, DevParams P,
                                                      double* dr_dgamma, double* fz) {
  __shared__ double X[24], vj[36], wdet[NQ], jxB[NQ][3];
  const int tid = threadIdx.x;
  for (int64_t cell = blockIdx.x; cell < ncells; cell += gridDim.x) {
    __syncthreads();
    const unsigned long long sgn = sign ? sign[cell] : 0ull;
    if (tid < 24) X[tid] = cellX[cell * 24 + tid];
    if (tid < 36) vj[tid] = xfull[gidx[cell * ND + OJ + tid]] * (((sgn >> tid) & 1ull) ? -1.0 : 1.0);
    __syncthreads();
    if (tid < NQ) {
      const int q = tid;
      double J[3][3];
      for (int i = 0; i < 3; ++i)
        for (int a = 0; a < 3; ++a) {
          double s = 0.0;
          for (int v = 0; v < 8; ++v) s += X[3 * v + i] * geo->gq1[q][v][a];
          J[i][a] = s;
        }
      double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                   J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                   J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
      wdet[q] = geo->w[q] * det;
      double j[3] = {0, 0, 0};
      for (int b = 0; b < 36; ++b) {
        const int d = b / 12;
        for (int i = 0; i < 3; ++i) j[i] += vj[b] * J[i][d] / det * tb->rt[q][b];
      }
      jxB[q][0] = j[1] * P.B[2] - j[2] * P.B[1];
      jxB[q][1] = j[2] * P.B[0] - j[0] * P.B[2];
      jxB[q][2] = j[0] * P.B[1] - j[1] * P.B[0];
    }
    __syncthreads();
    if (tid < 81) {
      const int c = tid / 27, n = tid % 27;
      double s = 0.0, m = 0.0;
      for (int q = 0; q < NQ; ++q) {
        s += wdet[q] * (-jxB[q][c] * tb->n2[q][n]);
        m += wdet[q] * tb->n2[q][n];
      }
      const int32_t rr = row[cell * ND + tid];
      if (dr_dgamma && rr >= 0) atomicAdd(&dr_dgamma[rr], s);
      if (fz && c == 2) fz[cell * 27 + n] = m;
    }
  }
}

// ---------------------------------------------------------------------- dR/dα and dR/dβ
// The residual of res_fluid_h1_hdiv (src/weakforms.jl:255-281) is linear in β (viscous term
// ∫∇u⊙∇v, :264) and in α (convection ∫v·((∇u)ᵀ·u), :277-279, conv at :670), so on the u rows
//   ∂R/∂β = ∫ Σ_i ∂_i u_c ∂_i N_n,   ∂R/∂α = ∫ N_n ((∇u)ᵀ·u)_c   (zero without convection).
// In the MHD scaling (src/Applications/expansion.jl:113-123) Ha enters through α and β.
// One CTA per cell: threads < 27 form the geometry and the state at their point; the 81 u
// rows then sum over the points.
__global__ void __launch_bounds__(128) k_param_derivs_ab(int64_t ncells, const double* __restrict__ cellX,
                                                         const int32_t* __restrict__ gidx,
                                                         const int32_t* __restrict__ row,
                                                         const double* __restrict__ xfull,
                                                         const DevTables<double>* __restrict__ tb,
                                                         const GeoTables* __restrict__ geo, int convection,
                                                         double* dr_dalpha, double* dr_dbeta) {
  __shared__ double X[24], vu[81], wdet[NQ], Ji[NQ][9], gu[NQ][9], cv[NQ][3];
  const int tid = threadIdx.x;
  for (int64_t cell = blockIdx.x; cell < ncells; cell += gridDim.x) {
    __syncthreads();
    if (tid < 24) X[tid] = cellX[cell * 24 + tid];
    if (tid < 81) vu[tid] = xfull[gidx[cell * ND + OU + tid]];
    __syncthreads();
    if (tid < NQ) {
      const int q = tid;
      double J[3][3];
      for (int i = 0; i < 3; ++i)
        for (int a = 0; a < 3; ++a) {
          double s = 0.0;
          for (int v = 0; v < 8; ++v) s += X[3 * v + i] * geo->gq1[q][v][a];
          J[i][a] = s;
        }
      const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                         J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                         J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
      const double id = 1.0 / det;
      double I[3][3];  // (J⁻¹)_{a i}
      I[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) * id;
      I[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
      I[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
      I[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) * id;
      I[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
      I[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
      I[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) * id;
      I[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
      I[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
      wdet[q] = geo->w[q] * det;
      for (int k = 0; k < 9; ++k) Ji[q][k] = I[k / 3][k % 3];
      double u[3] = {0, 0, 0}, g[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};  // g[i][c] = ∂_i u_c
      for (int n = 0; n < 27; ++n) {
        double gn[3];
        for (int i = 0; i < 3; ++i)
          gn[i] = I[0][i] * tb->g2[q][n][0] + I[1][i] * tb->g2[q][n][1] + I[2][i] * tb->g2[q][n][2];
        for (int c = 0; c < 3; ++c) {
          const double val = vu[c * 27 + n];
          u[c] += val * tb->n2[q][n];
          for (int i = 0; i < 3; ++i) g[i][c] += val * gn[i];
        }
      }
      for (int i = 0; i < 3; ++i)
        for (int c = 0; c < 3; ++c) gu[q][i * 3 + c] = g[i][c];
      for (int c = 0; c < 3; ++c) cv[q][c] = g[0][c] * u[0] + g[1][c] * u[1] + g[2][c] * u[2];
    }
    __syncthreads();
    if (tid < 81) {
      const int c = tid / 27, n = tid % 27;
      double sb = 0.0, sa = 0.0;
      for (int q = 0; q < NQ; ++q) {
        double gd = 0.0;
        for (int i = 0; i < 3; ++i) {
          const double gn =
              Ji[q][0 * 3 + i] * tb->g2[q][n][0] + Ji[q][1 * 3 + i] * tb->g2[q][n][1] + Ji[q][2 * 3 + i] * tb->g2[q][n][2];
          gd += gu[q][i * 3 + c] * gn;
        }
        sb += wdet[q] * gd;
        sa += wdet[q] * tb->n2[q][n] * cv[q][c];
      }
      const int32_t rr = row[cell * ND + tid];
      if (rr >= 0) {
        if (dr_dbeta) atomicAdd(&dr_dbeta[rr], sb);
        if (dr_dalpha && convection != 0) atomicAdd(&dr_dalpha[rr], sa);
      }
    }
  }
}

}  // namespace gbmhd

using namespace gbmhd;

// ---------------------------------------------------------------------- host side
template <typename T>
static size_t cells_smem() {
  return ((sizeof(DevTables<T>) + 15) & ~size_t(15)) + ((sizeof(GeoTables) + 15) & ~size_t(15)) +
         sizeof(CellWork<T>);
}

template <typename T, bool JAC, bool RES>
static int launch_cells(gbmhd_ctx* ctx, KArgs& a, const void* tab) {
  auto kern = k_cells<T, JAC, RES>;
  const size_t sm = cells_smem<T>();
  GB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  int occ = 0;
  GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, CELL_THREADS, sm));
  if (occ < 1) { ctx->err = "assembly kernel does not fit on an SM"; return -2; }
  int64_t grid = (int64_t)ctx->num_sms * occ;
  if (grid > a.ncells) grid = a.ncells;
  if (grid < 1) grid = 1;
  const GeoTables* geo = reinterpret_cast<const GeoTables*>(
      reinterpret_cast<const char*>(ctx->d_tab64) + ((sizeof(DevTables<double>) + 255) & ~size_t(255)));
  { kern<<<(unsigned)grid, CELL_THREADS, sm, ctx->stream>>>(a, reinterpret_cast<const DevTables<T>*>(tab), geo); gbmhd::count_launch(); }
  GB_CUDA(cudaGetLastError());
  return 0;
}

static int launch_residual(gbmhd_ctx* ctx, KArgs& a) {
  if (ctx->prm.zeta_u != 0.0) return launch_cells<double, false, true>(ctx, a, ctx->d_tab64);
  const size_t sm = ((sizeof(DevTables<double>) + 15) & ~size_t(15)) + sizeof(ResWarp) * RF_WARPS;
  GB_CUDA(cudaFuncSetAttribute(k_residual_flux, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  int occ = 0;
  GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_residual_flux, RF_WARPS * 32, sm));
  if (occ < 1) { ctx->err = "residual kernel does not fit on an SM"; return -2; }
  int64_t grid = std::min<int64_t>((int64_t)ctx->num_sms * occ, (a.ncells + RF_WARPS - 1) / RF_WARPS);
  const GeoTables* geo = reinterpret_cast<const GeoTables*>(
      reinterpret_cast<const char*>(ctx->d_tab64) + ((sizeof(DevTables<double>) + 255) & ~size_t(255)));
  { k_residual_flux<<<(unsigned)std::max<int64_t>(grid, 1), RF_WARPS * 32, sm, ctx->stream>>>(a, reinterpret_cast<const DevTables<double>*>(ctx->d_tab64), geo); gbmhd::count_launch(); }
  GB_CUDA(cudaGetLastError());
  return 0;
}

int gb_upload_tables(gbmhd_ctx* ctx) {
  RefTables R;
  build_ref_tables(R);
  DevTables<double> t64;
  DevTables<float> t32;
  GeoTables g;
  auto fill = [&](auto& t) {
    using TT = std::remove_reference_t<decltype(t.w[0])>;
    for (int q = 0; q < NQ; ++q) {
      t.w[q] = (TT)R.w[q];
      for (int v = 0; v < 8; ++v)
        for (int a = 0; a < 3; ++a) t.gq1[q][v][a] = (TT)R.gq1[q][v][a];
      for (int n = 0; n < 27; ++n) {
        t.n2[q][n] = (TT)R.n2[q][n];
        for (int a = 0; a < 3; ++a) t.g2[q][n][a] = (TT)R.g2[q][n][a];
      }
      for (int k = 0; k < 4; ++k) t.p1[q][k] = (TT)R.p1[q][k];
      for (int k = 0; k < 8; ++k) t.q1[q][k] = (TT)R.q1[q][k];
      for (int b = 0; b < 36; ++b) {
        t.rt[q][b] = (TT)R.rt[q][b];
        t.rtdiv[q][b] = (TT)R.rtdiv[q][b];
      }
    }
  };
  fill(t64);
  fill(t32);
  for (int q = 0; q < NQ; ++q) {
    g.w[q] = R.w[q];
    for (int v = 0; v < 8; ++v)
      for (int a = 0; a < 3; ++a) g.gq1[q][v][a] = R.gq1[q][v][a];
  }
  FacetTables F;
  for (int t = 0; t < NQF; ++t) F.fw[t] = R.fw[t];
  for (int f = 0; f < 6; ++f)
    for (int t = 0; t < NQF; ++t) {
      for (int v = 0; v < 8; ++v)
        for (int a = 0; a < 3; ++a) F.fgq1[f][t][v][a] = R.fgq1[f][t][v][a];
      for (int b = 0; b < 36; ++b) {
        F.frt[f][t][b] = R.frt[f][t][b];
        for (int a = 0; a < 3; ++a) F.frtg[f][t][b][a] = R.frtg[f][t][b][a];
      }
    }
  const size_t o64 = (sizeof(DevTables<double>) + 255) & ~size_t(255);
  GB_CUDA(cudaMalloc(&ctx->d_tab64, o64 + sizeof(GeoTables)));
  GB_CUDA(cudaMalloc(&ctx->d_tab32, sizeof(DevTables<float>)));
  GB_CUDA(cudaMalloc(&ctx->d_ftab, sizeof(FacetTables)));
  GB_CUDA(cudaMemcpy(ctx->d_tab64, &t64, sizeof(t64), cudaMemcpyHostToDevice));
  GB_CUDA(cudaMemcpy(reinterpret_cast<char*>(ctx->d_tab64) + o64, &g, sizeof(g), cudaMemcpyHostToDevice));
  GB_CUDA(cudaMemcpy(ctx->d_tab32, &t32, sizeof(t32), cudaMemcpyHostToDevice));
  GB_CUDA(cudaMemcpy(ctx->d_ftab, &F, sizeof(F), cudaMemcpyHostToDevice));
  return 0;
}

// The state-independent terms of the FP64 Jacobian (every term but convection: viscous, AL,
// pressure, Lorentz, Ohm, and the thin-wall facets) into ctx->d_val64s, once per parameter
// set.  The Jacobian is affine in the state apart from convection, so a Jacobian at any state
// is this copy plus the convection terms there: the per-step assembly does the u–u
// convection pairs only.  Returns -1 (whole assembly instead) when the copy does not fit.
static int static_jacobian(gbmhd_ctx* ctx, KArgs a, FArgs fa, const FacetTables* ft) {
  if (ctx->val64s_off) return -1;
  if (!ctx->d_val64s) {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess ||
        free_b < sizeof(double) * (size_t)ctx->nnz + ((size_t)4 << 30) ||
        cudaMalloc(&ctx->d_val64s, sizeof(double) * std::max<int64_t>(ctx->nnz, 1)) != cudaSuccess) {
      cudaGetLastError();
      ctx->d_val64s = nullptr;
      ctx->val64s_off = true;
      return -1;
    }
  }
  if (ctx->val64s_gen == ctx->params_gen) return 0;
  GB_CUDA(cudaMemsetAsync(ctx->d_val64s, 0, sizeof(double) * ctx->nnz, ctx->stream));
  a.val = ctx->d_val64s;
  a.r = nullptr;
  a.jpart = 1;
  fa.val = ctx->d_val64s;
  fa.r = nullptr;
  int rc = launch_cells<double, true, false>(ctx, a, ctx->d_tab64);
  if (rc) return rc;
  { if (ctx->nfacets) k_facets<double, true, false><<<(unsigned)ctx->nfacets, 64, 0, ctx->stream>>>(fa, ft); gbmhd::count_launch(); }
  GB_CUDA(cudaGetLastError());
  ctx->val64s_gen = ctx->params_gen;
  return 0;
}

// Residual (FP64) into d_r (if non-null) and Jacobian (precision) into the CSR values.
int gb_assemble_device(gbmhd_ctx* ctx, const double* d_x, double* d_r, int want_jac, int precision) {
  if (ctx->ndofs > 0)
    GB_CUDA(cudaMemcpyAsync(ctx->d_xfull, d_x, sizeof(double) * ctx->ndofs, cudaMemcpyDeviceToDevice,
                            ctx->stream));
  if (d_r) GB_CUDA(cudaMemsetAsync(d_r, 0, sizeof(double) * ctx->ndofs, ctx->stream));
  KArgs a{};
  a.ncells = ctx->ncells;
  a.cellX = ctx->d_cellX;
  a.gidx = ctx->d_gidx;
  a.row = ctx->d_row;
  a.sign = reinterpret_cast<const unsigned long long*>(ctx->d_sign);
  a.xfull = ctx->d_xfull;
  a.fcell = ctx->d_fcell;
  a.rowptr = ctx->d_rowptr;
  a.cls = ctx->d_class;
  a.offtab = ctx->d_offtab;
  a.r = d_r;
  a.prm = ctx->prm;
  FArgs fa{};
  fa.nfacets = ctx->nfacets;
  fa.fcell = ctx->d_fcellid;
  fa.flface = ctx->d_flface;
  fa.fprm = ctx->d_fprm;
  fa.cellX = ctx->d_cellX;
  fa.gidx = ctx->d_gidx;
  fa.row = ctx->d_row;
  fa.sign = a.sign;
  fa.xfull = ctx->d_xfull;
  fa.rowptr = ctx->d_rowptr;
  fa.cls = ctx->d_class;
  fa.offtab = ctx->d_offtab;
  fa.r = d_r;
  fa.dr_dcw = nullptr;
  const FacetTables* ft = reinterpret_cast<const FacetTables*>(ctx->d_ftab);
  int rc = 0;
  if (want_jac) {
    if (precision == GBMHD_MIXED) {
      GB_CUDA(cudaMemsetAsync(ctx->d_val32, 0, sizeof(float) * ctx->nnz, ctx->stream));
      a.val = ctx->d_val32;
      fa.val = ctx->d_val32;
      if (d_r) {
        if ((rc = launch_residual(ctx, a))) return rc;
      }
      if ((rc = launch_cells<float, true, false>(ctx, a, ctx->d_tab32))) return rc;
      if (ctx->nfacets) {
        { if (d_r) k_facets<double, false, true><<<(unsigned)ctx->nfacets, 64, 0, ctx->stream>>>(fa, ft); gbmhd::count_launch(); }
        { k_facets<float, true, false><<<(unsigned)ctx->nfacets, 64, 0, ctx->stream>>>(fa, ft); gbmhd::count_launch(); }
      }
    } else if ((rc = static_jacobian(ctx, a, fa, ft)) == 0) {
      // FP64: the cached state-independent terms, then the convection terms at this state
      GB_CUDA(cudaMemcpyAsync(ctx->d_val64, ctx->d_val64s, sizeof(double) * ctx->nnz, cudaMemcpyDeviceToDevice,
                              ctx->stream));
      a.val = ctx->d_val64;
      fa.val = ctx->d_val64;
      if (ctx->prm.convection != 0) {
        a.jpart = 2;
        if ((rc = launch_cells<double, true, false>(ctx, a, ctx->d_tab64))) return rc;
        a.jpart = 0;
      }
      if (d_r) {
        if ((rc = launch_residual(ctx, a))) return rc;
        { if (ctx->nfacets) k_facets<double, false, true><<<(unsigned)ctx->nfacets, 64, 0, ctx->stream>>>(fa, ft); gbmhd::count_launch(); }
      }
    } else {
      if (rc != -1) return rc;  // a launch of the state-independent pass failed
      GB_CUDA(cudaMemsetAsync(ctx->d_val64, 0, sizeof(double) * ctx->nnz, ctx->stream));
      a.val = ctx->d_val64;
      fa.val = ctx->d_val64;
      if (d_r) {
        if ((rc = launch_cells<double, true, false>(ctx, a, ctx->d_tab64))) return rc;
        if ((rc = launch_residual(ctx, a))) return rc;
        { if (ctx->nfacets) k_facets<double, true, true><<<(unsigned)ctx->nfacets, 64, 0, ctx->stream>>>(fa, ft); gbmhd::count_launch(); }
      } else {
        if ((rc = launch_cells<double, true, false>(ctx, a, ctx->d_tab64))) return rc;
        { if (ctx->nfacets) k_facets<double, true, false><<<(unsigned)ctx->nfacets, 64, 0, ctx->stream>>>(fa, ft); gbmhd::count_launch(); }
      }
    }
    ctx->jac_precision = precision;
  } else if (d_r) {
    if ((rc = launch_residual(ctx, a))) return rc;
    { if (ctx->nfacets) k_facets<double, false, true><<<(unsigned)ctx->nfacets, 64, 0, ctx->stream>>>(fa, ft); gbmhd::count_launch(); }
  }
  GB_CUDA(cudaGetLastError());
  return 0;
}

int gb_param_derivs(gbmhd_ctx* ctx, const double* d_x, double* d_dr_dgamma, double* d_dr_dcw, double* d_fz,
                    double* d_dr_dalpha, double* d_dr_dbeta) {
  if (ctx->ndofs > 0)
    GB_CUDA(cudaMemcpyAsync(ctx->d_xfull, d_x, sizeof(double) * ctx->ndofs, cudaMemcpyDeviceToDevice,
                            ctx->stream));
  if (d_dr_dgamma) GB_CUDA(cudaMemsetAsync(d_dr_dgamma, 0, sizeof(double) * ctx->ndofs, ctx->stream));
  if (d_dr_dcw) GB_CUDA(cudaMemsetAsync(d_dr_dcw, 0, sizeof(double) * ctx->ndofs, ctx->stream));
  if (d_dr_dalpha) GB_CUDA(cudaMemsetAsync(d_dr_dalpha, 0, sizeof(double) * ctx->ndofs, ctx->stream));
  if (d_dr_dbeta) GB_CUDA(cudaMemsetAsync(d_dr_dbeta, 0, sizeof(double) * ctx->ndofs, ctx->stream));
  const GeoTables* geo = reinterpret_cast<const GeoTables*>(
      reinterpret_cast<const char*>(ctx->d_tab64) + ((sizeof(DevTables<double>) + 255) & ~size_t(255)));
  int64_t grid = ctx->num_sms * 8;
  if (grid > ctx->ncells) grid = ctx->ncells;
  if (grid < 1) grid = 1;
  if (d_dr_dalpha || d_dr_dbeta) {
    { k_param_derivs_ab<<<(unsigned)grid, 128, 0, ctx->stream>>>(
        ctx->ncells, ctx->d_cellX, ctx->d_gidx, ctx->d_row, ctx->d_xfull,
        reinterpret_cast<const DevTables<double>*>(ctx->d_tab64), geo, ctx->prm.convection, d_dr_dalpha, d_dr_dbeta); gbmhd::count_launch(); }
    GB_CUDA(cudaGetLastError());
  }
  { k_param_derivs<<<(unsigned)grid, 128, 0, ctx->stream>>>(
      ctx->ncells, ctx->d_cellX, ctx->d_gidx, ctx->d_row, reinterpret_cast<const unsigned long long*>(ctx->d_sign),
      ctx->d_xfull, reinterpret_cast<const DevTables<double>*>(ctx->d_tab64), geo, ctx->prm, d_dr_dgamma, d_fz); gbmhd::count_launch(); }
  GB_CUDA(cudaGetLastError());
  if (d_dr_dcw && ctx->nfacets) {
    FArgs fa{};
    fa.nfacets = ctx->nfacets;
    fa.fcell = ctx->d_fcellid;
    fa.flface = ctx->d_flface;
    fa.fprm = ctx->d_fprm;
    fa.cellX = ctx->d_cellX;
    fa.gidx = ctx->d_gidx;
    fa.row = ctx->d_row;
    fa.sign = reinterpret_cast<const unsigned long long*>(ctx->d_sign);
    fa.xfull = ctx->d_xfull;
    fa.rowptr = ctx->d_rowptr;
    fa.cls = ctx->d_class;
    fa.offtab = ctx->d_offtab;
    fa.val = nullptr;
    fa.r = nullptr;
    fa.dr_dcw = d_dr_dcw;
    { k_facets<double, false, false><<<(unsigned)ctx->nfacets, 64, 0, ctx->stream>>>(
        fa, reinterpret_cast<const FacetTables*>(ctx->d_ftab)); gbmhd::count_launch(); }
    GB_CUDA(cudaGetLastError());
  }
  return 0;
}
