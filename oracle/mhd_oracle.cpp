// FP64 CPU oracle for the inductionless-MHD Newton assembly (test infrastructure only).
//
// This file is a plain restatement of the reference's cell integrands, written
// for checking the CUDA library; nothing in the product links it.  Only the
// tests, the smoke check and the CPU-baseline leg of bench.py load it.
//
// Reference behaviour restated here (paths inside GridapMHD.jl):
//   src/weakforms.jl:37-43     setup_variable: ∇u, div u = tr ∇u, ∇j, div j
//   src/weakforms.jl:255-281   res_fluid_h1_hdiv (integrand and signs)
//   src/weakforms.jl:283-312   jac_fluid_h1_hdiv (Newton / Picard convection)
//   src/weakforms.jl:670       conv(u,∇u) = (∇u)ᵀ·u
//   src/weakforms.jl:672-681   Πp = local L2 projection of div u onto the p space
//   src/weakforms.jl:716-719   res_φ_bcs
//   src/weakforms.jl:721-733   res/jac_thin_wall (residual uses the state x, see below)
//   src/parameters.jl:381-389  quadrature degree q = 5 -> 3 Gauss points per direction
//   src/parameters.jl:436-441  u: Q2 vector Lagrange, p: discontinuous P1 (space=:P)
//   src/parameters.jl:521-526  j: Raviart-Thomas order 1, φ: discontinuous Q1
//
// Reference defect handled: res_thin_wall reads `dx` that is not in scope
// (src/weakforms.jl:721-726).  The evident intent, τ∫(s·n)(j·n − jw + cw n·∇j·n),
// is evaluated with the state j.
//
// Local dof layout of one cell (129 entries):
//   [0,81)    u, component-major: c*27 + node, node = a + 3b + 9c over the 3x3x3
//             Lagrange nodes at ξ ∈ {0, 1/2, 1}
//   [81,85)   p, nodal P1 at (0,0,0),(1,0,0),(0,1,0),(0,0,1) of the reference cube
//   [85,121)  j, Raviart-Thomas: component d block of 12, index q + 3*(l1 + 2*l2),
//             ψ = L2_q(ξ_d) L1_l1(ξ_o1) L1_l2(ξ_o2) e_d  (o1 < o2 the other axes)
//   [121,129) φ, nodal Q1 at the 8 vertices (a + 2b + 4c)
// The RT face dofs (q = 0 or 2) are the +axis normal flux density at the face
// vertices; the contravariant Piola map j = J ĵ / det J pushes them forward.
//
// The gradient of a Piola-mapped field is taken with the Jacobian held constant
// inside the cell (exact on the box cells of every structured mesh used here).

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

constexpr int NU = 81, NP = 4, NJ = 36, NPHI = 8, ND = 129;
constexpr int OU = 0, OP = 81, OJ = 85, OPHI = 121;

// ---------------------------------------------------------------- quadrature
void gauss_legendre01(int n, double* x, double* w) {
  // Newton iteration on P_n; nodes mapped from [-1,1] to [0,1].
  for (int i = 0; i < n; ++i) {
    double t = std::cos(M_PI * (i + 0.75) / (n + 0.5));
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = t;
      for (int k = 2; k <= n; ++k) {
        double p2 = ((2.0 * k - 1.0) * t * p1 - (k - 1.0) * p0) / k;
        p0 = p1; p1 = p2;
      }
      double dp = n * (t * p1 - p0) / (t * t - 1.0);
      double dt = p1 / dp;
      t -= dt;
      if (std::fabs(dt) < 1e-16) break;
    }
    double p0 = 1.0, p1 = t;
    for (int k = 2; k <= n; ++k) {
      double p2 = ((2.0 * k - 1.0) * t * p1 - (k - 1.0) * p0) / k;
      p0 = p1; p1 = p2;
    }
    double dp = n * (t * p1 - p0) / (t * t - 1.0);
    x[i] = 0.5 * (1.0 - t);
    w[i] = 0.5 * 2.0 / ((1.0 - t * t) * dp * dp);
  }
}

// ---------------------------------------------------------------- 1D bases
inline double lag2(int a, double t) {
  switch (a) { case 0: return 2.0 * (t - 0.5) * (t - 1.0);
               case 1: return -4.0 * t * (t - 1.0);
               default: return 2.0 * t * (t - 0.5); }
}
inline double dlag2(int a, double t) {
  switch (a) { case 0: return 4.0 * t - 3.0;
               case 1: return 4.0 - 8.0 * t;
               default: return 4.0 * t - 1.0; }
}
inline double lag1(int a, double t) { return a == 0 ? 1.0 - t : t; }
inline double dlag1(int a, double) { return a == 0 ? -1.0 : 1.0; }

// ---------------------------------------------------------------- reference fields at a point
struct RefBasis {
  double q2[27], dq2[27][3];     // scalar Q2 nodal basis
  double q1[8], dq1[8][3];       // Q1 (geometry and φ)
  double p1[4], dp1[4][3];       // P1 nodal on the cube
  double rt[36][3], rtdiv[36], rtgrad[36][3][3];  // rtgrad[b][a][m] = ∂_a ψ̂_m
};

void eval_ref(const double xi[3], RefBasis& B) {
  for (int c = 0; c < 3; ++c)
    for (int b = 0; b < 3; ++b)
      for (int a = 0; a < 3; ++a) {
        int n = a + 3 * b + 9 * c;
        double la = lag2(a, xi[0]), lb = lag2(b, xi[1]), lc = lag2(c, xi[2]);
        B.q2[n] = la * lb * lc;
        B.dq2[n][0] = dlag2(a, xi[0]) * lb * lc;
        B.dq2[n][1] = la * dlag2(b, xi[1]) * lc;
        B.dq2[n][2] = la * lb * dlag2(c, xi[2]);
      }
  for (int c = 0; c < 2; ++c)
    for (int b = 0; b < 2; ++b)
      for (int a = 0; a < 2; ++a) {
        int n = a + 2 * b + 4 * c;
        double la = lag1(a, xi[0]), lb = lag1(b, xi[1]), lc = lag1(c, xi[2]);
        B.q1[n] = la * lb * lc;
        B.dq1[n][0] = dlag1(a, xi[0]) * lb * lc;
        B.dq1[n][1] = la * dlag1(b, xi[1]) * lc;
        B.dq1[n][2] = la * lb * dlag1(c, xi[2]);
      }
  B.p1[0] = 1.0 - xi[0] - xi[1] - xi[2];
  B.p1[1] = xi[0]; B.p1[2] = xi[1]; B.p1[3] = xi[2];
  for (int d = 0; d < 3; ++d) B.dp1[0][d] = -1.0;
  for (int k = 1; k < 4; ++k)
    for (int d = 0; d < 3; ++d) B.dp1[k][d] = (k - 1 == d) ? 1.0 : 0.0;
  std::memset(B.rt, 0, sizeof(B.rt));
  std::memset(B.rtgrad, 0, sizeof(B.rtgrad));
  for (int d = 0; d < 3; ++d) {
    int o1 = (d == 0) ? 1 : 0, o2 = (d == 2) ? 1 : 2;
    for (int l2 = 0; l2 < 2; ++l2)
      for (int l1 = 0; l1 < 2; ++l1)
        for (int q = 0; q < 3; ++q) {
          int b = d * 12 + q + 3 * (l1 + 2 * l2);
          double fq = lag2(q, xi[d]), f1 = lag1(l1, xi[o1]), f2 = lag1(l2, xi[o2]);
          B.rt[b][d] = fq * f1 * f2;
          B.rtdiv[b] = dlag2(q, xi[d]) * f1 * f2;
          B.rtgrad[b][d][d] = dlag2(q, xi[d]) * f1 * f2;
          B.rtgrad[b][o1][d] = fq * dlag1(l1, xi[o1]) * f2;
          B.rtgrad[b][o2][d] = fq * f1 * dlag1(l2, xi[o2]);
        }
  }
}

// ---------------------------------------------------------------- physical fields at a point
struct PhysBasis {
  double x[3];
  double J[3][3], Jinv[3][3], det;
  double u[27], gu[27][3];     // scalar Q2 values and physical gradients
  double p[4];
  double phi[8];
  double s[36][3], divs[36], gs[36][3][3];  // gs[b][i][k] = ∂_i ψ_k
};

void inv3(const double A[3][3], double Ai[3][3], double& det) {
  det = A[0][0] * (A[1][1] * A[2][2] - A[1][2] * A[2][1]) -
        A[0][1] * (A[1][0] * A[2][2] - A[1][2] * A[2][0]) +
        A[0][2] * (A[1][0] * A[2][1] - A[1][1] * A[2][0]);
  double id = 1.0 / det;
  Ai[0][0] = (A[1][1] * A[2][2] - A[1][2] * A[2][1]) * id;
  Ai[0][1] = (A[0][2] * A[2][1] - A[0][1] * A[2][2]) * id;
  Ai[0][2] = (A[0][1] * A[1][2] - A[0][2] * A[1][1]) * id;
  Ai[1][0] = (A[1][2] * A[2][0] - A[1][0] * A[2][2]) * id;
  Ai[1][1] = (A[0][0] * A[2][2] - A[0][2] * A[2][0]) * id;
  Ai[1][2] = (A[0][2] * A[1][0] - A[0][0] * A[1][2]) * id;
  Ai[2][0] = (A[1][0] * A[2][1] - A[1][1] * A[2][0]) * id;
  Ai[2][1] = (A[0][1] * A[2][0] - A[0][0] * A[2][1]) * id;
  Ai[2][2] = (A[0][0] * A[1][1] - A[0][1] * A[1][0]) * id;
}

void eval_phys(const double* X /*[8][3]*/, const double xi[3], PhysBasis& P) {
  RefBasis R;
  eval_ref(xi, R);
  for (int i = 0; i < 3; ++i) {
    P.x[i] = 0.0;
    for (int a = 0; a < 3; ++a) P.J[i][a] = 0.0;
  }
  for (int v = 0; v < 8; ++v)
    for (int i = 0; i < 3; ++i) {
      P.x[i] += X[3 * v + i] * R.q1[v];
      for (int a = 0; a < 3; ++a) P.J[i][a] += X[3 * v + i] * R.dq1[v][a];
    }
  inv3(P.J, P.Jinv, P.det);
  for (int n = 0; n < 27; ++n) {
    P.u[n] = R.q2[n];
    for (int i = 0; i < 3; ++i) {
      double g = 0.0;
      for (int a = 0; a < 3; ++a) g += P.Jinv[a][i] * R.dq2[n][a];
      P.gu[n][i] = g;
    }
  }
  for (int k = 0; k < 4; ++k) P.p[k] = R.p1[k];
  for (int k = 0; k < 8; ++k) P.phi[k] = R.q1[k];
  double id = 1.0 / P.det;
  for (int b = 0; b < 36; ++b) {
    for (int i = 0; i < 3; ++i) {
      double v = 0.0;
      for (int m = 0; m < 3; ++m) v += P.J[i][m] * R.rt[b][m];
      P.s[b][i] = v * id;
    }
    P.divs[b] = R.rtdiv[b] * id;
    for (int i = 0; i < 3; ++i)
      for (int k = 0; k < 3; ++k) {
        double g = 0.0;
        for (int a = 0; a < 3; ++a)
          for (int m = 0; m < 3; ++m) g += P.Jinv[a][i] * P.J[k][m] * R.rtgrad[b][a][m];
        P.gs[b][i][k] = g * id;
      }
  }
}

inline void cross(const double a[3], const double b[3], double c[3]) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

// Reference face f (0..5): axis = f/2, side = f%2 (ξ_axis = side).
void face_point(int f, double s, double t, double xi[3]) {
  int ax = f / 2, side = f % 2;
  int o1 = (ax == 0) ? 1 : 0, o2 = (ax == 2) ? 1 : 2;
  xi[ax] = side; xi[o1] = s; xi[o2] = t;
}

}  // namespace

extern "C" {

// Parameters of the fluid integrand (src/weakforms.jl:71-83 retrieve_fluid_params).
struct OrcFluid {
  double alpha, beta, gamma, sigma;
  double B[3];
  double f[3];        // used when f_cell is null
  double g[3];
  double zeta_u, zeta_j;
  int32_t convection; // 0 none, 1 picard, 2 newton
  const double* f_cell;  // [ncells][3] or null
};

// Boundary facets carrying the thin-wall law or a weak potential value.
struct OrcFacets {
  int64_t n;
  const int32_t* cell;   // cell index
  const int8_t* lface;   // local face 0..5 (axis*2 + side)
  const double* tau;     // thin wall penalty  (per facet)
  const double* cw;      // wall conductance ratio
  const double* jw;      // prescribed wall current
  const double* phi0;    // weak potential value (src/weakforms.jl:716-719); may be null
};

int orc_version() { return 1; }

void orc_gauss01(int n, double* x, double* w) { gauss_legendre01(n, x, w); }

// Residual (r_cell, [ncells][129]) and optionally the Jacobian (K_cell,
// [ncells][129][129], row = test dof, column = trial dof) of every cell.
// x_cell holds the 129 local state values per cell (free and Dirichlet).
void orc_assemble_cells(int64_t ncells, const double* cell_X /*[ncells][8][3]*/,
                        const double* x_cell, const OrcFluid* fl, const OrcFacets* fc,
                        double* r_cell, double* K_cell, int nthreads) {
  double gx[3], gw[3];
  gauss_legendre01(3, gx, gw);
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads)
  for (int64_t c = 0; c < ncells; ++c) {
    const double* X = cell_X + 24 * c;
    const double* xl = x_cell + ND * c;
    double* r = r_cell ? r_cell + ND * c : nullptr;
    double* K = K_cell ? K_cell + (int64_t)ND * ND * c : nullptr;
    if (r) std::memset(r, 0, sizeof(double) * ND);
    if (K) std::memset(K, 0, sizeof(double) * ND * ND);
    const double* fvec = fl->f_cell ? fl->f_cell + 3 * c : fl->f;
    std::vector<PhysBasis> PB(27);
    std::vector<double> dV(27);
    for (int qk = 0; qk < 3; ++qk)
      for (int qj = 0; qj < 3; ++qj)
        for (int qi = 0; qi < 3; ++qi) {
          int q = qi + 3 * qj + 9 * qk;
          double xi[3] = {gx[qi], gx[qj], gx[qk]};
          eval_phys(X, xi, PB[q]);
          dV[q] = gw[qi] * gw[qj] * gw[qk] * PB[q].det;
        }
    // Local L2 projection onto the p space (src/weakforms.jl:672-681): mass matrix
    // Mp and moments of div of every u basis function.
    double Mp[4][4] = {{0}}, Mpi[4][4];
    std::vector<double> Bdiv(4 * NU, 0.0);  // Bdiv[k*81 + b] = ∫ ψ_k div φ_b
    for (int q = 0; q < 27; ++q) {
      const PhysBasis& P = PB[q];
      for (int k = 0; k < 4; ++k) {
        for (int l = 0; l < 4; ++l) Mp[k][l] += P.p[k] * P.p[l] * dV[q];
        for (int cc = 0; cc < 3; ++cc)
          for (int n = 0; n < 27; ++n) Bdiv[k * NU + cc * 27 + n] += P.p[k] * P.gu[n][cc] * dV[q];
      }
    }
    {  // invert the 4x4 p mass matrix by Gauss-Jordan
      double A[4][8];
      for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 8; ++j) A[i][j] = j < 4 ? Mp[i][j] : (j - 4 == i ? 1.0 : 0.0);
      for (int i = 0; i < 4; ++i) {
        int piv = i;
        for (int k = i + 1; k < 4; ++k) if (std::fabs(A[k][i]) > std::fabs(A[piv][i])) piv = k;
        if (piv != i) for (int j = 0; j < 8; ++j) std::swap(A[i][j], A[piv][j]);
        double d = A[i][i];
        for (int j = 0; j < 8; ++j) A[i][j] /= d;
        for (int k = 0; k < 4; ++k) if (k != i) {
          double m = A[k][i];
          for (int j = 0; j < 8; ++j) A[k][j] -= m * A[i][j];
        }
      }
      for (int i = 0; i < 4; ++i) for (int j = 0; j < 4; ++j) Mpi[i][j] = A[i][j + 4];
    }
    // Projection coefficients of div u (state).
    double divmom[4] = {0, 0, 0, 0}, pic[4] = {0, 0, 0, 0};
    for (int k = 0; k < 4; ++k)
      for (int b = 0; b < NU; ++b) divmom[k] += Bdiv[k * NU + b] * xl[OU + b];
    for (int k = 0; k < 4; ++k)
      for (int l = 0; l < 4; ++l) pic[k] += Mpi[k][l] * divmom[l];

    for (int q = 0; q < 27; ++q) {
      const PhysBasis& P = PB[q];
      const double w = dV[q];
      // state at the point
      double u[3] = {0, 0, 0}, gu[3][3] = {{0}};  // gu[i][k] = ∂_i u_k
      for (int cc = 0; cc < 3; ++cc)
        for (int n = 0; n < 27; ++n) {
          double val = xl[OU + cc * 27 + n];
          u[cc] += val * P.u[n];
          for (int i = 0; i < 3; ++i) gu[i][cc] += val * P.gu[n][i];
        }
      double divu = gu[0][0] + gu[1][1] + gu[2][2];
      double p = 0.0;
      for (int k = 0; k < 4; ++k) p += xl[OP + k] * P.p[k];
      double j[3] = {0, 0, 0}, divj = 0.0;
      for (int b = 0; b < 36; ++b) {
        double val = xl[OJ + b];
        for (int i = 0; i < 3; ++i) j[i] += val * P.s[b][i];
        divj += val * P.divs[b];
      }
      double phi = 0.0;
      for (int k = 0; k < 8; ++k) phi += xl[OPHI + k] * P.phi[k];
      double pi_divu = 0.0;
      for (int k = 0; k < 4; ++k) pi_divu += pic[k] * P.p[k];
      double jxB[3], uxB[3];
      cross(j, fl->B, jxB);
      cross(u, fl->B, uxB);
      double conv[3];  // (∇u)ᵀ·u : conv_c = Σ_k ∂_k u_c u_k
      for (int cc = 0; cc < 3; ++cc) {
        conv[cc] = 0.0;
        for (int k = 0; k < 3; ++k) conv[cc] += gu[k][cc] * u[k];
      }
      if (r) {
        // u rows
        for (int cc = 0; cc < 3; ++cc)
          for (int n = 0; n < 27; ++n) {
            double vv = P.u[n];
            double gradterm = 0.0;
            for (int i = 0; i < 3; ++i) gradterm += gu[i][cc] * P.gu[n][i];
            double divv = P.gu[n][cc];
            double val = fl->beta * gradterm - p * divv - fl->gamma * jxB[cc] * vv - fvec[cc] * vv;
            if (fl->convection != 0) val += fl->alpha * vv * conv[cc];
            if (fl->zeta_u != 0.0) val += fl->zeta_u * pi_divu * divv;
            r[OU + cc * 27 + n] += w * val;
          }
        for (int k = 0; k < 4; ++k) r[OP + k] += w * (-divu * P.p[k]);
        for (int b = 0; b < 36; ++b) {
          double js = 0.0, uBs = 0.0, gs = 0.0;
          for (int i = 0; i < 3; ++i) {
            js += j[i] * P.s[b][i];
            uBs += uxB[i] * P.s[b][i];
            gs += fl->g[i] * P.s[b][i];
          }
          double val = js - fl->sigma * phi * P.divs[b] - fl->sigma * uBs - gs;
          if (fl->zeta_j != 0.0) val += fl->zeta_j * divj * P.divs[b];
          r[OJ + b] += w * val;
        }
        for (int k = 0; k < 8; ++k) r[OPHI + k] += w * (-divj * P.phi[k]);
      }
      if (K) {
        auto Kat = [&](int row, int col) -> double& { return K[(int64_t)row * ND + col]; };
        // u-u
        for (int cc = 0; cc < 3; ++cc)
          for (int a = 0; a < 27; ++a) {
            int row = OU + cc * 27 + a;
            double va = P.u[a];
            for (int dd = 0; dd < 3; ++dd)
              for (int b = 0; b < 27; ++b) {
                int col = OU + dd * 27 + b;
                double val = 0.0;
                if (cc == dd) {
                  double gg = 0.0;
                  for (int i = 0; i < 3; ++i) gg += P.gu[a][i] * P.gu[b][i];
                  val += fl->beta * gg;
                  if (fl->convection != 0) {
                    double ugb = 0.0;  // ((∇du)ᵀ u)_c with du = φ_b e_c
                    for (int k = 0; k < 3; ++k) ugb += P.gu[b][k] * u[k];
                    val += fl->alpha * va * ugb;
                  }
                }
                if (fl->convection == 2) {
                  // ((∇u)ᵀ du)_c with du = φ_b e_d  ->  ∂_d u_c φ_b
                  val += fl->alpha * va * gu[dd][cc] * P.u[b];
                }
                Kat(row, col) += w * val;
              }
          }
        // u-p and p-u
        for (int cc = 0; cc < 3; ++cc)
          for (int a = 0; a < 27; ++a)
            for (int k = 0; k < 4; ++k) {
              double v = -P.p[k] * P.gu[a][cc] * w;
              Kat(OU + cc * 27 + a, OP + k) += v;
              Kat(OP + k, OU + cc * 27 + a) += v;
            }
        // u-j: −γ (dj × B)·v
        for (int b = 0; b < 36; ++b) {
          double sxB[3];
          cross(P.s[b], fl->B, sxB);
          for (int cc = 0; cc < 3; ++cc)
            for (int a = 0; a < 27; ++a)
              Kat(OU + cc * 27 + a, OJ + b) += w * (-fl->gamma * sxB[cc] * P.u[a]);
        }
        // j-u: −σ (du × B)·s
        for (int dd = 0; dd < 3; ++dd) {
          double e[3] = {0, 0, 0};
          e[dd] = 1.0;
          double eB[3];
          cross(e, fl->B, eB);
          for (int a = 0; a < 36; ++a) {
            double eBs = eB[0] * P.s[a][0] + eB[1] * P.s[a][1] + eB[2] * P.s[a][2];
            for (int b = 0; b < 27; ++b)
              Kat(OJ + a, OU + dd * 27 + b) += w * (-fl->sigma * eBs * P.u[b]);
          }
        }
        // j-j
        for (int a = 0; a < 36; ++a)
          for (int b = 0; b < 36; ++b) {
            double ss = P.s[a][0] * P.s[b][0] + P.s[a][1] * P.s[b][1] + P.s[a][2] * P.s[b][2];
            double val = ss;
            if (fl->zeta_j != 0.0) val += fl->zeta_j * P.divs[a] * P.divs[b];
            Kat(OJ + a, OJ + b) += w * val;
          }
        // j-φ and φ-j
        for (int a = 0; a < 36; ++a)
          for (int k = 0; k < 8; ++k) {
            Kat(OJ + a, OPHI + k) += w * (-fl->sigma * P.phi[k] * P.divs[a]);
            Kat(OPHI + k, OJ + a) += w * (-P.divs[a] * P.phi[k]);
          }
      }
    }
    // AL u term in the Jacobian: ζᵤ ∫ Πp(div du) div v = ζᵤ Bdivᵀ Mp⁻¹ Bdiv
    if (K && fl->zeta_u != 0.0) {
      for (int a = 0; a < NU; ++a)
        for (int b = 0; b < NU; ++b) {
          double v = 0.0;
          for (int k = 0; k < 4; ++k)
            for (int l = 0; l < 4; ++l) v += Bdiv[k * NU + a] * Mpi[k][l] * Bdiv[l * NU + b];
          K[(int64_t)(OU + a) * ND + OU + b] += fl->zeta_u * v;
        }
    }
  }

  // Boundary facets (serial: a cell may own several facets).
  if (fc && fc->n > 0) {
    for (int64_t e = 0; e < fc->n; ++e) {
      int c = fc->cell[e];
      int f = fc->lface[e];
      const double* X = cell_X + 24 * (int64_t)c;
      const double* xl = x_cell + ND * (int64_t)c;
      double* r = r_cell ? r_cell + ND * (int64_t)c : nullptr;
      double* K = K_cell ? K_cell + (int64_t)ND * ND * c : nullptr;
      int ax = f / 2, side = f % 2;
      for (int tj = 0; tj < 3; ++tj)
        for (int ti = 0; ti < 3; ++ti) {
          double xi[3];
          face_point(f, gx[ti], gx[tj], xi);
          PhysBasis P;
          eval_phys(X, xi, P);
          // outward normal: ± J⁻ᵀ e_ax ; area element det J |J⁻ᵀ e_ax|
          double nn[3];
          for (int i = 0; i < 3; ++i) nn[i] = P.Jinv[ax][i] * (side ? 1.0 : -1.0);
          double nl = std::sqrt(nn[0] * nn[0] + nn[1] * nn[1] + nn[2] * nn[2]);
          for (int i = 0; i < 3; ++i) nn[i] /= nl;
          double dA = gw[ti] * gw[tj] * std::fabs(P.det) * nl;
          double sn[36], gnn[36];
          for (int b = 0; b < 36; ++b) {
            sn[b] = P.s[b][0] * nn[0] + P.s[b][1] * nn[1] + P.s[b][2] * nn[2];
            double g = 0.0;
            for (int i = 0; i < 3; ++i)
              for (int k = 0; k < 3; ++k) g += nn[i] * P.gs[b][i][k] * nn[k];
            gnn[b] = g;
          }
          double tau = fc->tau ? fc->tau[e] : 0.0;
          double cw = fc->cw ? fc->cw[e] : 0.0;
          double jw = fc->jw ? fc->jw[e] : 0.0;
          double phi0 = fc->phi0 ? fc->phi0[e] : 0.0;
          if (r) {
            double jn = 0.0, jnn = 0.0;
            for (int b = 0; b < 36; ++b) {
              jn += xl[OJ + b] * sn[b];
              jnn += xl[OJ + b] * gnn[b];
            }
            for (int a = 0; a < 36; ++a)
              r[OJ + a] += dA * (tau * sn[a] * (jn - jw + cw * jnn) + sn[a] * phi0);
          }
          if (K && tau != 0.0) {
            for (int a = 0; a < 36; ++a)
              for (int b = 0; b < 36; ++b)
                K[(int64_t)(OJ + a) * ND + OJ + b] += dA * tau * sn[a] * (sn[b] + cw * gnn[b]);
          }
        }
    }
  }
}

// Derivative of the cell residuals with respect to scalar parameters, at the
// state x: dR/dγ (−∫(j×B)·v), dR/dcw per thin-wall facet summed into one
// vector (τ∫(s·n)(n·∇j·n)), and the per-cell body-force moments ∫ v_z dΩ.
void orc_param_derivs(int64_t ncells, const double* cell_X, const double* x_cell,
                      const OrcFluid* fl, const OrcFacets* fc,
                      double* dr_dgamma /*[ncells][129]*/, double* dr_dcw /*[ncells][129]*/,
                      double* fz_moment /*[ncells][27]*/) {
  double gx[3], gw[3];
  gauss_legendre01(3, gx, gw);
  for (int64_t c = 0; c < ncells; ++c) {
    const double* X = cell_X + 24 * c;
    const double* xl = x_cell + ND * c;
    if (dr_dgamma) std::memset(dr_dgamma + ND * c, 0, sizeof(double) * ND);
    if (dr_dcw) std::memset(dr_dcw + ND * c, 0, sizeof(double) * ND);
    if (fz_moment) std::memset(fz_moment + 27 * c, 0, sizeof(double) * 27);
    for (int qk = 0; qk < 3; ++qk)
      for (int qj = 0; qj < 3; ++qj)
        for (int qi = 0; qi < 3; ++qi) {
          double xi[3] = {gx[qi], gx[qj], gx[qk]};
          PhysBasis P;
          eval_phys(X, xi, P);
          double w = gw[qi] * gw[qj] * gw[qk] * P.det;
          double j[3] = {0, 0, 0};
          for (int b = 0; b < 36; ++b)
            for (int i = 0; i < 3; ++i) j[i] += xl[OJ + b] * P.s[b][i];
          double jxB[3];
          cross(j, fl->B, jxB);
          for (int cc = 0; cc < 3; ++cc)
            for (int n = 0; n < 27; ++n) {
              if (dr_dgamma) dr_dgamma[ND * c + OU + cc * 27 + n] += w * (-jxB[cc] * P.u[n]);
              if (fz_moment && cc == 2) fz_moment[27 * c + n] += w * P.u[n];
            }
        }
  }
  if (fc && dr_dcw) {
    for (int64_t e = 0; e < fc->n; ++e) {
      int c = fc->cell[e];
      int f = fc->lface[e];
      const double* X = cell_X + 24 * (int64_t)c;
      const double* xl = x_cell + ND * (int64_t)c;
      int ax = f / 2, side = f % 2;
      for (int tj = 0; tj < 3; ++tj)
        for (int ti = 0; ti < 3; ++ti) {
          double xi[3];
          face_point(f, gx[ti], gx[tj], xi);
          PhysBasis P;
          eval_phys(X, xi, P);
          double nn[3];
          for (int i = 0; i < 3; ++i) nn[i] = P.Jinv[ax][i] * (side ? 1.0 : -1.0);
          double nl = std::sqrt(nn[0] * nn[0] + nn[1] * nn[1] + nn[2] * nn[2]);
          for (int i = 0; i < 3; ++i) nn[i] /= nl;
          double dA = gw[ti] * gw[tj] * std::fabs(P.det) * nl;
          double jnn = 0.0, sn[36];
          for (int b = 0; b < 36; ++b) {
            sn[b] = P.s[b][0] * nn[0] + P.s[b][1] * nn[1] + P.s[b][2] * nn[2];
            double g = 0.0;
            for (int i = 0; i < 3; ++i)
              for (int k = 0; k < 3; ++k) g += nn[i] * P.gs[b][i][k] * nn[k];
            jnn += xl[OJ + b] * g;
          }
          double tau = fc->tau ? fc->tau[e] : 0.0;
          for (int a = 0; a < 36; ++a) dr_dcw[ND * c + OJ + a] += dA * tau * sn[a] * jnn;
        }
    }
  }
}

// ∂R/∂β and ∂R/∂α on the u rows (the residual is linear in both): the viscous term
// ∫∇u⊙∇v and the convection term ∫v·((∇u)ᵀ·u) of res_fluid_h1_hdiv
// (src/weakforms.jl:264, :277-279; conv at :670).  The convection derivative is zero for
// convection = :none.  In the MHD scaling (src/Applications/expansion.jl:113-123) Ha enters
// through α = 1/N = Re/Ha² and β = 1/Ha², so dJ/dHa needs these two.
void orc_param_derivs_ab(int64_t ncells, const double* cell_X, const double* x_cell, const OrcFluid* fl,
                         double* dr_dalpha /*[ncells][129]*/, double* dr_dbeta /*[ncells][129]*/) {
  double gx[3], gw[3];
  gauss_legendre01(3, gx, gw);
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < ncells; ++c) {
    const double* X = cell_X + 24 * c;
    const double* xl = x_cell + ND * c;
    std::memset(dr_dalpha + ND * c, 0, sizeof(double) * ND);
    std::memset(dr_dbeta + ND * c, 0, sizeof(double) * ND);
    for (int qk = 0; qk < 3; ++qk)
      for (int qj = 0; qj < 3; ++qj)
        for (int qi = 0; qi < 3; ++qi) {
          double xi[3] = {gx[qi], gx[qj], gx[qk]};
          PhysBasis P;
          eval_phys(X, xi, P);
          const double w = gw[qi] * gw[qj] * gw[qk] * P.det;
          double u[3] = {0, 0, 0}, gu[3][3] = {{0}};  // gu[i][k] = ∂_i u_k
          for (int cc = 0; cc < 3; ++cc)
            for (int n = 0; n < 27; ++n) {
              const double val = xl[OU + cc * 27 + n];
              u[cc] += val * P.u[n];
              for (int i = 0; i < 3; ++i) gu[i][cc] += val * P.gu[n][i];
            }
          double conv[3];  // (∇u)ᵀ·u
          for (int cc = 0; cc < 3; ++cc) {
            conv[cc] = 0.0;
            for (int k = 0; k < 3; ++k) conv[cc] += gu[k][cc] * u[k];
          }
          for (int cc = 0; cc < 3; ++cc)
            for (int n = 0; n < 27; ++n) {
              double g = 0.0;
              for (int i = 0; i < 3; ++i) g += gu[i][cc] * P.gu[n][i];
              dr_dbeta[ND * c + OU + cc * 27 + n] += w * g;
              if (fl->convection != 0) dr_dalpha[ND * c + OU + cc * 27 + n] += w * P.u[n] * conv[cc];
            }
        }
  }
}

// Field evaluation for post-processing: at every cell, `npts1d`^3 Gauss points,
// write the physical point, weight·det J, u, ∇u (9, [i][k] = ∂_i u_k), p, j, div j, φ.
// out layout per point: 3 + 1 + 3 + 9 + 1 + 3 + 1 + 1 = 22 doubles.
void orc_eval_fields(int64_t ncells, const double* cell_X, const double* x_cell, int npts1d,
                     double* out) {
  std::vector<double> gx(npts1d), gw(npts1d);
  gauss_legendre01(npts1d, gx.data(), gw.data());
  const int np3 = npts1d * npts1d * npts1d;
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < ncells; ++c) {
    const double* X = cell_X + 24 * c;
    const double* xl = x_cell + ND * c;
    for (int qk = 0; qk < npts1d; ++qk)
      for (int qj = 0; qj < npts1d; ++qj)
        for (int qi = 0; qi < npts1d; ++qi) {
          int q = qi + npts1d * (qj + npts1d * qk);
          double xi[3] = {gx[qi], gx[qj], gx[qk]};
          PhysBasis P;
          eval_phys(X, xi, P);
          double* o = out + 22 * ((int64_t)c * np3 + q);
          std::memset(o, 0, sizeof(double) * 22);
          o[0] = P.x[0]; o[1] = P.x[1]; o[2] = P.x[2];
          o[3] = gw[qi] * gw[qj] * gw[qk] * P.det;
          for (int cc = 0; cc < 3; ++cc)
            for (int n = 0; n < 27; ++n) {
              double val = xl[OU + cc * 27 + n];
              o[4 + cc] += val * P.u[n];
              for (int i = 0; i < 3; ++i) o[7 + 3 * i + cc] += val * P.gu[n][i];
            }
          for (int k = 0; k < 4; ++k) o[16] += xl[OP + k] * P.p[k];
          for (int b = 0; b < 36; ++b) {
            for (int i = 0; i < 3; ++i) o[17 + i] += xl[OJ + b] * P.s[b][i];
            o[20] += xl[OJ + b] * P.divs[b];
          }
          for (int k = 0; k < 8; ++k) o[21] += xl[OPHI + k] * P.phi[k];
        }
  }
}

// Reference basis values at an arbitrary reference point (used by tests to check
// interpolation properties of the restated bases).
void orc_ref_basis(const double* xi, double* q2, double* rt /*[36][3]*/, double* rtdiv,
                   double* p1, double* q1) {
  RefBasis R;
  eval_ref(xi, R);
  if (q2) std::memcpy(q2, R.q2, sizeof(R.q2));
  if (rt) std::memcpy(rt, R.rt, sizeof(R.rt));
  if (rtdiv) std::memcpy(rtdiv, R.rtdiv, sizeof(R.rtdiv));
  if (p1) std::memcpy(p1, R.p1, sizeof(R.p1));
  if (q1) std::memcpy(q1, R.q1, sizeof(R.q1));
}

}  // extern "C"
