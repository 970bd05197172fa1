// Built-in reference-element tables of the H1-HDiv spaces at the Gauss points.
//
// Spaces (GridapMHD src/parameters.jl:436-441, :521-526): u Q2 Lagrange
// (component-major), p P1 on the cube, j Raviart-Thomas order 1, φ Q1.
// Quadrature: degree q = 5 (src/parameters.jl:381-389), i.e. 3 Gauss-Legendre
// points per direction on cells and on faces (src/parameters.jl:617-639).
#include <cmath>
#include <cstring>

#include "internal.h"

namespace gbmhd {
namespace {

const double kGx[3] = {0.5 - 0.5 * 0.7745966692414833770358531, 0.5, 0.5 + 0.5 * 0.7745966692414833770358531};
const double kGw[3] = {5.0 / 18.0, 8.0 / 18.0, 5.0 / 18.0};

double L2(int a, double t) {
  return a == 0 ? (2 * t - 1) * (t - 1) : (a == 1 ? 4 * t * (1 - t) : t * (2 * t - 1));
}
double dL2(int a, double t) { return a == 0 ? 4 * t - 3 : (a == 1 ? 4 - 8 * t : 4 * t - 1); }
double L1(int a, double t) { return a ? t : 1 - t; }
double dL1(int a) { return a ? 1.0 : -1.0; }

// RT function b: axis d, quadratic index q, linear indices l1 (axis o1), l2 (axis o2).
void rt_decode(int b, int& d, int& q, int& l1, int& l2, int& o1, int& o2) {
  d = b / 12;
  int r = b % 12;
  q = r % 3;
  l1 = (r / 3) % 2;
  l2 = (r / 3) / 2;
  o1 = d == 0 ? 1 : 0;
  o2 = d == 2 ? 1 : 2;
}

void rt_eval(int b, const double xi[3], double& val, double& div, double grad[3]) {
  int d, q, l1, l2, o1, o2;
  rt_decode(b, d, q, l1, l2, o1, o2);
  double fq = L2(q, xi[d]), f1 = L1(l1, xi[o1]), f2 = L1(l2, xi[o2]);
  val = fq * f1 * f2;
  div = dL2(q, xi[d]) * f1 * f2;
  grad[d] = div;
  grad[o1] = fq * dL1(l1) * f2;
  grad[o2] = fq * f1 * dL1(l2);
}

void q1_grads(const double xi[3], double g[8][3]) {
  for (int v = 0; v < 8; ++v) {
    int a = v & 1, b = (v >> 1) & 1, c = (v >> 2) & 1;
    g[v][0] = dL1(a) * L1(b, xi[1]) * L1(c, xi[2]);
    g[v][1] = L1(a, xi[0]) * dL1(b) * L1(c, xi[2]);
    g[v][2] = L1(a, xi[0]) * L1(b, xi[1]) * dL1(c);
  }
}

}  // namespace

void build_ref_tables(RefTables& T) {
  std::memset(&T, 0, sizeof(T));
  for (int k = 0; k < 3; ++k)
    for (int j = 0; j < 3; ++j)
      for (int i = 0; i < 3; ++i) {
        int q = i + 3 * j + 9 * k;
        double xi[3] = {kGx[i], kGx[j], kGx[k]};
        T.w[q] = kGw[i] * kGw[j] * kGw[k];
        q1_grads(xi, T.gq1[q]);
        for (int n = 0; n < 27; ++n) {
          int a = n % 3, b = (n / 3) % 3, c = n / 9;
          T.n2[q][n] = L2(a, xi[0]) * L2(b, xi[1]) * L2(c, xi[2]);
          T.g2[q][n][0] = dL2(a, xi[0]) * L2(b, xi[1]) * L2(c, xi[2]);
          T.g2[q][n][1] = L2(a, xi[0]) * dL2(b, xi[1]) * L2(c, xi[2]);
          T.g2[q][n][2] = L2(a, xi[0]) * L2(b, xi[1]) * dL2(c, xi[2]);
        }
        T.p1[q][0] = 1 - xi[0] - xi[1] - xi[2];
        T.p1[q][1] = xi[0]; T.p1[q][2] = xi[1]; T.p1[q][3] = xi[2];
        for (int v = 0; v < 8; ++v)
          T.q1[q][v] = L1(v & 1, xi[0]) * L1((v >> 1) & 1, xi[1]) * L1((v >> 2) & 1, xi[2]);
        for (int b = 0; b < 36; ++b) {
          double g[3];
          rt_eval(b, xi, T.rt[q][b], T.rtdiv[q][b], g);
        }
      }
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) T.fw[i + 3 * j] = kGw[i] * kGw[j];
  for (int f = 0; f < 6; ++f) {
    int ax = f / 2, side = f % 2;
    int o1 = ax == 0 ? 1 : 0, o2 = ax == 2 ? 1 : 2;
    for (int j = 0; j < 3; ++j)
      for (int i = 0; i < 3; ++i) {
        int t = i + 3 * j;
        double xi[3];
        xi[ax] = side; xi[o1] = kGx[i]; xi[o2] = kGx[j];
        q1_grads(xi, T.fgq1[f][t]);
        for (int b = 0; b < 36; ++b) {
          double div;
          rt_eval(b, xi, T.frt[f][t][b], div, T.frtg[f][t][b]);
        }
      }
  }
}

void build_post_tables(PostTables& T) {
  // 4-point Gauss-Legendre on [0,1]
  const double t0 = 0.3399810435848562648, t1 = 0.8611363115940525752;
  const double w0 = 0.6521451548625461427, w1 = 0.3478548451374538574;
  const double gx[4] = {0.5 - 0.5 * t1, 0.5 - 0.5 * t0, 0.5 + 0.5 * t0, 0.5 + 0.5 * t1};
  const double gw[4] = {0.5 * w1, 0.5 * w0, 0.5 * w0, 0.5 * w1};
  std::memset(&T, 0, sizeof(T));
  for (int k = 0; k < 4; ++k)
    for (int j = 0; j < 4; ++j)
      for (int i = 0; i < 4; ++i) {
        const int q = i + 4 * j + 16 * k;
        const double xi[3] = {gx[i], gx[j], gx[k]};
        T.w[q] = gw[i] * gw[j] * gw[k];
        for (int v = 0; v < 8; ++v) T.q1[q][v] = L1(v & 1, xi[0]) * L1((v >> 1) & 1, xi[1]) * L1((v >> 2) & 1, xi[2]);
        q1_grads(xi, T.gq1[q]);
        for (int n = 0; n < 27; ++n) {
          const int a = n % 3, b = (n / 3) % 3, c = n / 9;
          T.n2[q][n] = L2(a, xi[0]) * L2(b, xi[1]) * L2(c, xi[2]);
          T.g2[q][n][0] = dL2(a, xi[0]) * L2(b, xi[1]) * L2(c, xi[2]);
          T.g2[q][n][1] = L2(a, xi[0]) * dL2(b, xi[1]) * L2(c, xi[2]);
          T.g2[q][n][2] = L2(a, xi[0]) * L2(b, xi[1]) * dL2(c, xi[2]);
        }
        for (int b = 0; b < 36; ++b) {
          double div, g[3];
          rt_eval(b, xi, T.rt[q][b], div, g);
        }
      }
}

}  // namespace gbmhd
