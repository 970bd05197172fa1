// Post-processing of hunt() on the device: error and solution norms against the analytic
// Hunt solution (GridapMHD src/Applications/hunt.jl:238-260; analytical_hunt_u/j at
// :372-457), integrated with the degree-6 rule (4 Gauss points per direction).
//
// One CTA per cell, one thread per integration point.  A thread maps its point (trilinear
// geometry, FP64), forms u_h, ∇u_h and the Piola-mapped j_h from the cell's dof values,
// sums the two Fourier series (and their gradient for the H1 error) up to 2·nsums terms,
// keeping the partial sums at nsums, and contributes w·det J times the nine integrands.
// The CTA reduces its points; the host adds the per-cell sums in cell order, so the result
// does not depend on scheduling.
#include <cmath>
#include <vector>

#include "internal.h"

namespace gbmhd {
namespace {

struct HuntScalars {
  double a, l, mu, grad_pz, sigma, u_scale, j_scale, s;
  int n1, n2;  // terms of the series: k < n1 (nsums), k < n2 (2·nsums)
};

// per Fourier term k: α_k, N, r1, r2, 1/(1+exp(−2 r1)), 1/(1+exp(−2 r2)), (−1)^k
constexpr int TERM = 7;

__global__ void __launch_bounds__(NQP) k_hunt_norms(int64_t ncells, const double* __restrict__ cellX,
                                                    const int32_t* __restrict__ gidx,
                                                    const uint64_t* __restrict__ sign,
                                                    const double* __restrict__ xfull,
                                                    const PostTables* __restrict__ T,
                                                    const double* __restrict__ terms, HuntScalars hs,
                                                    double* __restrict__ partial) {
  __shared__ double X[24];
  __shared__ double v[81 + 36];
  __shared__ unsigned long long sg;
  __shared__ double red[NQP / 32][9];
  const int p = threadIdx.x, lane = p & 31, warp = p >> 5;
  for (int64_t cell = blockIdx.x; cell < ncells; cell += gridDim.x) {
    __syncthreads();
    if (p < 24) X[p] = cellX[cell * 24 + p];
    for (int a = p; a < 81; a += NQP) v[a] = xfull[gidx[cell * ND + OU + a]];
    if (p < 36) v[81 + p] = xfull[gidx[cell * ND + OJ + p]];
    if (p == 0) sg = sign ? sign[cell] : 0ull;
    __syncthreads();
    // geometry
    double J[3][3], x[3];
    for (int i = 0; i < 3; ++i) {
      x[i] = 0.0;
      for (int v8 = 0; v8 < 8; ++v8) x[i] += X[3 * v8 + i] * T->q1[p][v8];
      for (int e = 0; e < 3; ++e) {
        double t = 0.0;
        for (int v8 = 0; v8 < 8; ++v8) t += X[3 * v8 + i] * T->gq1[p][v8][e];
        J[i][e] = t;
      }
    }
    const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                       J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                       J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
    const double id = 1.0 / det;
    double Ji[3][3];  // Ji[e][i] = ∂ξ_e/∂x_i
    Ji[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) * id;
    Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
    Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
    Ji[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) * id;
    Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
    Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
    Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) * id;
    Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
    Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
    // u_h and ∇u_h (gu[i][c] = ∂_i u_c) on the mesh
    double u[3] = {0.0, 0.0, 0.0}, gu[3][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
    for (int n = 0; n < 27; ++n) {
      const double nv = T->n2[p][n];
      double G[3];
      for (int i = 0; i < 3; ++i)
        G[i] = Ji[0][i] * T->g2[p][n][0] + Ji[1][i] * T->g2[p][n][1] + Ji[2][i] * T->g2[p][n][2];
      for (int c = 0; c < 3; ++c) {
        const double val = v[c * 27 + n];
        u[c] += val * nv;
        for (int i = 0; i < 3; ++i) gu[i][c] += val * G[i];
      }
    }
    // j_h = Σ_b (±x_b) J e_d(b) rt_b / det J
    double ja[3] = {0.0, 0.0, 0.0};  // per reference axis d
    for (int b = 0; b < 36; ++b) {
      const double sgb = ((sg >> b) & 1ull) ? -1.0 : 1.0;
      ja[b / 12] += sgb * v[81 + b] * T->rt[p][b];
    }
    double jh[3];
    for (int i = 0; i < 3; ++i) jh[i] = (J[i][0] * ja[0] + J[i][1] * ja[1] + J[i][2] * ja[2]) * id;
    // the analytic fields at the physical point
    const double xi = hs.s * x[0] / hs.a, eta = hs.s * x[1] / hs.a;
    const bool inside = !(xi > 1.0 || xi < -1.0 || eta > 1.0 || eta < -1.0);
    double V[2] = {0.0, 0.0}, Vx[2] = {0.0, 0.0}, Vy[2] = {0.0, 0.0}, Hdx[2] = {0.0, 0.0}, Hdy[2] = {0.0, 0.0};
    if (inside) {
      double sV = 0.0, sVx = 0.0, sVy = 0.0, sHdx = 0.0, sHdy = 0.0;
      for (int k = 0; k < hs.n2; ++k) {
        const double* t = terms + TERM * k;
        const double ak = t[0], N = t[1], r1 = t[2], r2 = t[3], d1 = t[4], d2 = t[5], sk = t[6];
        const double e11 = exp(-r1 * (1.0 - eta)), e12 = exp(-r1 * (1.0 + eta));
        const double e21 = exp(-r2 * (1.0 - eta)), e22 = exp(-r2 * (1.0 + eta));
        double sn, cs;
        sincos(ak * xi, &sn, &cs);
        const double V2 = (r2 / N) * (e11 + e12) * d1, V3 = (r1 / N) * (e21 + e22) * d2;
        const double V2e = (r2 / N) * r1 * (e11 - e12) * d1, V3e = (r1 / N) * r2 * (e21 - e22) * d2;  // d/dη
        const double cu = 2.0 * sk / (hs.l * ak * ak * ak);
        sV += cu * cs * (1.0 - V2 - V3);
        sVx += -cu * ak * sn * (1.0 - V2 - V3);  // d/dξ
        sVy += cu * cs * (-V2e - V3e);           // d/dη
        const double H2 = (r2 / N) * (e11 - e12) * d1, H3 = (r1 / N) * (e21 - e22) * d2;
        const double H2y = (r2 / N) * (e11 + e12) * (r1 / hs.a) * d1, H3y = (r1 / N) * (e21 + e22) * (r2 / hs.a) * d2;
        sHdx += -2.0 * sk * sn / (hs.a * hs.l * ak * ak) * (H2 - H3);
        sHdy += cu * cs * (H2y - H3y);
        if (k + 1 == hs.n1) { V[0] = sV; Vx[0] = sVx; Vy[0] = sVy; Hdx[0] = sHdx; Hdy[0] = sHdy; }
      }
      V[1] = sV; Vx[1] = sVx; Vy[1] = sVy; Hdx[1] = sHdx; Hdy[1] = sHdy;
    }
    const double cu_ = (-hs.grad_pz) * hs.a * hs.a / hs.mu;              // u_z = V·cu_
    const double cj_ = hs.a * hs.a * sqrt(hs.sigma) / sqrt(hs.mu) * (-hs.grad_pz);
    const double wd = T->w[p] * det * hs.s * hs.s * hs.s;
    double uhp[3], guhp[3][3], jhp[3];
    for (int c = 0; c < 3; ++c) { uhp[c] = hs.u_scale * u[c]; jhp[c] = hs.j_scale * jh[c]; }
    for (int i = 0; i < 3; ++i)
      for (int c = 0; c < 3; ++c) guhp[i][c] = hs.u_scale * gu[i][c] / hs.s;
    double acc[9];
    for (int r = 0; r < 2; ++r) {
      const double uz = V[r] * cu_, duzx = Vx[r] * cu_ / hs.a, duzy = Vy[r] * cu_ / hs.a;
      const double jx = cj_ * Hdy[r], jy = -cj_ * Hdx[r];
      const double eu[3] = {-uhp[0], -uhp[1], uz - uhp[2]};
      double ge = 0.0;  // |∇u_a − ∇u_h|², ∇u_a has ∂_x u_z and ∂_y u_z only
      for (int i = 0; i < 3; ++i)
        for (int c = 0; c < 3; ++c) {
          const double ga = (c == 2 && i == 0) ? duzx : (c == 2 && i == 1) ? duzy : 0.0;
          const double d = ga - guhp[i][c];
          ge += d * d;
        }
      const double e2 = eu[0] * eu[0] + eu[1] * eu[1] + eu[2] * eu[2];
      const double ej[3] = {jx - jhp[0], jy - jhp[1], -jhp[2]};
      acc[3 * r + 0] = wd * (ge + e2);
      acc[3 * r + 1] = wd * e2;
      acc[3 * r + 2] = wd * (ej[0] * ej[0] + ej[1] * ej[1] + ej[2] * ej[2]);
    }
    double u2 = 0.0, g2 = 0.0;
    for (int c = 0; c < 3; ++c) {
      u2 += uhp[c] * uhp[c];
      for (int i = 0; i < 3; ++i) g2 += guhp[i][c] * guhp[i][c];
    }
    acc[6] = wd * (g2 + u2);
    acc[7] = wd * u2;
    acc[8] = wd * (jhp[0] * jhp[0] + jhp[1] * jhp[1] + jhp[2] * jhp[2]);
    for (int k = 0; k < 9; ++k) {
      double t = acc[k];
      for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
      if (lane == 0) red[warp][k] = t;
    }
    __syncthreads();
    if (p < 9) {
      double t = 0.0;
      for (int w = 0; w < NQP / 32; ++w) t += red[w][p];
      partial[cell * 9 + p] = t;
    }
  }
}

}  // namespace
}  // namespace gbmhd

using namespace gbmhd;

extern "C" int gbmhd_hunt_errors(gbmhd_ctx* ctx, const double* x_free, const gbmhd_hunt_analytic* an, double* out) {
  if (!ctx) return -1;
  if (!x_free || !an || !out) { ctx->err = "hunt_errors: NULL argument"; return -1; }
  if (!(an->L > 0.0) || !(an->mu > 0.0) || !(an->sigma >= 0.0) || !(an->length_scale > 0.0) || an->nsums < 0 ||
      an->nsums > 100000 || !std::isfinite(an->Ha) || !std::isfinite(an->grad_pz) || !std::isfinite(an->u_scale) ||
      !std::isfinite(an->j_scale)) {
    ctx->err = "hunt_errors: invalid analytic parameters";
    return -1;
  }
  if (!ctx->d_posttab) {
    PostTables h;
    build_post_tables(h);
    GB_CUDA(cudaMalloc(&ctx->d_posttab, sizeof(PostTables)));
    GB_CUDA(cudaMemcpy(ctx->d_posttab, &h, sizeof(PostTables), cudaMemcpyHostToDevice));
  }
  // per-term constants of both series (src/Applications/hunt.jl:390-395, :432-437); l = b/a = 1
  const int n2 = 2 * an->nsums + 1;
  std::vector<double> terms((size_t)TERM * n2);
  for (int k = 0; k < n2; ++k) {
    const double ak = (k + 0.5) * 3.14159265358979323846;
    const double N = std::sqrt(an->Ha * an->Ha + 4.0 * ak * ak);
    const double r1 = 0.5 * (an->Ha + N), r2 = 0.5 * (-an->Ha + N);
    double* t = terms.data() + (size_t)TERM * k;
    t[0] = ak; t[1] = N; t[2] = r1; t[3] = r2;
    t[4] = 1.0 / (1.0 + std::exp(-2.0 * r1));
    t[5] = 1.0 / (1.0 + std::exp(-2.0 * r2));
    t[6] = (k % 2) ? -1.0 : 1.0;
  }
  double *d_terms = nullptr, *d_part = nullptr;
  GB_CUDA(cudaMallocAsync(&d_terms, sizeof(double) * terms.size(), ctx->stream));
  GB_CUDA(cudaMallocAsync(&d_part, sizeof(double) * 9 * std::max<int64_t>(ctx->ncells, 1), ctx->stream));
  GB_CUDA(cudaMemcpyAsync(d_terms, terms.data(), sizeof(double) * terms.size(), cudaMemcpyHostToDevice, ctx->stream));
  GB_CUDA(cudaMemcpyAsync(ctx->d_xfull, x_free, sizeof(double) * ctx->ndofs, cudaMemcpyHostToDevice, ctx->stream));
  HuntScalars hs{an->L, 1.0, an->mu, an->grad_pz, an->sigma, an->u_scale, an->j_scale, an->length_scale,
                 an->nsums + 1, n2};
  const int64_t grid = std::max<int64_t>(1, std::min<int64_t>(ctx->ncells, (int64_t)ctx->num_sms * 32));
  if (ctx->ncells > 0) {
    k_hunt_norms<<<(unsigned)grid, NQP, 0, ctx->stream>>>(ctx->ncells, ctx->d_cellX, ctx->d_gidx, ctx->d_sign,
                                                         ctx->d_xfull, reinterpret_cast<const PostTables*>(ctx->d_posttab),
                                                         d_terms, hs, d_part);
    gbmhd::count_launch();
    GB_CUDA(cudaGetLastError());
  }
  std::vector<double> part((size_t)9 * ctx->ncells);
  if (ctx->ncells > 0)
    GB_CUDA(cudaMemcpyAsync(part.data(), d_part, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, ctx->stream));
  GB_CUDA(cudaFreeAsync(d_terms, ctx->stream));
  GB_CUDA(cudaFreeAsync(d_part, ctx->stream));
  GB_CUDA(cudaStreamSynchronize(ctx->stream));
  double sum[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int64_t c = 0; c < ctx->ncells; ++c)
    for (int k = 0; k < 9; ++k) sum[k] += part[(size_t)9 * c + k];
  // order of out: eu_h1, eu_l2, ej_l2, eu_ref_h1, eu_ref_l2, ej_ref_l2, uh_h1, uh_l2, jh_l2
  for (int k = 0; k < 9; ++k) out[k] = std::sqrt(std::max(0.0, sum[k]));
  return 0;
}

// ---------------------------------------------------------------- fields at the Q2 nodes (VTK)
// The solution at the 27 nodes ξ ∈ {0, ½, 1}³ of every cell, for a field file of order 2 like
// the post-processing of hunt() writes (src/Applications/hunt.jl:263-273): per node the
// physical point, u_h, p_h, j_h (contravariant Piola map), φ_h, div u_h and div j_h.  u_h is
// nodal (its dof values), the others are evaluated from the closed-form reference bases.
namespace gbmhd {
namespace {

constexpr int NODE_FIELDS = 13;

__device__ __forceinline__ double l2v(int a, double t) {
  return a == 0 ? (2 * t - 1) * (t - 1) : (a == 1 ? 4 * t * (1 - t) : t * (2 * t - 1));
}
__device__ __forceinline__ double l2d(int a, double t) { return a == 0 ? 4 * t - 3 : (a == 1 ? 4 - 8 * t : 4 * t - 1); }
__device__ __forceinline__ double l1v(int a, double t) { return a ? t : 1 - t; }
__device__ __forceinline__ double l1d(int a) { return a ? 1.0 : -1.0; }

__global__ void __launch_bounds__(32) k_node_fields(int64_t ncells, const double* __restrict__ cellX,
                                                    const int32_t* __restrict__ gidx,
                                                    const uint64_t* __restrict__ sign,
                                                    const double* __restrict__ xfull, double* __restrict__ out) {
  __shared__ double X[24], v[ND];
  __shared__ unsigned long long sg;
  const int t = threadIdx.x;
  for (int64_t cell = blockIdx.x; cell < ncells; cell += gridDim.x) {
    __syncwarp();
    if (t < 24) X[t] = cellX[cell * 24 + t];
    for (int a = t; a < ND; a += 32) v[a] = xfull[gidx[cell * ND + a]];
    if (t == 0) sg = sign ? sign[cell] : 0ull;
    __syncwarp();
    if (t < 27) {
      const int na = t % 3, nb = (t / 3) % 3, nc = t / 9;
      const double xi[3] = {0.5 * na, 0.5 * nb, 0.5 * nc};
      // trilinear geometry
      double x[3] = {0, 0, 0}, J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
      for (int vv = 0; vv < 8; ++vv) {
        const int a = vv & 1, b = (vv >> 1) & 1, c = (vv >> 2) & 1;
        const double f = l1v(a, xi[0]) * l1v(b, xi[1]) * l1v(c, xi[2]);
        const double g[3] = {l1d(a) * l1v(b, xi[1]) * l1v(c, xi[2]), l1v(a, xi[0]) * l1d(b) * l1v(c, xi[2]),
                             l1v(a, xi[0]) * l1v(b, xi[1]) * l1d(c)};
        for (int i = 0; i < 3; ++i) {
          x[i] += X[3 * vv + i] * f;
          for (int e = 0; e < 3; ++e) J[i][e] += X[3 * vv + i] * g[e];
        }
      }
      const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                         J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                         J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
      const double id = 1.0 / det;
      double Ji[3][3];  // Ji[e][i] = ∂ξ_e/∂x_i
      Ji[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) * id;
      Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
      Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
      Ji[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) * id;
      Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
      Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
      Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) * id;
      Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
      Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
      // div u_h: Σ_n Σ_c u_{c,n} ∂_c N_n
      double divu = 0.0;
      for (int n = 0; n < 27; ++n) {
        const int a = n % 3, b = (n / 3) % 3, c = n / 9;
        const double g[3] = {l2d(a, xi[0]) * l2v(b, xi[1]) * l2v(c, xi[2]),
                             l2v(a, xi[0]) * l2d(b, xi[1]) * l2v(c, xi[2]),
                             l2v(a, xi[0]) * l2v(b, xi[1]) * l2d(c, xi[2])};
        for (int cc = 0; cc < 3; ++cc)
          divu += v[OU + cc * 27 + n] * (Ji[0][cc] * g[0] + Ji[1][cc] * g[1] + Ji[2][cc] * g[2]);
      }
      // p_h (P1: 1 − ξ1 − ξ2 − ξ3, ξ1, ξ2, ξ3) and φ_h (Q1 at the vertices)
      const double p = v[OP] * (1 - xi[0] - xi[1] - xi[2]) + v[OP + 1] * xi[0] + v[OP + 2] * xi[1] + v[OP + 3] * xi[2];
      double phi = 0.0;
      for (int vv = 0; vv < 8; ++vv)
        phi += v[OPHI + vv] * l1v(vv & 1, xi[0]) * l1v((vv >> 1) & 1, xi[1]) * l1v((vv >> 2) & 1, xi[2]);
      // j_h = J ĵ / det J, div j_h = div ĵ / det J (RT: b = d·12 + q + 3(l1 + 2 l2))
      double ja[3] = {0, 0, 0}, dj = 0.0;
      for (int b = 0; b < 36; ++b) {
        const int d = b / 12, r = b % 12, q = r % 3, la = (r / 3) % 2, lb = (r / 3) / 2;
        const int o1 = d == 0 ? 1 : 0, o2 = d == 2 ? 1 : 2;
        const double sgb = ((sg >> b) & 1ull) ? -1.0 : 1.0;
        const double w = sgb * v[OJ + b] * l1v(la, xi[o1]) * l1v(lb, xi[o2]);
        ja[d] += w * l2v(q, xi[d]);
        dj += w * l2d(q, xi[d]);
      }
      double* o = out + ((size_t)cell * 27 + t) * NODE_FIELDS;
      o[0] = x[0]; o[1] = x[1]; o[2] = x[2];
      o[3] = v[OU + na + 3 * nb + 9 * nc]; o[4] = v[OU + 27 + na + 3 * nb + 9 * nc]; o[5] = v[OU + 54 + na + 3 * nb + 9 * nc];
      o[6] = p;
      for (int i = 0; i < 3; ++i) o[7 + i] = (J[i][0] * ja[0] + J[i][1] * ja[1] + J[i][2] * ja[2]) * id;
      o[10] = phi;
      o[11] = divu;
      o[12] = dj * id;
    }
  }
}

}  // namespace
}  // namespace gbmhd

extern "C" int gbmhd_node_fields(gbmhd_ctx* ctx, const double* x_free, double* out) {
  if (!ctx) return -1;
  if (!x_free || !out) { ctx->err = "node_fields: NULL argument"; return -1; }
  const size_t nout = (size_t)ctx->ncells * 27 * gbmhd::NODE_FIELDS;
  double* d_out = nullptr;
  GB_CUDA(cudaMallocAsync(&d_out, sizeof(double) * std::max<size_t>(nout, 1), ctx->stream));
  GB_CUDA(cudaMemcpyAsync(ctx->d_xfull, x_free, sizeof(double) * ctx->ndofs, cudaMemcpyHostToDevice, ctx->stream));
  if (ctx->ncells > 0) {
    const int64_t grid = std::max<int64_t>(1, std::min<int64_t>(ctx->ncells, (int64_t)ctx->num_sms * 64));
    gbmhd::k_node_fields<<<(unsigned)grid, 32, 0, ctx->stream>>>(ctx->ncells, ctx->d_cellX, ctx->d_gidx, ctx->d_sign,
                                                                ctx->d_xfull, d_out);
    gbmhd::count_launch();
    GB_CUDA(cudaGetLastError());
  }
  GB_CUDA(cudaMemcpyAsync(out, d_out, sizeof(double) * nout, cudaMemcpyDeviceToHost, ctx->stream));
  GB_CUDA(cudaFreeAsync(d_out, ctx->stream));
  GB_CUDA(cudaStreamSynchronize(ctx->stream));
  return 0;
}
