// C-ABI entry points of libgbmhd (declared in include/gbmhd.h).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstring>
#include <string>
#include <vector>

#include "internal.h"
#include "solver.h"

using namespace gbmhd;

static thread_local std::string g_create_err;
static std::atomic<int64_t> g_launches{0}, g_gemms{0};

namespace gbmhd {
void count_launch(int64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
int64_t launch_count() { return g_launches.load(std::memory_order_relaxed); }
void count_gemm(int64_t n) { g_gemms.fetch_add(n, std::memory_order_relaxed); }
}  // namespace gbmhd

extern "C" int gbmhd_counters(int64_t* kernel_launches, int64_t* gemm_calls) {
  if (kernel_launches) *kernel_launches = g_launches.load();
  if (gemm_calls) *gemm_calls = g_gemms.load();
  return 0;
}

extern "C" int gbmhd_version(void) { return 1; }

extern "C" const char* gbmhd_last_error(const gbmhd_ctx* ctx) {
  return ctx ? ctx->err.c_str() : g_create_err.c_str();
}

static void free_ctx(gbmhd_ctx* c) {
  if (!c) return;
  solver_destroy(c);
  void* ptrs[] = {c->d_cellX, c->d_gidx, c->d_row, c->d_sign, c->d_xfull, c->d_fcell, c->d_fcellid,
                  c->d_flface, c->d_fprm, c->d_tab64, c->d_tab32, c->d_ftab, c->d_rowptr, c->d_col,
                  c->d_class, c->d_offtab, c->d_val64, c->d_val32, c->d_r, c->d_xtmp, c->d_posttab, c->d_val64s};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

extern "C" void gbmhd_destroy(gbmhd_ctx* ctx) { free_ctx(ctx); }

extern "C" void* gbmhd_get_stream(const gbmhd_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

static int set_params_impl(gbmhd_ctx* ctx, const gbmhd_params* p, bool first) {
  if (!p) { ctx->err = "params is NULL"; return -1; }
  const double sc[] = {p->alpha, p->beta, p->gamma, p->sigma, p->B[0], p->B[1], p->B[2], p->f[0], p->f[1],
                       p->f[2], p->g[0], p->g[1], p->g[2], p->zeta_u, p->zeta_j};
  for (double v : sc)
    if (!std::isfinite(v)) { ctx->err = "non-finite physical parameter"; return -1; }
  if (p->convection < 0 || p->convection > 2) { ctx->err = "convection must be 0, 1 or 2"; return -1; }
  DevParams& d = ctx->prm;
  d.alpha = p->alpha; d.beta = p->beta; d.gamma = p->gamma; d.sigma = p->sigma;
  for (int i = 0; i < 3; ++i) { d.B[i] = p->B[i]; d.f[i] = p->f[i]; d.g[i] = p->g[i]; }
  d.zeta_u = p->zeta_u; d.zeta_j = p->zeta_j;
  d.convection = p->convection;
  d.has_fcell = p->f_cell != nullptr;
  if (p->f_cell) {
    for (int64_t i = 0; i < 3 * ctx->ncells; ++i)
      if (!std::isfinite(p->f_cell[i])) { ctx->err = "non-finite cellwise body force"; return -1; }
    if (!ctx->d_fcell) GB_CUDA(cudaMalloc(&ctx->d_fcell, sizeof(double) * 3 * ctx->ncells));
    GB_CUDA(cudaMemcpy(ctx->d_fcell, p->f_cell, sizeof(double) * 3 * ctx->ncells, cudaMemcpyHostToDevice));
  }
  // facets
  if (p->nfacets < 0) { ctx->err = "nfacets < 0"; return -1; }
  if (!first && p->nfacets != ctx->nfacets) {
    if (ctx->d_fcellid) cudaFree(ctx->d_fcellid);
    if (ctx->d_flface) cudaFree(ctx->d_flface);
    if (ctx->d_fprm) cudaFree(ctx->d_fprm);
    ctx->d_fcellid = nullptr; ctx->d_flface = nullptr; ctx->d_fprm = nullptr;
  }
  ctx->nfacets = p->nfacets;
  if (p->nfacets > 0) {
    if (!p->facet_cell || !p->facet_lface) { ctx->err = "facet arrays are NULL"; return -1; }
    std::vector<double> prm(4 * p->nfacets);
    for (int64_t e = 0; e < p->nfacets; ++e) {
      if (p->facet_cell[e] < 0 || p->facet_cell[e] >= ctx->ncells) { ctx->err = "facet cell out of range"; return -1; }
      if (p->facet_lface[e] < 0 || p->facet_lface[e] > 5) { ctx->err = "facet local face out of range"; return -1; }
      prm[4 * e + 0] = p->facet_tau ? p->facet_tau[e] : 0.0;
      prm[4 * e + 1] = p->facet_cw ? p->facet_cw[e] : 0.0;
      prm[4 * e + 2] = p->facet_jw ? p->facet_jw[e] : 0.0;
      prm[4 * e + 3] = p->facet_phi0 ? p->facet_phi0[e] : 0.0;
      for (int k = 0; k < 4; ++k)
        if (!std::isfinite(prm[4 * e + k])) { ctx->err = "non-finite facet parameter"; return -1; }
    }
    if (!ctx->d_fcellid) GB_CUDA(cudaMalloc(&ctx->d_fcellid, sizeof(int32_t) * p->nfacets));
    if (!ctx->d_flface) GB_CUDA(cudaMalloc(&ctx->d_flface, sizeof(int8_t) * p->nfacets));
    if (!ctx->d_fprm) GB_CUDA(cudaMalloc(&ctx->d_fprm, sizeof(double) * 4 * p->nfacets));
    GB_CUDA(cudaMemcpy(ctx->d_fcellid, p->facet_cell, sizeof(int32_t) * p->nfacets, cudaMemcpyHostToDevice));
    GB_CUDA(cudaMemcpy(ctx->d_flface, p->facet_lface, sizeof(int8_t) * p->nfacets, cudaMemcpyHostToDevice));
    GB_CUDA(cudaMemcpy(ctx->d_fprm, prm.data(), sizeof(double) * 4 * p->nfacets, cudaMemcpyHostToDevice));
  }
  return 0;
}

extern "C" int gbmhd_set_params(gbmhd_ctx* ctx, const gbmhd_params* p) {
  if (!ctx) return -1;
  GB_CUDA(cudaStreamSynchronize(ctx->stream));  // no kernel of this context may read the old values
  ctx->params_gen++;
  return set_params_impl(ctx, p, false);
}

extern "C" int gbmhd_create(gbmhd_ctx** out, const gbmhd_mesh* mesh, const gbmhd_dofmap* dofs,
                            const gbmhd_params* params) {
  g_create_err.clear();
  if (!out || !mesh || !dofs || !params) { g_create_err = "NULL argument"; return -1; }
  *out = nullptr;
  if (mesh->ncells <= 0 || !mesh->cell_coords) { g_create_err = "mesh has no cells"; return -1; }
  if (!dofs->cell_dofs) { g_create_err = "cell_dofs is NULL"; return -1; }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    g_create_err = "no CUDA device available";
    return -2;
  }
  gbmhd_ctx* ctx = new gbmhd_ctx();
  auto fail = [&](int rc) {
    g_create_err = ctx->err;
    free_ctx(ctx);
    return rc;
  };
  cudaGetDevice(&ctx->device);
  cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, ctx->device);
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
    ctx->err = "cudaStreamCreate failed";
    return fail(-2);
  }
  const int64_t nc = mesh->ncells;
  ctx->ncells = nc;
  for (int f = 0; f < 4; ++f) {
    if (dofs->nfree[f] < 0 || dofs->ndir[f] < 0) { ctx->err = "negative dof count"; return fail(-1); }
    ctx->nfree[f] = dofs->nfree[f];
    ctx->ndir[f] = dofs->ndir[f];
  }
  ctx->offs[0] = 0;
  for (int f = 1; f < 4; ++f) ctx->offs[f] = ctx->offs[f - 1] + ctx->nfree[f - 1];
  ctx->ndofs = ctx->offs[3] + ctx->nfree[3];
  if (ctx->ndofs >= (int64_t)1 << 31) { ctx->err = "more than 2^31 dofs"; return fail(-1); }
  int64_t doffs[4];
  doffs[0] = ctx->ndofs;
  for (int f = 1; f < 4; ++f) doffs[f] = doffs[f - 1] + ctx->ndir[f - 1];
  ctx->nfull = doffs[3] + ctx->ndir[3];
  for (int i = 0; i < 24 * nc; ++i)
    if (!std::isfinite(mesh->cell_coords[i])) { ctx->err = "non-finite cell coordinate"; return fail(-1); }
  // per-cell rows and value indices
  std::vector<int32_t> row(nc * ND), gidx(nc * ND);
  for (int64_t c = 0; c < nc; ++c)
    for (int a = 0; a < ND; ++a) {
      const int f = a < OP ? 0 : (a < OJ ? 1 : (a < OPHI ? 2 : 3));
      const int32_t id = dofs->cell_dofs[c * ND + a];
      if (id >= 0) {
        if (id >= ctx->nfree[f]) { ctx->err = "free dof id out of range"; return fail(-1); }
        row[c * ND + a] = (int32_t)(ctx->offs[f] + id);
        gidx[c * ND + a] = (int32_t)(ctx->offs[f] + id);
      } else {
        const int64_t d = -(int64_t)id - 1;
        if (d >= ctx->ndir[f]) { ctx->err = "Dirichlet dof id out of range"; return fail(-1); }
        row[c * ND + a] = -1;
        gidx[c * ND + a] = (int32_t)(doffs[f] + d);
      }
    }
  std::vector<double> xfull(ctx->nfull, 0.0);
  for (int f = 0; f < 4; ++f)
    if (dofs->dir_values[f])
      for (int64_t d = 0; d < ctx->ndir[f]; ++d) {
        if (!std::isfinite(dofs->dir_values[f][d])) { ctx->err = "non-finite Dirichlet value"; return fail(-1); }
        xfull[doffs[f] + d] = dofs->dir_values[f][d];
      }
  std::vector<uint64_t> sign;
  if (dofs->cell_sign_j) {
    sign.assign(nc, 0);
    for (int64_t c = 0; c < nc; ++c)
      for (int b = 0; b < 36; ++b) {
        int8_t s = dofs->cell_sign_j[c * 36 + b];
        if (s != 1 && s != -1) { ctx->err = "RT sign must be +1 or -1"; return fail(-1); }
        if (s < 0) sign[c] |= (1ull << b);
      }
  }
  Pattern P;
  std::string perr = build_pattern(nc, ctx->ndofs, row.data(), P);
  if (!perr.empty()) { ctx->err = perr; return fail(-1); }
  ctx->nnz = P.nnz;
  ctx->nclass = P.nclass;
  ctx->h_cell_row = row;
  ctx->h_cellX.assign(mesh->cell_coords, mesh->cell_coords + 24 * nc);
#define ALLOC_COPY(dst, src, bytes)                                                 \
  do {                                                                              \
    cudaError_t e_ = cudaMalloc((void**)&(dst), (bytes));                           \
    if (e_ == cudaSuccess) e_ = cudaMemcpy((dst), (src), (bytes), cudaMemcpyHostToDevice); \
    if (e_ != cudaSuccess) { ctx->err = std::string("device allocation: ") + cudaGetErrorString(e_); return fail(-2); } \
  } while (0)
  ALLOC_COPY(ctx->d_cellX, mesh->cell_coords, sizeof(double) * 24 * nc);
  ALLOC_COPY(ctx->d_gidx, gidx.data(), sizeof(int32_t) * ND * nc);
  ALLOC_COPY(ctx->d_row, row.data(), sizeof(int32_t) * ND * nc);
  if (!sign.empty()) ALLOC_COPY(ctx->d_sign, sign.data(), sizeof(uint64_t) * nc);
  ALLOC_COPY(ctx->d_xfull, xfull.data(), sizeof(double) * std::max<int64_t>(ctx->nfull, 1));
  ALLOC_COPY(ctx->d_rowptr, P.rowptr.data(), sizeof(int64_t) * (ctx->ndofs + 1));
  ALLOC_COPY(ctx->d_col, P.col.data(), sizeof(int32_t) * std::max<int64_t>(P.nnz, 1));
  ALLOC_COPY(ctx->d_class, P.cell_class.data(), sizeof(int32_t) * nc);
  ALLOC_COPY(ctx->d_offtab, P.offtab.data(), sizeof(uint16_t) * P.offtab.size());
#undef ALLOC_COPY
  ctx->h_rowptr.swap(P.rowptr);
  ctx->h_col.swap(P.col);
  if (cudaMalloc(&ctx->d_r, sizeof(double) * std::max<int64_t>(ctx->ndofs, 1)) != cudaSuccess ||
      cudaMalloc(&ctx->d_xtmp, sizeof(double) * std::max<int64_t>(ctx->ndofs, 1)) != cudaSuccess) {
    ctx->err = "device allocation of work vectors failed";
    return fail(-2);
  }
  int rc = gb_upload_tables(ctx);
  if (rc) return fail(rc);
  rc = set_params_impl(ctx, params, true);
  if (rc) return fail(rc);
  *out = ctx;
  return 0;
}

extern "C" int gbmhd_sizes(const gbmhd_ctx* ctx, int64_t* ndofs, int64_t* nnz, int64_t* ncells) {
  if (!ctx) return -1;
  if (ndofs) *ndofs = ctx->ndofs;
  if (nnz) *nnz = ctx->nnz;
  if (ncells) *ncells = ctx->ncells;
  return 0;
}

static int ensure_values(gbmhd_ctx* ctx, int precision) {
  if (precision == GBMHD_MIXED) {
    if (!ctx->d_val32) GB_CUDA(cudaMalloc(&ctx->d_val32, sizeof(float) * std::max<int64_t>(ctx->nnz, 1)));
  } else {
    if (!ctx->d_val64) GB_CUDA(cudaMalloc(&ctx->d_val64, sizeof(double) * std::max<int64_t>(ctx->nnz, 1)));
  }
  return 0;
}

extern "C" int gbmhd_assemble_device(gbmhd_ctx* ctx, const double* d_x, double* d_r, int32_t want_jacobian,
                                     int32_t precision) {
  if (!ctx) return -1;
  if (!d_x) { ctx->err = "x is NULL"; return -1; }
  if (precision != GBMHD_FP64 && precision != GBMHD_MIXED) { ctx->err = "unknown precision"; return -1; }
  if (want_jacobian) {
    int rc = ensure_values(ctx, precision);
    if (rc) return rc;
  }
  int rc = gb_assemble_device(ctx, d_x, d_r, want_jacobian, precision);
  if (rc) return rc;
  return 0;
}

extern "C" int gbmhd_assemble(gbmhd_ctx* ctx, const double* x, double* r_out, int32_t want_jacobian,
                              int32_t precision) {
  if (!ctx) return -1;
  if (!x) { ctx->err = "x is NULL"; return -1; }
  GB_CUDA(cudaMemcpyAsync(ctx->d_xtmp, x, sizeof(double) * ctx->ndofs, cudaMemcpyHostToDevice, ctx->stream));
  int rc = gbmhd_assemble_device(ctx, ctx->d_xtmp, r_out ? ctx->d_r : nullptr, want_jacobian, precision);
  if (rc) return rc;
  if (r_out)
    GB_CUDA(cudaMemcpyAsync(r_out, ctx->d_r, sizeof(double) * ctx->ndofs, cudaMemcpyDeviceToHost, ctx->stream));
  GB_CUDA(cudaStreamSynchronize(ctx->stream));
  return 0;
}

extern "C" int gbmhd_get_csr(gbmhd_ctx* ctx, int64_t* rowptr, int32_t* col, double* val) {
  if (!ctx) return -1;
  GB_CUDA(cudaStreamSynchronize(ctx->stream));
  if (rowptr) GB_CUDA(cudaMemcpy(rowptr, ctx->d_rowptr, sizeof(int64_t) * (ctx->ndofs + 1), cudaMemcpyDeviceToHost));
  if (col) GB_CUDA(cudaMemcpy(col, ctx->d_col, sizeof(int32_t) * ctx->nnz, cudaMemcpyDeviceToHost));
  if (val) {
    if (ctx->jac_precision == GBMHD_FP64) {
      GB_CUDA(cudaMemcpy(val, ctx->d_val64, sizeof(double) * ctx->nnz, cudaMemcpyDeviceToHost));
    } else if (ctx->jac_precision == GBMHD_MIXED) {
      std::vector<float> tmp(ctx->nnz);
      GB_CUDA(cudaMemcpy(tmp.data(), ctx->d_val32, sizeof(float) * ctx->nnz, cudaMemcpyDeviceToHost));
      for (int64_t i = 0; i < ctx->nnz; ++i) val[i] = tmp[i];
    } else {
      ctx->err = "no Jacobian has been assembled";
      return -1;
    }
  }
  return 0;
}
