// Newton driver, FGMRES and block preconditioner (placeholder until the solver lands).
#include "solver.h"

struct Solver {};

void solver_destroy(gbmhd_ctx* ctx) {
  delete ctx->solver;
  ctx->solver = nullptr;
}

extern "C" int gbmhd_newton_solve_device(gbmhd_ctx* ctx, double*, const gbmhd_solve_opts*, gbmhd_report*) {
  if (ctx) ctx->err = "solver not built";
  return -1;
}
extern "C" int gbmhd_newton_solve(gbmhd_ctx* ctx, double*, const gbmhd_solve_opts*, gbmhd_report*) {
  if (ctx) ctx->err = "solver not built";
  return -1;
}
extern "C" int gbmhd_adjoint(gbmhd_ctx* ctx, const double*, const gbmhd_objective*, const gbmhd_solve_opts*,
                             double*, int64_t, double*, gbmhd_report*) {
  if (ctx) ctx->err = "solver not built";
  return -1;
}
