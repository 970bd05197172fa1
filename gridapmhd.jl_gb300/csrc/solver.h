// Linear/nonlinear solver interface of libgbmhd (solver.cu).
#pragma once
#include "internal.h"

void solver_destroy(gbmhd_ctx* ctx);
