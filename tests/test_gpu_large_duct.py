"""Mixed precision against FP64 on a duct large enough for the multi-tile solve kernels.

The smaller GPU tests have fronts whose boundary and eliminated blocks fit in one row tile
of the TMA-staged sweeps (at most 256 rows). The 24x24x4 Hunt duct at Ha = 500 with tanh
stretching has levels with up to ~1,500 boundary rows and several column chunks. Those
levels exercise:
- the fused vector gather of the forward sweep;
- the direct accumulation into x of the backward sweep;
- the multi-column transposed sweeps of the adjoint;
- the register-resident pivot kernel on levels with few fronts.

Tolerances: the mixed solution must agree with the FP64 GPU solution to 1e-8 relative L2
per field (pressure modulo a constant). The mixed adjoint gradients (dJ/dγ, dJ/dcw) must
agree with the FP64 ones to 1e-6 relative.
"""
import numpy as np
import pytest

from gbmhd.objectives import flow_rate
from helpers import gpu_context, hunt_case
from test_gpu_newton import field_rel_errors

pytestmark = pytest.mark.gpu


def test_mixed_matches_fp64_on_24x24x4_ha500(gpu_lib):
    mesh, dm, params = hunt_case(nc=(24, 24), nz=4, Ha=500.0, Re=1.0, beta_map=3.0, cw=0.1, Lz=0.2)
    ctx = gpu_context(mesh, dm, params)
    x64, rep64, rc64 = ctx.newton_solve(np.zeros(dm.ndofs), precision=0, max_newton=12, newton_rtol=1e-12,
                                        restart=200, max_linear=600, linear_rtol=1e-10)
    assert rc64 == 0, rep64
    g = flow_rate(mesh, dm, 0.1)
    dJ64, _, arep64, arc64 = ctx.adjoint(x64, g, with_cells=False, precision=0, restart=200, max_linear=600,
                                         linear_rtol=1e-9)
    assert arc64 == 0, arep64

    x32, rep32, rc32 = ctx.newton_solve(np.zeros(dm.ndofs), precision=1, max_newton=12, newton_rtol=1e-12,
                                        restart=200, max_linear=600, linear_rtol=1e-3)
    assert rc32 == 0, rep32
    assert rep32["final_residual"] <= 1e-9 * rep32["initial_residual"], rep32
    # FP32 factors precondition: the whole solve stays far from the iteration cap
    assert rep32["linear_iters"] <= 400, rep32
    errs = field_rel_errors(dm, x32, x64)
    assert max(errs.values()) <= 1e-8, errs

    dJ32, _, arep32, arc32 = ctx.adjoint(x32, g, with_cells=False, precision=1, restart=200, max_linear=600,
                                         linear_rtol=1e-9)
    assert arc32 == 0, arep32
    for k in range(2):
        assert abs(dJ32[k] - dJ64[k]) <= 1e-6 * abs(dJ64[k]), (k, dJ32[:2], dJ64[:2])
