"""GPU discrete adjoint against the oracle's adjoint (direct solves with the reference-restated
assembly) and against central finite differences of the GPU Newton solve."""
import numpy as np
import pytest

from adjoint_ref import oracle_adjoint
from gbmhd.objectives import flow_rate
from helpers import gpu_context, hunt_case, oracle_problem
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _case():
    rng = np.random.default_rng(0)
    mesh, dm, params = hunt_case(nc=(6, 6), nz=4, Ha=20.0, Re=10.0, beta_map=2.5, cw=0.1, Lz=0.2)
    fz = rng.uniform(0.9, 1.1, mesh.ncells)
    params["f_cell"] = np.stack([0 * fz, 0 * fz, fz], 1)
    return mesh, dm, params


@pytest.mark.parametrize("precision", [0, 1])
def test_adjoint_matches_oracle(gpu_lib, precision):
    mesh, dm, params = _case()
    g = flow_rate(mesh, dm, 0.1)
    prob = oracle_problem(mesh, dm, params)
    xref, _ = O.newton_direct(prob, np.zeros(dm.ndofs), gauge=[dm.offsets["p"]], rtol=1e-14, maxiter=10)
    dgam, dcw, dfz, _ = oracle_adjoint(prob, dm, xref, g, [dm.offsets["p"]])
    ctx = gpu_context(mesh, dm, params)
    # the FP64 residual of this case bottoms out near 1e-12 (assembly round-off), so the
    # absolute stop sits just above it
    x, rep, rc = ctx.newton_solve(np.zeros(dm.ndofs), precision=precision, max_newton=12, newton_rtol=1e-12,
                                  newton_atol=1e-11, restart=40, max_linear=400,
                                  linear_rtol=1e-4 if precision else 1e-8)
    assert rc == 0, rep
    out, lam, arep, arc = ctx.adjoint(x, g, with_cells=True, precision=precision, restart=40, max_linear=400,
                                      linear_rtol=1e-10)
    assert arc == 0, arep
    assert abs(out[0] - dgam) <= 1e-6 * abs(dgam)
    assert abs(out[1] - dcw) <= 1e-6 * abs(dcw)
    assert np.linalg.norm(out[4:] - dfz) <= 1e-6 * np.linalg.norm(dfz)


def test_adjoint_matches_gpu_finite_differences(gpu_lib):
    mesh, dm, params = _case()
    g = flow_rate(mesh, dm, 0.1)
    ctx = gpu_context(mesh, dm, params)
    opts = dict(precision=0, max_newton=12, newton_rtol=1e-13, newton_atol=1e-14, restart=40, max_linear=400,
                linear_rtol=1e-10)
    x, rep, rc = ctx.newton_solve(np.zeros(dm.ndofs), **opts)
    out, lam, arep, arc = ctx.adjoint(x, g, with_cells=False, precision=0, restart=40, max_linear=400,
                                      linear_rtol=1e-11)
    # FD step 1e-4 (relative): the states come from iterative Newton solves converged to
    # ‖r‖ ~ 1e-14, whose error (~1e-11 in J) enters the quotient as 1/h, while the central
    # difference's truncation error is O(h²); the CPU test checks step 1e-6 with direct solves.
    h = 1e-4
    gam = params["gamma"]
    Js = []
    for s in (+1, -1):
        ctx.set_params(dict(params, gamma=gam * (1 + s * h)))
        xs, _, _ = ctx.newton_solve(x, **opts)
        Js.append(g @ xs)
    ctx.set_params(params)
    fd = (Js[0] - Js[1]) / (2 * h * gam)
    assert abs(fd - out[0]) <= 1e-6 * abs(out[0]), (fd, out[0])
