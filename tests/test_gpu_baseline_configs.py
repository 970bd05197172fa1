"""Parity at the sizes of the benchmark configurations.

* 32x32x3 duct (tanh stretching β = 2, Ha = 100, Re = 10, cw = 0.1): the GPU Newton
  solution, FP64 and mixed, against the oracle's FP64 solution of the same mesh (SuperLU,
  committed as tests/golden/cfg2_solution.npz by tests/golden/make_cfg2.py).
* 64x64x4 duct (β = 3, Ha = 500, Re = 1, cw = 0.1): the mixed solution against the plain FP64
  GPU path driven to ‖r‖ ≤ 1e-12‖r0‖.  No CPU direct solve finishes at 976,920 dofs; the FP64
  GPU path is the reference there, certified against the oracle on the smaller ducts.
* 48x48x4 duct (β = 2.5, Ha = 200, Re = 10, cw = 0.1, f_z ~ U[0.9, 1.1] per cell, seed 0):
  the adjoint gradient of the axial flow rate at mid-length w.r.t. Ha, cw and the f_z field
  (along a direction of positive per-cell weights, seed 1), against central finite differences
  of FP64 GPU Newton solves (relative steps 1e-6 and 1e-4), and
  against the gradient formed with the oracle's FP64 assembly (its residual at the GPU state,
  its transposed Jacobian applied to the GPU's λ, and its ∂R/∂θ).

Tolerances: 1e-8 relative L2 per field (pressure modulo a constant); 1e-6 relative on every
gradient component against the oracle-assembly gradient and the 1e-4-step differences, 1e-5
against the 1e-6-step differences (their noise floor, see the test).
"""
import os

import numpy as np
import pytest

from adjoint_ref import oracle_param_derivs
from gbmhd.objectives import flow_rate, ha_gradient
from helpers import gpu_context, hunt_case, oracle_problem
from test_gpu_newton import field_rel_errors

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CFG2 = dict(nc=(32, 32), nz=3, Ha=100.0, Re=10.0, beta_map=2.0, cw=0.1, Lz=0.2)
CFG3 = dict(nc=(64, 64), nz=4, Ha=500.0, Re=1.0, beta_map=3.0, cw=0.1, Lz=0.2)
CFG4 = dict(nc=(48, 48), nz=4, Ha=200.0, Re=10.0, beta_map=2.5, cw=0.1, Lz=0.2)


@pytest.mark.parametrize("precision", [0, 1])
def test_cfg2_32x32x3_matches_oracle(gpu_lib, precision):
    path = os.path.join(GOLDEN, "cfg2_solution.npz")
    if not os.path.exists(path):
        pytest.skip("tests/golden/cfg2_solution.npz not generated")
    xref = np.load(path)["x"]
    mesh, dm, params = hunt_case(**CFG2)
    assert xref.shape == (dm.ndofs,)
    ctx = gpu_context(mesh, dm, params)
    x, rep, rc = ctx.newton_solve(np.zeros(dm.ndofs), precision=precision, max_newton=12, newton_rtol=1e-12,
                                  newton_atol=0.0, restart=200, max_linear=600,
                                  linear_rtol=1e-3 if precision else 1e-8)
    assert rc == 0 and rep["converged"], rep
    errs = field_rel_errors(dm, x, xref)
    for f, e in errs.items():
        assert e <= 1e-8, (f, e, errs, rep)


def test_cfg3_64x64x4_mixed_matches_fp64(gpu_lib):
    mesh, dm, params = hunt_case(**CFG3)
    ctx = gpu_context(mesh, dm, params)
    x64, rep64, rc64 = ctx.newton_solve(np.zeros(dm.ndofs), precision=0, max_newton=12, newton_rtol=1e-12,
                                        restart=200, max_linear=600, linear_rtol=1e-10)
    # the FP64 path's residual floor here is 2e-14 … 2e-13 absolute (‖r0‖ = 5.2e-3): it may end
    # on the step cap instead of the floor rule, with the state as accurate as the floor allows
    assert rc64 in (0, 1) and rep64["final_residual"] <= 1e-10 * rep64["initial_residual"], rep64
    x32, rep32, rc32 = ctx.newton_solve(np.zeros(dm.ndofs), precision=1, max_newton=12, newton_rtol=1e-12,
                                        restart=200, max_linear=600, linear_rtol=1e-3)
    assert rc32 == 0, rep32
    errs = field_rel_errors(dm, x32, x64)
    assert max(errs.values()) <= 1e-8, errs


def _cfg4():
    mesh, dm, params = hunt_case(**CFG4)
    rng = np.random.default_rng(0)
    fz = rng.uniform(0.9, 1.1, mesh.ncells)
    params["f_cell"] = np.stack([0 * fz, 0 * fz, fz], 1)
    return mesh, dm, params


def test_cfg4_48x48x4_adjoint_gradient(gpu_lib):
    mesh, dm, params = _cfg4()
    Ha, Re = CFG4["Ha"], CFG4["Re"]
    g = flow_rate(mesh, dm, 0.1)
    ctx = gpu_context(mesh, dm, params)
    base = dict(precision=0, restart=200, max_linear=600)
    # to the FP64 residual's floor: the round-off of the assembly, whose atomic adds run in
    # arbitrary order, at γ = 4000 (measured 1e-12 … 5e-11 absolute from run to run)
    x, rep, rc = ctx.newton_solve(np.zeros(dm.ndofs), max_newton=12, newton_rtol=1e-14, newton_atol=0.0,
                                  linear_rtol=1e-12, **base)
    assert rep["final_residual"] <= 2e-8 * rep["initial_residual"], rep
    dJ, lam, arep, arc = ctx.adjoint(x, g, with_cells=True, linear_rtol=1e-10, **base)
    assert arc == 0, arep
    dJ_dHa = ha_gradient(dJ, Ha, Re, "cfd")

    # (1) the gradient formed with the oracle's FP64 assembly at the GPU's state and λ
    prob = oracle_problem(mesh, dm, params)
    r0, _ = prob.residual_jacobian(np.zeros(dm.ndofs), want_jac=False)
    r, A = prob.residual_jacobian(x)
    assert np.linalg.norm(r) <= 2e-8 * np.linalg.norm(r0), (np.linalg.norm(r), np.linalg.norm(r0))
    assert np.linalg.norm(A.T @ lam - g) <= 1e-9 * np.linalg.norm(g)
    dRg, dRc, fzm = oracle_param_derivs(prob, x)
    gd = dm.global_cell_dofs()[:, 54:81]
    lz = np.where(gd >= 0, lam[np.maximum(gd, 0)], 0.0)
    ref = dict(gamma=-lam @ dRg, cw=-lam @ dRc)
    assert abs(dJ[0] - ref["gamma"]) <= 1e-6 * abs(ref["gamma"]), (dJ[0], ref)
    assert abs(dJ[1] - ref["cw"]) <= 1e-6 * abs(ref["cw"]), (dJ[1], ref)
    dfz_ref = np.sum(lz * fzm, 1)
    assert np.linalg.norm(dJ[4:] - dfz_ref) <= 1e-6 * np.linalg.norm(dfz_ref)

    # (2) central finite differences of FP64 GPU Newton solves from x.  The J of a solve carries
    # the FP64 residual floor (1e-12 … 5e-11 absolute, the assembly's atomic adds in arbitrary
    # order): measured 3e-14 … 1.4e-13 in J, i.e. mostly 1e-8 … 5e-6 of the gradient at a
    # relative step of 1e-6, with one cw difference at 2.5e-5 in four runs.  So the 1e-6 step is
    # checked to 5e-5, and a 1e-4 step (truncation O(h²) ~ 1e-8, noise 100x smaller) to the
    # 1e-6 target.
    fd_opts = dict(max_newton=6, newton_rtol=0.0, newton_atol=0.0, linear_rtol=1e-12, **base)

    def J(p):
        ctx.set_params(p)
        xs, _, _ = ctx.newton_solve(x, **fd_opts)
        return g @ xs

    f = params["facets"]
    w = np.random.default_rng(1).uniform(0.5, 1.5, mesh.ncells) * params["f_cell"][:, 2]
    adj = {"Ha": dJ_dHa, "cw": dJ[1], "f_z": float(dJ[4:] @ w)}
    for h, tol in ((1e-6, 5e-5), (1e-4, 1e-6)):
        fd = {}
        pp = dict(params, gamma=(Ha * (1 + h)) ** 2 / Re)
        pm = dict(params, gamma=(Ha * (1 - h)) ** 2 / Re)
        fd["Ha"] = (J(pp) - J(pm)) / (2 * h * Ha)
        fd["cw"] = (J(dict(params, facets=dict(f, cw=f["cw"] * (1 + h)))) -
                    J(dict(params, facets=dict(f, cw=f["cw"] * (1 - h))))) / (2 * h * f["cw"][0])
        fp, fm = params["f_cell"].copy(), params["f_cell"].copy()
        fp[:, 2] += h * w
        fm[:, 2] -= h * w
        fd["f_z"] = (J(dict(params, f_cell=fp)) - J(dict(params, f_cell=fm))) / (2 * h)
        ctx.set_params(params)
        print(f"cfg4 gradient, step {h:g}: adjoint", adj, "finite differences", fd,
              "relative", {k: abs(fd[k] - adj[k]) / abs(adj[k]) for k in adj})
        for k in adj:
            assert abs(fd[k] - adj[k]) <= tol * abs(adj[k]), (h, k, fd[k], adj[k])
