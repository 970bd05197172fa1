"""Sudden expansion (non-zero Dirichlet inlet, natural outlet, insulating walls) on the GPU
against the oracle's FP64 direct Newton."""
import numpy as np
import pytest

from helpers import expansion_case, gpu_context, oracle_problem
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _rel(a, b, modulo_const=False):
    a, b = a.copy(), b.copy()
    if modulo_const:
        a -= a.mean(); b -= b.mean()
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("precision", [0, 1])
def test_expansion_newton_matches_oracle(gpu_lib, precision):
    mesh, dm, params = expansion_case()
    prob = oracle_problem(mesh, dm, params)
    # insulating walls everywhere: φ is defined up to a constant
    xref, info = O.newton_direct(prob, np.zeros(dm.ndofs), gauge=[dm.offsets["phi"]], rtol=1e-13, maxiter=12)
    ctx = gpu_context(mesh, dm, params)
    x, rep, rc = ctx.newton_solve(np.zeros(dm.ndofs), precision=precision, max_newton=15, newton_rtol=1e-11,
                                  newton_atol=1e-14, restart=60, max_linear=400,
                                  linear_rtol=1e-4 if precision else 1e-8)
    assert rc == 0, rep
    s = dm.split(x)
    r = dm.split(xref)
    assert _rel(s["u"], r["u"]) <= 1e-8
    assert _rel(s["j"], r["j"]) <= 1e-8
    assert _rel(s["p"], r["p"]) <= 1e-8
    assert _rel(s["phi"], r["phi"], modulo_const=True) <= 1e-8


@pytest.mark.parametrize("precision", [0, 1])
def test_expansion_pressure_drop_adjoint_matches_oracle(gpu_lib, precision):
    """The pressure-drop objective's gradient on the GPU (MHD scaling: dJ/dα, dJ/dβ, dJ/dγ and
    the cellwise f_z, with dJ/dHa by the chain rule) against the oracle's adjoint (direct
    solves, reference-restated assembly)."""
    from adjoint_ref import oracle_adjoint, oracle_adjoint_ab
    from gbmhd.objectives import ha_gradient, pressure_drop
    Ha, Re = 20.0, 10.0
    mesh, dm, params = expansion_case(Ha=Ha, Re=Re)
    fz = np.linspace(0.4, 0.6, mesh.ncells)
    params["f_cell"] = np.stack([0 * fz, 0 * fz, fz], 1)
    gauge = [dm.offsets["phi"]]
    g = pressure_drop(mesh, dm)
    prob = oracle_problem(mesh, dm, params)
    xref, _ = O.newton_direct(prob, np.zeros(dm.ndofs), gauge=gauge, rtol=1e-14, maxiter=12)
    dgam, _, dfz, lam = oracle_adjoint(prob, dm, xref, g, gauge)
    dal, dbe = oracle_adjoint_ab(prob, lam, xref)
    ctx = gpu_context(mesh, dm, params)
    x, rep, rc = ctx.newton_solve(np.zeros(dm.ndofs), precision=precision, max_newton=15, newton_rtol=1e-12,
                                  newton_atol=1e-14, restart=60, max_linear=400,
                                  linear_rtol=1e-4 if precision else 1e-8)
    assert rc == 0, rep
    out, glam, arep, arc = ctx.adjoint(x, g, with_cells=True, precision=precision, restart=60, max_linear=400,
                                       linear_rtol=1e-10)
    assert arc == 0, arep
    for name, a, b in (("gamma", out[0], dgam), ("alpha", out[2], dal), ("beta", out[3], dbe)):
        assert abs(a - b) <= 1e-6 * abs(b), (name, a, b)
    assert np.linalg.norm(out[4:] - dfz) <= 1e-6 * np.linalg.norm(dfz)
    ref = ha_gradient(np.array([dgam, 0.0, dal, dbe]), Ha, Re, "mhd")
    assert abs(ha_gradient(out, Ha, Re, "mhd") - ref) <= 1e-6 * abs(ref)
