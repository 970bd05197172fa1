"""The oracle's discrete adjoint against central finite differences (CPU)."""
import numpy as np

from adjoint_ref import oracle_adjoint
from gbmhd.objectives import flow_rate
from helpers import hunt_case, oracle_problem
from oracle import oracle as O


def _solve(mesh, dm, params):
    prob = oracle_problem(mesh, dm, params)
    x, _ = O.newton_direct(prob, np.zeros(dm.ndofs), gauge=[dm.offsets["p"]], rtol=1e-14, maxiter=10)
    return prob, x


def test_oracle_adjoint_matches_finite_differences():
    rng = np.random.default_rng(0)
    base = dict(nc=(3, 3), nz=2, Ha=6.0, Re=5.0, beta_map=1.5, cw=0.1, Lz=0.2, zeta_u=1.0, zeta_j=1.0)
    mesh, dm, params = hunt_case(**base)
    fz = rng.uniform(0.9, 1.1, mesh.ncells)
    fcell = np.stack([0 * fz, 0 * fz, fz], 1)
    params["f_cell"] = fcell
    g = flow_rate(mesh, dm, 0.1)
    prob, x = _solve(mesh, dm, params)
    dgam, dcw, dfz, _ = oracle_adjoint(prob, dm, x, g, [dm.offsets["p"]])

    def J_of(p):
        _, xx = _solve(mesh, dm, p)
        return g @ xx
    h = 1e-6
    for key, ref in (("gamma", dgam),):
        pp, pm = dict(params), dict(params)
        pp[key] = params[key] * (1 + h); pm[key] = params[key] * (1 - h)
        fd = (J_of(pp) - J_of(pm)) / (2 * h * params[key])
        assert abs(fd - ref) <= 1e-6 * abs(ref), (key, fd, ref)
    # cw (all thin-wall facets together)
    pp, pm = dict(params), dict(params)
    f = params["facets"]
    cw0 = f["cw"][0]
    pp["facets"] = dict(f, cw=f["cw"] * (1 + h)); pm["facets"] = dict(f, cw=f["cw"] * (1 - h))
    fd = (J_of(pp) - J_of(pm)) / (2 * h * cw0)
    assert abs(fd - dcw) <= 1e-6 * abs(dcw), (fd, dcw)
    # two cells of the body-force field
    for c in (0, mesh.ncells - 1):
        fp, fm = fcell.copy(), fcell.copy()
        fp[c, 2] *= 1 + h; fm[c, 2] *= 1 - h
        fd = (J_of(dict(params, f_cell=fp)) - J_of(dict(params, f_cell=fm))) / (2 * h * fcell[c, 2])
        assert abs(fd - dfz[c]) <= 1e-6 * abs(dfz).max(), (c, fd, dfz[c])


def test_oracle_adjoint_pressure_drop_on_expansion():
    """The inlet−outlet pressure drop of the sudden expansion (the second objective of the
    adjoint) against central finite differences in γ and in the body force of one cell."""
    from gbmhd.objectives import pressure_drop
    from helpers import expansion_case
    mesh, dm, params = expansion_case(Ha=8.0, Re=4.0)
    fz = np.full(mesh.ncells, 0.5)
    params["f_cell"] = np.stack([0 * fz, 0 * fz, fz], 1)
    gauge = [dm.offsets["phi"]]
    g = pressure_drop(mesh, dm)

    def solve(p):
        prob = oracle_problem(mesh, dm, p)
        x, _ = O.newton_direct(prob, np.zeros(dm.ndofs), gauge=gauge, rtol=1e-14, maxiter=12)
        return prob, x

    prob, x = solve(params)
    dgam, _, dfz, _ = oracle_adjoint(prob, dm, x, g, gauge)
    h = 1e-6
    Jp = g @ solve(dict(params, gamma=params["gamma"] * (1 + h)))[1]
    Jm = g @ solve(dict(params, gamma=params["gamma"] * (1 - h)))[1]
    fd = (Jp - Jm) / (2 * h * params["gamma"])
    assert abs(fd - dgam) <= 1e-6 * abs(dgam), (fd, dgam)
    c = mesh.ncells // 2
    fp, fm = params["f_cell"].copy(), params["f_cell"].copy()
    fp[c, 2] *= 1 + h
    fm[c, 2] *= 1 - h
    fd = (g @ solve(dict(params, f_cell=fp))[1] - g @ solve(dict(params, f_cell=fm))[1]) / (2 * h * fz[c])
    assert abs(fd - dfz[c]) <= 1e-6 * abs(dfz).max(), (fd, dfz[c])


def test_oracle_dJ_dHa_mhd_scaling():
    """dJ/dHa of the expansion's pressure drop in the MHD scaling (α = Re/Ha², β = 1/Ha²,
    γ = 1): the adjoint's dJ/dα and dJ/dβ through the chain rule of gbmhd.objectives against
    central finite differences in Ha (step 1e-6 relative) with direct solves."""
    from adjoint_ref import oracle_adjoint_ab
    from gbmhd.objectives import ha_gradient, pressure_drop
    from helpers import expansion_case
    Ha, Re = 8.0, 4.0
    mesh, dm, params = expansion_case(Ha=Ha, Re=Re)
    gauge = [dm.offsets["phi"]]
    g = pressure_drop(mesh, dm)

    def solve(ha):
        _, _, p = expansion_case(Ha=ha, Re=Re)
        prob = oracle_problem(mesh, dm, p)
        x, _ = O.newton_direct(prob, np.zeros(dm.ndofs), gauge=gauge, rtol=1e-14, maxiter=12)
        return prob, x

    prob, x = solve(Ha)
    dgam, dcw, _, lam = oracle_adjoint(prob, dm, x, g, gauge)
    dal, dbe = oracle_adjoint_ab(prob, lam, x)
    dJ = np.array([dgam, dcw, dal, dbe])
    ref = ha_gradient(dJ, Ha, Re, "mhd")
    h = 1e-6
    fd = (g @ solve(Ha * (1 + h))[1] - g @ solve(Ha * (1 - h))[1]) / (2 * h * Ha)
    assert abs(fd - ref) <= 1e-6 * abs(ref), (fd, ref)
    # each of dJ/dα and dJ/dβ on its own
    for key, val in (("alpha", dal), ("beta", dbe)):
        pp, pm = dict(params), dict(params)
        pp[key] = params[key] * (1 + h)
        pm[key] = params[key] * (1 - h)
        Jp = g @ O.newton_direct(oracle_problem(mesh, dm, pp), np.zeros(dm.ndofs), gauge=gauge, rtol=1e-14,
                                 maxiter=12)[0]
        Jm = g @ O.newton_direct(oracle_problem(mesh, dm, pm), np.zeros(dm.ndofs), gauge=gauge, rtol=1e-14,
                                 maxiter=12)[0]
        fd = (Jp - Jm) / (2 * h * params[key])
        assert abs(fd - val) <= 1e-6 * abs(val), (key, fd, val)


def test_ha_gradient_chain_rule_cfd():
    """CFD scaling: γ = Ha²/Re, so dJ/dHa = dJ/dγ · 2Ha/Re; unknown scalings are rejected."""
    import pytest
    from gbmhd.objectives import ha_gradient
    assert ha_gradient(np.array([3.0, 0.0, 0.0, 0.0]), 50.0, 10.0, "cfd") == 3.0 * 2 * 50.0 / 10.0
    with pytest.raises(ValueError):
        ha_gradient(np.zeros(4), 1.0, 1.0, "other")
