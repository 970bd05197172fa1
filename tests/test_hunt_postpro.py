"""hunt() post-processing restated in the oracle: the analytic Hunt gradient and the error
norms, pinned against the reference's published error norms (golden vectors)."""
import json
import os

import numpy as np
import pytest

from gbmhd.fespace import build_dofmap
from gbmhd.mesh import hunt_generate_base_mesh
from oracle import oracle as O

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "published_hunt.json")))


@pytest.mark.parametrize("Ha", [5.0, 50.0, 500.0])
def test_analytic_gradient_matches_finite_differences(Ha):
    rng = np.random.default_rng(0)
    x = np.c_[rng.uniform(-0.95, 0.95, (40, 2)), np.zeros(40)]
    g = O.analytical_hunt_grad_u(1.0, 1.0, 1.3, -0.7, Ha, 12, x)
    h = 1e-6
    for i in range(2):
        xp, xm = x.copy(), x.copy()
        xp[:, i] += h
        xm[:, i] -= h
        fd = (O.analytical_hunt_u(1.0, 1.0, 1.3, -0.7, Ha, 12, xp) - O.analytical_hunt_u(1.0, 1.0, 1.3, -0.7, Ha, 12, xm)) / (2 * h)
        scale = max(np.abs(g[:, i, 2]).max(), 1e-12)
        assert np.abs(fd[:, 2] - g[:, i, 2]).max() <= 1e-7 * scale + 1e-12
    assert np.all(g[:, :, 0:2] == 0.0) and np.all(g[:, 2, :] == 0.0)


def test_published_hunt_errors_nc10():
    """Reference hunt(nc=(10,10), B=(0,50,0), L=1, kmap=1, Re=1, nsums=500): eu_ref_l2,
    ej_ref_l2 and eu_ref_h1 (2·nsums Fourier terms) of the discrete solution
    (analysis/gadi/results/2023_04/eaab9d1.../hconv_ha00050ns500/summary.csv:7)."""
    r = next(r for r in GOLD if r["case"] == "nc=10, Ha=50")
    Ha = float(r["Ha"])
    m = hunt_generate_base_mesh((10, 10), Ha=Ha, nz=3, BL_adapted=False, kmap_x=1, kmap_y=1)
    dm = build_dofmap(m, ["conducting", "insulating"], ["insulating"])
    fl = O.Fluid(alpha=1.0, beta=1.0, gamma=Ha ** 2, B=(0, 1, 0), f=(0, 0, 1), convection=2)
    prob = O.OracleProblem(m.cell_coords(), dm.global_cell_dofs(), dm.ndofs, dm.cell_values, fl)
    x, _ = O.newton_direct(prob, np.zeros(dm.ndofs), gauge=[dm.offsets["p"]], rtol=1e-12)
    # hunt(): μ = ρν = 1, grad_pz = −f_z/ρ = −1, uh = u0 ūh, jh = σ u0 B0 j̄h = Ha j̄h
    e = O.hunt_errors(m.cell_coords(), dm.cell_values(x), L=1.0, mu=1.0, grad_pz=-1.0, sigma=1.0, Ha=Ha,
                      nsums=int(r["nsums"]), u_scale=1.0, j_scale=Ha)
    for k in ("eu_ref_l2", "ej_ref_l2", "eu_ref_h1", "uh_l2", "uh_h1", "jh_l2"):
        assert abs(e[k] / float(r[k]) - 1) < 1e-10, (k, e[k], r[k])
