"""hunt() post-processing on the device (gbmhd_hunt_errors) against the oracle's restatement
and, end to end through the host mirror hunt(), against the reference's published norms."""
import json
import os

import numpy as np
import pytest

from helpers import gpu_context, hunt_case
from oracle import oracle as O

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "published_hunt.json")))


@pytest.mark.parametrize("scales", [dict(u_scale=1.0, j_scale=1.0, length_scale=1.0, L=1.0),
                                    dict(u_scale=1.7, j_scale=20.0, length_scale=2.0, L=2.0)])
def test_hunt_errors_match_oracle(gpu_lib, scales):
    mesh, dm, params = hunt_case(nc=(8, 8), nz=3, Ha=20.0, Re=1.0, beta_map=2.0)
    ctx = gpu_context(mesh, dm, params)
    x, rep, rc = ctx.newton_solve(np.zeros(dm.ndofs), precision=0, max_newton=12, newton_rtol=1e-12,
                                  restart=60, max_linear=400, linear_rtol=1e-10)
    assert rc == 0, rep
    kw = dict(mu=1.0, grad_pz=-1.0, sigma=1.0, Ha=20.0, nsums=30, **scales)
    got = ctx.hunt_errors(x, **kw)
    ref = O.hunt_errors(mesh.cell_coords(), dm.cell_values(x), **kw)
    for k, v in ref.items():
        assert abs(got[k] - v) <= 1e-10 * abs(v) + 1e-300, (k, got[k], v)


def test_host_hunt_matches_published_norms(gpu_lib):
    """hunt(nc=(10,10), B=(0,50,0), L=1, kmap=1, Re=1, nsums=500) through the host mirror:
    GPU Newton solve, then the GPU post-processing, against the published eu_ref_l2,
    ej_ref_l2, eu_ref_h1, uh_l2, uh_h1 and jh_l2
    (analysis/gadi/results/2023_04/eaab9d1.../hconv_ha00050ns500/summary.csv:7)."""
    from gbmhd.main import hunt
    r = next(r for r in GOLD if r["case"] == "nc=10, Ha=50")
    info = hunt(nc=(10, 10), B=(0.0, 50.0, 0.0), L=1.0, kmap_x=1, kmap_y=1, BL_adapted=False, nsums=int(r["nsums"]))
    assert info.get("converged", True)
    for k in ("eu_ref_l2", "ej_ref_l2", "eu_ref_h1", "uh_l2", "uh_h1", "jh_l2"):
        assert abs(info[k] / float(r[k]) - 1) < 1e-7, (k, info[k], r[k])
    assert info["time_post_process"] > 0.0
