"""The adjoint's objectives (gbmhd/objectives.py) on manufactured fields their discrete
spaces represent exactly: the flow rate through a cross-section (Q2 velocity) and the
inlet−outlet pressure drop (dP1 pressure)."""
import numpy as np

from gbmhd.objectives import flow_rate, pressure_drop
from helpers import expansion_case, hunt_case

OU, OP = 0, 81


def _q2_node_coords(X):
    """Physical coordinates of the 27 Q2 nodes of each cell, node n = a + 3b + 9c at (a, b, c)/2."""
    out = np.zeros((X.shape[0], 27, 3))
    for n in range(27):
        xi = np.array([n % 3, (n // 3) % 3, n // 9]) / 2.0
        for v in range(8):
            w = 1.0
            for d in range(3):
                w *= xi[d] if (v >> d) & 1 else 1.0 - xi[d]
            out[:, n, :] += w * X[:, v, :]
    return out


def test_flow_rate_of_biquadratic_profile():
    """u_z = (1 − x²)(1 − y²) is biquadratic and zero on the walls: its Q2 interpolant on the
    (axis-aligned, stretched) Hunt cells is exact, and ∫ u_z dA over [−1, 1]² is 16/9."""
    mesh, dm, _ = hunt_case(nc=(6, 5), nz=4, Lz=0.2, beta_map=2.0)
    X = mesh.cell_coords()
    P = _q2_node_coords(X)
    gd = dm.global_cell_dofs()
    x = np.zeros(dm.ndofs)
    rows = gd[:, OU + 2 * 27:OU + 3 * 27]
    m = rows >= 0
    f = (1 - P[..., 0] ** 2) * (1 - P[..., 1] ** 2)
    x[rows[m]] = f[m]
    for z0 in (0.0, 0.1, 0.15):
        J = flow_rate(mesh, dm, z0) @ x
        assert abs(J - 16.0 / 9.0) < 1e-12, (z0, J)


def test_flow_rate_is_linear_and_only_reads_uz():
    mesh, dm, _ = hunt_case(nc=(4, 4), nz=3)
    g = flow_rate(mesh, dm, 0.0)
    nz = np.nonzero(g)[0]
    assert len(nz) > 0
    assert np.all((nz >= dm.offsets["u"]) & (nz < dm.offsets["u"] + dm.nfree["u"]))


def test_pressure_drop_of_linear_pressure():
    """p = x (the flow axis) is in dP1 on axis-aligned boxes; the volume-weighted means on the
    inlet and outlet cells are their volume-weighted centroid x."""
    mesh, dm, _ = expansion_case()
    X = mesh.cell_coords()
    gd = dm.global_cell_dofs()
    lo = X[:, 0, :]
    h = X[:, 7, :] - X[:, 0, :]
    assert np.allclose(X[:, 1, 1:], X[:, 0, 1:]) and np.allclose(X[:, 2, [0, 2]], X[:, 0, [0, 2]])  # boxes
    x = np.zeros(dm.ndofs)
    # p = p0 ψ0 + p1 ξ1 + p2 ξ2 + p3 ξ3 with ψ0 = 1 − ξ1 − ξ2 − ξ3: p = x_lo + h_x ξ1
    x[gd[:, OP + 0]] = lo[:, 0]
    x[gd[:, OP + 1]] = lo[:, 0] + h[:, 0]
    x[gd[:, OP + 2]] = lo[:, 0]
    x[gd[:, OP + 3]] = lo[:, 0]
    J = pressure_drop(mesh, dm) @ x
    bc, _, bt = mesh.boundary_faces()
    vol = np.prod(h, axis=1)
    mid = lo[:, 0] + 0.5 * h[:, 0]

    def mean_x(tag):
        c = np.unique(bc[bt == mesh.tag_names.index(tag)])
        return np.sum(vol[c] * mid[c]) / np.sum(vol[c])

    expect = mean_x("inlet") - mean_x("outlet")
    assert abs(J - expect) < 1e-12 * max(1.0, abs(expect)), (J, expect)
    # a constant pressure has no drop
    xc = np.zeros(dm.ndofs)
    xc[gd[:, OP:OP + 4].ravel()] = 3.0
    assert abs(pressure_drop(mesh, dm) @ xc) < 1e-12
