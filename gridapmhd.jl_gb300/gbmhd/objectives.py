"""Linear objectives J(x) for the discrete adjoint and their gradients ∂J/∂x.

* ``flow_rate``: J = ∫ u_z dA over the cross-section plane z = z0 (a plane of
  cell faces), the axial flow rate of the Hunt duct.
* ``pressure_drop``: J = mean p over the inlet cells − mean p over the outlet
  cells (cells touching the inlet / outlet boundary), for the expansion.

The reference has no adjoint; these functionals define what the gradient is
taken of.  They are linear in the free dof vector, so ∂J/∂x is constant.
"""
from __future__ import annotations

import numpy as np

from .fespace import DofMap, OP, OU
from .mesh import StructuredMesh

_GX = np.array([0.5 - 0.5 * np.sqrt(0.6), 0.5, 0.5 + 0.5 * np.sqrt(0.6)])
_GW = np.array([5.0, 8.0, 5.0]) / 18.0


def _lag2(a, t):
    return [(2 * t - 1) * (t - 1), 4 * t * (1 - t), t * (2 * t - 1)][a]


def _dq1(xi):
    g = np.zeros((8, 3))
    for v in range(8):
        a, b, c = v & 1, (v >> 1) & 1, (v >> 2) & 1
        l = [(1 - xi[0], xi[0]), (1 - xi[1], xi[1]), (1 - xi[2], xi[2])]
        d = [-1.0, 1.0]
        g[v, 0] = d[a] * l[1][b] * l[2][c]
        g[v, 1] = l[0][a] * d[b] * l[2][c]
        g[v, 2] = l[0][a] * l[1][b] * d[c]
    return g


def flow_rate(mesh: StructuredMesh, dm: DofMap, z0: float) -> np.ndarray:
    """∂J/∂x for J = ∫_{z=z0} u_z dA (faces ξ3 = 0 of the cells whose lower z face is at z0)."""
    X = mesh.cell_coords()
    zlo = X[:, 0, 2]
    tol = 1e-9 * max(1.0, abs(z0))
    cells = np.nonzero(np.abs(zlo - z0) < tol)[0]
    if len(cells) == 0:
        raise ValueError(f"no cell face lies on z = {z0}")
    g = np.zeros(dm.ndofs)
    gd = dm.global_cell_dofs()
    for tj in range(3):
        for ti in range(3):
            xi = np.array([_GX[ti], _GX[tj], 0.0])
            G = _dq1(xi)
            J = np.einsum("cvi,va->cia", X[cells], G)            # (nc, 3, 3)
            cof = np.cross(J[:, :, 0], J[:, :, 1])                # area vector of the ξ3 face
            dA = _GW[ti] * _GW[tj] * np.linalg.norm(cof, axis=1)
            for n in range(27):
                a, b, c = n % 3, (n // 3) % 3, n // 9
                if c != 0:
                    continue
                N = _lag2(a, xi[0]) * _lag2(b, xi[1])
                rows = gd[cells, OU + 2 * 27 + n]
                m = rows >= 0
                np.add.at(g, rows[m], dA[m] * N)
    return g


def pressure_drop(mesh: StructuredMesh, dm: DofMap, inlet_tag="inlet", outlet_tag="outlet") -> np.ndarray:
    """∂J/∂x for J = (cell-volume-weighted mean p on inlet cells) − (same on outlet cells)."""
    bc, bf, bt = mesh.boundary_faces()
    X = mesh.cell_coords()
    gd = dm.global_cell_dofs()
    g = np.zeros(dm.ndofs)
    for tag, sign in ((inlet_tag, 1.0), (outlet_tag, -1.0)):
        cells = np.unique(bc[bt == mesh.tag_names.index(tag)])
        # ∫_cell p = Σ_k p_k ∫ ψ_k ; with ψ = (1−ξ1−ξ2−ξ3, ξ1, ξ2, ξ3) on the reference cube
        vol = np.zeros(len(cells))
        mom = np.zeros((len(cells), 4))
        for k3 in range(3):
            for k2 in range(3):
                for k1 in range(3):
                    xi = np.array([_GX[k1], _GX[k2], _GX[k3]])
                    w = _GW[k1] * _GW[k2] * _GW[k3]
                    J = np.einsum("cvi,va->cia", X[cells], _dq1(xi))
                    det = np.linalg.det(J)
                    psi = np.array([1 - xi.sum(), xi[0], xi[1], xi[2]])
                    vol += w * det
                    mom += (w * det)[:, None] * psi[None, :]
        V = vol.sum()
        for k in range(4):
            rows = gd[cells, OP + k]
            np.add.at(g, rows, sign * mom[:, k] / V)
    return g


def ha_gradient(dJ: np.ndarray, Ha: float, Re: float, scaling: str = "cfd") -> float:
    """dJ/dHa from gbmhd_adjoint's parameter gradient dJ = [dJ/dγ, dJ/dcw, dJ/dα, dJ/dβ, ...].

    * ``"cfd"`` scaling (src/Applications/hunt.jl:125-128): α = 1, β = 1/Re, γ = N = Ha²/Re,
      so dJ/dHa = dJ/dγ · 2Ha/Re.
    * ``"mhd"`` scaling (src/Applications/expansion.jl:113-123): α = 1/N = Re/Ha², β = 1/Ha²,
      γ = 1, so dJ/dHa = −(2/Ha³)(Re·dJ/dα + dJ/dβ).
    """
    if scaling == "cfd":
        return float(dJ[0]) * 2.0 * Ha / Re
    if scaling == "mhd":
        return -2.0 / Ha ** 3 * (Re * float(dJ[2]) + float(dJ[3]))
    raise ValueError(f"unknown scaling {scaling!r}: expected 'cfd' or 'mhd'")
