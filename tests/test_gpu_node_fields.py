"""The device field evaluation at the Q2 nodes (gbmhd_node_fields, the data of the VTK output)
against the oracle's restatement of the bases, with the trilinear geometry and the Piola map
formed in numpy, on a perturbed (non-affine) stretched duct with a random state."""
import numpy as np
import pytest

from helpers import gpu_context, hunt_case, random_state
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _ref(xi):
    q2 = np.zeros(27); rt = np.zeros((36, 3)); rtdiv = np.zeros(36); p1 = np.zeros(4); q1 = np.zeros(8)
    O.lib().orc_ref_basis(O._dp(np.asarray(xi, float)), O._dp(q2), O._dp(rt), O._dp(rtdiv), O._dp(p1), O._dp(q1))
    return q2, rt, rtdiv, p1, q1


def test_node_fields_match_the_oracle_bases(gpu_lib):
    mesh, dm, params = hunt_case(nc=(3, 3), nz=3, beta_map=2.0, perturb=0.15, cw=0.1)
    x = random_state(dm, seed=3)
    ctx = gpu_context(mesh, dm, params)
    out = ctx.node_fields(x)
    X = mesh.cell_coords()
    xc = dm.cell_values(x)
    for c in range(mesh.ncells):
        for n in range(27):
            xi = np.array([0.5 * (n % 3), 0.5 * ((n // 3) % 3), 0.5 * (n // 9)])
            q2, rt, rtdiv, p1, q1 = _ref(xi)
            # trilinear map and its Jacobian (closed-form gradients of the Q1 vertex functions)
            pt = q1 @ X[c]
            J = np.zeros((3, 3))
            for v in range(8):
                a, b, cc = v & 1, (v >> 1) & 1, (v >> 2) & 1
                L = [(1 - xi[0], xi[0]), (1 - xi[1], xi[1]), (1 - xi[2], xi[2])]
                d = (-1.0, 1.0)
                g = np.array([d[a] * L[1][b] * L[2][cc], L[0][a] * d[b] * L[2][cc], L[0][a] * L[1][b] * d[cc]])
                J += np.outer(X[c, v], g)
            det = np.linalg.det(J)
            u = np.array([xc[c, 27 * k:27 * k + 27] @ q2 for k in range(3)])
            p = xc[c, 81:85] @ p1
            j = J @ (xc[c, 85:121] @ rt) / det
            divj = xc[c, 85:121] @ rtdiv / det
            phi = xc[c, 121:129] @ q1
            o = out[c, n]
            assert np.allclose(o[0:3], pt, atol=1e-12)
            assert np.allclose(o[3:6], u, atol=1e-12)
            assert abs(o[6] - p) <= 1e-12 and abs(o[10] - phi) <= 1e-12
            scale = max(1.0, np.abs(j).max())
            assert np.abs(o[7:10] - j).max() <= 1e-12 * scale, (o[7:10], j)
            assert abs(o[12] - divj) <= 1e-12 * max(1.0, abs(divj))
