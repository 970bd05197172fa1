"""Properties of the library's local basis that the Julia change of basis relies on
(gridapmhd.jl_gb300/julia/GridapMHDGB300.jl, `LocalMaps`), checked on the oracle's
restatement of the basis (orc_ref_basis).

The shim converts between Gridap's dof values (face and interior moments for RT1,
src/parameters.jl:521-526; nodal values for Q2, P1, Q1, :436-441) and the library's
coefficients with M[i,k] = σᵢ(ψₖ), block by block: 4 x 4 per face, then the cell interior.
That is consistent across the two cells of a face only if
  * each RT face function has zero normal flux through every other face, and each interior
    function zero normal flux through all faces (M block triangular, face blocks depend on
    the face alone);
  * the four face functions of a face are independent on that face (the face block is
    invertible whatever moments Gridap uses), and all 36 are independent in the cell;
  * the Q2, P1 and Q1 functions are unisolvent (the nodal maps are invertible), the Q2 ones
    Kronecker at the 27 nodes (the u map is the node permutation).
"""
import ctypes as C

import numpy as np

from oracle import oracle as O


def ref_basis(xi):
    q2 = np.zeros(27); rt = np.zeros((36, 3)); rtdiv = np.zeros(36); p1 = np.zeros(4); q1 = np.zeros(8)
    O.lib().orc_ref_basis(O._dp(np.asarray(xi, float)), O._dp(q2), O._dp(rt), O._dp(rtdiv), O._dp(p1), O._dp(q1))
    return q2, rt, p1, q1


def rt_class(b):
    """(axis d, q) of RT function b: q = 0 / 2 face ξ_d = 0 / 1, q = 1 interior."""
    return b // 12, (b % 12) % 3


def face_points(axis, side, rng, n=12):
    P = rng.uniform(0.05, 0.95, (n, 3))
    P[:, axis] = side
    return P


def test_rt_face_functions_carry_flux_through_their_own_face_only():
    rng = np.random.default_rng(0)
    for axis in range(3):
        for side in (0, 1):
            pts = face_points(axis, side, rng)
            flux = np.array([ref_basis(x)[1][:, axis] for x in pts])   # (points, 36): ψ·e_axis
            for b in range(36):
                d, q = rt_class(b)
                own = d == axis and q == 2 * side
                if not own:
                    assert np.abs(flux[:, b]).max() <= 1e-14, (b, axis, side)
            own = [b for b in range(36) if rt_class(b) == (axis, 2 * side)]
            assert len(own) == 4
            # the four traces are independent on the face: rank 4 at 12 face points
            assert np.linalg.matrix_rank(flux[:, own], tol=1e-10) == 4


def test_rt_interior_functions_have_no_face_flux_and_all_36_are_independent():
    rng = np.random.default_rng(1)
    interior = [b for b in range(36) if rt_class(b)[1] == 1]
    assert len(interior) == 12
    for axis in range(3):
        for side in (0, 1):
            for x in face_points(axis, side, rng, 6):
                assert np.abs(ref_basis(x)[1][interior, axis]).max() <= 1e-14
    vals = np.array([ref_basis(x)[1] for x in rng.uniform(0, 1, (40, 3))])           # (40, 36, 3)
    A = vals.transpose(0, 2, 1).reshape(-1, 36)                                       # rows: point x component
    assert np.linalg.matrix_rank(A, tol=1e-10) == 36


def test_lagrange_bases_are_unisolvent_and_q2_is_nodal():
    nodes = [(a / 2, b / 2, c / 2) for c in range(3) for b in range(3) for a in range(3)]  # n = a + 3b + 9c
    Q2 = np.array([ref_basis(x)[0] for x in nodes])
    assert np.allclose(Q2, np.eye(27), atol=1e-14)
    verts = [(a, b, c) for c in (0, 1) for b in (0, 1) for a in (0, 1)]
    Q1 = np.array([ref_basis(x)[3] for x in verts])
    assert np.allclose(Q1, np.eye(8), atol=1e-14)
    rng = np.random.default_rng(2)
    P1 = np.array([ref_basis(x)[2] for x in rng.uniform(0, 1, (10, 3))])
    assert np.linalg.matrix_rank(P1, tol=1e-10) == 4
