"""The FP64 Jacobian's state-independent part, checked on the CPU with the oracle.

The library assembles the FP64 Jacobian as a cached part (every term but convection:
viscous, augmented-Lagrangian, pressure, Lorentz, Ohm, thin-wall facets), assembled once per
parameter set, plus a convection-only pass at each state (csrc/assemble.cu, KArgs::jpart).
That is exact only if the Jacobian is affine in the state outside the u–u block.  Here the
oracle's Jacobians at two random states must differ in u–u entries only, for a Hunt duct
with thin walls and both augmented-Lagrangian terms, with Picard and Newton convection, and
for the expansion in the MHD scaling."""
import numpy as np
import pytest

from helpers import expansion_case, hunt_case, oracle_problem, random_state

CASES = {
    "hunt_newton_al": lambda: hunt_case(nc=(4, 4), nz=3, Ha=50.0, Re=10.0, cw=0.05, zeta_u=3.0, zeta_j=2.0),
    "hunt_picard": lambda: hunt_case(nc=(4, 4), nz=3, Ha=20.0, Re=10.0, cw=0.01, convection=1),
    "expansion_mhd_thin_wall": lambda: expansion_case(thin_wall=(100.0, 0.1)),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_jacobian_is_affine_in_the_state_outside_the_velocity_block(name):
    mesh, dm, params = CASES[name]()
    prob = oracle_problem(mesh, dm, params)
    _, J1 = prob.residual_jacobian(random_state(dm, seed=1, scale=0.5))
    _, J2 = prob.residual_jacobian(random_state(dm, seed=2, scale=0.5))
    D = (J1 - J2).tocoo()
    scale = max(abs(J1).max(), abs(J2).max())
    nu = dm.nfree["u"]  # the free vector is ordered [u; p; j; φ]
    outside = (D.row >= nu) | (D.col >= nu)
    assert np.abs(D.data[outside]).max(initial=0.0) <= 1e-13 * scale
    # and the convection part is really there: the u–u block does change with the state
    assert np.abs(D.data[~outside]).max(initial=0.0) > 1e-8 * scale
