"""GPU assembly against the FP64 oracle: CSR pattern bit-exact, values within tolerance."""
import numpy as np
import pytest

from helpers import gpu_context, hunt_case, oracle_problem, random_state

pytestmark = pytest.mark.gpu

CASES = {
    "uniform": dict(nc=(4, 4), nz=3, Ha=10.0, Re=10.0),
    "tanh_thinwall": dict(nc=(5, 4), nz=3, Ha=20.0, Re=5.0, beta_map=2.0, cw=0.01),
    "trilinear_al": dict(nc=(3, 3), nz=2, Ha=7.0, Re=3.0, beta_map=1.0, perturb=0.2, cw=0.1, zeta_u=2.0,
                         zeta_j=3.0, convection=2),
    "picard": dict(nc=(3, 4), nz=3, Ha=4.0, Re=2.0, convection=1),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_assembly_fp64_matches_oracle(gpu_lib, name):
    mesh, dm, params = hunt_case(**CASES[name])
    prob = oracle_problem(mesh, dm, params)
    x = random_state(dm, seed=7, scale=0.3)
    r_ref, A_ref = prob.residual_jacobian(x)
    ctx = gpu_context(mesh, dm, params)
    r = ctx.assemble(x, want_jacobian=True, precision=0)
    rowptr, col, val = ctx.csr()
    assert ctx.nnz == A_ref.nnz
    assert np.array_equal(rowptr, A_ref.indptr)          # pattern: bit-exact
    assert np.array_equal(col, A_ref.indices)
    scale = np.abs(A_ref.data).max()
    assert np.abs(val - A_ref.data).max() <= 1e-12 * scale
    assert np.abs(r - r_ref).max() <= 1e-12 * np.abs(r_ref).max()


@pytest.mark.parametrize("name", sorted(CASES))
def test_assembly_mixed_matches_oracle(gpu_lib, name):
    mesh, dm, params = hunt_case(**CASES[name])
    prob = oracle_problem(mesh, dm, params)
    x = random_state(dm, seed=11, scale=0.3)
    r_ref, A_ref = prob.residual_jacobian(x)
    ctx = gpu_context(mesh, dm, params)
    r = ctx.assemble(x, want_jacobian=True, precision=1)
    rowptr, col, val = ctx.csr()
    assert np.array_equal(col, A_ref.indices)
    # FP32 element matrices: error relative to the largest entry of each row
    rows = np.repeat(np.arange(len(rowptr) - 1), np.diff(rowptr))
    rowmax = np.maximum.reduceat(np.abs(A_ref.data), rowptr[:-1])
    assert (np.abs(val - A_ref.data) / rowmax[rows]).max() <= 2e-5
    # the residual stays FP64 in the mixed path
    assert np.abs(r - r_ref).max() <= 1e-12 * np.abs(r_ref).max()


def test_cellwise_force_and_set_params(gpu_lib):
    mesh, dm, params = hunt_case(nc=(3, 3), nz=2, Ha=5.0, Re=2.0)
    rng = np.random.default_rng(0)
    fz = rng.uniform(0.9, 1.1, mesh.ncells)
    params2 = dict(params, f_cell=np.stack([0 * fz, 0 * fz, fz], 1))
    ctx = gpu_context(mesh, dm, params)
    ctx.set_params(params2)
    x = random_state(dm, seed=2, scale=0.1)
    r = ctx.assemble(x, want_jacobian=False)
    r_ref, _ = oracle_problem(mesh, dm, params2).residual_jacobian(x, want_jac=False)
    assert np.abs(r - r_ref).max() <= 1e-12 * np.abs(r_ref).max()
