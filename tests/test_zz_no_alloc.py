"""Allocation-free parameter gradient (gbmhd_param_gradient_noalloc) through the C ABI.

The entry point turns an adjoint vector λ into dJ/dγ and dJ/dcw with scratch held in a
file-scope device array.  It must agree with gbmhd_adjoint (which allocates) on the same
state and λ, on two calls in a row, and the second call must leave the device's free
memory unchanged.  The file name sorts last so that the test also runs after every other
GPU test in one session; it passes alone too.
"""
import numpy as np
import pytest

from gbmhd.objectives import flow_rate
from helpers import gpu_context, hunt_case

pytestmark = pytest.mark.gpu


def test_noalloc_gradient_matches_adjoint(gpu_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    # Thin-wall Hunt duct: both γ and cw enter the residual.
    mesh, dm, params = hunt_case(nc=(6, 6), nz=4, Ha=20.0, Re=10.0, beta_map=2.5, cw=0.1, Lz=0.2)
    ctx = gpu_context(mesh, dm, params)
    x, rep, rc = ctx.newton_solve(np.zeros(dm.ndofs), precision=0, max_newton=12, newton_rtol=1e-12,
                                  newton_atol=1e-13, restart=40, max_linear=400, linear_rtol=1e-8)
    assert rc == 0, rep
    g = flow_rate(mesh, dm, 0.1)
    ref, lam, arep, arc = ctx.adjoint(x, g, with_cells=False, precision=0, restart=40, max_linear=400,
                                      linear_rtol=1e-10)
    assert arc == 0, arep
    assert ref[0] != 0.0 and ref[1] != 0.0, ref

    d_x = torch.from_numpy(x).cuda()
    d_lam = torch.from_numpy(lam).cuda()
    d_out = torch.empty(2, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    results = []
    for call in range(2):
        d_out.fill_(float("nan"))
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        rc = gpu_lib.gbmhd_param_gradient_noalloc(ctx.h, d_x.data_ptr(), d_lam.data_ptr(), d_out.data_ptr())
        assert rc == 0, gpu_lib.gbmhd_last_error(ctx.h)
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info()[0]
        if call == 1:  # the first call may load the module that holds the scratch array
            assert free_after == free_before, (free_before, free_after)
        res = d_out.cpu().numpy().copy()
        results.append(res)
        # Same math as gbmhd_adjoint's ∂R/∂θ kernels, summed in another order.
        assert abs(res[0] - ref[0]) <= 1e-11 * abs(ref[0]), (call, res, ref[:2])
        assert abs(res[1] - ref[1]) <= 1e-11 * abs(ref[1]), (call, res, ref[:2])
    # fixed reduction order: the two calls agree bit for bit
    assert np.array_equal(results[0], results[1]), results


def test_noalloc_rejects_null_arguments(gpu_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    mesh, dm, params = hunt_case(nc=(4, 4), nz=3)
    ctx = gpu_context(mesh, dm, params)
    d_out = torch.empty(2, dtype=torch.float64, device="cuda")
    rc = gpu_lib.gbmhd_param_gradient_noalloc(ctx.h, None, None, d_out.data_ptr())
    assert rc == -1
    assert b"NULL" in gpu_lib.gbmhd_last_error(ctx.h)


def test_noalloc_without_thin_wall_facets(gpu_lib):
    """A duct without thin-wall facets: dJ/dcw is 0 and dJ/dγ still matches gbmhd_adjoint."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    mesh, dm, params = hunt_case(nc=(4, 4), nz=4, Ha=10.0, Re=10.0, cw=0.0, Lz=0.2)
    assert params["facets"] is None
    ctx = gpu_context(mesh, dm, params)
    x, rep, rc = ctx.newton_solve(np.zeros(dm.ndofs), precision=0, max_newton=12, newton_rtol=1e-12,
                                  newton_atol=1e-13, restart=40, max_linear=400, linear_rtol=1e-8)
    assert rc == 0, rep
    ref, lam, arep, arc = ctx.adjoint(x, flow_rate(mesh, dm, 0.1), with_cells=False, precision=0, restart=40,
                                      max_linear=400, linear_rtol=1e-10)
    assert arc == 0, arep
    d_x = torch.from_numpy(x).cuda()
    d_lam = torch.from_numpy(lam).cuda()
    d_out = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = gpu_lib.gbmhd_param_gradient_noalloc(ctx.h, d_x.data_ptr(), d_lam.data_ptr(), d_out.data_ptr())
    assert rc == 0, gpu_lib.gbmhd_last_error(ctx.h)
    torch.cuda.synchronize()
    res = d_out.cpu().numpy()
    assert res[1] == 0.0, res
    assert abs(res[0] - ref[0]) <= 1e-11 * abs(ref[0]), (res, ref[:2])


def test_noalloc_rejects_more_facets_than_the_scratch_holds(gpu_lib):
    """65,537 facet entries (one wall face repeated, τ = 0) exceed the 65,536 facet slots:
    the call returns -1 with a message and launches nothing."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    mesh, dm, params = hunt_case(nc=(4, 4), nz=3, Ha=10.0, Re=10.0, cw=0.1, Lz=0.2)
    f = params["facets"]
    n = 65537
    params["facets"] = dict(cell=np.full(n, f["cell"][0], np.int32), lface=np.full(n, f["lface"][0], np.int8),
                            tau=np.zeros(n), cw=np.full(n, 0.1), jw=np.zeros(n), phi0=None)
    ctx = gpu_context(mesh, dm, params)
    d = torch.zeros(ctx.ndofs, dtype=torch.float64, device="cuda")
    d_out = torch.empty(2, dtype=torch.float64, device="cuda")
    rc = gpu_lib.gbmhd_param_gradient_noalloc(ctx.h, d.data_ptr(), d.data_ptr(), d_out.data_ptr())
    assert rc == -1
    assert b"facets exceed the scratch limit" in gpu_lib.gbmhd_last_error(ctx.h)
