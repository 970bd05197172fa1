"""GPU Newton solve (FGMRES + Badia2024 block preconditioner with the multifrontal (u,j)
solve) against the oracle's FP64 Newton + direct-solve solution."""
import numpy as np
import pytest

from helpers import gpu_context, hunt_case, oracle_problem
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def field_rel_errors(dm, x, xref, p_scale=1.0):
    """Relative L2 error of each field's dof vector.  The pressure is compared modulo a
    constant and relative to max(‖p_ref‖, p_scale·sqrt(n_p)): the fully developed Hunt
    pressure is constant, so its reference vector is round-off after the gauge."""
    out = {}
    for f in ("u", "p", "j", "phi"):
        a = x[dm.offsets[f]:dm.offsets[f] + dm.nfree[f]].copy()
        b = xref[dm.offsets[f]:dm.offsets[f] + dm.nfree[f]].copy()
        den = max(np.linalg.norm(b), 1e-300)
        if f == "p":
            a -= a.mean()
            b -= b.mean()
            den = max(np.linalg.norm(b), p_scale * np.sqrt(len(b)))
        out[f] = np.linalg.norm(a - b) / den
    return out


CASES = {
    # the shape of the CPU-runnable configuration: 8x8x3, Lz=0.2, Ha=10, Re=10, cw=0.01
    "cfg1": dict(nc=(8, 8), nz=3, Ha=10.0, Re=10.0, cw=0.01, Lz=0.2),
    # stretched, high Ha, small
    "ha200": dict(nc=(6, 6), nz=4, Ha=200.0, Re=10.0, beta_map=2.5, cw=0.1, Lz=0.2),
}


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("precision", [0, 1])
def test_newton_matches_direct_oracle(gpu_lib, name, precision):
    mesh, dm, params = hunt_case(**CASES[name])
    prob = oracle_problem(mesh, dm, params)
    xref, info = O.newton_direct(prob, np.zeros(dm.ndofs), gauge=[dm.offsets["p"]], rtol=1e-13, maxiter=10)
    ctx = gpu_context(mesh, dm, params)
    # Stop on the relative residual alone: at Ha = 200 an absolute 1e-10 leaves p at ~1e-8.
    x, rep, rc = ctx.newton_solve(np.zeros(dm.ndofs), precision=precision, max_newton=12, newton_rtol=1e-12,
                                  newton_atol=0.0, restart=40, max_linear=400,
                                  linear_rtol=1e-4 if precision else 1e-8)
    assert rc == 0 and rep["converged"], rep
    errs = field_rel_errors(dm, x, xref)
    for f, e in errs.items():
        assert e <= 1e-8, (f, e, rep)


def test_badia2024_block_preconditioner_fp64(gpu_lib):
    """The Badia2024 block-triangular preconditioner (src/Solvers/badia2024.jl:2-48), which
    needs the augmented-Lagrangian weights; they vanish at the discrete solution, so the
    solution is the one of the plain weak form."""
    mesh, dm, params = hunt_case(nc=(8, 8), nz=3, Ha=10.0, Re=10.0, cw=0.01, Lz=0.2, zeta_u=10.0, zeta_j=10.0)
    mesh0, dm0, params0 = hunt_case(nc=(8, 8), nz=3, Ha=10.0, Re=10.0, cw=0.01, Lz=0.2)
    prob = oracle_problem(mesh0, dm0, params0)
    xref, info = O.newton_direct(prob, np.zeros(dm0.ndofs), gauge=[dm0.offsets["p"]], rtol=1e-13, maxiter=10)
    ctx = gpu_context(mesh, dm, params)
    x, rep, rc = ctx.newton_solve(np.zeros(dm.ndofs), precision=0, max_newton=12, newton_rtol=1e-10,
                                  newton_atol=1e-10, restart=40, max_linear=400, linear_rtol=1e-8,
                                  preconditioner=1)
    assert rc == 0 and rep["converged"], rep
    assert rep["linear_iters"] <= 60
    errs = field_rel_errors(dm, x, xref)
    for f in ("u", "j", "phi"):
        assert errs[f] <= 1e-7, (f, errs)



def test_stagnation_safeguard_refactors_then_falls_back_to_fp64(gpu_lib, monkeypatch):
    """The mixed-precision safeguard: the diagnostic stagnation test (GBMHD_STAG_ITERS=1,
    GBMHD_STAG_REL=0) declares every FP32-preconditioned linear solve stagnated after one
    iteration, so the first step refactors in FP32, stagnates again and moves to FP64 factors
    for the rest of the solve.  Two refactorizations, and the solution still matches the
    oracle's direct Newton."""
    monkeypatch.setenv("GBMHD_STAG_ITERS", "1")
    monkeypatch.setenv("GBMHD_STAG_REL", "0")
    mesh, dm, params = hunt_case(**CASES["cfg1"])
    prob = oracle_problem(mesh, dm, params)
    xref, _ = O.newton_direct(prob, np.zeros(dm.ndofs), gauge=[dm.offsets["p"]], rtol=1e-13, maxiter=10)
    ctx = gpu_context(mesh, dm, params)
    x, rep, rc = ctx.newton_solve(np.zeros(dm.ndofs), precision=1, max_newton=12, newton_rtol=1e-12,
                                  newton_atol=0.0, restart=40, max_linear=400, linear_rtol=1e-4)
    assert rc == 0 and rep["converged"], rep
    assert rep["pc_refactorizations"] == 2, rep
    for f, e in field_rel_errors(dm, x, xref).items():
        assert e <= 1e-8, (f, e, rep)


def test_sweep_wait_timeout_is_reported(gpu_lib, monkeypatch):
    """A TMA sweep whose mbarrier wait gives up (here: a wait limit of zero spins, set through
    the diagnostic GBMHD_SWEEP_WAIT_LIMIT before the factors are created) drains its copies in
    flight, sets the device error flag, and the Newton step that used it fails with -3 and the
    timeout message.  A new context (default limit) on the same device then solves normally."""
    from gbmhd.lib import GbmhdError
    mesh, dm, params = hunt_case(**CASES["cfg1"])
    monkeypatch.setenv("GBMHD_SWEEP_WAIT_LIMIT", "0")
    monkeypatch.setenv("GBMHD_STAG_ITERS", "100000")
    ctx = gpu_context(mesh, dm, params)
    with pytest.raises(GbmhdError, match="timed out"):
        ctx.newton_solve(np.zeros(dm.ndofs), precision=1, max_newton=3, newton_rtol=1e-12, newton_atol=0.0,
                         restart=20, max_linear=20, linear_rtol=1e-4)
    monkeypatch.delenv("GBMHD_SWEEP_WAIT_LIMIT")
    monkeypatch.delenv("GBMHD_STAG_ITERS")
    ctx2 = gpu_context(mesh, dm, params)
    x, rep, rc = ctx2.newton_solve(np.zeros(dm.ndofs), precision=1, max_newton=12, newton_rtol=1e-12,
                                   newton_atol=0.0, restart=40, max_linear=400, linear_rtol=1e-4)
    assert rc == 0 and rep["converged"], rep
