"""Sudden expansion (non-zero Dirichlet inlet, natural outlet, insulating walls) on the GPU
against the oracle's FP64 direct Newton."""
import numpy as np
import pytest

from helpers import expansion_case, gpu_context, oracle_problem
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _rel(a, b, modulo_const=False):
    a, b = a.copy(), b.copy()
    if modulo_const:
        a -= a.mean(); b -= b.mean()
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("precision", [0, 1])
def test_expansion_newton_matches_oracle(gpu_lib, precision):
    mesh, dm, params = expansion_case()
    prob = oracle_problem(mesh, dm, params)
    # insulating walls everywhere: φ is defined up to a constant
    xref, info = O.newton_direct(prob, np.zeros(dm.ndofs), gauge=[dm.offsets["phi"]], rtol=1e-13, maxiter=12)
    ctx = gpu_context(mesh, dm, params)
    x, rep, rc = ctx.newton_solve(np.zeros(dm.ndofs), precision=precision, max_newton=15, newton_rtol=1e-11,
                                  newton_atol=1e-14, restart=60, max_linear=400,
                                  linear_rtol=1e-4 if precision else 1e-8)
    assert rc == 0, rep
    s = dm.split(x)
    r = dm.split(xref)
    assert _rel(s["u"], r["u"]) <= 1e-8
    assert _rel(s["j"], r["j"]) <= 1e-8
    assert _rel(s["p"], r["p"]) <= 1e-8
    assert _rel(s["phi"], r["phi"], modulo_const=True) <= 1e-8
