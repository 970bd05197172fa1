"""Host check of the LU form of the multifrontal fronts (the algorithm of csrc/mf_numeric.cu).

A numpy emulation of the device algorithm, step for step, on the library's own symbolic
structure (csrc/mf_symbolic.cpp, compiled with g++):

* factorization: per front, blocked right-looking LU of the eliminated block by panels of PW
  pivots; every NB-pivot diagonal block is replaced by its inverse (partial pivoting inside the
  block only), the rows below it are multiplied by that inverse (L), the rest of the panel is
  updated, the panel's later blocks update their rows beyond the panel (U), and the trailing
  submatrix takes one rank-PW update.  A front then holds [D⁻¹\\L11 , U11 ; L21 , S].
* solves: both sweeps in super-blocks of SB rows: a substitution chain over the NB-blocks
  inside a super-block, and a GEMV for the rows (forward) or columns (backward) beyond it; the
  transposed solve (adjoint) runs the same structure on Uᵀ and Lᵀ.

The emulated factors must solve the Jacobian (and its transpose) to round-off.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from helpers import hunt_case, oracle_problem
from test_mf_host import harness, symbolic  # noqa: F401  (fixture)

NB, PW = 64, 128


def factor_front(M, E):
    """In-place LU form of the front M (n x n) over its first E pivots."""
    for p in range(0, E, PW):
        pw = min(PW, E - p)
        for k in range(p, p + pw, NB):
            kb = min(NB, p + pw - k)
            K = slice(k, k + kb)
            P = np.linalg.inv(M[K, K])
            M[k + kb:, K] = M[k + kb:, K] @ P
            M[k + kb:, k + kb:p + pw] -= M[k + kb:, K] @ M[K, k + kb:p + pw]
            M[K, K] = P
        for k in range(p + NB, p + pw, NB):
            kb = min(NB, p + pw - k)
            M[k:k + kb, p + pw:] -= M[k:k + kb, p:k] @ M[p:k, p + pw:]
        M[p + pw:, p + pw:] -= M[p + pw:, p:p + pw] @ M[p:p + pw, p + pw:]


def blocks(s0, s1):
    return [(k, min(k + NB, s1)) for k in range(s0, s1, NB)]


def emulate_lu(S, A, reg, SB):
    lev, storage = S["levels"], int(S["sizes"][0])
    F = np.zeros(storage)
    n_of = lambda f: int(lev[S["f_level"][f]][2])
    E_of = lambda f: int(lev[S["f_level"][f]][0])
    front = lambda f: F[S["f_off"][f]:S["f_off"][f] + n_of(f) ** 2].reshape(n_of(f), n_of(f), order="F")
    for l in range(len(lev)):
        E, B, n, first, count, off, ab, ae, cb, ce = (int(v) for v in lev[l])
        for f in range(first, first + count):
            for i in range(S["f_ne"][f], E):
                F[S["f_off"][f] + i + i * n] = 1.0
        F[S["ah_dst"][ab:ae]] = A.data[S["ah_src"][ab:ae]]
        if l == len(lev) - 1:
            F[S["reg_dst"]] += reg[S["reg_dof"]]
        for c in S["child_list"][cb:ce]:
            nb = S["f_nb"][c]
            pos = S["ea_pos"][S["ea_ptr"][c]:S["ea_ptr"][c] + nb]
            Ec = E_of(c)
            front(S["f_parent"][c])[np.ix_(pos, pos)] += front(c)[Ec:Ec + nb, Ec:Ec + nb]
        for f in range(first, first + count):
            factor_front(front(f), E)

    def idx(f):
        return (S["elim"][S["elim_ptr"][f]:S["elim_ptr"][f + 1]], S["bnd"][S["bnd_ptr"][f]:S["bnd_ptr"][f + 1]])

    def sbs(E):
        return [(s, min(s + SB, E)) for s in range(0, E, SB)]

    def solve(b0):
        b, x, ts = b0.copy(), np.zeros_like(b0), {}
        for l in range(len(lev)):
            E, B, n, first, count = (int(v) for v in lev[l][:5])
            for f in range(first, first + count):
                el, bd = idx(f)
                M = front(f)
                t = np.zeros(E)
                t[:len(el)] = b[el]
                for s0, s1 in sbs(E):
                    for k, k1 in blocks(s0, s1):          # unit lower chain inside the super-block
                        t[k1:s1] -= M[k1:s1, k:k1] @ t[k:k1]
                    t[s1:E] -= M[s1:E, s0:s1] @ t[s0:s1]  # rows beyond: eliminated ...
                    np.add.at(b, bd, -(M[E:E + len(bd), s0:s1] @ t[s0:s1]))  # ... and boundary
                ts[f] = t
        for l in range(len(lev) - 1, -1, -1):
            E, B, n, first, count = (int(v) for v in lev[l][:5])
            for f in range(first, first + count):
                el, bd = idx(f)
                M = front(f)
                z = ts[f].copy()
                xe = np.zeros(E)
                for s0, s1 in reversed(sbs(E)):
                    z[s0:s1] -= M[s0:s1, s1:E] @ xe[s1:E] + M[s0:s1, E:E + len(bd)] @ x[bd]
                    for k, k1 in reversed(blocks(s0, s1)):  # upper chain with the block inverses
                        xe[k:k1] = M[k:k1, k:k1] @ (z[k:k1] - M[k:k1, k1:s1] @ xe[k1:s1])
                x[el] = xe[:len(el)]
        return x

    def solve_t(b0):
        b, x, ts = b0.copy(), np.zeros_like(b0), {}
        for l in range(len(lev)):
            E, B, n, first, count = (int(v) for v in lev[l][:5])
            for f in range(first, first + count):
                el, bd = idx(f)
                M = front(f)
                t = np.zeros(E)
                t[:len(el)] = b[el]
                for s0, s1 in sbs(E):
                    for k, k1 in blocks(s0, s1):          # Uᵀ chain: y_k = D_k⁻ᵀ t_k
                        t[k:k1] = M[k:k1, k:k1].T @ t[k:k1]
                        t[k1:s1] -= M[k:k1, k1:s1].T @ t[k:k1]
                    t[s1:E] -= M[s0:s1, s1:E].T @ t[s0:s1]
                    np.add.at(b, bd, -(M[s0:s1, E:E + len(bd)].T @ t[s0:s1]))
                ts[f] = t
        for l in range(len(lev) - 1, -1, -1):
            E, B, n, first, count = (int(v) for v in lev[l][:5])
            for f in range(first, first + count):
                el, bd = idx(f)
                M = front(f)
                z = ts[f].copy()
                xe = np.zeros(E)
                for s0, s1 in reversed(sbs(E)):
                    z[s0:s1] -= M[s1:E, s0:s1].T @ xe[s1:E] + M[E:E + len(bd), s0:s1].T @ x[bd]
                    for k, k1 in reversed(blocks(s0, s1)):  # Lᵀ chain (unit upper)
                        xe[k:k1] = z[k:k1] - M[k1:s1, k:k1].T @ xe[k1:s1]
                x[el] = xe[:len(el)]
        return x

    return solve, solve_t


def _regularised(mesh, dm, params, S, A):
    X = mesh.cell_coords()
    vol = np.abs(np.linalg.det(np.stack([X[:, 1] - X[:, 0], X[:, 2] - X[:, 0], X[:, 4] - X[:, 0]], 2)))
    gd = dm.global_cell_dofs()
    reg = np.zeros(dm.ndofs)
    for k in range(4):
        reg[gd[:, 81 + k]] = -vol / params["beta"] / 3
    for k in range(8):
        reg[gd[:, 121 + k]] = -vol / 27
    K = A + sp.diags(np.where(np.isin(np.arange(dm.ndofs), S["reg_dof"]), reg, 0.0))
    return reg, K


@pytest.mark.parametrize("SB", [64, 192, 512])
def test_lu_fronts_solve_the_jacobian(harness, SB):  # noqa: F811
    mesh, dm, params = hunt_case(nc=(6, 5), nz=3, Ha=10.0, Re=10.0, cw=0.01, Lz=0.2)
    prob = oracle_problem(mesh, dm, params)
    r, A = prob.residual_jacobian(np.zeros(dm.ndofs))
    S = symbolic(harness, mesh, dm, True)
    reg, K = _regularised(mesh, dm, params, S, A)
    solve, solve_t = emulate_lu(S, A, reg, SB)
    rng = np.random.default_rng(0)
    x = rng.standard_normal(dm.ndofs)
    assert np.linalg.norm(solve(K @ x) - x) <= 1e-8 * np.linalg.norm(x)
    assert np.linalg.norm(solve_t(K.T @ x) - x) <= 1e-8 * np.linalg.norm(x)


def test_lu_fronts_solve_the_uj_block(harness):  # noqa: F811
    """The (u,j) block of the Badia2024 preconditioner (no regularisation)."""
    mesh, dm, params = hunt_case(nc=(6, 5), nz=3, Ha=10.0, Re=10.0, cw=0.01, Lz=0.2, zeta_u=10.0, zeta_j=10.0)
    prob = oracle_problem(mesh, dm, params)
    r, A = prob.residual_jacobian(np.zeros(dm.ndofs))
    S = symbolic(harness, mesh, dm, False)
    solve, solve_t = emulate_lu(S, A, np.zeros(dm.ndofs), 128)
    uj = np.zeros(dm.ndofs, bool)
    uj[S["elim"]] = True
    Auj = A[uj][:, uj]
    rng = np.random.default_rng(1)
    x = np.zeros(dm.ndofs)
    x[uj] = rng.standard_normal(int(uj.sum()))
    b = np.zeros(dm.ndofs)
    b[uj] = Auj @ x[uj]
    assert np.linalg.norm(solve(b)[uj] - x[uj]) <= 1e-8 * np.linalg.norm(x)
    bt = np.zeros(dm.ndofs)
    bt[uj] = Auj.T @ x[uj]
    assert np.linalg.norm(solve_t(bt)[uj] - x[uj]) <= 1e-8 * np.linalg.norm(x)
