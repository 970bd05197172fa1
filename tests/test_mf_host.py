"""Host logic of the multifrontal factorization, checked on the CPU.

The library's symbolic analysis (csrc/mf_symbolic.cpp, csrc/pattern.cpp) is compiled
with g++ and run on small meshes; a numpy emulation of the numeric phase (front
assembly, extend-add, Gauss-Jordan elimination, both sweeps) then has to solve the
Jacobian assembled by the oracle."""
import ctypes as C
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest
import scipy.sparse as sp

from helpers import hunt_case, oracle_problem

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "gridapmhd.jl_gb300", "csrc")


@pytest.fixture(scope="module")
def harness():
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    d = tempfile.mkdtemp()
    so = os.path.join(d, "libmfh.so")
    inc = ["-I" + CSRC, "-I/usr/local/cuda/include"]
    subprocess.run(["g++", "-O2", "-fopenmp", "-fPIC", "-shared", "-std=c++17", *inc, "-o", so,
                    os.path.join(os.path.dirname(__file__), "mf_harness.cpp"), os.path.join(CSRC, "mf_symbolic.cpp"),
                    os.path.join(CSRC, "pattern.cpp")], check=True)
    return C.CDLL(so)


def _load(d, name, dt):
    return np.fromfile(os.path.join(d, name), dtype=dt)


def symbolic(harness, mesh, dm, mono):
    gd = np.ascontiguousarray(dm.global_cell_dofs().astype(np.int32))
    X = np.ascontiguousarray(mesh.cell_coords())
    d = tempfile.mkdtemp()
    rc = harness.mf_harness(C.c_int64(mesh.ncells), X.ctypes.data_as(C.c_void_p), gd.ctypes.data_as(C.c_void_p),
                            C.c_int64(dm.ndofs), C.c_int(1 if mono else 0), d.encode())
    assert rc == 0
    S = {k: _load(d, k, t) for k, t in (("rowptr", np.int64), ("col", np.int32), ("levels", np.int64),
                                        ("f_ne", np.int32), ("f_nb", np.int32), ("f_level", np.int32),
                                        ("f_parent", np.int32), ("f_off", np.int64), ("elim_ptr", np.int64),
                                        ("bnd_ptr", np.int64), ("elim", np.int32), ("bnd", np.int32),
                                        ("ah_src", np.int32), ("ah_dst", np.int64), ("child_list", np.int32),
                                        ("ea_ptr", np.int64), ("ea_pos", np.int32), ("reg_dst", np.int64),
                                        ("reg_dof", np.int32), ("sizes", np.int64))}
    S["levels"] = S["levels"].reshape(-1, 10)
    return S


def emulate(S, A, reg):
    """Factor with the library's algorithm in FP64 and return the solve operator."""
    lev, storage = S["levels"], int(S["sizes"][0])
    F = np.zeros(storage)
    n_of = lambda f: int(lev[S["f_level"][f]][2])
    E_of = lambda f: int(lev[S["f_level"][f]][0])
    for l in range(len(lev)):
        E, B, n, first, count, off, ab, ae, cb, ce = (int(v) for v in lev[l])
        for f in range(first, first + count):
            for i in range(S["f_ne"][f], E):
                F[S["f_off"][f] + i + i * n] = 1.0
        F[S["ah_dst"][ab:ae]] = A.data[S["ah_src"][ab:ae]]
        if l == len(lev) - 1:
            F[S["reg_dst"]] += reg[S["reg_dof"]]
        for c in S["child_list"][cb:ce]:
            p, nc, Ec, nb = S["f_parent"][c], n_of(c), E_of(c), S["f_nb"][c]
            Mc = F[S["f_off"][c]:S["f_off"][c] + nc * nc].reshape(nc, nc, order="F")
            Mp = F[S["f_off"][p]:S["f_off"][p] + n_of(p) ** 2].reshape(n_of(p), n_of(p), order="F")
            pos = S["ea_pos"][S["ea_ptr"][c]:S["ea_ptr"][c] + nb]
            Mp[np.ix_(pos, pos)] += Mc[Ec:Ec + nb, Ec:Ec + nb]
        for f in range(first, first + count):
            M = F[S["f_off"][f]:S["f_off"][f] + n * n].reshape(n, n, order="F")
            P = np.linalg.inv(M[:E, :E])
            W = P @ M[:E, E:]
            G = -M[E:, :E] @ P
            Sc = M[E:, E:] - M[E:, :E] @ W
            M[:E, :E], M[:E, E:], M[E:, :E], M[E:, E:] = P, W, G, Sc

    def solve(b0):
        b, x, ts = b0.copy(), np.zeros_like(b0), {}
        for l in range(len(lev)):
            E, B, n, first, count = (int(v) for v in lev[l][:5])
            for f in range(first, first + count):
                el = S["elim"][S["elim_ptr"][f]:S["elim_ptr"][f + 1]]
                bd = S["bnd"][S["bnd_ptr"][f]:S["bnd_ptr"][f + 1]]
                t = np.zeros(E)
                t[:len(el)] = b[el]
                ts[f] = t
                M = F[S["f_off"][f]:S["f_off"][f] + n * n].reshape(n, n, order="F")
                if len(bd):
                    np.add.at(b, bd, M[E:E + len(bd), :E] @ t)
        for l in range(len(lev) - 1, -1, -1):
            E, B, n, first, count = (int(v) for v in lev[l][:5])
            for f in range(first, first + count):
                el = S["elim"][S["elim_ptr"][f]:S["elim_ptr"][f + 1]]
                bd = S["bnd"][S["bnd_ptr"][f]:S["bnd_ptr"][f + 1]]
                M = F[S["f_off"][f]:S["f_off"][f] + n * n].reshape(n, n, order="F")
                x[el] = M[:len(el), :E] @ ts[f] - M[:len(el), E:E + len(bd)] @ x[bd]
        return x
    return solve


@pytest.mark.parametrize("mono", [True, False])
def test_symbolic_structure(harness, mono):
    mesh, dm, params = hunt_case(nc=(6, 5), nz=3, Ha=10.0, Re=10.0, cw=0.01, Lz=0.2)
    S = symbolic(harness, mesh, dm, mono)
    gd = dm.global_cell_dofs()
    sysd = np.unique(gd[:, np.r_[0:129] if mono else np.r_[0:81, 85:121]])
    sysd = sysd[sysd >= 0]
    # every dof of the system is eliminated exactly once
    assert np.array_equal(np.sort(S["elim"]), sysd)
    # the root has no boundary; every other front's boundary lies in its parent's front
    root = len(S["f_ne"]) - 1
    assert S["f_nb"][root] == 0 and S["f_parent"][root] == -1
    # arrowheads cover each nonzero of the system block exactly once
    nnz_sys = 0
    rp, col = S["rowptr"], S["col"]
    inset = np.zeros(dm.ndofs, bool)
    inset[sysd] = True
    for r in sysd:
        nnz_sys += int(inset[col[rp[r]:rp[r + 1]]].sum())
    assert len(S["ah_src"]) == nnz_sys
    assert len(np.unique(S["ah_dst"])) == len(S["ah_dst"])


@pytest.mark.parametrize("mono", [True, False])
@pytest.mark.parametrize("case", [dict(nc=(6, 5), nz=3, Ha=10.0, Re=10.0, cw=0.01, Lz=0.2),
                                  dict(nc=(16, 16), nz=4, Ha=500.0, Re=1.0, beta_map=3.0, cw=0.1, Lz=0.2)])
def test_levels_keep_eliminated_and_boundary_dofs_apart(harness, mono, case):
    """The TMA sweeps read b at a level's eliminated dofs while other CTAs of the same
    launch add into b at the level's boundary dofs, and the backward sweep adds into x at
    the eliminated dofs while reading x at the boundary ones.  Both need: no dof is
    eliminated by one front of a level and a boundary dof of another front of that level,
    and each front's eliminated and boundary dofs are distinct."""
    mesh, dm, params = hunt_case(**case)
    S = symbolic(harness, mesh, dm, mono)
    for L in S["levels"]:
        E, B, n, first, count = (int(v) for v in L[:5])
        el = np.concatenate([S["elim"][S["elim_ptr"][f]:S["elim_ptr"][f + 1]] for f in range(first, first + count)])
        bd = np.concatenate([S["bnd"][S["bnd_ptr"][f]:S["bnd_ptr"][f + 1]] for f in range(first, first + count)])
        assert len(np.unique(el)) == len(el)
        assert len(np.intersect1d(el, bd)) == 0
        for f in range(first, first + count):
            b = S["bnd"][S["bnd_ptr"][f]:S["bnd_ptr"][f + 1]]
            assert len(np.unique(b)) == len(b)


def test_emulated_factorization_solves_the_jacobian(harness):
    from oracle import oracle as O  # noqa: F401
    mesh, dm, params = hunt_case(nc=(6, 5), nz=3, Ha=10.0, Re=10.0, cw=0.01, Lz=0.2)
    prob = oracle_problem(mesh, dm, params)
    r, A = prob.residual_jacobian(np.zeros(dm.ndofs))
    S = symbolic(harness, mesh, dm, True)
    assert np.array_equal(S["rowptr"], A.indptr) and np.array_equal(S["col"], A.indices)
    # root regularisation of the global constant modes, as the library does
    X = mesh.cell_coords()
    vol = np.abs(np.linalg.det(np.stack([X[:, 1] - X[:, 0], X[:, 2] - X[:, 0], X[:, 4] - X[:, 0]], 2)))
    gd = dm.global_cell_dofs()
    reg = np.zeros(dm.ndofs)
    for k in range(4):
        reg[gd[:, 81 + k]] = -vol / params["beta"] / 3
    for k in range(8):
        reg[gd[:, 121 + k]] = -vol / 27
    solve = emulate(S, A, reg)
    rng = np.random.default_rng(0)
    x = rng.standard_normal(dm.ndofs)
    K = A + sp.diags(np.where(np.isin(np.arange(dm.ndofs), S["reg_dof"]), reg, 0.0))
    assert np.linalg.norm(solve(K @ x) - x) <= 1e-8 * np.linalg.norm(x)
