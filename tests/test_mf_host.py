"""Host logic of the multifrontal factorization, checked on the CPU.

The library's symbolic analysis (csrc/mf_symbolic.cpp, csrc/pattern.cpp) is compiled
with g++ and run on small meshes, and its structure is checked here; test_mf_lu_host.py
emulates the numeric phase on it."""
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
    with tempfile.TemporaryDirectory() as d:  # the arrays are read into memory, the files removed
        rc = harness.mf_harness(C.c_int64(mesh.ncells), X.ctypes.data_as(C.c_void_p),
                                gd.ctypes.data_as(C.c_void_p), C.c_int64(dm.ndofs), C.c_int(1 if mono else 0),
                                d.encode())
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


@pytest.mark.parametrize("mono", [True, False])
@pytest.mark.parametrize("case", [dict(nc=(8, 8), nz=3, Ha=10.0, Re=10.0, cw=0.01, Lz=0.2),
                                  dict(nc=(16, 16), nz=4, Ha=500.0, Re=1.0, beta_map=3.0, cw=0.1, Lz=0.2)])
def test_groups_of_one_height_are_independent(harness, mono, case):
    """The sweeps and the FP32 factorization run the level groups of one tree height side by
    side (csrc/mf_numeric.cu: lheight from f_parent, one run per height).  That needs: a
    parent follows its children in the front order (the heights are computed in one pass);
    the fronts of a group share one height and a height's groups are consecutive; no front's
    parent lies in a group of its own height; and every boundary dof of a front is
    eliminated by one of its ancestors, so groups of one height write disjoint eliminated
    dofs and only add (atomically) into higher fronts' dofs."""
    mesh, dm, params = hunt_case(**case)
    S = symbolic(harness, mesh, dm, mono)
    fp = S["f_parent"]
    nf = len(fp)
    fh = np.zeros(nf, np.int64)
    for f in range(nf):
        if fp[f] >= 0:
            assert fp[f] > f
            fh[fp[f]] = max(fh[fp[f]], fh[f] + 1)
    lev_h = []
    lev_of = np.zeros(nf, np.int64)
    for l, L in enumerate(S["levels"]):
        first, count = int(L[3]), int(L[4])
        assert count > 0
        assert len(set(fh[first:first + count].tolist())) == 1
        lev_h.append(int(fh[first]))
        lev_of[first:first + count] = l
    assert lev_h == sorted(lev_h)  # each height's groups are consecutive
    for f in range(nf):
        if fp[f] >= 0:
            assert lev_h[lev_of[fp[f]]] > lev_h[lev_of[f]]
    owner = np.full(dm.ndofs, -1, np.int64)
    for f in range(nf):
        owner[S["elim"][S["elim_ptr"][f]:S["elim_ptr"][f + 1]]] = f
    for f in range(nf):
        anc, p = set(), fp[f]
        while p >= 0:
            anc.add(int(p))
            p = fp[p]
        for d in S["bnd"][S["bnd_ptr"][f]:S["bnd_ptr"][f + 1]]:
            assert int(owner[d]) in anc, (f, d)
    # at least one height has several groups in the larger case (the concurrency is exercised)
    if case["nc"] == (16, 16):
        assert any(lev_h.count(h) > 1 for h in set(lev_h))
