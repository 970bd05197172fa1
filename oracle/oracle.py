"""FP64 CPU oracle harness (test infrastructure only; never on the product path).

Drives ``liboracle.so`` (mhd_oracle.cpp) and restates, with numpy/scipy:

* Gridap's ``SparseMatrixAssembler`` for the consecutive [u;p;j;φ] free
  vector: every touched element block is inserted in full, Dirichlet rows and
  columns are dropped (GridapMHD src/main.jl:218-224);
* the ``:julia`` solver, ``NewtonSolver(LUSolver())`` (src/main.jl:181-186),
  with SuperLU in place of UMFPACK and an explicit tolerance;
* the post-processing norms of ``_hunt`` (src/Applications/hunt.jl:238-260),
  including the analytic Hunt solution (src/Applications/hunt.jl:372-457).

Constant-mode gauges: when u is Dirichlet on the whole boundary, the pressure
is defined up to a constant; when j·n is Dirichlet on the whole boundary, φ
is too.  The direct solve drops one dof of each such field (row and column);
comparisons are then made modulo the constant.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess
from dataclasses import dataclass, field
from typing import Optional, Sequence

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


def build():
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        _LIB = C.CDLL(path)
        _LIB.orc_assemble_cells.restype = None
        _LIB.orc_param_derivs.restype = None
        _LIB.orc_param_derivs_ab.restype = None
        _LIB.orc_eval_fields.restype = None
    return _LIB


class OrcFluid(C.Structure):
    _fields_ = [("alpha", C.c_double), ("beta", C.c_double), ("gamma", C.c_double), ("sigma", C.c_double),
                ("B", C.c_double * 3), ("f", C.c_double * 3), ("g", C.c_double * 3),
                ("zeta_u", C.c_double), ("zeta_j", C.c_double), ("convection", C.c_int32),
                ("f_cell", C.POINTER(C.c_double))]


class OrcFacets(C.Structure):
    _fields_ = [("n", C.c_int64), ("cell", C.POINTER(C.c_int32)), ("lface", C.POINTER(C.c_int8)),
                ("tau", C.POINTER(C.c_double)), ("cw", C.POINTER(C.c_double)), ("jw", C.POINTER(C.c_double)),
                ("phi0", C.POINTER(C.c_double))]


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


@dataclass
class Fluid:
    alpha: float = 1.0
    beta: float = 1.0
    gamma: float = 1.0
    sigma: float = 1.0
    B: Sequence[float] = (0.0, 1.0, 0.0)
    f: Sequence[float] = (0.0, 0.0, 0.0)
    g: Sequence[float] = (0.0, 0.0, 0.0)
    zeta_u: float = 0.0
    zeta_j: float = 0.0
    convection: int = 2
    f_cell: Optional[np.ndarray] = None


@dataclass
class Facets:
    cell: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    lface: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int8))
    tau: Optional[np.ndarray] = None
    cw: Optional[np.ndarray] = None
    jw: Optional[np.ndarray] = None
    phi0: Optional[np.ndarray] = None


def _c_fluid(fl: Fluid):
    s = OrcFluid()
    s.alpha, s.beta, s.gamma, s.sigma = fl.alpha, fl.beta, fl.gamma, fl.sigma
    s.B[:] = list(fl.B); s.f[:] = list(fl.f); s.g[:] = list(fl.g)
    s.zeta_u, s.zeta_j, s.convection = fl.zeta_u, fl.zeta_j, int(fl.convection)
    keep = None
    if fl.f_cell is not None:
        keep = np.ascontiguousarray(fl.f_cell, dtype=np.float64)
        s.f_cell = _dp(keep)
    return s, keep


def _c_facets(fc: Optional[Facets]):
    s = OrcFacets()
    if fc is None or len(fc.cell) == 0:
        s.n = 0
        return s, []
    keep = [np.ascontiguousarray(fc.cell, np.int32), np.ascontiguousarray(fc.lface, np.int8)]
    s.n = len(fc.cell)
    s.cell = keep[0].ctypes.data_as(C.POINTER(C.c_int32))
    s.lface = keep[1].ctypes.data_as(C.POINTER(C.c_int8))
    for name in ("tau", "cw", "jw", "phi0"):
        v = getattr(fc, name)
        if v is not None:
            a = np.ascontiguousarray(v, np.float64)
            keep.append(a)
            setattr(s, name, _dp(a))
    return s, keep


def assemble_cells(cell_X, x_cell, fl: Fluid, fc: Optional[Facets] = None, want_jac=True, nthreads=None):
    L = lib()
    nc = cell_X.shape[0]
    cell_X = np.ascontiguousarray(cell_X, np.float64)
    x_cell = np.ascontiguousarray(x_cell, np.float64)
    r = np.empty((nc, 129))
    K = np.empty((nc, 129, 129)) if want_jac else None
    sf, k1 = _c_fluid(fl)
    sc, k2 = _c_facets(fc)
    L.orc_assemble_cells(C.c_int64(nc), _dp(cell_X), _dp(x_cell), C.byref(sf), C.byref(sc), _dp(r),
                         _dp(K) if K is not None else None, C.c_int(nthreads or os.cpu_count() or 1))
    return r, K


def touched_mask():
    f = np.empty(129, dtype=np.int64)
    f[0:81] = 0; f[81:85] = 1; f[85:121] = 2; f[121:129] = 3
    m = np.zeros((129, 129), bool)
    for (a, b) in {(0, 0), (0, 1), (0, 2), (1, 0), (2, 2), (2, 3), (2, 0), (3, 2)}:
        m[np.ix_(f == a, f == b)] = True
    return m


class OracleProblem:
    """Global FP64 assembly over a mesh and dof map produced by the host mirror."""

    def __init__(self, cell_X, gdofs, ndofs, cell_values_fn, fluid: Fluid, facets: Optional[Facets] = None):
        self.cell_X = np.ascontiguousarray(cell_X, np.float64)
        self.gdofs = gdofs            # (ncells,129) global free ids, -1 for Dirichlet
        self.ndofs = ndofs
        self.cell_values = cell_values_fn
        self.fluid = fluid
        self.facets = facets
        mask = touched_mask()
        rows = np.broadcast_to(gdofs[:, :, None], (len(gdofs), 129, 129))
        cols = np.broadcast_to(gdofs[:, None, :], (len(gdofs), 129, 129))
        keep = mask[None] & (rows >= 0) & (cols >= 0)
        self._sel = np.nonzero(keep.reshape(len(gdofs), -1))
        self._ri = rows.reshape(len(gdofs), -1)[self._sel]
        self._ci = cols.reshape(len(gdofs), -1)[self._sel]

    def residual_jacobian(self, x, want_jac=True):
        xc = self.cell_values(x)
        r_cell, K_cell = assemble_cells(self.cell_X, xc, self.fluid, self.facets, want_jac)
        g = self.gdofs
        m = g >= 0
        r = np.bincount(g[m], weights=r_cell[m], minlength=self.ndofs)
        if not want_jac:
            return r, None
        vals = K_cell.reshape(len(g), -1)[self._sel]
        A = sp.coo_matrix((vals, (self._ri, self._ci)), shape=(self.ndofs, self.ndofs)).tocsr()
        A.sum_duplicates()
        A.sort_indices()
        return r, A


def problem_from_case(mesh, dm, params) -> OracleProblem:
    """The oracle's problem for a (mesh, dof map, parameters) workload of the host mirror
    (gbmhd.cases): the same cells, dof numbering, Dirichlet values and physical parameters."""
    fl = Fluid(alpha=params["alpha"], beta=params["beta"], gamma=params["gamma"], sigma=params["sigma"],
               B=params["B"], f=params["f"], zeta_u=params["zeta_u"], zeta_j=params["zeta_j"],
               convection=params["convection"], f_cell=params.get("f_cell"))
    fc = None
    if params.get("facets") is not None:
        q = params["facets"]
        fc = Facets(cell=q["cell"], lface=q["lface"], tau=q["tau"], cw=q["cw"], jw=q["jw"], phi0=q.get("phi0"))
    return OracleProblem(mesh.cell_coords(), dm.global_cell_dofs(), dm.ndofs, dm.cell_values, fl, fc)


def newton_direct(prob: OracleProblem, x0, gauge: Sequence[int] = (), rtol=1e-10, atol=0.0, maxiter=10,
                  verbose=False):
    """Newton with a sparse direct solve (SuperLU), dropping the gauge dofs."""
    x = np.array(x0, dtype=float, copy=True)
    keep = np.ones(prob.ndofs, bool)
    keep[list(gauge)] = False
    idx = np.nonzero(keep)[0]
    r, A = prob.residual_jacobian(x)
    r0 = np.linalg.norm(r)
    hist = [r0]
    it = 0
    while it < maxiter:
        if hist[-1] <= max(atol, rtol * r0) and it > 0:
            break
        Ar = A[idx][:, idx].tocsc()
        dx = np.zeros_like(x)
        dx[idx] = spla.spsolve(Ar, -r[idx], permc_spec="COLAMD")
        x += dx
        it += 1
        r, A = prob.residual_jacobian(x)
        hist.append(np.linalg.norm(r))
        if verbose:
            print(f"newton {it}: |r| = {hist[-1]:.3e}")
        if hist[-1] <= max(atol, rtol * r0):
            break
    return x, dict(nls_iters=it, residuals=hist)


def newton_chord(prob: OracleProblem, x0, gauge: Sequence[int] = (), rtol=1e-13, atol=0.0, maxiter=60,
                 verbose=False):
    """Newton's root with one SuperLU factorization (the chord method).

    The residual is evaluated exactly at every step (FP64 assembly); only the Jacobian is
    frozen at x0.  The iteration therefore converges to the same root as the Newton
    iteration of the :julia solver (src/main.jl:181-186), only more slowly.  This is
    for meshes where SuperLU takes minutes per factorization (the 32x32x3 duct)."""
    x = np.array(x0, dtype=float, copy=True)
    keep = np.ones(prob.ndofs, bool)
    keep[list(gauge)] = False
    idx = np.nonzero(keep)[0]
    r, A = prob.residual_jacobian(x)
    lu = spla.splu(A[idx][:, idx].tocsc(), permc_spec="COLAMD")
    del A
    r0 = np.linalg.norm(r)
    hist = [r0]
    it = 0
    while it < maxiter and hist[-1] > max(atol, rtol * r0):
        x[idx] -= lu.solve(r[idx])
        it += 1
        r, _ = prob.residual_jacobian(x, want_jac=False)
        hist.append(np.linalg.norm(r))
        if verbose:
            print(f"chord {it}: |r| = {hist[-1]:.3e}", flush=True)
        if it > 3 and hist[-1] > 0.9 * hist[-2]:
            break
    return x, dict(nls_iters=it, residuals=hist)


def eval_fields(cell_X, x_cell, npts1d=4):
    L = lib()
    nc = cell_X.shape[0]
    out = np.empty((nc, npts1d ** 3, 22))
    L.orc_eval_fields(C.c_int64(nc), _dp(np.ascontiguousarray(cell_X)), _dp(np.ascontiguousarray(x_cell)),
                      C.c_int(npts1d), _dp(out))
    return out.reshape(-1, 22)


def field_norms(cell_X, x_cell, npts1d=4):
    """L2 norms of u and j and H1 norm of u (degree 2(order+1) rule, src/Applications/hunt.jl:245)."""
    F = eval_fields(cell_X, x_cell, npts1d)
    w = F[:, 3]
    u, gu, j = F[:, 4:7], F[:, 7:16], F[:, 17:20]
    return dict(uh_l2=math.sqrt(np.sum(w * np.sum(u * u, 1))),
                uh_h1=math.sqrt(np.sum(w * (np.sum(u * u, 1) + np.sum(gu * gu, 1)))),
                jh_l2=math.sqrt(np.sum(w * np.sum(j * j, 1))))


def analytical_hunt_u(a, b, mu, grad_pz, Ha, n, x):
    """Restatement of analytical_hunt_u (src/Applications/hunt.jl:372-410), vectorised."""
    l = b / a
    xi, eta = x[:, 0] / a, x[:, 1] / a
    V = np.zeros(len(x))
    for k in range(n + 1):
        ak = (k + 0.5) * math.pi / l
        N = math.sqrt(Ha ** 2 + 4 * ak ** 2)
        r1, r2 = 0.5 * (Ha + N), 0.5 * (-Ha + N)
        V2 = (r2 / N) * (np.exp(-r1 * (1 - eta)) + np.exp(-r1 * (1 + eta))) / (1 + math.exp(-2 * r1))
        V3 = (r1 / N) * (np.exp(-r2 * (1 - eta)) + np.exp(-r2 * (1 + eta))) / (1 + math.exp(-2 * r2))
        V += 2 * (-1) ** k * np.cos(ak * xi) / (l * ak ** 3) * (1 - V2 - V3)
    uz = V / mu * (-grad_pz) * a ** 2
    out = np.zeros((len(x), 3))
    out[:, 2] = uz
    out[(np.abs(xi) > 1) | (np.abs(eta) > 1)] = 0.0
    return out


def analytical_hunt_j(a, b, sigma, mu, grad_pz, Ha, n, x):
    """Restatement of analytical_hunt_j (src/Applications/hunt.jl:413-457), vectorised."""
    l = b / a
    xi, eta = x[:, 0] / a, x[:, 1] / a
    Hdx = np.zeros(len(x)); Hdy = np.zeros(len(x))
    for k in range(n + 1):
        ak = (k + 0.5) * math.pi / l
        N = math.sqrt(Ha ** 2 + 4 * ak ** 2)
        r1, r2 = 0.5 * (Ha + N), 0.5 * (-Ha + N)
        den1, den2 = 1 + math.exp(-2 * r1), 1 + math.exp(-2 * r2)
        num = np.exp(-r1 * (1 - eta)) - np.exp(-r1 * (1 + eta))
        num_dy = np.exp(-r1 * (1 - eta)) * (r1 / a) + np.exp(-r1 * (1 + eta)) * (r1 / a)
        H2, H2dy = (r2 / N) * (num / den1), (r2 / N) * (num_dy / den1)
        num = np.exp(-r2 * (1 - eta)) - np.exp(-r2 * (1 + eta))
        num_dy = np.exp(-r2 * (1 - eta)) * (r2 / a) + np.exp(-r2 * (1 + eta)) * (r2 / a)
        H3, H3dy = (r1 / N) * (num / den2), (r1 / N) * (num_dy / den2)
        Hdx += -2 * (-1) ** k * np.sin(ak * xi) / (a * l * ak ** 2) * (H2 - H3)
        Hdy += 2 * (-1) ** k * np.cos(ak * xi) / (l * ak ** 3) * (H2dy - H3dy)
    out = np.zeros((len(x), 3))
    out[:, 0] = a ** 2 * sigma ** 0.5 / mu ** 0.5 * (-grad_pz) * Hdy
    out[:, 1] = a ** 2 * sigma ** 0.5 / mu ** 0.5 * (-grad_pz) * (-Hdx)
    out[(np.abs(xi) > 1) | (np.abs(eta) > 1)] = 0.0
    return out


def analytical_hunt_grad_u(a, b, mu, grad_pz, Ha, n, x):
    """∇ of analytical_hunt_u (src/Applications/hunt.jl:372-410) as [point][i][k] = ∂_i u_k: the
    derivative of its Fourier series term by term (the reference differentiates the same
    function with dual numbers when it forms ∇(u − uh), :250).  Only ∂_x u_z and ∂_y u_z are
    nonzero."""
    l = b / a
    xi, eta = x[:, 0] / a, x[:, 1] / a
    dxi = np.zeros(len(x)); deta = np.zeros(len(x))
    for k in range(n + 1):
        ak = (k + 0.5) * math.pi / l
        N = math.sqrt(Ha ** 2 + 4 * ak ** 2)
        r1, r2 = 0.5 * (Ha + N), 0.5 * (-Ha + N)
        den1, den2 = 1 + math.exp(-2 * r1), 1 + math.exp(-2 * r2)
        e11, e12 = np.exp(-r1 * (1 - eta)), np.exp(-r1 * (1 + eta))
        e21, e22 = np.exp(-r2 * (1 - eta)), np.exp(-r2 * (1 + eta))
        V2 = (r2 / N) * (e11 + e12) / den1
        V3 = (r1 / N) * (e21 + e22) / den2
        dV2 = (r2 / N) * r1 * (e11 - e12) / den1
        dV3 = (r1 / N) * r2 * (e21 - e22) / den2
        c = 2 * (-1) ** k / (l * ak ** 3)
        dxi += -c * ak * np.sin(ak * xi) * (1 - V2 - V3)
        deta += c * np.cos(ak * xi) * (-dV2 - dV3)
    s = (-grad_pz) * a ** 2 / mu / a
    out = np.zeros((len(x), 3, 3))
    out[:, 0, 2] = s * dxi
    out[:, 1, 2] = s * deta
    out[(np.abs(xi) > 1) | (np.abs(eta) > 1)] = 0.0
    return out


def hunt_errors(cell_X, x_cell, L=1.0, mu=1.0, grad_pz=-1.0, sigma=1.0, Ha=10.0, nsums=10, u_scale=1.0,
                j_scale=1.0, length_scale=1.0):
    """The nine norms of hunt()'s post-processing (src/Applications/hunt.jl:238-260) with the
    degree-6 rule (4 Gauss points per direction): eu_h1, eu_l2, ej_l2 (nsums terms), the
    same with 2·nsums terms (…_ref), and uh_h1, uh_l2, jh_l2.  length_scale warps the mesh
    (src/Applications/hunt.jl:352-357): points and measure scale, gradients of uh by 1/s."""
    F = eval_fields(cell_X, x_cell, 4)
    s = length_scale
    xp = s * F[:, 0:3]
    w = F[:, 3] * s ** 3
    uh = u_scale * F[:, 4:7]
    guh = u_scale * F[:, 7:16].reshape(-1, 3, 3) / s
    jh = j_scale * F[:, 17:20]
    out = {}
    for tag, n in (("", nsums), ("_ref", 2 * nsums)):
        ua = analytical_hunt_u(L, L, mu, grad_pz, Ha, n, xp)
        gua = analytical_hunt_grad_u(L, L, mu, grad_pz, Ha, n, xp)
        ja = analytical_hunt_j(L, L, sigma, mu, grad_pz, Ha, n, xp)
        eu2 = np.sum((ua - uh) ** 2, 1)
        ge2 = np.sum((gua - guh) ** 2, (1, 2))
        out[f"eu{tag}_h1"] = math.sqrt(np.sum(w * (ge2 + eu2)))
        out[f"eu{tag}_l2"] = math.sqrt(np.sum(w * eu2))
        out[f"ej{tag}_l2"] = math.sqrt(np.sum(w * np.sum((ja - jh) ** 2, 1)))
    out["uh_h1"] = math.sqrt(np.sum(w * (np.sum(uh * uh, 1) + np.sum(guh * guh, (1, 2)))))
    out["uh_l2"] = math.sqrt(np.sum(w * np.sum(uh * uh, 1)))
    out["jh_l2"] = math.sqrt(np.sum(w * np.sum(jh * jh, 1)))
    return out
