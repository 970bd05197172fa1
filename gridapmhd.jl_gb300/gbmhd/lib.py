"""ctypes binding of libgbmhd (include/gbmhd.h).

This is the reference-facing boundary as a Python host sees it; the Julia
host binds the same symbols with ``ccall`` (julia/GridapMHDGB300.jl).  There is no
CPU fallback: if the CUDA library is missing or no GPU is present, calls fail.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "libgbmhd.so")

GBMHD_FP64 = 0
GBMHD_MIXED = 1
GBMHD_MIXED_F64OP = 2
GBMHD_PC_MONOLITHIC = 0
GBMHD_PC_BADIA2024 = 1

SYMBOLS = ["gbmhd_version", "gbmhd_create", "gbmhd_set_params", "gbmhd_sizes", "gbmhd_assemble",
           "gbmhd_assemble_device", "gbmhd_get_csr", "gbmhd_newton_solve", "gbmhd_newton_solve_device",
           "gbmhd_adjoint", "gbmhd_param_gradient_noalloc", "gbmhd_get_stream", "gbmhd_diag_uj_solve_error", "gbmhd_sweep_stats", "gbmhd_hunt_errors", "gbmhd_diag_tc_gemm", "gbmhd_diag_pivot_inverse", "gbmhd_diag_pc_compare", "gbmhd_node_fields", "gbmhd_counters", "gbmhd_last_error", "gbmhd_destroy"]

_dp = C.POINTER(C.c_double)
_i32p = C.POINTER(C.c_int32)
_i8p = C.POINTER(C.c_int8)


class Mesh(C.Structure):
    _fields_ = [("ncells", C.c_int64), ("cell_coords", _dp)]


class DofMap(C.Structure):
    _fields_ = [("nfree", C.c_int64 * 4), ("ndir", C.c_int64 * 4), ("cell_dofs", _i32p),
                ("dir_values", _dp * 4), ("cell_sign_j", _i8p)]


class Params(C.Structure):
    _fields_ = [("alpha", C.c_double), ("beta", C.c_double), ("gamma", C.c_double), ("sigma", C.c_double),
                ("B", C.c_double * 3), ("f", C.c_double * 3), ("g", C.c_double * 3),
                ("zeta_u", C.c_double), ("zeta_j", C.c_double), ("convection", C.c_int32),
                ("f_cell", _dp), ("nfacets", C.c_int64), ("facet_cell", _i32p), ("facet_lface", _i8p),
                ("facet_tau", _dp), ("facet_cw", _dp), ("facet_jw", _dp), ("facet_phi0", _dp)]


class SolveOpts(C.Structure):
    _fields_ = [("precision", C.c_int32), ("max_newton", C.c_int32), ("newton_rtol", C.c_double),
                ("newton_atol", C.c_double), ("restart", C.c_int32), ("max_linear", C.c_int32),
                ("linear_rtol", C.c_double), ("verbose", C.c_int32), ("preconditioner", C.c_int32)]


class Report(C.Structure):
    _fields_ = [("newton_iters", C.c_int32), ("linear_iters", C.c_int32), ("converged", C.c_int32),
                ("initial_residual", C.c_double), ("final_residual", C.c_double),
                ("time_assembly_s", C.c_double), ("time_setup_pc_s", C.c_double),
                ("time_linear_s", C.c_double), ("time_total_s", C.c_double),
                ("residual_history", C.c_double * 64), ("pc_refactorizations", C.c_int32)]

    def as_dict(self):
        n = min(self.newton_iters + 1, 64)
        return dict(newton_iters=self.newton_iters, linear_iters=self.linear_iters,
                    converged=bool(self.converged), initial_residual=self.initial_residual,
                    final_residual=self.final_residual, time_assembly_s=self.time_assembly_s,
                    time_setup_pc_s=self.time_setup_pc_s, time_linear_s=self.time_linear_s,
                    time_total_s=self.time_total_s, residual_history=list(self.residual_history[:n]),
                    pc_refactorizations=self.pc_refactorizations)


class HuntAnalytic(C.Structure):
    _fields_ = [("L", C.c_double), ("mu", C.c_double), ("grad_pz", C.c_double), ("sigma", C.c_double),
                ("Ha", C.c_double), ("nsums", C.c_int32), ("u_scale", C.c_double), ("j_scale", C.c_double),
                ("length_scale", C.c_double)]


HUNT_NORMS = ("eu_h1", "eu_l2", "ej_l2", "eu_ref_h1", "eu_ref_l2", "ej_ref_l2", "uh_h1", "uh_l2", "jh_l2")


class Objective(C.Structure):
    _fields_ = [("dJdx", _dp), ("n_theta_cells", C.c_int32)]


class GbmhdError(RuntimeError):
    pass


_LIB = None


def load(path: Optional[str] = None):
    """Load libgbmhd.so; raises if it has not been built (no fallback)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    p = path or LIBPATH
    if not os.path.exists(p):
        raise GbmhdError(f"libgbmhd.so not found at {p}; build it with gbmhd._build.build()")
    L = C.CDLL(p)
    L.gbmhd_version.restype = C.c_int
    L.gbmhd_last_error.restype = C.c_char_p
    L.gbmhd_last_error.argtypes = [C.c_void_p]
    L.gbmhd_create.argtypes = [C.POINTER(C.c_void_p), C.POINTER(Mesh), C.POINTER(DofMap), C.POINTER(Params)]
    L.gbmhd_set_params.argtypes = [C.c_void_p, C.POINTER(Params)]
    L.gbmhd_sizes.argtypes = [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    L.gbmhd_assemble.argtypes = [C.c_void_p, _dp, _dp, C.c_int32, C.c_int32]
    L.gbmhd_assemble_device.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32]
    L.gbmhd_get_csr.argtypes = [C.c_void_p, C.POINTER(C.c_int64), _i32p, _dp]
    L.gbmhd_newton_solve.argtypes = [C.c_void_p, _dp, C.POINTER(SolveOpts), C.POINTER(Report)]
    L.gbmhd_newton_solve_device.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(SolveOpts), C.POINTER(Report)]
    L.gbmhd_adjoint.argtypes = [C.c_void_p, _dp, C.POINTER(Objective), C.POINTER(SolveOpts), _dp, C.c_int64,
                                _dp, C.POINTER(Report)]
    L.gbmhd_param_gradient_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.gbmhd_get_stream.argtypes = [C.c_void_p]
    L.gbmhd_get_stream.restype = C.c_void_p
    L.gbmhd_diag_uj_solve_error.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, _dp]
    L.gbmhd_sweep_stats.argtypes = [C.c_void_p, C.POINTER(C.c_int64), _dp, _dp]
    L.gbmhd_diag_tc_gemm.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_float, C.c_void_p, C.c_int32, C.c_int64,
                                      C.c_void_p, C.c_int32, C.c_int64, C.c_float, C.c_void_p, C.c_int32,
                                      C.c_int64, C.c_int32, C.POINTER(C.c_int32)]
    L.gbmhd_diag_pc_compare.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, _dp]
    L.gbmhd_diag_pivot_inverse.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p,
                                            C.c_int32, _dp, C.POINTER(C.c_int32)]
    L.gbmhd_node_fields.argtypes = [C.c_void_p, _dp, _dp]
    L.gbmhd_hunt_errors.argtypes = [C.c_void_p, _dp, C.POINTER(HuntAnalytic), _dp]
    L.gbmhd_counters.argtypes = [C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    L.gbmhd_destroy.argtypes = [C.c_void_p]
    L.gbmhd_destroy.restype = None
    _LIB = L
    return L


def _ptr(a, t=_dp):
    return a.ctypes.data_as(t) if a is not None else None


class Context:
    """Owns one gbmhd_ctx: mesh, dofs, CSR pattern and device buffers."""

    def __init__(self, cell_coords: np.ndarray, cell_dofs: np.ndarray, nfree, ndir, dir_values, params: dict,
                 cell_sign_j: Optional[np.ndarray] = None):
        self.L = load()
        self._keep = []
        self.ncells = int(cell_coords.shape[0])
        cc = self._k(np.ascontiguousarray(cell_coords, np.float64).reshape(self.ncells, 24))
        cd = self._k(np.ascontiguousarray(cell_dofs, np.int32))
        m = Mesh(self.ncells, _ptr(cc))
        d = DofMap()
        d.nfree[:] = [int(v) for v in nfree]
        d.ndir[:] = [int(v) for v in ndir]
        d.cell_dofs = _ptr(cd, _i32p)
        for i, v in enumerate(dir_values):
            if v is not None and len(v):
                d.dir_values[i] = _ptr(self._k(np.ascontiguousarray(v, np.float64)))
        if cell_sign_j is not None:
            d.cell_sign_j = _ptr(self._k(np.ascontiguousarray(cell_sign_j, np.int8)), _i8p)
        p = self._params(params)
        h = C.c_void_p()
        rc = self.L.gbmhd_create(C.byref(h), C.byref(m), C.byref(d), C.byref(p))
        if rc != 0:
            raise GbmhdError(f"gbmhd_create failed ({rc}): {self.L.gbmhd_last_error(None).decode()}")
        self.h = h
        n, nnz, nc = C.c_int64(), C.c_int64(), C.c_int64()
        self.L.gbmhd_sizes(self.h, C.byref(n), C.byref(nnz), C.byref(nc))
        self.ndofs, self.nnz = n.value, nnz.value

    def _k(self, a):
        self._keep.append(a)
        return a

    def _params(self, q: dict) -> Params:
        p = Params()
        p.alpha, p.beta, p.gamma, p.sigma = (float(q.get(k, d)) for k, d in
                                              (("alpha", 1.0), ("beta", 1.0), ("gamma", 1.0), ("sigma", 1.0)))
        p.B[:] = [float(v) for v in q.get("B", (0, 0, 0))]
        p.f[:] = [float(v) for v in q.get("f", (0, 0, 0))]
        p.g[:] = [float(v) for v in q.get("g", (0, 0, 0))]
        p.zeta_u, p.zeta_j = float(q.get("zeta_u", 0.0)), float(q.get("zeta_j", 0.0))
        p.convection = int(q.get("convection", 2))
        if q.get("f_cell") is not None:
            p.f_cell = _ptr(self._k(np.ascontiguousarray(q["f_cell"], np.float64)))
        fc = q.get("facets")
        if fc is not None and len(fc["cell"]):
            p.nfacets = len(fc["cell"])
            p.facet_cell = _ptr(self._k(np.ascontiguousarray(fc["cell"], np.int32)), _i32p)
            p.facet_lface = _ptr(self._k(np.ascontiguousarray(fc["lface"], np.int8)), _i8p)
            for name in ("tau", "cw", "jw", "phi0"):
                if fc.get(name) is not None:
                    setattr(p, "facet_" + name, _ptr(self._k(np.ascontiguousarray(fc[name], np.float64))))
        return p

    def _check(self, rc, what):
        if rc < 0:
            raise GbmhdError(f"{what} failed ({rc}): {self.L.gbmhd_last_error(self.h).decode()}")
        return rc

    def set_params(self, params: dict):
        self._check(self.L.gbmhd_set_params(self.h, C.byref(self._params(params))), "gbmhd_set_params")

    def assemble(self, x: np.ndarray, want_jacobian=True, precision=GBMHD_FP64, want_residual=True):
        x = np.ascontiguousarray(x, np.float64)
        assert x.shape == (self.ndofs,)
        r = np.empty(self.ndofs) if want_residual else None
        self._check(self.L.gbmhd_assemble(self.h, _ptr(x), _ptr(r), int(want_jacobian), int(precision)),
                    "gbmhd_assemble")
        return r

    def assemble_device(self, d_x: int, d_r: int, want_jacobian=True, precision=GBMHD_FP64):
        self._check(self.L.gbmhd_assemble_device(self.h, C.c_void_p(d_x), C.c_void_p(d_r), int(want_jacobian),
                                                 int(precision)), "gbmhd_assemble_device")

    def csr(self):
        rowptr = np.empty(self.ndofs + 1, np.int64)
        col = np.empty(self.nnz, np.int32)
        val = np.empty(self.nnz, np.float64)
        self._check(self.L.gbmhd_get_csr(self.h, rowptr.ctypes.data_as(C.POINTER(C.c_int64)),
                                         _ptr(col, _i32p), _ptr(val)), "gbmhd_get_csr")
        return rowptr, col, val

    def newton_solve(self, x0: np.ndarray, **opts):
        x = np.array(x0, dtype=np.float64, copy=True)
        o = make_opts(**opts)
        rep = Report()
        rc = self._check(self.L.gbmhd_newton_solve(self.h, _ptr(x), C.byref(o), C.byref(rep)),
                         "gbmhd_newton_solve")
        return x, rep.as_dict(), rc

    def newton_solve_device(self, d_x: int, **opts):
        o = make_opts(**opts)
        rep = Report()
        rc = self._check(self.L.gbmhd_newton_solve_device(self.h, C.c_void_p(d_x), C.byref(o), C.byref(rep)),
                         "gbmhd_newton_solve_device")
        return rep.as_dict(), rc

    def adjoint(self, x: np.ndarray, dJdx: np.ndarray, with_cells=True, **opts):
        x = np.ascontiguousarray(x, np.float64)
        g = np.ascontiguousarray(dJdx, np.float64)
        obj = Objective(_ptr(g), 1 if with_cells else 0)
        nth = 4 + (self.ncells if with_cells else 0)
        out = np.zeros(nth)
        lam = np.zeros(self.ndofs)
        o = make_opts(**opts)
        rep = Report()
        rc = self._check(self.L.gbmhd_adjoint(self.h, _ptr(x), C.byref(obj), C.byref(o), _ptr(out), nth, _ptr(lam),
                                              C.byref(rep)), "gbmhd_adjoint")
        return out, lam, rep.as_dict(), rc

    def uj_solve_error(self, d_state: int, precision=GBMHD_MIXED) -> float:
        e = C.c_double()
        self._check(self.L.gbmhd_diag_uj_solve_error(self.h, C.c_void_p(d_state), int(precision), C.byref(e)),
                    "gbmhd_diag_uj_solve_error")
        return e.value

    def node_fields(self, x: np.ndarray) -> np.ndarray:
        """(ncells, 27, 13): point, u, p, j, φ, div u, div j at the Q2 nodes (gbmhd_node_fields)."""
        x = np.ascontiguousarray(x, np.float64)
        out = np.empty((self.ncells, 27, 13))
        self._check(self.L.gbmhd_node_fields(self.h, _ptr(x), _ptr(out)), "gbmhd_node_fields")
        return out

    def pc_compare(self, d_state: int, transpose=False) -> float:
        """‖y32 − y64‖/‖y64‖ for y = P⁻¹b (P⁻ᵀb), FP32 against FP64 factors (gbmhd_diag_pc_compare)."""
        e = C.c_double()
        self._check(self.L.gbmhd_diag_pc_compare(self.h, C.c_void_p(d_state), int(bool(transpose)), C.byref(e)),
                    "gbmhd_diag_pc_compare")
        return e.value

    def sweep_stats(self):
        """(solves, device seconds, factor bytes per solve) of the multifrontal sweeps since the last call."""
        a, t, b = C.c_int64(), C.c_double(), C.c_double()
        self._check(self.L.gbmhd_sweep_stats(self.h, C.byref(a), C.byref(t), C.byref(b)), "gbmhd_sweep_stats")
        return a.value, t.value, b.value

    def hunt_errors(self, x, *, L=1.0, mu=1.0, grad_pz=-1.0, sigma=1.0, Ha=10.0, nsums=10, u_scale=1.0,
                    j_scale=1.0, length_scale=1.0):
        """Norms of the hunt() post-processing (src/Applications/hunt.jl:238-260) on the device:
        a dict with eu_h1, eu_l2, ej_l2, eu_ref_h1, eu_ref_l2, ej_ref_l2, uh_h1, uh_l2, jh_l2."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        if x.shape != (self.ndofs,):
            raise ValueError(f"x must have shape ({self.ndofs},)")
        a = HuntAnalytic(L, mu, grad_pz, sigma, Ha, nsums, u_scale, j_scale, length_scale)
        out = np.zeros(9)
        self._check(self.L.gbmhd_hunt_errors(self.h, _ptr(x), C.byref(a), _ptr(out)), "gbmhd_hunt_errors")
        return dict(zip(HUNT_NORMS, out.tolist()))

    def stream(self) -> int:
        return int(self.L.gbmhd_get_stream(self.h) or 0)

    def close(self):
        if getattr(self, "h", None):
            self.L.gbmhd_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def counters() -> dict:
    """Kernel launches and cuBLAS GEMM calls made by libgbmhd so far."""
    L = load()
    a, b = C.c_int64(), C.c_int64()
    L.gbmhd_counters(C.byref(a), C.byref(b))
    return {"launches": a.value, "gemm_calls": b.value}


def make_opts(precision=GBMHD_MIXED, max_newton=10, newton_rtol=1e-10, newton_atol=0.0, restart=30,
              max_linear=500, linear_rtol=1e-3, verbose=0, preconditioner=GBMHD_PC_MONOLITHIC) -> SolveOpts:
    o = SolveOpts()
    o.preconditioner = int(preconditioner)
    o.precision, o.max_newton = int(precision), int(max_newton)
    o.newton_rtol, o.newton_atol = float(newton_rtol), float(newton_atol)
    o.restart, o.max_linear, o.linear_rtol, o.verbose = int(restart), int(max_linear), float(linear_rtol), int(verbose)
    return o
