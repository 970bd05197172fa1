"""Host-side mirror of ``GridapMHD.main(params)`` and ``GridapMHD.hunt(...)``.

The parameter dictionaries, their defaults and their validation follow
GridapMHD src/parameters.jl (``add_default_params`` :85-137, ``params_fluid``
:693-723, ``params_bcs`` :777-813, ``params_bcs_thin_wall`` :938-947,
``default_solver_params`` :221-287) for the keys this hot path uses; the
solver symbol ``"gb300"`` selects the GPU library, as a ``:gb300`` method
set would in Julia (src/main.jl:173-190).  ``main`` returns
``(xh, full_params, output)`` like src/main.jl:122-169.

Unicode keys of the reference (``"α"``, ``"ζᵤ"``, ``"φ"`` ...) and ASCII
aliases (``"alpha"``, ``"zeta_u"``, ``"phi"``) are both accepted.
"""
from __future__ import annotations

import json
import math
import os
import time
from dataclasses import dataclass
from typing import Any, Dict, Optional

import numpy as np

from . import lib
from .fespace import DofMap, build_dofmap
from .mesh import StructuredMesh, hunt_generate_base_mesh, hunt_stretch_map, tanh_map

ALIASES = {"alpha": "α", "beta": "β", "gamma": "γ", "sigma": "σ", "zeta_u": "ζᵤ", "zeta_j": "ζⱼ", "phi": "φ",
           "tau": "τ", "mu": "μ", "zetau": "ζᵤ", "zetaj": "ζⱼ"}


def _canon(d: Dict) -> Dict:
    return {ALIASES.get(k, k): v for k, v in d.items()}


def _check_unused(sub: Dict, mandatory: Dict, params: Dict, where: str):
    """src/parameters.jl:47-55."""
    if params.get("check_valid", True):
        for k in sub:
            if k not in mandatory:
                raise KeyError(f"Key :{k} is not a valid key in params{where}. "
                               "Set params[:check_valid] = false to ignore invalid keys.")


def _check_mandatory(sub, mandatory, where):
    if not isinstance(sub, dict):
        raise TypeError(f"The params{where} has to be a Dict")
    for k, m in mandatory.items():
        if m and k not in sub:
            raise KeyError(f"Key :{k} is a mandatory key in params{where}, but it is not provided.")


def default_solver_params(solver: str = "gb300") -> Dict:
    """``default_solver_params(::Val{:gb300})`` (pattern of src/parameters.jl:221-287)."""
    if solver != "gb300":
        raise ValueError(f"solver {solver!r} is not provided by this library; use 'gb300'")
    return {"solver": "gb300", "matrix_type": "SparseMatrixCSR{0,Float64,Int64}", "vector_type": "Vector{Float64}",
            "solver_postpro": gb300_postpro, "niter": 10, "niter_ls": 40, "rtol": 1e-10, "atol": 0.0,
            "precision": "mixed", "max_linear": 500, "linear_rtol": 1e-6, "verbose": 0}


def gb300_postpro(report: Dict, info: Dict):
    """``solver_postpro`` hook (src/parameters.jl:305-338): iteration counts and residuals."""
    info["nls_iters"] = report["newton_iters"]
    info["ls_iters"] = report["linear_iters"]
    info["nls_residuals"] = report["residual_history"]


def uses_petsc(solver) -> bool:
    return False


def space_uses_multigrid(solver):
    return [False] * 4


def params_fluid(params: Dict) -> Dict:
    mandatory = {"domain": True, "α": True, "β": True, "γ": True, "B": True, "f": False, "σ": False, "ζᵤ": False,
                 "ζⱼ": False, "g": False, "divg": False, "convection": False, "μ": False}
    fl = _canon(params["fluid"])
    _check_mandatory(fl, mandatory, "[:fluid]")
    out = {"σ": 1.0, "f": (0.0, 0.0, 0.0), "ζᵤ": 0.0, "ζⱼ": 0.0, "g": (0.0, 0.0, 0.0), "divg": 0.0,
           "convection": "newton", "μ": 6}
    out.update(fl)
    _check_unused(out, mandatory, params, "[:fluid]")
    if out["convection"] not in ("none", "newton", "picard"):
        raise ValueError("convection must be one of none, newton, picard")
    if out["domain"] is not None:
        raise NotImplementedError("only a fluid domain equal to the whole model is supported (no solid)")
    return out


def params_bcs(params: Dict) -> Dict:
    mandatory = {"u": True, "j": True, "φ": False, "t": False, "thin_wall": False, "stabilization": False}
    b = _canon(params["bcs"])
    _check_mandatory(b, mandatory, "[:bcs]")
    out = {"φ": [], "t": [], "thin_wall": [], "stabilization": []}
    out.update(b)
    _check_unused(out, mandatory, params, "[:bcs]")
    if out["t"]:
        raise NotImplementedError("Boundary tranction not yet implemented")  # src/weakforms.jl:162-164
    if out["stabilization"]:
        raise NotImplementedError("skeleton stabilisation is outside this hot path")
    u = dict(out["u"])
    _check_mandatory(u, {"tags": True, "values": False}, "[:bcs][:u]")
    _check_unused(u, {"tags": True, "values": False}, params, "[:bcs][:u]")
    j = dict(out["j"])
    _check_mandatory(j, {"tags": True, "values": False}, "[:bcs][:j]")
    tw = out["thin_wall"]
    tw = [tw] if isinstance(tw, dict) else list(tw)
    tw2 = []
    for i, d in enumerate(tw):
        d = _canon(d)
        m = {"domain": True, "cw": True, "τ": True, "jw": False}
        _check_mandatory(d, m, f"[:bcs][:thin_wall][{i + 1}]")
        d = {"jw": 0.0, **d}
        _check_unused(d, m, params, f"[:bcs][:thin_wall][{i + 1}]")
        tw2.append(d)
    out["thin_wall"] = tw2
    ph = out["φ"]
    ph = [ph] if isinstance(ph, dict) else list(ph)
    for i, d in enumerate(ph):
        _check_mandatory(d, {"domain": True, "value": True}, f"[:bcs][:φ][{i + 1}]")
    out["φ"] = ph
    out["u"], out["j"] = u, j
    return out


def params_solver(params: Dict) -> Dict:
    s = params["solver"]
    if isinstance(s, str):
        return default_solver_params(s)
    if "solver" not in s:
        raise KeyError("params[:solver] must contain :solver")
    out = default_solver_params(s["solver"])
    out.update(s)
    return out


def params_fespaces(params: Dict) -> Dict:
    fe = dict(params.get("fespaces") or {})
    out = {"order_u": 2, "order_j": fe.get("order_u", 2), "p_constraint": None, "φ_constraint": None,
           "rt_scaling": None, "fluid_disc": "Qk_dPkm1", "current_disc": "RT"}
    out.update(_canon(fe))
    _check_unused(out, {k: False for k in ("order_u", "order_j", "p_constraint", "φ_constraint", "rt_scaling",
                                           "fluid_disc", "current_disc")}, params, "[:fespaces]")
    if out["order_u"] != 2 or out["order_j"] != 2 or out["fluid_disc"] != "Qk_dPkm1" or out["current_disc"] != "RT":
        raise NotImplementedError("the GPU hot path implements Q2/dP1/RT1/dQ1 (order 2, :Qk_dPkm1, :RT) only")
    out["formulation"] = "H1HDiv"
    out["q"] = 5  # src/parameters.jl:381-389 with k_u = k_j = 2
    return out


def add_default_params(_params: Dict) -> Dict:
    """``add_default_params`` (src/parameters.jl:85-137) for the keys of this hot path."""
    mandatory = {"ptimer": False, "debug": False, "solve": True, "res_assemble": False, "jac_assemble": False,
                 "model": True, "fluid": True, "solid": False, "bcs": True, "fespaces": False, "solver": True,
                 "multigrid": False, "check_valid": False, "transient": False, "continuation": False, "x0": False}
    _check_mandatory(_params, mandatory, "")
    p = {"debug": False, "res_assemble": False, "jac_assemble": False, "solid": None, "fespaces": None,
         "multigrid": None, "check_valid": True, "transient": None, "continuation": None, "x0": "zero"}
    p.update(_params)
    _check_unused(p, mandatory, p, "")
    if p.get("solid") is not None or p.get("transient") is not None or p.get("continuation") is not None:
        raise NotImplementedError("solid domains, transient and continuation runs are outside this hot path")
    p["fespaces"] = params_fespaces(p)
    p["fluid"] = params_fluid(p)
    p["bcs"] = params_bcs(p)
    p["solver"] = params_solver(p)
    return p


@dataclass
class FEFunction:
    """Free dof values of the multi-field solution with the data to split them."""
    free_values: np.ndarray
    dofmap: DofMap
    mesh: StructuredMesh

    def field(self, name: str) -> np.ndarray:
        return self.dofmap.split(self.free_values)[name]

    def cell_values(self) -> np.ndarray:
        return self.dofmap.cell_values(self.free_values)


def _facets(mesh: StructuredMesh, bcs: Dict):
    bc, bf, bt = mesh.boundary_faces()
    cells, faces, tau, cw, jw, phi0 = [], [], [], [], [], []
    for d in bcs["thin_wall"]:
        tag = d["domain"]
        sel = bt == mesh.tag_names.index(tag)
        n = int(sel.sum())
        cells.append(bc[sel]); faces.append(bf[sel])
        tau.append(np.full(n, float(d["τ"]))); cw.append(np.full(n, float(d["cw"])))
        jw.append(np.full(n, float(d["jw"]))); phi0.append(np.zeros(n))
    for d in bcs["φ"]:
        sel = bt == mesh.tag_names.index(d["domain"])
        n = int(sel.sum())
        cells.append(bc[sel]); faces.append(bf[sel])
        tau.append(np.zeros(n)); cw.append(np.zeros(n)); jw.append(np.zeros(n))
        phi0.append(np.full(n, float(d["value"])))
    if not cells:
        return None
    return dict(cell=np.concatenate(cells).astype(np.int32), lface=np.concatenate(faces).astype(np.int8),
                tau=np.concatenate(tau), cw=np.concatenate(cw), jw=np.concatenate(jw), phi0=np.concatenate(phi0))


def _tags(t):
    return [t] if isinstance(t, str) else list(t)


def lib_params(fluid: Dict, facets, ncells: int) -> Dict:
    conv = {"none": 0, "picard": 1, "newton": 2}[fluid["convection"]]
    f = fluid["f"]
    q = dict(alpha=fluid["α"], beta=fluid["β"], gamma=fluid["γ"], sigma=fluid["σ"], B=tuple(fluid["B"]),
             g=tuple(fluid["g"]), zeta_u=fluid["ζᵤ"], zeta_j=fluid["ζⱼ"], convection=conv, facets=facets)
    f = np.asarray(f, dtype=float)
    if f.shape == (3,):
        q["f"] = tuple(f)
    elif f.shape == (ncells, 3):
        q["f"] = (0.0, 0.0, 0.0)
        q["f_cell"] = f
    else:
        raise ValueError("fluid f must be a 3-vector or a (ncells,3) cellwise field")
    return q


def setup(params: Dict):
    """Spaces, dof map and library context (the ``setup_fe_spaces`` + ``_fe_operator`` stage)."""
    mesh: StructuredMesh = params["model"]
    bcs = params["bcs"]
    u_values = bcs["u"].get("values")
    fn = u_values if callable(u_values) else None
    dm = build_dofmap(mesh, _tags(bcs["u"]["tags"]), _tags(bcs["j"]["tags"]), u_values=fn)
    facets = _facets(mesh, bcs)
    q = lib_params(params["fluid"], facets, mesh.ncells)
    ctx = lib.Context(mesh.cell_coords(), dm.cell_dofs, [dm.nfree[f] for f in ("u", "p", "j", "phi")],
                      [dm.ndir[f] for f in ("u", "p", "j", "phi")],
                      [dm.dir_values.get(f) for f in ("u", "p", "j", "phi")], q)
    return dm, ctx


def main(_params: Dict, output: Optional[Dict] = None):
    """Solve the MHD problem (src/main.jl:122-169) on the GPU: returns (xh, full_params, output)."""
    output = {} if output is None else output
    params = add_default_params(_params)
    timer = params.setdefault("ptimer", {})
    t0 = time.perf_counter()
    dm, ctx = setup(params)
    timer["fe_spaces"] = time.perf_counter() - t0
    x0 = params["x0"]
    x = np.zeros(dm.ndofs) if (isinstance(x0, str) and x0 == "zero") else np.asarray(x0, dtype=float).copy()
    if params["debug"]:
        rng = np.random.default_rng(1234)
        x = rng.random(dm.ndofs)
    elif params["solve"]:
        s = params["solver"]
        t1 = time.perf_counter()
        prec = lib.GBMHD_MIXED if s["precision"] == "mixed" else lib.GBMHD_FP64
        x, rep, rc = ctx.newton_solve(x, precision=prec, max_newton=s["niter"], newton_rtol=s["rtol"],
                                      newton_atol=s["atol"], restart=s["niter_ls"], max_linear=s["max_linear"],
                                      linear_rtol=s["linear_rtol"], verbose=s["verbose"])
        timer["solve"] = time.perf_counter() - t1
        s["solver_postpro"](rep, output)
        output["gpu_report"] = rep
        if rc != 0:
            output["converged"] = False
    if params["res_assemble"]:
        t1 = time.perf_counter()
        ctx.assemble(x, want_jacobian=False)
        timer["residual"] = time.perf_counter() - t1
    if params["jac_assemble"]:
        t1 = time.perf_counter()
        ctx.assemble(x, want_jacobian=True, precision=lib.GBMHD_FP64, want_residual=False)
        timer["jacobian"] = time.perf_counter() - t1
    params["_context"] = ctx
    return FEFunction(x, dm, params["model"]), params, output


def hunt(*, nc=(4, 4), ν=1.0, ρ=1.0, σ=1.0, B=(0.0, 10.0, 0.0), f=(0.0, 0.0, 1.0), ζᵤ=0.0, ζⱼ=0.0, L=1.0,
         u0=1.0, B0=None, tw=0.0, order=2, nsums=10, title="hunt", path=".", debug=False, res_assemble=False,
         jac_assemble=False, solve=True, solver="gb300", formulation="cfd", initial_value="zero",
         convection="newton", BL_adapted=True, kmap_x=1, kmap_y=1, nz=3, Lz=0.1, map_beta=None, cw=0.0, τ=100.0,
         write=False, vtk=False, **kw) -> Dict[str, Any]:
    """``hunt(; kwargs...)`` (src/Applications/hunt.jl:1-304) on the GPU.

    Extra keywords for the duct configurations of the GPU benchmark: ``nz``,
    ``Lz`` (axial cells and length; the reference hard-codes 3 and 0.1),
    ``map_beta`` (tanh stretching instead of the Smolentsev/power maps) and
    ``cw``/``τ`` (thin-wall law on the Hartmann walls, src/weakforms.jl:721-733).
    With ``vtk=True`` the fields uh, ph, jh, phi, div_uh and div_jh are written to
    ``<path>/<title>.vtu`` at order 2, as the reference does (src/Applications/hunt.jl:263-273;
    the fields are evaluated on the device, gbmhd_node_fields, and carry the solved units).
    Returns the ``info`` dict the reference saves to BSON."""
    if kw:
        raise TypeError(f"unexpected keyword(s) {sorted(kw)}")
    if tw > 0.0:
        raise NotImplementedError("resolved solid walls (tw>0) are outside this hot path")
    if order != 2:
        raise NotImplementedError("order 2 only")
    if formulation not in ("cfd", "mhd"):
        raise ValueError("formulation must be :cfd or :mhd")
    info: Dict[str, Any] = {}
    tpre = time.perf_counter()
    B0 = float(np.linalg.norm(B)) if B0 is None else float(B0)
    Re = u0 * L / ν
    Ha = B0 * L * math.sqrt(σ / (ρ * ν))
    N = Ha ** 2 / Re
    fbar = (L / (ρ * u0 ** 2)) * np.asarray(f, dtype=float)
    Bbar = np.asarray(B, dtype=float) / B0
    if formulation == "cfd":
        alpha, beta, gamma = 1.0, 1.0 / Re, N
    else:
        alpha, beta, gamma = 1.0 / N, 1.0 / Ha ** 2, 1.0
        fbar = fbar / N
    cmap = tanh_map(map_beta) if map_beta is not None else hunt_stretch_map(L + tw, Ha, kmap_x, kmap_y, BL_adapted)
    model = hunt_generate_base_mesh(tuple(nc), L=L, tw=tw, Ha=Ha, nz=nz, Lz=Lz, map=cmap)
    params = {"debug": debug, "solve": solve, "res_assemble": res_assemble, "jac_assemble": jac_assemble,
              "model": model, "solver": solver,
              "fluid": {"domain": None, "α": alpha, "β": beta, "γ": gamma, "f": tuple(fbar), "B": tuple(Bbar),
                        "ζᵤ": ζᵤ, "ζⱼ": ζⱼ, "convection": convection},
              "bcs": {"u": {"tags": ["conducting", "insulating"]}, "j": {"tags": "insulating"}},
              "x0": initial_value}
    if cw > 0.0:
        params["bcs"]["thin_wall"] = [{"domain": "conducting", "cw": cw, "τ": τ}]
    tpre = time.perf_counter() - tpre
    xh, full, info = main(params, output=info)
    info["time_pre_process"] = tpre
    for k, v in full["ptimer"].items():
        info[f"time_{k}"] = v
    dm = xh.dofmap
    # post-processing (src/Applications/hunt.jl:211-260) on the device: the solved fields
    # rescaled to physical units (uh = u0 ūh, jh = σ u0 B0 j̄h) against the analytic Hunt
    # solution with nsums and 2·nsums Fourier terms, on the mesh warped by L
    tpost = time.perf_counter()
    norms = full["_context"].hunt_errors(xh.free_values, L=L, mu=ρ * ν, grad_pz=-float(f[2]) / ρ, sigma=σ,
                                          Ha=Ha, nsums=nsums, u_scale=u0, j_scale=σ * u0 * B0, length_scale=L)
    info.update(norms)
    info["time_post_process"] = time.perf_counter() - tpost
    info.update(nc=list(nc), ncells=model.ncells, ndofs_u=dm.nfree["u"], ndofs_p=dm.nfree["p"],
                ndofs_j=dm.nfree["j"], ndofs_φ=dm.nfree["phi"], ndofs=dm.ndofs, Re=Re, Ha=Ha, nsums=nsums,
                kmap=[kmap_x, kmap_y], title=title)
    info["xh"] = xh
    if vtk:
        from .vtk import write_vtu
        tv = time.perf_counter()
        os.makedirs(path, exist_ok=True)
        info["vtk_file"] = write_vtu(os.path.join(path, f"{title}.vtu"),
                                     full["_context"].node_fields(xh.free_values))
        info["time_vtk"] = time.perf_counter() - tv
    if write:
        os.makedirs(path, exist_ok=True)
        with open(os.path.join(path, f"{title}.json"), "w") as fh:
            json.dump({k: v for k, v in info.items() if k not in ("xh", "gpu_report")}, fh, indent=1, default=str)
    return info
