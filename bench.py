"""Benchmark: mixed-precision Newton solve of the inductionless-MHD Hunt duct on one GPU.

Workload (the GPU-scale duct configuration): Hunt duct [-1,1]^2 x 0.2, 64x64x4 hex
cells, x,y stretched by tanh(3x)/tanh(3), periodic in z; Ha=500, Re=1 (CFD scaling
α=1, β=1/Re, γ=Ha²/Re), B=(0,1,0), f=(0,0,1); thin-wall law cw=0.1 (τ=100) on the
Hartmann walls, insulating side walls, no-slip walls; no augmented-Lagrangian terms
(ζᵤ=ζⱼ=0: the reference's own Jacobian).  One step = one full Newton solve from x0 = 0
to ‖r‖ ≤ 1e-12‖r0‖: every residual/Jacobian assembly, the nested-dissection
multifrontal factorization of the Jacobian (FP32) and all FGMRES iterations (FP64).

--impl reference times the FP64 CPU restatement of the reference path (the oracle:
OpenMP cell assembly + SuperLU Newton, the semantics of GridapMHD's :julia solver)
on a bounded sample of the same duct (a 6x6x4 mesh per step), in the same unit; once, outside
the steps, it also reports the oracle's Newton throughput on 6x6x4, 8x8x4 and 10x10x4 samples
and its element assembly on the full 64x64x4 duct (cpu_context).
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for p in (ROOT, os.path.join(ROOT, "gridapmhd.jl_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np

ZETA = 0.0
CFG = dict(nc=(64, 64), nz=4, Lz=0.2, beta_map=3.0, Ha=500.0, Re=1.0, cw=0.1, tau=100.0, zeta=ZETA)
SAMPLE_NC = (6, 6)      # bounded CPU sample per reference step
SWEEP_NC = ((6, 6), (8, 8), (10, 10))
# smaller duct for kernel-level profiling captures (fits a few GB on the device)
CFG_SMALL = dict(nc=(32, 32), nz=4, Lz=0.2, beta_map=2.0, Ha=100.0, Re=10.0, cw=0.1, tau=100.0, zeta=0.0)
METRIC = "Newton-solve throughput (cells/s), Hunt 64x64x4 Ha=500, mixed precision"


def workload(nc, nz, Lz, beta_map, Ha, Re, cw, tau, zeta, convection=2):
    from gbmhd.cases import hunt_case
    return hunt_case(nc=nc, nz=nz, Ha=Ha, Re=Re, beta_map=beta_map, Lz=Lz, cw=cw, tau=tau, zeta_u=zeta,
                     zeta_j=zeta, convection=convection)


class Clocks:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    def __init__(self):
        self.samples, self.proc = [], None

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0],
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                                         text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([s.strip() for s in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                pass
        sm = [float(s[0]) for s in self.samples if s and s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if len(s) > 1 and s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if len(s) > 3 + i and s[3 + i].strip() == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "fallback": True}


def cpu_sample(steps=1, nc=None):
    """Oracle FP64 Newton (OpenMP element assembly + SuperLU direct solves, the semantics of
    GridapMHD's :julia solver) on a small sample of the same duct (default 6x6x4)."""
    from oracle import oracle as O
    cfg = dict(CFG, nc=nc or SAMPLE_NC, zeta=0.0)
    mesh, dm, params = workload(**cfg)
    prob = O.problem_from_case(mesh, dm, params)
    times = []
    for _ in range(steps):
        t = time.perf_counter()
        O.newton_direct(prob, np.zeros(dm.ndofs), gauge=[dm.offsets["p"]], rtol=1e-10, maxiter=10)
        times.append(time.perf_counter() - t)
    return mesh.ncells, times


def cpu_context():
    """Measured once, outside the steps: the oracle's Newton throughput at growing sample sizes
    (the direct solve's fill grows much faster than the mesh), and its element assembly (the
    residual and the 129 x 129 cell Jacobians) on the full 64x64x4 duct on all host threads."""
    from oracle import oracle as O
    sweep = {}
    for nc in SWEEP_NC:
        n, t = cpu_sample(1, nc)
        sweep[f"{nc[0]}x{nc[1]}x4"] = {"cells": n, "seconds": t[0], "cells_per_s": n / t[0]}
    mesh, dm, params = workload(**CFG)
    fl = O.Fluid(alpha=params["alpha"], beta=params["beta"], gamma=params["gamma"], sigma=params["sigma"],
                 B=params["B"], f=params["f"])
    fc = O.Facets(**{k: v for k, v in params["facets"].items()})
    X, xc = mesh.cell_coords(), dm.cell_values(np.zeros(dm.ndofs))
    t = time.perf_counter()
    O.assemble_cells(X, xc, fl, fc, True)
    ta = time.perf_counter() - t
    return {"newton_sample_sweep": sweep,
            "element_assembly_64x64x4": {"cells_per_s": mesh.ncells / ta, "seconds": ta,
                                         "note": "same configuration; element residuals and Jacobians of all "
                                                 "16,384 cells, FP64, OpenMP on all host threads (no global "
                                                 "CSR insertion)"}}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle as O
    O.build()
    W, K = args.warmup, args.steps
    nc, times = cpu_sample(W + K)
    tk = times[W:]
    sec = float(np.mean(tk))
    val = nc / sec
    cores = os.cpu_count()
    line = {"metric": METRIC, "value": val, "unit": "cells/s", "n_gpus": args.gpus, "steps": K, "warmup": W,
            "ms_per_step": 1e3 * sec, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": f"hunt duct {SAMPLE_NC[0]}x{SAMPLE_NC[1]}x4 sample (Lz=0.2, tanh 3, Ha=500, Re=1, "
                                   "cw=0.1)", "full_workload": "hunt duct 64x64x4", "same_config": False,
                       "solver": "Newton + SuperLU (direct), the :julia solver's semantics"},
            "cpu_baseline": {"value": val, "unit": "cells/s", "cores": cores, "kind": "port",
                             "sample": f"Newton solve of the {SAMPLE_NC[0]}x{SAMPLE_NC[1]}x4 mesh ({nc} cells); "
                                       "element assembly on all host threads, SuperLU single-threaded; the "
                                       "full 976,920-dof duct does not factor with SuperLU in a bounded time"},
            "e2e": {"value": val, "unit": "cells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if not args.no_cpu:
        line["cpu_context"] = cpu_context()
    print(json.dumps(line))


def compare_paths(args, ctx, mesh, dm, d_x_mixed, stream, opts):
    """Outside the timed region: the adjoint gradient of the axial flow rate at mid-length with
    respect to (Ha, cw, f_z per cell) right after the mixed Newton solve (its factors are
    reused), then the plain FP64 GPU path on the same duct: its Newton solve and the per-field
    difference of the mixed solution from it."""
    import torch
    from gbmhd import lib
    from gbmhd.objectives import flow_rate
    out = {}
    x_mixed = d_x_mixed.cpu().numpy()
    g = flow_rate(mesh, dm, 0.1)
    ctx.sweep_stats()  # reset the sweep timers
    t = time.perf_counter()
    # λ to a relative residual of 1e-8 (the gradient target is 1e-6 relative)
    dJ, lam, arep, arc = ctx.adjoint(x_mixed, g, with_cells=True, precision=lib.GBMHD_MIXED, restart=200,
                                     max_linear=600, linear_rtol=1e-8)
    ta = time.perf_counter() - t
    sw_n, sw_s, sw_bytes = ctx.sweep_stats()  # transposed preconditioner applications
    out["adjoint"] = {"seconds": ta, "rc": int(arc), "linear_iters": arep["linear_iters"],
                      "time_setup_pc_s": arep["time_setup_pc_s"],
                      "time_assembly_s": arep["time_assembly_s"], "time_linear_s": arep["time_linear_s"],
                      "transposed_sweeps": {"applications": sw_n,
                                            "ms_per_application": 1e3 * sw_s / sw_n if sw_n else None,
                                            "achieved_gbs": sw_bytes * sw_n / sw_s / 1e9 if sw_s > 0 else None},
                      "n_theta": int(len(dJ)),
                      "dJ_dgamma": float(dJ[0]), "dJ_dcw": float(dJ[1]),
                      "objective": "axial flow rate at z = 0.1",
                      "note": "host call (gbmhd_adjoint) at the mixed solution: FP64 transposed Jacobian, "
                              "the Newton solve's FP32 factors, FGMRES to 1e-8"}
    d64 = torch.zeros_like(d_x_mixed)
    # the FP64 reference is driven to ‖r‖ ≤ 1e-12 ‖r0‖
    o64 = dict(opts, precision=lib.GBMHD_FP64, newton_rtol=1e-12, linear_rtol=1e-10)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    rep64, rc64 = ctx.newton_solve_device(d64.data_ptr(), **o64)
    e1.record(stream)
    torch.cuda.synchronize()
    t64 = e0.elapsed_time(e1) / 1e3
    x64 = d64.cpu().numpy()
    errs = {}
    for f in ("u", "p", "j", "phi"):
        a = x_mixed[dm.offsets[f]:dm.offsets[f] + dm.nfree[f]].copy()
        b = x64[dm.offsets[f]:dm.offsets[f] + dm.nfree[f]].copy()
        den = max(np.linalg.norm(b), 1e-300)
        if f == "p":  # up to a constant, relative to unit pressure (the Hunt pressure is constant)
            a -= a.mean()
            b -= b.mean()
            den = max(np.linalg.norm(b), np.sqrt(len(b)))
        errs[f] = float(np.linalg.norm(a - b) / den)
    out["fp64_gpu"] = {"newton_solve_s": t64, "converged": bool(rc64 == 0), "newton_iters": rep64["newton_iters"],
                       "linear_iters": rep64["linear_iters"], "time_setup_pc_s": rep64["time_setup_pc_s"],
                       "mixed_rel_l2_error_vs_fp64": errs}
    return out


def run_ours(args):
    import torch
    from gbmhd import _build, lib
    from gbmhd.cases import gpu_context
    _build.build()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    dev = torch.device("cuda")
    t0 = time.perf_counter()
    cfg = CFG_SMALL if args.small else CFG
    mesh, dm, params = workload(**cfg)
    ctx = gpu_context(mesh, dm, params)
    t_setup = time.perf_counter() - t0
    n = ctx.ndofs
    stream = torch.cuda.ExternalStream(ctx.stream())
    d_x = torch.zeros(n, dtype=torch.float64, device=dev)
    opts = dict(precision=lib.GBMHD_MIXED, max_newton=12, newton_rtol=1e-12, restart=200, max_linear=600,
                linear_rtol=1e-3)
    reps = []
    for _ in range(args.warmup):
        d_x.zero_()
        torch.cuda.synchronize()
        rep, rc = ctx.newton_solve_device(d_x.data_ptr(), **opts)
        if rc != 0:
            raise RuntimeError(f"Newton did not converge (warm-up): {rep}")
        reps.append(rep)
    torch.cuda.synchronize()
    L0 = lib.counters()
    ctx.sweep_stats()  # reset the sweep timers
    clk = Clocks()
    clk.start()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            d_x.zero_()
        rep, rc = ctx.newton_solve_device(d_x.data_ptr(), **opts)
        if rc != 0:
            raise RuntimeError(f"Newton did not converge: {rep}")
        reps.append(rep)
    e1.record(stream)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = clk.stop()
    L1 = lib.counters()
    sw_n, sw_s, sw_bytes = ctx.sweep_stats()
    ms = e0.elapsed_time(e1) / args.steps
    if world > 1:
        t = torch.tensor([ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = world * mesh.ncells / (ms / 1e3)
    last = reps[-1]
    # e2e: host C-ABI call, host buffers (pinned), H2D of x0 and D2H of the solution inside
    x_host = torch.zeros(n, dtype=torch.float64).pin_memory()
    xh = x_host.numpy()
    te = []
    for _ in range(0 if args.no_e2e else max(1, args.steps)):
        xh[:] = 0.0
        t = time.perf_counter()
        x_out, rep_e, rc = ctx.newton_solve(xh, **opts)
        te.append(time.perf_counter() - t)
    e2e_value = world * mesh.ncells / float(np.mean(te)) if te else None
    # assembly throughput and the dominant-kernel roofline (FP32 Jacobian + FP64 residual)
    d_r = torch.empty(n, dtype=torch.float64, device=dev)
    for _ in range(3):
        ctx.assemble_device(d_x.data_ptr(), d_r.data_ptr(), True, lib.GBMHD_MIXED)
    torch.cuda.synchronize()
    a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    nrep = 10
    a0.record(stream)
    for _ in range(nrep):
        ctx.assemble_device(d_x.data_ptr(), d_r.data_ptr(), True, lib.GBMHD_MIXED)
    a1.record(stream)
    torch.cuda.synchronize()
    asm_ms = a0.elapsed_time(a1) / nrep
    j0, j1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    j0.record(stream)
    for _ in range(nrep):
        ctx.assemble_device(d_x.data_ptr(), 0, True, lib.GBMHD_MIXED)
    j1.record(stream)
    torch.cuda.synchronize()
    jac_ms = j0.elapsed_time(j1) / nrep
    # algorithmic bytes of one FP32 Jacobian assembly: 4 B per element-matrix contribution
    # (14,913 per cell) + per-cell reads (coords 192 B, dof ids 2x516 B, state 1032 B)
    alg_bytes = mesh.ncells * (14913 * 4 + 192 + 2 * 516 + 1032)
    pk = peaks()
    asm_achieved = alg_bytes / (jac_ms / 1e3) / 1e9
    # dominant kernels: the multifrontal solve sweeps; algorithmic bytes = the FP32 factor
    # entries one preconditioner application reads (forward: the unit-lower L, E²/2 + nb·E
    # per front; backward: U with the block inverses, E²/2 + E·nb), timed by CUDA events on
    # the context stream around every application
    sw_achieved = sw_bytes * sw_n / sw_s / 1e9 if sw_s > 0 else None
    extra = {} if args.no_compare else compare_paths(args, ctx, mesh, dm, d_x, stream, opts)
    line = {"metric": METRIC, "value": value, "unit": "cells/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (Jacobian, preconditioner) / f64 (residual, Krylov, update)",
            "data": "synthetic",
            "config": {"workload": f"hunt duct {cfg['nc'][0]}x{cfg['nc'][1]}x{cfg['nz']}, Lz={cfg['Lz']}, "
                                   f"tanh({cfg['beta_map']:g}x) stretching, Ha={cfg['Ha']:g}, Re={cfg['Re']:g}, "
                                   f"cw={cfg['cw']:g}, zeta={cfg['zeta']:g}", "ncells": mesh.ncells, "ndofs": n,
                       "nnz": ctx.nnz,
                       "precision": "mixed", "newton_rtol": 1e-12,
                       "l2": "inputs larger than L2 (Jacobian values alone 0.78 GB)"},
            "newton_solve_s": ms / 1e3, "newton_iters": last["newton_iters"], "linear_iters": last["linear_iters"],
            "linear_iters_per_step": [r["linear_iters"] for r in reps[-args.steps:]],
            "pc_refactorizations": sum(r["pc_refactorizations"] for r in reps),
            "residual_history": [float("%.3e" % v) for v in last.get("residual_history", [])],
            "time_split_s": {k: last[k] for k in ("time_assembly_s", "time_setup_pc_s", "time_linear_s")},
            "assembly_cells_per_s": mesh.ncells / (asm_ms / 1e3), "jacobian_cells_per_s": mesh.ncells / (jac_ms / 1e3),
            "setup_s": t_setup,
            "e2e": {"value": e2e_value, "unit": "cells/s", "h2d_bytes_per_step": 8 * n, "d2h_bytes_per_step": 8 * n},
            "gpu_launches": int(L1["launches"] - L0["launches"]),
            "library_gemm_calls": int(L1["gemm_calls"] - L0["gemm_calls"]),
            "roofline": {"kernel": "multifrontal preconditioner application: one CUDA graph launch of the LU sweeps "
                                   "(k_chain_fwd + k_rect_tma forward, k_rect_tma + k_chain_bwd backward, over all "
                                   "levels and super-blocks)", "bound": "hbm",
                         "achieved": sw_achieved, "peak": pk.get("hbm_gbs"), "unit": "GB/s",
                         "frac": sw_achieved / pk.get("hbm_gbs") if sw_achieved else None,
                         "traffic": None, "bytes_per_application": sw_bytes, "applications": sw_n,
                         "ms_per_application": 1e3 * sw_s / sw_n if sw_n else None,
                         "share_of_step": sw_s / (args.steps * ms / 1e3),
                         "note": "of measured" if not pk.get("fallback") else "of fallback"},
            "roofline_assembly": {"kernel": "k_cells<float,JAC> (FP32 Jacobian assembly)", "bound": "hbm",
                                  "achieved": asm_achieved, "peak": pk.get("hbm_gbs"), "unit": "GB/s",
                                  "frac": asm_achieved / pk.get("hbm_gbs"),
                                  "note": "of measured" if not pk.get("fallback") else "of fallback"},
            "clocks": clocks}
    line.update(extra)
    if extra.get("adjoint"):
        # spec ratio: plain FP64 GPU Newton solve ÷ (mixed Newton solve + adjoint gradient)
        line["fp64_newton_over_mixed_newton_plus_adjoint"] = (
            extra["fp64_gpu"]["newton_solve_s"] / (ms / 1e3 + extra["adjoint"]["seconds"]))
    if not args.no_cpu and rank == 0:
        nc_s, times = cpu_sample(1)
        line["cpu_baseline"] = {"value": nc_s / times[0], "unit": "cells/s", "cores": os.cpu_count(), "kind": "port",
                                "sample": f"FP64 oracle Newton + SuperLU on the {SAMPLE_NC[0]}x{SAMPLE_NC[1]}x4 "
                                          f"duct ({nc_s} cells)"}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


# The sudden-expansion configuration: 3-D channel of rectangular section, inlet 1 (z) x 0.5 (y),
# expanding 4x in y at x = 0, 2 upstream and 8 downstream; ~97k hexes graded toward the walls
# and the step (more cells along the channel than across it: the factors of the 3-D separators
# must fit in one GPU's memory); Ha = 1000, Re = 10, MHD scaling; parabolic inlet of mean 1 over
# the outlet section; thin-wall law with cw = 0 (insulating) and τ = 100 on the walls; natural
# outlet.  Objective: mean inlet pressure − mean outlet pressure.
EXPANSION = dict(n_up=24, n_down=330, n_y_in=12, n_y_out=12, n_z=8, L_up=2.0, L_down=8.0, grading=4.0,
                 Ha=1000.0, Re=10.0, thin_wall=(100.0, 0.0))


def run_expansion(args):
    """The expansion configuration end to end on the GPU: mixed-precision Newton solve, adjoint
    gradient of the pressure drop w.r.t. (Ha, cw) and its check against central finite
    differences of further Newton solves.  One JSON line; not part of the default bench."""
    import torch
    from gbmhd import _build, lib
    from gbmhd.cases import expansion_case, gpu_context
    from gbmhd.objectives import ha_gradient, pressure_drop
    _build.build()
    cfg = dict(EXPANSION)
    if args.small:
        cfg.update(n_up=6, n_down=40, n_y_in=6, n_y_out=6, n_z=6)
    t0 = time.perf_counter()
    mesh, dm, params = expansion_case(**cfg)
    ctx = gpu_context(mesh, dm, params)
    t_setup = time.perf_counter() - t0
    g = pressure_drop(mesh, dm)
    opts = dict(precision=lib.GBMHD_MIXED, max_newton=20, newton_rtol=1e-12, restart=100, max_linear=800,
                linear_rtol=1e-3)
    t = time.perf_counter()
    x, rep, rc = ctx.newton_solve(np.zeros(dm.ndofs), **opts)
    t_newton = time.perf_counter() - t
    sw_n, sw_s, sw_bytes = ctx.sweep_stats()
    out = {"metric": "expansion: mixed Newton solve + pressure-drop adjoint (Ha, cw)", "impl": "ours",
           "config": {"workload": f"sudden expansion {mesh.ncells} cells (nx {cfg['n_up']}+{cfg['n_down']}, "
                                  f"ny {cfg['n_y_in']}+2x{cfg['n_y_out']}, nz {cfg['n_z']}), Ha=1000, Re=10, "
                                  "MHD scaling, thin wall cw=0 tau=100", "ncells": mesh.ncells, "ndofs": dm.ndofs,
                      "nnz": ctx.nnz},
           "setup_host_s": t_setup, "newton_solve_s": t_newton, "newton_rc": int(rc), "report": rep,
           "preconditioner": {"applications": sw_n, "ms_per_application": 1e3 * sw_s / sw_n if sw_n else None,
                              "factor_gbytes_read_per_application": sw_bytes / 1e9}}
    if rc != 0:
        print(json.dumps(out))
        return
    Ha, Re = cfg["Ha"], cfg["Re"]
    t = time.perf_counter()
    dJ, lam, arep, arc = ctx.adjoint(x, g, with_cells=False, precision=lib.GBMHD_MIXED, restart=100, max_linear=800,
                                     linear_rtol=1e-8)
    t_adj = time.perf_counter() - t
    dHa = ha_gradient(dJ, Ha, Re, "mhd")
    out.update(adjoint_s=t_adj, adjoint_rc=int(arc), adjoint_linear_iters=arep["linear_iters"], J=float(g @ x),
               dJ_dHa=dHa, dJ_dcw=float(dJ[1]), dJ_dalpha=float(dJ[2]), dJ_dbeta=float(dJ[3]))
    # central finite differences (step 1e-6 relative in Ha, 1e-4 absolute in cw around 0)
    def J_of(p):
        ctx.set_params(p)
        xs, r, c = ctx.newton_solve(x, **dict(opts, newton_rtol=0.0, newton_atol=0.0, max_newton=6,
                                              linear_rtol=1e-10))
        return float(g @ xs)
    h = 1e-6
    p0 = dict(params)
    N = lambda ha: ha ** 2 / Re
    pp = dict(p0, alpha=1.0 / N(Ha * (1 + h)), beta=1.0 / (Ha * (1 + h)) ** 2)
    pm = dict(p0, alpha=1.0 / N(Ha * (1 - h)), beta=1.0 / (Ha * (1 - h)) ** 2)
    fd_ha = (J_of(pp) - J_of(pm)) / (2 * h * Ha)
    f = p0["facets"]
    hc = 1e-4
    fd_cw = (J_of(dict(p0, facets=dict(f, cw=f["cw"] + hc))) - J_of(dict(p0, facets=dict(f, cw=f["cw"] - hc)))) / (2 * hc)
    ctx.set_params(p0)
    out.update(fd_dJ_dHa=fd_ha, fd_dJ_dcw=fd_cw, rel_err_dHa=abs(fd_ha - dHa) / abs(dHa),
               rel_err_dcw=abs(fd_cw - dJ[1]) / abs(dJ[1]) if dJ[1] != 0 else None,
               gpu_mem_gb=torch.cuda.mem_get_info()[1] / 1e9 - torch.cuda.mem_get_info()[0] / 1e9)
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--small", action="store_true", help="32x32x3 duct (profiling captures)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-compare", action="store_true", help="skip the FP64-path and adjoint comparison")
    ap.add_argument("--expansion", action="store_true",
                    help="the sudden-expansion configuration (~97k cells, Ha=1000) instead of the duct bench")
    args = ap.parse_args()
    if args.expansion:
        run_expansion(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
