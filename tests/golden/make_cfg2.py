"""Golden FP64 solution of the 32x32x3 stretched duct (Ha=100, Re=10, cw=0.1) from the CPU
oracle (FP64 assembly, one SuperLU factorization, chord iterations to the Newton root), for
the GPU parity test at that size.

    python tests/golden/make_cfg2.py
writes tests/golden/cfg2_norms.json and tests/golden/cfg2_solution.npz (about half an hour
on 8 cores: the SuperLU factorization of the 182,034-dof Jacobian dominates).
"""
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "gridapmhd.jl_gb300"), os.path.join(ROOT, "tests")):
    sys.path.insert(0, p)

import numpy as np  # noqa: E402

from helpers import hunt_case, oracle_problem  # noqa: E402
from oracle import oracle as O  # noqa: E402

CFG2 = dict(nc=(32, 32), nz=3, Ha=100.0, Re=10.0, beta_map=2.0, cw=0.1, Lz=0.2)


def main():
    mesh, dm, params = hunt_case(**CFG2)
    prob = oracle_problem(mesh, dm, params)
    t = time.time()
    x, info = O.newton_chord(prob, np.zeros(dm.ndofs), gauge=[dm.offsets["p"]], rtol=1e-14, maxiter=60,
                             verbose=True)
    el = time.time() - t
    nrm = O.field_norms(mesh.cell_coords(), dm.cell_values(x))
    sp = dm.split(x)
    p = sp["p"] - sp["p"].mean()
    out = dict(config=CFG2, ndofs=dm.ndofs, nls_iters=info["nls_iters"], residuals=[float(v) for v in info["residuals"]],
               norms={k: float(v) for k, v in nrm.items()},
               dof_norms={"u": float(np.linalg.norm(sp["u"])), "j": float(np.linalg.norm(sp["j"])),
                          "phi": float(np.linalg.norm(sp["phi"])), "p_modulo_const": float(np.linalg.norm(p))},
               seconds=el)
    np.savez_compressed(os.path.join(HERE, "cfg2_solution.npz"), x=x)
    with open(os.path.join(HERE, "cfg2_norms.json"), "w") as fh:
        json.dump(out, fh, indent=1)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
