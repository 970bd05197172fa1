"""Problem builders shared by the tests (host mirror + oracle on the same inputs)."""
import numpy as np

from gbmhd.cases import expansion_case, gpu_context, hunt_case  # noqa: F401  (re-exported)
from oracle import oracle as O


def oracle_problem(mesh, dm, params):
    return O.problem_from_case(mesh, dm, params)


def random_state(dm, seed=1, scale=1.0):
    rng = np.random.default_rng(seed)
    return scale * rng.standard_normal(dm.ndofs)
