"""The float-float pivot-block inverses of the FP32 factorization (64 x 64 diagonal blocks,
partial pivoting inside the block).

All four kernel variants run the same float-float operations on every entry in the same
order, so they must agree bit for bit; against an FP64 inverse of the same FP32 block, the
error of the FP32-rounded result is bounded by a few units of FP32 rounding relative to
|A⁻¹| (the float-float arithmetic carries ~48 bits, so κ(A) barely enters).  Blocks: random
ones whose row scales span e^6 (so the pivot order is not the identity), a
permuted diagonally dominant one, a short last block (kb < 64) and a singular one (status
1, no fault).  The timing line compares the variants at the launch widths of the top and
bottom levels of a 64×64×4 factorization."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

VARIANTS = (0, 1, 2, 3)


def _fronts(count, n, kb, seed, kind="random"):
    rng = np.random.default_rng(seed)
    F = np.zeros((count, n, n), np.float32)  # F[f, col, row]: column-major fronts
    for f in range(count):
        if kind == "random":
            A = rng.standard_normal((kb, kb)) * np.exp(rng.uniform(-3, 3, (kb, 1)))
        elif kind == "dominant":
            A = rng.standard_normal((kb, kb)) + np.diag(rng.uniform(20, 40, kb))
            A = A[rng.permutation(kb)]
        else:  # singular: a zero column
            A = rng.standard_normal((kb, kb))
            A[:, kb // 2] = 0.0
        F[f, :kb, :kb] = A.T.astype(np.float32)
        F[f, kb:, :] = rng.standard_normal((n - kb, n)).astype(np.float32)  # beyond the block
        F[f, :kb, kb:] = rng.standard_normal((kb, n - kb)).astype(np.float32)
    return F


def _run(gpu_lib, torch, F, kb, variant, reps=0):
    count, n = F.shape[0], F.shape[1]
    dF = torch.from_numpy(F).cuda()
    dP = torch.full((count, 64, 64), float("nan"), dtype=torch.float32, device="cuda")
    ms = C.c_double(0.0)
    st = C.c_int32(-1)
    rc = gpu_lib.gbmhd_diag_pivot_inverse(variant, count, n, kb, dF.data_ptr(), dP.data_ptr(), reps, C.byref(ms),
                                          C.byref(st))
    assert rc == 0, rc
    return dP.cpu().numpy(), st.value, ms.value


@pytest.mark.parametrize("case", [("random", 5, 64, 64), ("dominant", 3, 80, 64), ("random", 4, 72, 48)])
def test_pivot_inverse_variants_agree_and_invert(gpu_lib, case):
    torch = pytest.importorskip("torch")
    kind, count, n, kb = case
    F = _fronts(count, n, kb, seed=count * 100 + kb, kind=kind)
    outs = []
    for v in VARIANTS:
        P, st, _ = _run(gpu_lib, torch, F, kb, v)
        assert st == 0, (v, st)
        outs.append(P)
    for v in VARIANTS[1:]:
        assert np.array_equal(outs[0].view(np.uint32), outs[v].view(np.uint32)), v
    for f in range(count):
        A = F[f, :kb, :kb].T.astype(np.float64)
        X = np.linalg.inv(A)
        got = outs[0][f].T  # row-major view of the column-major block
        assert np.all(got[kb:, :] == 0) and np.all(got[:, kb:] == 0)
        err = np.abs(got[:kb, :kb] - X).max() / np.abs(X).max()
        assert err < 2e-6, (f, err)


def test_pivot_inverse_singular_block_sets_status(gpu_lib):
    torch = pytest.importorskip("torch")
    F = _fronts(2, 64, 64, seed=7, kind="singular")
    P0, st0, _ = _run(gpu_lib, torch, F, 64, 0)
    P3, st3, _ = _run(gpu_lib, torch, F, 64, 3)
    assert st0 == 1 and st3 == 1
    assert np.array_equal(P0.view(np.uint32), P3.view(np.uint32))


def test_pivot_inverse_timing(gpu_lib):
    torch = pytest.importorskip("torch")
    lines = []
    for count in (1, 8, 64, 256, 2048):
        F = _fronts(min(count, 16), 64, 64, seed=11)
        F = np.concatenate([F] * ((count + 15) // 16))[:count]
        times = []
        for v in VARIANTS:
            _, st, ms = _run(gpu_lib, torch, F, 64, v, reps=20)
            assert st == 0
            times.append(ms * 1e3)
        lines.append(f"{count} blocks: " + ", ".join(f"v{v} {t:.1f} us" for v, t in zip(VARIANTS, times)))
    print("\npivot inverse per launch: " + "; ".join(lines))
