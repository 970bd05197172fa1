"""The tensor-core FP32 GEMM of the factorization (tcgen05, three-way BF16 splits) against FP64
products of the same FP32 inputs.

The shapes are those of the LU panel and trailing updates: K of a pivot block or a panel
(8 … 128, not always a multiple of 16), M and N not multiples of the 128 x 128 tile, several
problems per launch, α = ±1, β ∈ {0, 1}, leading dimensions larger than the rows.  Tolerance:
relative to Σ_k |a_ik b_kj| + |β c_ij|, the worst entry error may be at most 4 times that of
an FP32 SGEMM (numpy's, on the same FP32 inputs) and at most 2e-6 (FP32 products of up to 128
terms)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [  # m, n, k, batch, alpha, beta
    (128, 128, 64, 1, 1.0, 0.0),
    (300, 64, 64, 3, 1.0, 0.0),
    (200, 40, 24, 2, -1.0, 1.0),
    (64, 500, 64, 2, -1.0, 1.0),
    (700, 650, 128, 2, -1.0, 1.0),
    (129, 257, 8, 1, -1.0, 1.0),
    (384, 384, 72, 4, -1.0, 1.0),
    (2048, 2048, 128, 4, -1.0, 1.0),  # a trailing update of the size of a top-level front
]


@pytest.mark.parametrize("shape", SHAPES)
def test_tc_gemm_matches_fp64(gpu_lib, shape):
    torch = pytest.importorskip("torch")
    m, n, k, batch, alpha, beta = shape
    lda, ldb, ldc = m + 8, k + 8, m + 16
    rng = np.random.default_rng(m * 7 + n * 3 + k)
    A = np.zeros((batch, k, lda), np.float32)   # column-major: A[b, col, row]
    B = np.zeros((batch, n, ldb), np.float32)
    Cm = np.zeros((batch, n, ldc), np.float32)
    A[:, :, :m] = rng.standard_normal((batch, k, m)) * np.exp(rng.uniform(-3, 3, (batch, k, 1)))
    B[:, :, :k] = rng.standard_normal((batch, n, k))
    Cm[:, :, :m] = rng.standard_normal((batch, n, m))
    dA, dB, dC = (torch.from_numpy(a).cuda() for a in (A, B, Cm))
    st = C.c_int32(-1)
    rc = gpu_lib.gbmhd_diag_tc_gemm(m, n, k, alpha, dA.data_ptr(), lda, k * lda, dB.data_ptr(), ldb, n * ldb, beta,
                                    dC.data_ptr(), ldc, n * ldc, batch, C.byref(st))
    assert rc == 0 and st.value == 0, (rc, st.value)
    out = dC.cpu().numpy()
    for b in range(batch):
        a = A[b, :, :m].T.astype(np.float64)           # m x k
        bb = B[b, :, :k].T.astype(np.float64)          # k x n
        c = Cm[b, :, :m].T.astype(np.float64)          # m x n
        ref = alpha * a @ bb + beta * c
        scale = np.abs(a) @ np.abs(bb) + abs(beta) * np.abs(c)
        got = out[b, :, :m].T.astype(np.float64)
        err = np.abs(got - ref) / scale
        sg = (np.float32(alpha) * (A[b, :, :m].T @ B[b, :, :k].T) + np.float32(beta) * Cm[b, :, :m].T).astype(np.float64)
        err_sgemm = np.abs(sg - ref) / scale
        assert err.max() <= min(2e-6, max(4 * err_sgemm.max(), 2e-7)), (b, err.max(), err_sgemm.max())
    # rows beyond m and the padding of every column are left untouched
    assert np.array_equal(out[:, :, m:], Cm[:, :, m:])
