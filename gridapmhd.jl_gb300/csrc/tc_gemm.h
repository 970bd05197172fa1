// FP32 strided-batched GEMM on the tcgen05 tensor cores (tc_gemm.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

namespace gbmhd {
// Device workspace (bytes) that tc_gemm_f32 needs for these sizes: the BF16 split images of A
// and Bᵀ (1.5 x their FP32 bytes, padded to 128-row blocks and K stages of 32).
size_t tc_gemm_workspace(int m, int n, int k, int batch);

// C = α·A·B + β·C for `batch` column-major problems (A m x k, B k x n, C m x n; strides sA, sB, sC
// between problems), 1 ≤ k ≤ 128, on `stream`.  FP32 accuracy from three-way BF16 splits.
// ws: a 16-byte aligned device workspace of at least tc_gemm_workspace(m, n, k, batch) bytes,
// used by this call's kernels only (stream order).  A tensor-core wait that times out sets
// *err = 2 (device) and leaves its tile unwritten.  Returns 0, or < 0 with *msg on invalid
// arguments (including a workspace too small) or a launch error.
int tc_gemm_f32(cudaStream_t stream, int m, int n, int k, float alpha, const float* A, int lda, long long sA,
                const float* B, int ldb, long long sB, float beta, float* C, int ldc, long long sC, int batch,
                void* ws, size_t ws_bytes, int32_t* err, std::string* msg);
}  // namespace gbmhd
