// FP32 strided-batched GEMM on the tcgen05 tensor cores (tc_gemm.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

namespace gbmhd {
// C = α·A·B + β·C for `batch` column-major problems (A m x k, B k x n, C m x n; strides sA, sB, sC
// between problems), 1 ≤ k ≤ 128, on `stream`.  FP32 accuracy from three-way BF16 splits.
// A tensor-core wait that times out sets *err = 2 (device) and leaves its tile unwritten.
// Returns 0, or < 0 with *msg on invalid arguments or a launch error.
int tc_gemm_f32(cudaStream_t stream, int m, int n, int k, float alpha, const float* A, int lda, long long sA,
                const float* B, int ldb, long long sB, float beta, float* C, int ldc, long long sC, int batch,
                int32_t* err, std::string* msg);
}  // namespace gbmhd
