// FP32 strided-batched GEMM on the tcgen05 tensor cores (sm_103a), for the dense updates of the
// multifrontal factorization:  C = α·A·B + β·C,  column-major, K ≤ 128.
//
// FP32 accuracy from BF16 tensor cores: every operand entry is split into three BF16 parts,
// a = a0 + a1 + a2 (a0 = bf16(a), a1 = bf16(a − a0), a2 = bf16(a − a0 − a1); 3 × 8 significant
// bits cover FP32's 24), and the product keeps the six cross terms of order ≥ 2⁻¹⁶ relative:
// a0b0 + a0b1 + a1b0 + a0b2 + a1b1 + a2b0.  The dropped terms are O(2⁻²⁴) relative, the size of
// FP32 rounding.  (This is the usual multi-word splitting of a wide product into narrow
// tensor-core products; the accumulation is FP32 in tensor memory.)
//
// One CTA per 128 x 128 tile of C (grid: M tiles, N tiles, batch), 256 threads:
//   - K is staged in halves of 64: threads 0..127 load row i of the A tile, threads 128..255
//     row j of the Bᵀ tile, split them and store the parts in shared memory in the canonical
//     K-major, no-swizzle layout (8-row x 16-byte core matrices: 16 B apart along a row group,
//     SBO = 128 B between row groups, LBO = 128 rows x 16 B between K groups of 8);
//   - thread 0 issues 4 K-steps x 6 products of tcgen05.mma.kind::f16 (M = 128, N = 128,
//     K = 16) into one FP32 accumulator of 128 tensor-memory columns, and commits them to an
//     mbarrier that every thread waits on (bounded spins);
//   - the epilogue reads the accumulator with tcgen05.ld (warp w: lanes 32·(w mod 4).., columns
//     64·(w / 4)..) and writes α·acc + β·C with coalesced column accesses.
// A wait that runs out sets *err = 2, waits once more (bounded) for the MMAs in flight, frees
// the tensor memory and leaves the tile unwritten.
#include <cuda_bf16.h>

#include "internal.h"
#include "tc_gemm.h"

namespace gbmhd {
namespace {

constexpr int TM = 128, TN = 128, KH = 64;  // tile rows, tile columns, K staged per half
constexpr int TC_THREADS = 256;
constexpr int PART_BYTES = TM * KH * 2;     // one BF16 part of one operand half: 16 KB
constexpr long TC_WAIT_LIMIT = 1L << 24;

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor, K-major, no swizzle (start, LBO, SBO in 16-byte units;
// bits 46-48 = 0b001 for tcgen05).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: D FP32, A and B BF16, both K-major, M = 128, N = 128.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TN >> 3) << 17) | ((uint32_t)(TM >> 4) << 24);

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate));
}

__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t phase, long limit) {
  for (long i = 0; i < limit; ++i) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(phase)
        : "memory");
    if (ok) return true;
  }
  return false;
}

// Split 8 consecutive K values of one row into three BF16 parts and store each as one
// 16-byte core-matrix row.
__device__ __forceinline__ void split_store(const float (&v)[8], unsigned char* p0, unsigned char* p1,
                                            unsigned char* p2) {
  __align__(16) __nv_bfloat16 h0[8], h1[8], h2[8];
#pragma unroll
  for (int u = 0; u < 8; ++u) {
    const __nv_bfloat16 a0 = __float2bfloat16_rn(v[u]);
    const float r1 = v[u] - __bfloat162float(a0);
    const __nv_bfloat16 a1 = __float2bfloat16_rn(r1);
    const float r2 = r1 - __bfloat162float(a1);
    h0[u] = a0;
    h1[u] = a1;
    h2[u] = __float2bfloat16_rn(r2);
  }
  *reinterpret_cast<uint4*>(p0) = *reinterpret_cast<const uint4*>(h0);
  *reinterpret_cast<uint4*>(p1) = *reinterpret_cast<const uint4*>(h1);
  *reinterpret_cast<uint4*>(p2) = *reinterpret_cast<const uint4*>(h2);
}

__global__ void __launch_bounds__(TC_THREADS, 2)
    k_tc_gemm(int m, int n, int k, float alpha, const float* __restrict__ A, int lda, long long sA,
              const float* __restrict__ B, int ldb, long long sB, float beta, float* __restrict__ C, int ldc,
              long long sC, int32_t* err) {
  extern __shared__ __align__(1024) unsigned char tc_smem[];
  // [A part 0..2][B part 0..2], each PART_BYTES
  __shared__ __align__(8) uint64_t done_bar;
  __shared__ uint32_t tmem_slot;
  __shared__ int failed;
  const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
  const int64_t bz = blockIdx.z;
  const float* Ab = A + bz * sA;
  const float* Bb = B + bz * sB;
  float* Cb = C + bz * sC;
  const int i0 = blockIdx.x * TM, j0 = blockIdx.y * TN;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_slot)),
                 "r"(TN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&done_bar)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    failed = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_slot;
  const uint32_t base = smem_addr(tc_smem);
  const int kpad = (k + 15) / 16 * 16;
  const int nhalf = (kpad + KH - 1) / KH;
  uint32_t phase = 0;
  for (int h = 0; h < nhalf; ++h) {
    // ---- stage K columns [h·KH, h·KH + KH) of the A rows and Bᵀ rows, split into parts
    const int kb0 = h * KH;
    const bool isA = tid < TM;
    const int row = isA ? tid : tid - TM;  // row of the A tile (i) or of the Bᵀ tile (j)
    const int gi = (isA ? i0 : j0) + row;
    const bool live = isA ? gi < m : gi < n;
    unsigned char* op = tc_smem + (isA ? 0 : 3 * PART_BYTES);
    // all KH loads of the row first (one memory round trip), then the splits
    float v[KH];
    const float* src = isA ? Ab + gi : Bb + (int64_t)gi * ldb;
    const int64_t stride = isA ? lda : 1;
    const int kn = live ? min(KH, k - kb0) : 0;
    if (!isA && kn == KH && (reinterpret_cast<uintptr_t>(src + kb0) & 15) == 0) {
      // a row of Bᵀ is K-contiguous: sixteen 16-byte loads
#pragma unroll
      for (int u = 0; u < KH / 4; ++u) {
        const float4 q = *reinterpret_cast<const float4*>(src + kb0 + 4 * u);
        v[4 * u] = q.x; v[4 * u + 1] = q.y; v[4 * u + 2] = q.z; v[4 * u + 3] = q.w;
      }
    } else {
#pragma unroll
      for (int u = 0; u < KH; ++u) v[u] = u < kn ? src[(int64_t)(kb0 + u) * stride] : 0.0f;
    }
#pragma unroll
    for (int kc = 0; kc < KH / 8; ++kc) {
      // core matrix (row group row/8, K group kc): kc·(128·16) + (row/8)·128 + (row%8)·16
      const int off = kc * (TM * 16) + (row >> 3) * 128 + (row & 7) * 16;
      split_store(*reinterpret_cast<const float(*)[8]>(v + 8 * kc), op + off, op + PART_BYTES + off,
                  op + 2 * PART_BYTES + off);
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    // ---- one thread issues the MMAs of this half and commits them to the barrier
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      const int ksteps = min(KH, kpad - kb0) / 16;
      const int pa[6] = {0, 0, 1, 0, 1, 2}, pb[6] = {0, 1, 0, 2, 1, 0};
      for (int ks = 0; ks < ksteps; ++ks)
        for (int t = 0; t < 6; ++t) {
          const uint32_t a_addr = base + pa[t] * PART_BYTES + ks * 2 * (TM * 16);
          const uint32_t b_addr = base + (3 + pb[t]) * PART_BYTES + ks * 2 * (TN * 16);
          const uint64_t ad = smem_desc(a_addr, TM * 16, 128), bd = smem_desc(b_addr, TN * 16, 128);
          mma_bf16(tmem, ad, bd, (h > 0 || ks > 0 || t > 0) ? 1u : 0u);
        }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_addr(&done_bar))
                   : "memory");
    }
    // ---- every thread waits for the MMAs (they read the shared memory about to be reused)
    if (!mbar_wait(&done_bar, phase, TC_WAIT_LIMIT)) {
      failed = 1;
      mbar_wait(&done_bar, phase, TC_WAIT_LIMIT);  // let the MMAs in flight finish
    }
    phase ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;");
    __syncthreads();
    if (failed) break;
  }
  if (!failed) {
    // ---- epilogue: warp w reads lanes 32·(w % 4).. (tile rows) and columns 64·(w / 4)..
    const int q = warp & 3, ch = warp >> 2;
    const int gi = i0 + 32 * q + lane;
    for (int cb = 0; cb < 2; ++cb) {
      const int c0 = 64 * ch + 32 * cb;
      uint32_t r[32];
      const uint32_t taddr = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
          "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
            "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
            "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (gi < m) {
#pragma unroll
        for (int c = 0; c < 32; ++c) {
          const int gj = j0 + c0 + c;
          if (gj < n) {
            float* p = Cb + gi + (int64_t)gj * ldc;
            const float acc = __uint_as_float(r[c]);
            *p = beta == 0.0f ? alpha * acc : fmaf(alpha, acc, beta * *p);
          }
        }
      }
    }
  } else if (tid == 0) {
    atomicExch(err, 2);
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TN));
}

}  // namespace

constexpr size_t kTcSmem = 6 * (size_t)PART_BYTES;  // 96 KB: two CTAs per SM

int tc_gemm_f32(cudaStream_t stream, int m, int n, int k, float alpha, const float* A, int lda, long long sA,
                const float* B, int ldb, long long sB, float beta, float* C, int ldc, long long sC, int batch,
                int32_t* err, std::string* msg) {
  if (m <= 0 || n <= 0 || batch <= 0) return 0;
  if (k <= 0 || k > 2 * KH) {
    if (msg) *msg = "tensor-core GEMM: K = " + std::to_string(k) + " outside [1, 128]";
    return -1;
  }
  if (batch > 65535) {
    if (msg) *msg = "tensor-core GEMM: batch " + std::to_string(batch) + " exceeds 65535";
    return -1;
  }
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(k_tc_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem);
    if (e != cudaSuccess) {
      if (msg) *msg = std::string("tensor-core GEMM: ") + cudaGetErrorString(e);
      return -2;
    }
    attr_set = true;
  }
  dim3 grid((unsigned)((m + TM - 1) / TM), (unsigned)((n + TN - 1) / TN), (unsigned)batch);
  k_tc_gemm<<<grid, TC_THREADS, kTcSmem, stream>>>(m, n, k, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, err);
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    if (msg) *msg = std::string("tensor-core GEMM launch: ") + cudaGetErrorString(e);
    return -2;
  }
  return 0;
}

}  // namespace gbmhd

// Diagnostic entry point (include/gbmhd.h): the GEMM above on device buffers, for tests.
extern "C" int gbmhd_diag_tc_gemm(int32_t m, int32_t n, int32_t k, float alpha, const float* A, int32_t lda,
                                  int64_t sA, const float* B, int32_t ldb, int64_t sB, float beta, float* C,
                                  int32_t ldc, int64_t sC, int32_t batch, int32_t* status) {
  int32_t* d_err = nullptr;
  if (cudaMalloc(&d_err, sizeof(int32_t)) != cudaSuccess) return -2;
  cudaMemset(d_err, 0, sizeof(int32_t));
  std::string msg;
  int rc = gbmhd::tc_gemm_f32(nullptr, m, n, k, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, batch, d_err, &msg);
  if (rc == 0 && cudaDeviceSynchronize() != cudaSuccess) rc = -2;
  int32_t h = 0;
  cudaMemcpy(&h, d_err, sizeof(int32_t), cudaMemcpyDeviceToHost);
  cudaFree(d_err);
  if (status) *status = h;
  return rc;
}
