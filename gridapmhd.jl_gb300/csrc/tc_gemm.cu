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
// Two launches per GEMM:
//   - k_tc_split writes the parts of every 128-row block of A and of Bᵀ, per K stage of
//     KC = 32, into a workspace in the exact shared-memory image an MMA stage reads: the
//     canonical K-major, no-swizzle layout (8-row x 16-byte core matrices: 16 B apart along
//     a row group, SBO = 128 B between row groups, LBO = 128 rows x 16 B between K groups of
//     8), three 8 KB parts per block and stage.  Each operand entry is split once, not once
//     per tile that reads it.
//   - k_tc_gemm, persistent and warp-specialized: one CTA per SM walks the 128 x 128 tiles
//     of C (all problems of the batch) with a ring of NST stages and two tensor-memory
//     accumulators, so that the epilogue of one tile overlaps the MMAs of the next.
//       warp 0 (producer): one thread copies a stage's A and B images (24 KB each) with
//         cp.async.bulk onto the stage's `full` barrier;
//       warp 1 (MMA): one thread issues 2 K-steps x 6 products of tcgen05.mma.kind::f16
//         (M = 128, N = 128, K = 16) per stage into the tile's FP32 accumulator (128
//         tensor-memory columns), commits each stage to its `empty` barrier and each tile
//         to `acc_full`;
//       warps 2-5 (epilogue): C moves in chunks of 32 columns through a ring of four
//         shared-memory buffers, loaded by TMA three chunks ahead and written back by TMA
//         stores (one thread issues both); warp w combines accumulator lanes 32·(w mod 4)..
//         (tcgen05.ld) with the chunk in place and arrives on `acc_empty` after each tile.
// Every wait is bounded.  One that runs out sets *err = 2 and an abort flag that ends the
// other roles' loops; the MMA thread then waits (bounded) for its MMAs in flight before the
// tensor memory is freed, and the tiles not finished are left unwritten.
#include <cuda.h>  // CUtensorMap (the encoder is reached through the runtime's driver entry point)
#include <cuda_bf16.h>

#include <algorithm>

#include "internal.h"
#include "tc_gemm.h"

namespace gbmhd {
namespace {

constexpr int TM = 128, TN = 128, KC = 32;  // tile rows, tile columns, K per stage
constexpr int NST = 3;                      // stages in the ring
constexpr int PART_BYTES = TM * KC * 2;     // one BF16 part of one 128-row block and stage: 8 KB
constexpr int IMG_BYTES = 3 * PART_BYTES;   // the three parts of one operand stage: 24 KB
constexpr int STAGE_BYTES = 2 * IMG_BYTES;  // A parts 0..2, B parts 0..2
constexpr int CW = 32, NCB = 4;            // C chunks of 32 columns, a ring of 4 buffers
constexpr int CHUNK_BYTES = CW * TM * 4;    // 16 KB
constexpr int CTILE_BYTES = NCB * CHUNK_BYTES;  // the C ring of the epilogue: 64 KB
constexpr int PROD_WARP = 0, MMA_WARP = 1, EPI_WARP0 = 2, EPI_WARPS = 4;
constexpr int TC_THREADS = 32 * (EPI_WARP0 + EPI_WARPS);
constexpr int ACC_COLS = 2 * TN;            // two accumulators
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

__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Waits for the phase of the given parity; false when the limit runs out (the abort flag is
// then raised) or another role raised the flag.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag) {
  for (long i = 0; i < TC_WAIT_LIMIT; ++i) {
    if (mbar_test(bar, parity)) return true;
    if ((i & 63) == 63 && *abort_flag) return false;
  }
  *abort_flag = 1;
  return false;
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
               : "memory");
}

// Split 8 consecutive K values of one row into three BF16 parts and store each as one
// 16-byte core-matrix row.
__device__ __forceinline__ uint32_t bf16x2(__nv_bfloat16 lo, __nv_bfloat16 hi) {
  return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

__device__ __forceinline__ void split_store(const float (&v)[8], unsigned char* p0, unsigned char* p1,
                                            unsigned char* p2) {
  uint32_t w0[4], w1[4], w2[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    __nv_bfloat16 a0[2], a1[2], a2[2];
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      const float x = v[2 * u + e];
      a0[e] = __float2bfloat16_rn(x);
      const float r1 = x - __bfloat162float(a0[e]);
      a1[e] = __float2bfloat16_rn(r1);
      a2[e] = __float2bfloat16_rn(r1 - __bfloat162float(a1[e]));
    }
    w0[u] = bf16x2(a0[0], a0[1]);
    w1[u] = bf16x2(a1[0], a1[1]);
    w2[u] = bf16x2(a2[0], a2[1]);
  }
  *reinterpret_cast<uint4*>(p0) = make_uint4(w0[0], w0[1], w0[2], w0[3]);
  *reinterpret_cast<uint4*>(p1) = make_uint4(w1[0], w1[1], w1[2], w1[3]);
  *reinterpret_cast<uint4*>(p2) = make_uint4(w2[0], w2[1], w2[2], w2[3]);
}

struct TileCoord {
  int mi, nj;
  int64_t bz;
};

__device__ __forceinline__ TileCoord tile_coord(int64_t tile, int mt, int nt) {
  TileCoord c;
  c.mi = (int)(tile % mt);
  const int64_t r = tile / mt;
  c.nj = (int)(r % nt);
  c.bz = r / nt;
  return c;
}

__device__ __forceinline__ void tma_load_c(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
      ::"r"(smem_addr(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
      : "memory");
}
__device__ __forceinline__ void tma_store_c(const CUtensorMap* map, int x, int y, int z, const void* src) {
  asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3}], [%4];"
               ::"l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_addr(src))
               : "memory");
}

__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}

// Split images of A (row blocks of A) and of Bᵀ (row blocks of Bᵀ = column blocks of B):
// block x of the grid: x < mt·nk → A block x / nk, stage x % nk; else B.  Thread = row.
__global__ void __launch_bounds__(TM) k_tc_split(int m, int n, int k, const float* __restrict__ A, int lda,
                                                 long long sA, const float* __restrict__ B, int ldb, long long sB,
                                                 int mt, int nt, int nk, unsigned char* __restrict__ ws) {
  const int64_t bz = blockIdx.y;
  const int x = blockIdx.x, row = threadIdx.x;
  const bool isA = x < mt * nk;
  const int blk = (isA ? x : x - mt * nk) / nk, kc = (isA ? x : x - mt * nk) % nk;
  const int g = blk * TM + row, kb0 = kc * KC;
  const int kn = (isA ? g < m : g < n) ? min(KC, k - kb0) : 0;
  float v[KC];
  if (isA) {
    const float* src = A + bz * sA + g;
#pragma unroll
    for (int u = 0; u < KC; ++u) v[u] = u < kn ? src[(int64_t)(kb0 + u) * lda] : 0.0f;
  } else {
    const float* src = B + bz * sB + (int64_t)g * ldb + kb0;
    if (kn == KC && (reinterpret_cast<uintptr_t>(src) & 15) == 0) {
#pragma unroll
      for (int u = 0; u < KC / 4; ++u) {
        const float4 q = *reinterpret_cast<const float4*>(src + 4 * u);
        v[4 * u] = q.x; v[4 * u + 1] = q.y; v[4 * u + 2] = q.z; v[4 * u + 3] = q.w;
      }
    } else {
#pragma unroll
      for (int u = 0; u < KC; ++u) v[u] = u < kn ? src[u] : 0.0f;
    }
  }
  const int64_t img = isA ? (bz * mt + blk) * nk + kc : (int64_t)gridDim.y * mt * nk + (bz * nt + blk) * nk + kc;
  unsigned char* op = ws + img * IMG_BYTES;
#pragma unroll
  for (int kg = 0; kg < KC / 8; ++kg) {
    // core matrix (row group row/8, K group kg): kg·(128·16) + (row/8)·128 + (row%8)·16
    const int off = kg * (TM * 16) + (row >> 3) * 128 + (row & 7) * 16;
    split_store(*reinterpret_cast<const float(*)[8]>(v + 8 * kg), op + off, op + PART_BYTES + off,
                op + 2 * PART_BYTES + off);
  }
}

__global__ void __launch_bounds__(TC_THREADS, 1)
    k_tc_gemm(const __grid_constant__ CUtensorMap cmap, int tma_c, int m, int n, int k, float alpha,
              const unsigned char* __restrict__ ws, float beta, float* __restrict__ C, int ldc, long long sC,
              int batch, int c16, int32_t* err) {
  // [NST][A parts 0..2 | B parts 0..2], then the C tile [TN columns][TM rows]
  extern __shared__ __align__(1024) unsigned char tc_smem[];
  __shared__ __align__(8) uint64_t full[NST], empty[NST], acc_full[2], acc_empty[2], drain_bar, cfull[NCB];
  __shared__ uint32_t tmem_slot;
  __shared__ int abort_flag;
  volatile int* abort_v = &abort_flag;
  const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
  const int mt = (m + TM - 1) / TM, nt = (n + TN - 1) / TN;
  const int64_t ntiles = (int64_t)mt * nt * batch;
  const int kpad = (k + 15) / 16 * 16;
  const int nk = (kpad + KC - 1) / KC;  // stages per tile
  if (warp == MMA_WARP) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_slot)),
                 "r"(ACC_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int s = 0; s < NST; ++s) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&full[s])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&empty[s])));
    }
    for (int b = 0; b < 2; ++b) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&acc_full[b])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(&acc_empty[b])), "r"(32 * EPI_WARPS));
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&drain_bar)));
    for (int i = 0; i < NCB; ++i) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&cfull[i])));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    abort_flag = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_slot;
  const uint32_t base = smem_addr(tc_smem);

  if (warp == PROD_WARP) {
    // ---------------------------------------------------------------- producer
    if (lane == 0) {
      const unsigned char* wsB = ws + (size_t)batch * mt * nk * IMG_BYTES;
      int s = 0;
      uint32_t ph = 0, last_ph[NST];
      bool go = true, used[NST];
      for (int i = 0; i < NST; ++i) { used[i] = false; last_ph[i] = 0; }
      for (int64_t tile = blockIdx.x; tile < ntiles && go; tile += gridDim.x) {
        const TileCoord tc = tile_coord(tile, mt, nt);
        const unsigned char* a = ws + ((tc.bz * mt + tc.mi) * nk) * (int64_t)IMG_BYTES;
        const unsigned char* b = wsB + ((tc.bz * nt + tc.nj) * nk) * (int64_t)IMG_BYTES;
        for (int kc = 0; kc < nk; ++kc) {
          if (!mbar_wait(&empty[s], ph ^ 1u, abort_v)) { go = false; break; }  // the MMAs released it
          unsigned char* st = tc_smem + (size_t)s * STAGE_BYTES;
          asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(&full[s])),
                       "r"(STAGE_BYTES)
                       : "memory");
          bulk_load(st, a + (int64_t)kc * IMG_BYTES, IMG_BYTES, &full[s]);
          bulk_load(st + IMG_BYTES, b + (int64_t)kc * IMG_BYTES, IMG_BYTES, &full[s]);
          used[s] = true;
          last_ph[s] = ph;
          if (++s == NST) { s = 0; ph ^= 1u; }
        }
      }
      if (*abort_v)  // let the copies in flight land before the CTA's shared memory is released
        for (int i = 0; i < NST; ++i)
          if (used[i])
            for (long w = 0; w < TC_WAIT_LIMIT && !mbar_test(&full[i], last_ph[i]); ++w) {
            }
    }
    __syncwarp();
  } else if (warp == MMA_WARP) {
    // ---------------------------------------------------------------- MMA issue
    if (lane == 0) {
      int s = 0, b = 0;
      uint32_t ph = 0, aph = 0;
      bool issued = false;
      for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        if (!mbar_wait(&acc_empty[b], aph ^ 1u, abort_v)) break;  // the epilogue has read this accumulator
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t d = tmem + (uint32_t)(b * TN);
        bool ok = true;
        for (int kc = 0; kc < nk; ++kc) {
          if (!mbar_wait(&full[s], ph, abort_v)) { ok = false; break; }
          asm volatile("tcgen05.fence::after_thread_sync;");
          const int ksteps = min(KC, kpad - kc * KC) / 16;
          const uint32_t st = base + (uint32_t)(s * STAGE_BYTES);
          const int pa[6] = {0, 0, 1, 0, 1, 2}, pb[6] = {0, 1, 0, 2, 1, 0};
          for (int ks = 0; ks < ksteps; ++ks)
#pragma unroll
            for (int t = 0; t < 6; ++t) {
              const uint32_t a_addr = st + pa[t] * PART_BYTES + ks * 2 * (TM * 16);
              const uint32_t b_addr = st + IMG_BYTES + pb[t] * PART_BYTES + ks * 2 * (TN * 16);
              mma_bf16(d, smem_desc(a_addr, TM * 16, 128), smem_desc(b_addr, TN * 16, 128),
                       (kc > 0 || ks > 0 || t > 0) ? 1u : 0u);
            }
          issued = true;
          mma_commit(&empty[s]);  // the stage is free once these MMAs have read it
          if (++s == NST) { s = 0; ph ^= 1u; }
        }
        if (!ok) break;
        mma_commit(&acc_full[b]);
        if (++b == 2) { b = 0; aph ^= 1u; }
      }
      if (issued && *abort_v) {  // let the MMAs in flight finish before the tensor memory is freed
        mma_commit(&drain_bar);
        for (long i = 0; i < TC_WAIT_LIMIT && !mbar_test(&drain_bar, 0u); ++i) {
        }
      }
    }
    __syncwarp();
  } else {
    // ---------------------------------------------------------------- epilogue
    // With a tensor map of C (tma_c): C moves in chunks of CW = 32 columns through a ring of
    // NCB = 4 shared-memory buffers [CW columns][TM rows]; thread 0 of the epilogue loads a
    // chunk with one TMA box copy three chunks ahead, the four warps combine it in place with
    // the accumulator columns (tcgen05.ld, lane = row), and thread 0 writes it back with one
    // TMA store (one bulk group per chunk; a buffer is reused once the store of its previous
    // chunk has read it).  TMA clips the box at the edges of C.  Without a tensor map (C or
    // its strides not 16-byte aligned) row gi is written directly from lane gi.
    const int q = warp & 3, et = tid - 32 * EPI_WARP0;
    const bool leader = et == 0;
    float* Cs = reinterpret_cast<float*>(tc_smem + (size_t)NST * STAGE_BYTES);
    const int64_t my_tiles = blockIdx.x < ntiles ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    const int64_t nchunks = my_tiles * NCB;
    const bool loads = tma_c && beta != 0.0f;
    auto issue_load = [&](int64_t g) {  // leader only
      const TileCoord tc = tile_coord(blockIdx.x + (g / NCB) * gridDim.x, mt, nt);
      const int bb = (int)(g % NCB);
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(&cfull[bb])),
                   "r"((uint32_t)CHUNK_BYTES)
                   : "memory");
      tma_load_c(Cs + (size_t)bb * CW * TM, &cmap, tc.mi * TM, tc.nj * TN + bb * CW, (int)tc.bz, &cfull[bb]);
    };
    // every chunk is loaded, in order: the load of chunk g is the (g / NCB)-th into its buffer
    int64_t issued = 0;  // chunks whose load has been issued (leader)
    int64_t drain_from = -1;  // the first chunk whose wait ran out (leader)
    if (leader && loads)
      for (; issued < (nchunks < NCB - 1 ? nchunks : (int64_t)(NCB - 1)); ++issued) issue_load(issued);
    int b = 0;
    uint32_t aph = 0;
    int64_t gc = 0;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
      const TileCoord tc = tile_coord(tile, mt, nt);
      const int i0 = tc.mi * TM, j0 = tc.nj * TN;
      float* Cb = C + tc.bz * sC;
      const bool ok = mbar_wait(&acc_full[b], aph, abort_v);
      // the stop decision is reduced over the epilogue warps so that all of them leave together
      // (the tensor-memory loads below are .sync.aligned, and the named barriers count all four)
      uint32_t stop;
      asm volatile(
          "{\n .reg .pred pin, pout;\n setp.ne.u32 pin, %1, 0;\n bar.red.or.pred pout, 1, %2, pin;\n"
          " selp.u32 %0, 1, 0, pout;\n}\n"
          : "=r"(stop)
          : "r"((!ok || *abort_v) ? 1u : 0u), "n"(32 * EPI_WARPS)
          : "memory");
      if (stop) break;
      asm volatile("tcgen05.fence::after_thread_sync;");
      const int rl = 32 * q + lane, gi = i0 + rl;
      for (int c = 0; c < NCB; ++c, ++gc) {
        const int c0 = CW * c;
        uint32_t r[32];
        const uint32_t taddr = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(b * TN + c0);
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
            "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
              "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
              "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
            : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (tma_c) {
          const int bb = (int)(gc % NCB);
          float* buf = Cs + (size_t)bb * CW * TM;
          if (loads) {
            if (!mbar_wait(&cfull[bb], (uint32_t)(gc / NCB) & 1u, abort_v)) {
              *abort_v = 1;
              if (leader && drain_from < 0) drain_from = gc;
            }
          } else {  // buf is free once the store of its previous chunk has read it
            if (leader) asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(NCB - 1) : "memory");
            asm volatile("bar.sync 1, %0;" ::"n"(32 * EPI_WARPS) : "memory");
          }
#pragma unroll
          for (int cc = 0; cc < 32; ++cc) {
            float* e = buf + cc * TM + rl;
            *e = fmaf(alpha, __uint_as_float(r[cc]), loads ? beta * *e : 0.0f);
          }
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          asm volatile("bar.sync 1, %0;" ::"n"(32 * EPI_WARPS) : "memory");  // the chunk is complete
          if (leader) {
            tma_store_c(&cmap, i0, j0 + c0, (int)tc.bz, buf);
            asm volatile("cp.async.bulk.commit_group;" ::: "memory");
            if (loads && issued < nchunks) {
              // the next load goes into the buffer whose store was committed one chunk ago
              asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
              issue_load(issued++);
            }
          }
        } else if (gi < m) {
#pragma unroll
          for (int cc = 0; cc < 32; ++cc) {
            const int gj = j0 + c0 + cc;
            if (gj < n) {
              float* e = Cb + gi + (int64_t)gj * ldc;
              *e = fmaf(alpha, __uint_as_float(r[cc]), beta != 0.0f ? beta * *e : 0.0f);
            }
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;");
      mbar_arrive(&acc_empty[b]);  // the accumulator may be overwritten
      if (++b == 2) { b = 0; aph ^= 1u; }
    }
    if (leader && tma_c) {
      asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");  // the stores have completed
      // loads issued for chunks not consumed (an abort): let them land before the CTA leaves
      for (int64_t g2 = drain_from >= 0 ? drain_from : gc; g2 < issued; ++g2)
        for (long w = 0; w < TC_WAIT_LIMIT && !mbar_test(&cfull[g2 % NCB], (uint32_t)(g2 / NCB) & 1u); ++w) {
        }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (*abort_v && tid == 0) atomicExch(err, 2);
  if (warp == MMA_WARP) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ACC_COLS));
}

}  // namespace

constexpr size_t kTcSmem = (size_t)NST * STAGE_BYTES + CTILE_BYTES;  // 208 KB: one CTA per SM

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_tiled_fn() {
  void* p = nullptr;
  cudaDriverEntryPointQueryResult q{};
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
      q == cudaDriverEntryPointSuccess)
    return reinterpret_cast<EncodeTiledFn>(p);
  return nullptr;
}

size_t tc_gemm_workspace(int m, int n, int k, int batch) {
  if (m <= 0 || n <= 0 || k <= 0 || batch <= 0) return 0;
  const int64_t mt = (m + TM - 1) / TM, nt = (n + TN - 1) / TN, nk = ((k + 15) / 16 * 16 + KC - 1) / KC;
  return (size_t)(batch * (mt + nt) * nk) * IMG_BYTES;
}

int tc_gemm_f32(cudaStream_t stream, int m, int n, int k, float alpha, const float* A, int lda, long long sA,
                const float* B, int ldb, long long sB, float beta, float* C, int ldc, long long sC, int batch,
                void* ws, size_t ws_bytes, int32_t* err, std::string* msg) {
  if (m <= 0 || n <= 0 || batch <= 0) return 0;
  if (k <= 0 || k > 128) {
    if (msg) *msg = "tensor-core GEMM: K = " + std::to_string(k) + " outside [1, 128]";
    return -1;
  }
  if (batch > 65535) {
    if (msg) *msg = "tensor-core GEMM: batch " + std::to_string(batch) + " exceeds 65535";
    return -1;
  }
  const size_t need = tc_gemm_workspace(m, n, k, batch);
  if (!ws || ws_bytes < need || reinterpret_cast<uintptr_t>(ws) % 16 != 0) {
    if (msg) *msg = "tensor-core GEMM: workspace of " + std::to_string(ws_bytes) + " bytes, " + std::to_string(need) +
                    " needed (16-byte aligned)";
    return -1;
  }
  static int attr_dev = -1, num_sms = 0;
  int dev = 0;
  cudaGetDevice(&dev);
  if (attr_dev != dev) {
    cudaError_t e = cudaFuncSetAttribute(k_tc_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) {
      if (msg) *msg = std::string("tensor-core GEMM: ") + cudaGetErrorString(e);
      return -2;
    }
    attr_dev = dev;
  }
  const int mt = (m + TM - 1) / TM, nt = (n + TN - 1) / TN, nk = ((k + 15) / 16 * 16 + KC - 1) / KC;
  dim3 gs((unsigned)((mt + nt) * nk), (unsigned)batch);
  k_tc_split<<<gs, TM, 0, stream>>>(m, n, k, A, lda, sA, B, ldb, sB, mt, nt, nk, static_cast<unsigned char*>(ws));
  count_launch();
  const int64_t tiles = (int64_t)mt * nt * batch;
  const unsigned grid = (unsigned)std::min<int64_t>(tiles, std::max(1, num_sms));
  // 16-byte C pieces: the base, the column stride and the problem stride keep 16-byte alignment
  const int c16 = (reinterpret_cast<uintptr_t>(C) % 16 == 0 && ldc % 4 == 0 && sC % 4 == 0) ? 1 : 0;
  // the epilogue's tensor map of C: rows x columns x problems, box TM rows x CW columns
  CUtensorMap cmap{};
  int tma_c = 0;
  if (c16 && (batch == 1 || sC > 0)) {
    static EncodeTiledFn enc = encode_tiled_fn();
    if (enc) {
      const cuuint64_t dims[3] = {(cuuint64_t)m, (cuuint64_t)n, (cuuint64_t)batch};
      const cuuint64_t strides[2] = {(cuuint64_t)ldc * sizeof(float),
                                     (cuuint64_t)(batch > 1 ? sC : (long long)ldc * n) * sizeof(float)};
      const cuuint32_t box[3] = {(cuuint32_t)TM, (cuuint32_t)CW, 1};
      const cuuint32_t estr[3] = {1, 1, 1};
      tma_c = enc(&cmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, C, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
    }
  }
  k_tc_gemm<<<grid, TC_THREADS, kTcSmem, stream>>>(cmap, tma_c, m, n, k, alpha, static_cast<const unsigned char*>(ws),
                                                   beta, C, ldc, sC, batch, c16, err);
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
  void* ws = nullptr;
  const size_t wsb = gbmhd::tc_gemm_workspace(m, n, k, batch);
  if (cudaMalloc(&d_err, sizeof(int32_t)) != cudaSuccess) return -2;
  if (wsb && cudaMalloc(&ws, wsb) != cudaSuccess) {
    cudaFree(d_err);
    return -2;
  }
  cudaMemset(d_err, 0, sizeof(int32_t));
  std::string msg;
  int rc = gbmhd::tc_gemm_f32(nullptr, m, n, k, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, batch, ws, wsb,
                              d_err, &msg);
  if (rc == 0 && cudaDeviceSynchronize() != cudaSuccess) rc = -2;
  int32_t h = 0;
  cudaMemcpy(&h, d_err, sizeof(int32_t), cudaMemcpyDeviceToHost);
  cudaFree(d_err);
  if (ws) cudaFree(ws);
  if (status) *status = h;
  return rc;
}
