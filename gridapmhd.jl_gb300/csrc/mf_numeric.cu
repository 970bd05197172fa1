// Numeric multifrontal factorization and solves of the (u,j) block (see mf.h).
#include <cublas_v2.h>
#include <cuda.h>  // CUtensorMap types; the encoder is reached through the runtime's driver entry point

#include <cstdlib>
#include <cstring>

#include "mf.h"

using namespace gbmhd;

namespace {

constexpr int NB = 64;   // Gauss-Jordan pivot block (inverted by one CTA)
constexpr long kSweepWaitDefault = 1L << 22;  // spin limit of the sweeps' mbarrier waits
// panel: the trailing part of a front is updated once per PW pivots.  PW = 256 halves the
// traffic again but multiplies the FP32 rounding of the panel's progressive inverse by the
// conditioning of a 256-pivot block: at Ha = 500 (64x64x4) one solve in three then needed
// 600+ FGMRES iterations instead of ~100.
constexpr int PW = 128;
static_assert(PW % NB == 0 && PW <= 256 && (PW & (PW - 1)) == 0, "k_panel_rows maps one thread per panel row");

struct DevSym {
  int32_t* f_ne = nullptr;
  int32_t* f_nb = nullptr;
  int64_t* f_off = nullptr;
  int64_t* elim_ptr = nullptr;
  int64_t* bnd_ptr = nullptr;
  int32_t* elim = nullptr;
  int32_t* bnd = nullptr;
  int32_t* ah_src = nullptr;
  int64_t* ah_dst = nullptr;
  int32_t* child_list = nullptr;
  int64_t* ea_ptr = nullptr;
  int32_t* ea_pos = nullptr;
  int32_t* f_parent = nullptr;
  int32_t* f_level = nullptr;
  int64_t* reg_dst = nullptr;
  int32_t* reg_dof = nullptr;
};

}  // namespace

struct MFNumeric {
  MFSymbolic S;
  DevSym d;
  cublasHandle_t blas = nullptr;
  int precision = -1;          // precision of the stored factors
  void* F = nullptr;           // front storage (float or double)
  size_t F_bytes = 0;
  void* Pbuf = nullptr;        // pivot inverses  [count][NB*NB]
  void* Cbuf = nullptr;        // column blocks   [count][n*NB]
  void* Tbuf = nullptr;        // row blocks      [count][NB*n]
  void* T2buf = nullptr;
  void* Rbuf = nullptr;        // panel rows before elimination   [count][PW*n]
  void* Nbuf = nullptr;        // eliminated panel columns        [count][n*PW]
  size_t work_bytes = 0;
  double* tsave = nullptr;     // forward-sweep values of the eliminated dofs
  double* ybuf = nullptr;      // backward-sweep accumulators (kept zero between solves)
  int64_t* tsave_off = nullptr;  // per front
  int64_t tsave_len = 0;
  int32_t* d_err = nullptr;    // device-side status (singular pivot block)
  int fp32_gemm_mode = 0;      // 0: BF16x9 emulated FP32, 1: plain FP32
  // TMA-staged sweeps (FP32 factors): one 3-D tensor map per level (rows x columns x fronts)
  std::vector<CUtensorMap> maps;
  std::vector<int> map_rows;      // row tile of each map
  std::vector<char> map_ok;
  const void* maps_base = nullptr;
  float2* vpk = nullptr;            // packed vector segments of one level (transposed sweeps)
  bool scaled = false;              // factors are those of Dr A Dc (monolithic)
  double* d_dr = nullptr;           // [ndofs] row scales (powers of two)
  double* d_dc = nullptr;           // [ndofs] column scales
  void* d_sval = nullptr;           // scaled copy of the Jacobian values [nnz] (value precision)
  size_t sval_bytes = 0;
  int32_t* d_sweep_err = nullptr;   // set by a sweep whose TMA wait timed out
  int32_t* h_sweep_err = nullptr;   // pinned copy, read at the next solve and by mf_check_sweeps
  long wait_limit = 0;              // spin limit of the sweeps' mbarrier waits
  // sweep timing: events around each solve, harvested when the next one starts
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  bool ev_pending = false;
  int64_t sweep_applies = 0;
  double sweep_seconds = 0.0;
  int64_t sweep_elems = 0;     // factor entries one solve reads (padding excluded)
};

int mf_precision(const MFNumeric* M) { return M ? M->precision : -1; }

static void harvest_sweep_time(MFNumeric* M, bool wait) {
  if (!M->ev_pending) return;
  if (wait) cudaEventSynchronize(M->ev1);
  else if (cudaEventQuery(M->ev1) != cudaSuccess) return;
  float ms = 0.0f;
  if (cudaEventElapsedTime(&ms, M->ev0, M->ev1) == cudaSuccess) {
    M->sweep_seconds += 1e-3 * ms;
    M->sweep_applies += 1;
  }
  M->ev_pending = false;
}

void mf_sweep_stats(MFNumeric* M, int64_t* applies, double* seconds, double* bytes_per_apply) {
  harvest_sweep_time(M, true);
  *applies = M->sweep_applies;
  *seconds = M->sweep_seconds;
  *bytes_per_apply = (double)M->sweep_elems * (M->precision == GBMHD_FP64 ? 8.0 : 4.0);
  M->sweep_applies = 0;
  M->sweep_seconds = 0.0;
}

#define MF_CUDA(call)                                                               \
  do {                                                                              \
    cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess) {                                                        \
      ctx->err = std::string("multifrontal: ") + #call + ": " + cudaGetErrorString(e_); \
      return -2;                                                                    \
    }                                                                               \
  } while (0)
#define MF_BLAS(call)                                                               \
  do {                                                                              \
    cublasStatus_t s_ = (call);                                                     \
    if (s_ != CUBLAS_STATUS_SUCCESS) {                                              \
      ctx->err = std::string("multifrontal: cuBLAS status ") + std::to_string((int)s_) + " in " + #call; \
      return -2;                                                                    \
    }                                                                               \
  } while (0)

template <typename V>
static int upload(gbmhd_ctx* ctx, V** dst, const std::vector<V>& src) {
  size_t bytes = sizeof(V) * std::max<size_t>(src.size(), 1);
  MF_CUDA(cudaMalloc((void**)dst, bytes));
  if (!src.empty()) MF_CUDA(cudaMemcpy(*dst, src.data(), sizeof(V) * src.size(), cudaMemcpyHostToDevice));
  return 0;
}

int mf_create(gbmhd_ctx* ctx, const MFSymbolic& S, MFNumeric** out) {
  // the solve sweeps stage a front's vector segment in shared memory and read fronts with
  // 16-byte vector loads: every front must start on a multiple of 8 entries with n % 8 == 0
  for (const MFLevel& L : S.levels)
    if (L.E % 8 || L.n % 8 || L.off % 64) {
      ctx->err = "multifrontal: front sizes are not padded to multiples of 8";
      *out = nullptr;
      return -1;
    }
  for (const MFLevel& L : S.levels)
    if (sizeof(double) * (size_t)L.n > 200 * 1024) {
      ctx->err = "multifrontal: front of " + std::to_string(L.n) + " dofs exceeds the solve kernels' staging limit";
      *out = nullptr;
      return -1;
    }
  MFNumeric* M = new MFNumeric();
  M->S = S;
  *out = M;
  int rc = 0;
  if ((rc = upload(ctx, &M->d.f_ne, S.f_ne)) || (rc = upload(ctx, &M->d.f_nb, S.f_nb)) ||
      (rc = upload(ctx, &M->d.f_off, S.f_off)) || (rc = upload(ctx, &M->d.elim_ptr, S.elim_ptr)) ||
      (rc = upload(ctx, &M->d.bnd_ptr, S.bnd_ptr)) || (rc = upload(ctx, &M->d.elim, S.elim)) ||
      (rc = upload(ctx, &M->d.bnd, S.bnd)) || (rc = upload(ctx, &M->d.ah_src, S.ah_src)) ||
      (rc = upload(ctx, &M->d.ah_dst, S.ah_dst)) || (rc = upload(ctx, &M->d.child_list, S.child_list)) ||
      (rc = upload(ctx, &M->d.ea_ptr, S.ea_ptr)) || (rc = upload(ctx, &M->d.ea_pos, S.ea_pos)) ||
      (rc = upload(ctx, &M->d.f_parent, S.f_parent)) || (rc = upload(ctx, &M->d.f_level, S.f_level)) ||
      (rc = upload(ctx, &M->d.reg_dst, S.reg_dst)) || (rc = upload(ctx, &M->d.reg_dof, S.reg_dof)))
    return rc;
  // forward-sweep buffers: E_l doubles per front
  std::vector<int64_t> toff(S.f_ne.size());
  int64_t t = 0;
  for (const MFLevel& L : S.levels)
    for (int64_t f = L.first; f < L.first + L.count; ++f) {
      toff[f] = t;
      t += L.E;
    }
  M->tsave_len = t;
  // forward reads rows E.. of the ne eliminated columns, backward rows 0..ne of the ne
  // eliminated and nb boundary columns
  M->sweep_elems = 0;
  for (size_t f = 0; f < S.f_ne.size(); ++f) {
    const int64_t ne = S.f_ne[f], nb = S.f_nb[f];
    M->sweep_elems += nb * ne + ne * (ne + nb);
  }
  {
    size_t vmax = 1;
    for (const MFLevel& L : S.levels) vmax = std::max(vmax, (size_t)L.count * L.n);
    MF_CUDA(cudaMalloc(&M->vpk, sizeof(float2) * vmax));
  }
  MF_CUDA(cudaMalloc(&M->d_sweep_err, sizeof(int32_t)));
  MF_CUDA(cudaMemset(M->d_sweep_err, 0, sizeof(int32_t)));
  MF_CUDA(cudaMallocHost(&M->h_sweep_err, sizeof(int32_t)));
  *M->h_sweep_err = 0;
  MF_CUDA(cudaEventCreate(&M->ev0));
  MF_CUDA(cudaEventCreate(&M->ev1));
  if ((rc = upload(ctx, &M->tsave_off, toff))) return rc;
  MF_CUDA(cudaMalloc(&M->tsave, sizeof(double) * std::max<int64_t>(t, 1)));
  MF_CUDA(cudaMalloc(&M->ybuf, sizeof(double) * std::max<int64_t>(t, 1)));
  MF_CUDA(cudaMemset(M->ybuf, 0, sizeof(double) * std::max<int64_t>(t, 1)));
  MF_CUDA(cudaMalloc(&M->d_err, sizeof(int32_t)));
  if (cublasCreate(&M->blas) != CUBLAS_STATUS_SUCCESS) {
    ctx->err = "multifrontal: cublasCreate failed";
    return -2;
  }
  MF_BLAS(cublasSetStream(M->blas, ctx->stream));
  // Front entries are finite (a singular pivot block raises the factorization error and a
  // non-finite FGMRES residual ends the solve), so the BF16x9 emulation need not scan its
  // operands for infinities and NaNs before every GEMM.
  MF_BLAS(cublasSetEmulationSpecialValuesSupport(M->blas, CUDA_EMULATION_SPECIAL_VALUES_SUPPORT_NONE));
  M->wait_limit = kSweepWaitDefault;
  if (const char* wl = std::getenv("GBMHD_SWEEP_WAIT_LIMIT")) M->wait_limit = std::max(0L, std::atol(wl));
  const char* mode = std::getenv("GBMHD_FP32_GEMM");
  M->fp32_gemm_mode = (mode && std::strcmp(mode, "fp32") == 0) ? 1 : 0;
  return 0;
}

void mf_destroy(MFNumeric* M) {
  if (!M) return;
  void* ptrs[] = {M->d.f_ne, M->d.f_nb, M->d.f_off, M->d.elim_ptr, M->d.bnd_ptr, M->d.elim, M->d.bnd,
                  M->d.ah_src, M->d.ah_dst, M->d.child_list, M->d.ea_ptr, M->d.ea_pos, M->d.f_parent,
                  M->d.f_level, M->d.reg_dst, M->d.reg_dof, M->F, M->Pbuf, M->Cbuf, M->Tbuf, M->T2buf, M->Rbuf, M->Nbuf, M->tsave, M->ybuf, M->tsave_off, M->d_err};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (M->blas) cublasDestroy(M->blas);
  if (M->vpk) cudaFree(M->vpk);
  if (M->d_dr) cudaFree(M->d_dr);
  if (M->d_dc) cudaFree(M->d_dc);
  if (M->d_sval) cudaFree(M->d_sval);
  if (M->d_sweep_err) cudaFree(M->d_sweep_err);
  if (M->h_sweep_err) cudaFreeHost(M->h_sweep_err);
  if (M->ev0) cudaEventDestroy(M->ev0);
  if (M->ev1) cudaEventDestroy(M->ev1);
  delete M;
}

// ------------------------------------------------------------------ kernels
template <typename T>
__global__ void k_pad_diag(T* F, int64_t off, int64_t count, int n, int E, const int32_t* f_ne, int64_t first) {
  const int64_t f = blockIdx.x;
  if (f >= count) return;
  const int ne = f_ne[first + f];
  T* M = F + off + f * (int64_t)n * n;
  for (int i = ne + threadIdx.x; i < E; i += blockDim.x) M[i + (int64_t)i * n] = (T)1;
}

template <typename T, typename V>
__global__ void k_arrowhead(const V* __restrict__ Aval, const int32_t* __restrict__ src,
                            const int64_t* __restrict__ dst, int64_t b, int64_t e, T* __restrict__ F) {
  for (int64_t i = b + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < e; i += (int64_t)gridDim.x * blockDim.x)
    F[dst[i]] = (T)Aval[src[i]];
}

// Diagonal regularisation of the p and φ pivots (monolithic factorization).
// ---- equilibration (monolithic factorization)
// Ruiz scaling of the Jacobian before it is factored: rows and columns are divided by the
// square roots of their largest entries, a few sweeps, with the scales rounded to powers of
// two so that scaling is exact in any precision.  The factors are those of Dr A Dc; a solve
// scales its right-hand side by Dr and its result by Dc.  Measured at Ha = 500 on the 64x64x4
// duct (FP32 emulation): the worst 64x64 pivot blocks drop from κ ~1e12 to ~1e9 and the FGMRES
// iterations per three digits from 20 to 11.
template <typename V>
__global__ void k_ruiz_max(int64_t n, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                           const V* __restrict__ val, const double* __restrict__ dr, const double* __restrict__ dc,
                           double* __restrict__ rmax, unsigned long long* __restrict__ cmax) {
  const int lane = threadIdx.x & 31;
  for (int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; r < n;
       r += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const double sr = dr[r];
    double m = 0.0;
    for (int64_t t = rowptr[r] + lane; t < rowptr[r + 1]; t += 32) {
      const int32_t c = col[t];
      const double a = fabs((double)val[t] * sr * dc[c]);
      m = fmax(m, a);
      // non-negative doubles order like their bit patterns
      atomicMax(&cmax[c], (unsigned long long)__double_as_longlong(a));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
    if (lane == 0) rmax[r] = m;
  }
}

__device__ __forceinline__ double pow2_rsqrt(double m) {  // 2^round(-log2(m)/2), 1 for m == 0
  if (!(m > 0.0)) return 1.0;
  return exp2(rint(-0.5 * log2(m)));
}

__global__ void k_ruiz_update(int64_t n, const double* __restrict__ rmax, const unsigned long long* __restrict__ cmax,
                              double* __restrict__ dr, double* __restrict__ dc) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    dr[i] *= pow2_rsqrt(rmax[i]);
    dc[i] *= pow2_rsqrt(__longlong_as_double((long long)cmax[i]));
  }
}

template <typename V>
__global__ void k_scale_vals(int64_t n, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                             const V* __restrict__ val, const double* __restrict__ dr, const double* __restrict__ dc,
                             V* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  for (int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; r < n;
       r += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const V sr = (V)dr[r];  // powers of two: exact in V
    for (int64_t t = rowptr[r] + lane; t < rowptr[r + 1]; t += 32) out[t] = val[t] * sr * (V)dc[col[t]];
  }
}

__global__ void k_fill(int64_t n, double a, double* __restrict__ v) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) v[i] = a;
}

__global__ void k_scale_vec(int64_t n, const double* __restrict__ s, double* __restrict__ v) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    v[i] *= s[i];
}

template <typename T>
__global__ void k_reg_add(T* F, const int64_t* __restrict__ dst, const int32_t* __restrict__ dof,
                          const double* __restrict__ reg, const double* __restrict__ dr, const double* __restrict__ dc,
                          int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t d = dof[i];
    F[dst[i]] += (T)(reg[d] * (dr ? dr[d] * dc[d] : 1.0));
  }
}

__device__ __forceinline__ void atomic_add_t(float* p, float v) { atomicAdd(p, v); }
__device__ __forceinline__ void atomic_add_t(double* p, double v) { atomicAdd(p, v); }

// Children of the current level add their Schur complement into the parent front.
template <typename T>
__global__ void k_extend_add(T* F, const int32_t* __restrict__ child_list, int64_t cb, const int32_t* __restrict__ f_nb,
                             const int64_t* __restrict__ f_off, const int32_t* __restrict__ f_parent,
                             const int32_t* __restrict__ f_level, const int64_t* __restrict__ ea_ptr,
                             const int32_t* __restrict__ ea_pos, const int* __restrict__ lev_n,
                             const int* __restrict__ lev_E) {
  const int32_t c = child_list[cb + blockIdx.x];
  const int nb = f_nb[c];
  const int lc = f_level[c];
  const int nc = lev_n[lc], Ec = lev_E[lc];
  const int32_t p = f_parent[c];
  const int np = lev_n[f_level[p]];
  const T* Sc = F + f_off[c];
  T* Fp = F + f_off[p];
  const int32_t* pos = ea_pos + ea_ptr[c];
  for (int j = blockIdx.y; j < nb; j += gridDim.y) {
    const int64_t pj = (int64_t)pos[j] * np;
    const T* colj = Sc + (int64_t)(Ec + j) * nc + Ec;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) atomic_add_t(&Fp[pos[i] + pj], colj[i]);
  }
}

// Inverse of the kb x kb pivot block of every front: in-place Gauss-Jordan with partial
// pivoting inside the block (row interchanges, undone as column interchanges at the end),
// computed in FP64 whatever the storage type and then rounded to it.  kb³ FP64 multiply-
// adds per block; the pivot search is one warp's shuffle argmax.  P[f] (NB x NB,
// column-major, ld NB, zero outside kb x kb).
template <typename T>
__global__ void __launch_bounds__(256) k_pivot_inverse(const T* __restrict__ F, int64_t off, int n, int k, int kb,
                                                       T* __restrict__ P, int32_t* err) {
  __shared__ double A[NB * NB];  // column-major, ld kb
  __shared__ double rowc[NB], mcol[NB];
  __shared__ int perm[NB], colsrc[NB];
  __shared__ int piv_row;
  const int64_t f = blockIdx.x;
  const T* M = F + off + f * (int64_t)n * n;
  const int tid = threadIdx.x;
  const int ti = tid & (NB - 1), tj = tid / NB;  // row, first column of this thread (4 column groups)
  constexpr int CG = 256 / NB;
  if (ti < kb)
    for (int j = tj; j < kb; j += CG) A[ti + j * kb] = (double)M[(k + ti) + (int64_t)(k + j) * n];
  __syncthreads();
  for (int c = 0; c < kb; ++c) {
    if (tid < 32) {  // argmax |A[i, c]| over rows c..kb-1 (ties: the lower row)
      double best = -1.0;
      int bi = c;
      for (int i = c + tid; i < kb; i += 32) {
        const double a = fabs(A[i + c * kb]);
        if (a > best) { best = a; bi = i; }
      }
      for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_down_sync(0xffffffffu, best, o);
        const int oi = __shfl_down_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
      }
      if (tid == 0) {
        piv_row = bi;
        perm[c] = bi;
        if (!(best > 0.0)) atomicExch(err, 1);
      }
    }
    __syncthreads();
    const int pr = piv_row;
    if (pr != c && tid < kb) {
      const double t = A[c + tid * kb];
      A[c + tid * kb] = A[pr + tid * kb];
      A[pr + tid * kb] = t;
    }
    __syncthreads();
    if (tid < kb) {
      const double d = A[c + c * kb];
      const double inv = d != 0.0 ? 1.0 / d : 0.0;
      rowc[tid] = tid == c ? inv : A[c + tid * kb] * inv;
      mcol[tid] = tid == c ? 0.0 : A[tid + c * kb];
    }
    __syncthreads();
    if (ti < kb) {
      const double mi = mcol[ti];
      for (int j = tj; j < kb; j += CG) {
        const int idx = ti + j * kb;
        A[idx] = ti == c ? rowc[j] : (j == c ? 0.0 : A[idx]) - mi * rowc[j];
      }
    }
    __syncthreads();
  }
  if (tid == 0) {  // undo the row interchanges as column interchanges, last first
    for (int j = 0; j < kb; ++j) colsrc[j] = j;
    for (int c = kb - 1; c >= 0; --c) {
      const int p = perm[c];
      const int t = colsrc[c];
      colsrc[c] = colsrc[p];
      colsrc[p] = t;
    }
  }
  __syncthreads();
  T* Pf = P + f * (int64_t)NB * NB;
  for (int j = tj; j < NB; j += CG)  // column-major, zero outside kb x kb
    Pf[ti + j * NB] = (ti < kb && j < kb) ? (T)A[ti + colsrc[j] * kb] : (T)0;
}

// The same in-place Gauss-Jordan for FP32 factors, in float-float arithmetic on the FP32
// pipes (~48 significant bits; the result is rounded to FP32).  GB300 issues FP64 at a
// small fraction of its FP32 rate: the kb³ updates cost ~14 FP32 operations each here
// instead of one FP64 FMA, which is still several times faster.  The per-column scalars
// (the pivot's reciprocal, the scaled pivot row) are float-float too; the pivot is chosen on
// the high parts.
// float-float product (Dekker via FMA) and reciprocal (one Newton step on the FP32 one)
__device__ __forceinline__ void df_mul(float ah, float al, float bh, float bl, float& h, float& l) {
  const float p = __fmul_rn(ah, bh);
  float e = fmaf(ah, bh, -p);
  e = fmaf(ah, bl, e);
  e = fmaf(al, bh, e);
  h = __fadd_rn(p, e);
  l = __fsub_rn(e, __fsub_rn(h, p));
}

__device__ __forceinline__ void df_rcp(float ah, float al, float& h, float& l) {
  const float x = __frcp_rn(ah);
  float e = fmaf(-ah, x, 1.0f);  // 1 − ah·x, exact
  e = fmaf(-al, x, e);
  const float d = __fmul_rn(x, e);
  h = __fadd_rn(x, d);
  l = __fsub_rn(d, __fsub_rn(h, x));
}

// The 64x64 block lives in registers: thread (row ti = tid mod 64, column group tj = tid / 64,
// CGN groups) holds the NB / CGN float-float entries A[ti, tj + CGN·u].  Per column step only
// column c, the pivot row and the old row c pass through shared memory, with two barriers:
//   (1) the two warps that hold column c copy it out and each reduces an argmax over its 32
//       rows (high parts; ties: the lower row);
//   (2) after the barrier: the pivot row's holders form the scaled pivot row r (r_c = 1 / pivot),
//       row c's holders copy the old row c (it moves to row pr), and threads < 64 form the
//       multipliers m_i = A[i, c] after the interchange;
//   (3) after the barrier every thread updates its entries: row c becomes r, the others
//       a − m_i r_j (column c: −m_i r_c).
// The start of a step reads nothing that the previous step's (3) still needs, so the two
// barriers per step suffice.  The chain of 64 steps is latency-bound: levels with few fronts
// (one CTA per front) use CGN = 16 (1024 threads, 4 entries each) so that every SM
// sub-partition has 8 warps to interleave; levels with many fronts use CGN = 4.
__device__ __forceinline__ void df_sub_prod(float ah, float al, float m_h, float m_l, float r_h, float r_l, float& oh,
                                            float& ol) {
  // p = m · r in float-float
  const float ph = __fmul_rn(m_h, r_h);
  float pl = fmaf(m_h, r_h, -ph);
  pl = fmaf(m_h, r_l, pl);
  pl = fmaf(m_l, r_h, pl);
  // a − p: TwoSum on the high parts, the low parts added to the error, renormalised by TwoSum
  const float sh = __fsub_rn(ah, ph);
  const float bv = __fsub_rn(sh, ah);
  const float e = __fadd_rn(__fsub_rn(ah, __fsub_rn(sh, bv)), __fsub_rn(-ph, bv));
  const float sl = __fadd_rn(e, __fsub_rn(al, pl));
  const float h = __fadd_rn(sh, sl);
  const float hv = __fsub_rn(h, sh);
  oh = h;
  ol = __fadd_rn(__fsub_rn(sh, __fsub_rn(h, hv)), __fsub_rn(sl, hv));
}

template <int CGN>
__global__ void __launch_bounds__(NB * CGN) k_pivot_inverse_df(const float* __restrict__ F, int64_t off, int n, int k,
                                                              int kb, float* __restrict__ P, int32_t* err) {
  static_assert(NB == 64 && NB % CGN == 0, "register layout: 64 rows x CGN column groups");
  constexpr int NU = NB / CGN;
  constexpr int LD = NB + 1;
  __shared__ float Ob[NB * LD];  // the result, column-major, before the column interchanges
  __shared__ float ch[NB], cl[NB], rh[NB], rl[NB], mh[NB], ml[NB], oh[NB], ol[NB];
  __shared__ float cand_v[2];
  __shared__ int cand_i[2];
  __shared__ int perm[NB], colsrc[NB];
  const int64_t f = blockIdx.x;
  const float* M = F + off + f * (int64_t)n * n;
  const int tid = threadIdx.x;
  const int ti = tid & (NB - 1), tj = tid >> 6, lane = tid & 31;
  float h[NU], l[NU];
#pragma unroll
  for (int u = 0; u < NU; ++u) {
    const int j = tj + CGN * u;
    h[u] = (ti < kb && j < kb) ? M[(k + ti) + (int64_t)(k + j) * n] : 0.0f;  // zero padding beyond kb
    l[u] = 0.0f;
  }
  for (int c = 0; c < kb; ++c) {
    const int uc = c / CGN;
    // (1)
    if (tj == c % CGN) {
      float vh = 0.0f, vl = 0.0f;
#pragma unroll
      for (int u = 0; u < NU; ++u)
        if (u == uc) { vh = h[u]; vl = l[u]; }
      ch[ti] = vh;
      cl[ti] = vl;
      float best = (ti >= c && ti < kb) ? fabsf(vh) : -1.0f;
      int bi = ti;
      for (int o = 16; o > 0; o >>= 1) {
        const float ob = __shfl_down_sync(0xffffffffu, best, o);
        const int oi = __shfl_down_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
      }
      if (lane == 0) {
        cand_v[ti >> 5] = best;
        cand_i[ti >> 5] = bi;
      }
    }
    __syncthreads();
    // (2)
    int pr = cand_i[0];
    float pbest = cand_v[0];
    if (cand_v[1] > pbest) { pbest = cand_v[1]; pr = cand_i[1]; }
    if (!(pbest > 0.0f)) pr = c;  // singular block: keep going, the error flag is set below
    if (ti == pr) {
      float ih = 0.0f, il = 0.0f;
      const float dh = ch[pr], dl = cl[pr];
      if (dh != 0.0f) df_rcp(dh, dl, ih, il);
#pragma unroll
      for (int u = 0; u < NU; ++u) {
        const int j = tj + CGN * u;
        if (j == c) { rh[j] = ih; rl[j] = il; }
        else df_mul(h[u], l[u], ih, il, rh[j], rl[j]);
      }
    }
    if (ti == c) {
#pragma unroll
      for (int u = 0; u < NU; ++u) {
        oh[tj + CGN * u] = h[u];
        ol[tj + CGN * u] = l[u];
      }
    }
    if (tid < NB) {
      const int i = tid;
      const int src = i == pr ? c : i;  // row i after the interchange holds the old row src
      if (i == c) { mh[i] = 0.0f; ml[i] = 0.0f; }
      else { mh[i] = ch[src]; ml[i] = cl[src]; }
      if (i == 0) {
        perm[c] = pr;
        if (!(pbest > 0.0f)) atomicExch(err, 1);
      }
    }
    __syncthreads();
    // (3)
    const float m_h = mh[ti], m_l = ml[ti];
    const bool from_c = ti == pr && pr != c;  // this row now holds the old row c
#pragma unroll
    for (int u = 0; u < NU; ++u) {
      const int j = tj + CGN * u;
      const float r_h = rh[j], r_l = rl[j];
      if (ti == c) {
        h[u] = r_h;
        l[u] = r_l;
      } else {
        float ah = from_c ? oh[j] : h[u], al = from_c ? ol[j] : l[u];
        if (j == c) { ah = 0.0f; al = 0.0f; }
        df_sub_prod(ah, al, m_h, m_l, r_h, r_l, h[u], l[u]);
      }
    }
  }
#pragma unroll
  for (int u = 0; u < NU; ++u) Ob[ti + (tj + CGN * u) * LD] = __fadd_rn(h[u], l[u]);
  if (tid == 0) {  // undo the row interchanges as column interchanges, last first
    for (int j = 0; j < kb; ++j) colsrc[j] = j;
    for (int c = kb - 1; c >= 0; --c) {
      const int p = perm[c];
      const int t = colsrc[c];
      colsrc[c] = colsrc[p];
      colsrc[p] = t;
    }
  }
  __syncthreads();
  float* Pf = P + f * (int64_t)NB * NB;
  for (int j = tj; j < NB; j += CGN)  // column-major, zero outside kb x kb
    Pf[ti + j * NB] = (ti < kb && j < kb) ? Ob[ti + colsrc[j] * LD] : 0.0f;
}

// Shared-memory variant (block in shared memory, 6 CTAs per SM): levels with many fronts,
// where the launch is throughput-bound rather than latency-bound.
__global__ void __launch_bounds__(256) k_pivot_inverse_df_smem(const float* __restrict__ F, int64_t off, int n, int k,
                                                          int kb, float* __restrict__ P, int32_t* err) {
  // column-major with leading dimension LD = NB + 1: row accesses (swap, pivot row) are
  // free of bank conflicts
  constexpr int LD = NB + 1;
  __shared__ float Ah[NB * LD], Al[NB * LD];
  __shared__ float rh[NB], rl[NB], mh[NB], ml[NB], ch[NB], cl[NB];
  __shared__ int perm[NB], colsrc[NB];
  __shared__ int piv_row;
  const int64_t f = blockIdx.x;
  const float* M = F + off + f * (int64_t)n * n;
  const int tid = threadIdx.x;
  const int ti = tid & (NB - 1), tj = tid / NB;  // row, first column of this thread (4 column groups)
  constexpr int CG = 256 / NB;
  if (ti < kb)
    for (int j = tj; j < kb; j += CG) {
      Ah[ti + j * LD] = M[(k + ti) + (int64_t)(k + j) * n];
      Al[ti + j * LD] = 0.0f;
    }
  __syncthreads();
  for (int c = 0; c < kb; ++c) {
    // (1) warp 0: argmax |A[i, c]| (high parts) over rows c..kb-1 (ties: the lower row), and
    //     a copy of column c, so that (2) can swap rows while reading the old column
    if (tid < 32) {
      float best = -1.0f;
      int bi = c;
      for (int i = tid; i < kb; i += 32) {
        const float h = Ah[i + c * LD];
        ch[i] = h;
        cl[i] = Al[i + c * LD];
        if (i >= c && fabsf(h) > best) { best = fabsf(h); bi = i; }
      }
      for (int o = 16; o > 0; o >>= 1) {
        const float ob = __shfl_down_sync(0xffffffffu, best, o);
        const int oi = __shfl_down_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
      }
      if (tid == 0) {
        piv_row = bi;
        perm[c] = bi;
        if (!(best > 0.0f)) atomicExch(err, 1);
      }
    }
    __syncthreads();
    // (2) thread j < kb: swap rows c and pr of column j, scale the new row c by 1 / pivot;
    //     multipliers m_i = A[i, c] after the swap (from the copy of column c)
    const int pr = piv_row;
    if (tid < kb) {
      const int j = tid;
      float ih = 0.0f, il = 0.0f;
      const float dh = ch[pr], dl = cl[pr];  // the pivot
      if (dh != 0.0f) df_rcp(dh, dl, ih, il);
      const float ah = Ah[pr + j * LD], al = Al[pr + j * LD];  // new row c, column j
      if (pr != c) {
        Ah[pr + j * LD] = Ah[c + j * LD];
        Al[pr + j * LD] = Al[c + j * LD];
      }
      if (j == c) { rh[j] = ih; rl[j] = il; }
      else df_mul(ah, al, ih, il, rh[j], rl[j]);
      const int i = tid;
      const int src = i == pr ? c : i;  // row i after the swap holds the old row src
      if (i == c) { mh[i] = 0.0f; ml[i] = 0.0f; }
      else { mh[i] = ch[src]; ml[i] = cl[src]; }
    }
    __syncthreads();
    // (3) rank-1 update of every row but c; row c becomes the scaled pivot row
    if (ti < kb) {
      const float m_h = mh[ti], m_l = ml[ti];
#pragma unroll
      for (int u = 0; u < NB / CG; ++u) {
        const int j = tj + u * CG;
        if (j >= kb) break;
        const int idx = ti + j * LD;
        const float r_h = rh[j], r_l = rl[j];
        if (ti == c) {
          Ah[idx] = r_h;
          Al[idx] = r_l;
          continue;
        }
        const float ah = j == c ? 0.0f : Ah[idx], al = j == c ? 0.0f : Al[idx];
        // p = m · r in float-float
        const float ph = __fmul_rn(m_h, r_h);
        float pl = fmaf(m_h, r_h, -ph);
        pl = fmaf(m_h, r_l, pl);
        pl = fmaf(m_l, r_h, pl);
        // a − p: TwoSum on the high parts, the low parts added to the error, renormalised by TwoSum
        const float sh = __fsub_rn(ah, ph);
        const float bv = __fsub_rn(sh, ah);
        const float e = __fadd_rn(__fsub_rn(ah, __fsub_rn(sh, bv)), __fsub_rn(-ph, bv));
        const float sl = __fadd_rn(e, __fsub_rn(al, pl));
        const float h = __fadd_rn(sh, sl);
        const float hv = __fsub_rn(h, sh);
        Ah[idx] = h;
        Al[idx] = __fadd_rn(__fsub_rn(sh, __fsub_rn(h, hv)), __fsub_rn(sl, hv));
      }
    }
    __syncthreads();
  }
  if (tid == 0) {  // undo the row interchanges as column interchanges, last first
    for (int j = 0; j < kb; ++j) colsrc[j] = j;
    for (int c = kb - 1; c >= 0; --c) {
      const int p = perm[c];
      const int t = colsrc[c];
      colsrc[c] = colsrc[p];
      colsrc[p] = t;
    }
  }
  __syncthreads();
  float* Pf = P + f * (int64_t)NB * NB;
  for (int j = tj; j < NB; j += CG)  // column-major, zero outside kb x kb
    Pf[ti + j * NB] = (ti < kb && j < kb) ? __fadd_rn(Ah[ti + colsrc[j] * LD], Al[ti + colsrc[j] * LD]) : 0.0f;
}

// C = M[:, K] with the K rows zeroed (n x kb); Tb = M[K, c0 : c0+cw] (kb x cw).  Grid
// (column groups, fronts).
template <typename T>
__global__ void __launch_bounds__(256) k_gj_copy(const T* __restrict__ F, int64_t off, int n, int k, int kb, int c0,
                                                 int cw, T* __restrict__ C, T* __restrict__ Tb) {
  const int64_t f = blockIdx.y;
  const T* M = F + off + f * (int64_t)n * n;
  T* Cf = C + f * (int64_t)n * NB;
  T* Tf = Tb + f * (int64_t)NB * n;
  for (int j = blockIdx.x; j < kb; j += gridDim.x)  // C: column k + j
    for (int i = threadIdx.x; i < n; i += blockDim.x)
      Cf[i + (int64_t)j * n] = (i >= k && i < k + kb) ? (T)0 : M[i + (int64_t)(k + j) * n];
  const int r = threadIdx.x & (NB - 1);
  for (int c = blockIdx.x * (256 / NB) + threadIdx.x / NB; c < cw; c += gridDim.x * (256 / NB))  // Tb: kb rows
    if (r < kb) Tf[r + (int64_t)c * NB] = M[(k + r) + (int64_t)(c0 + c) * n];
}

// M[K, c0 + c] = T2[:, c] for c < cw outside K; M[K, K] = P.
template <typename T>
__global__ void __launch_bounds__(256) k_gj_fix(T* __restrict__ F, int64_t off, int n, int k, int kb, int c0, int cw,
                                                const T* __restrict__ T2, const T* __restrict__ P) {
  const int64_t f = blockIdx.y;
  T* M = F + off + f * (int64_t)n * n;
  const T* T2f = T2 + f * (int64_t)NB * n;
  const T* Pf = P + f * (int64_t)NB * NB;
  const int r = threadIdx.x & (NB - 1);
  for (int c = blockIdx.x * (256 / NB) + threadIdx.x / NB; c < cw; c += gridDim.x * (256 / NB))
    if (r < kb) {
      const int cc = c0 + c;
      const bool inK = cc >= k && cc < k + kb;
      M[(k + r) + (int64_t)cc * n] = inK ? Pf[r + (int64_t)(cc - k) * NB] : T2f[r + (int64_t)c * NB];
    }
}

// Panel elimination helpers (panel = pivot columns [p, p + pw)):
// R = M[p : p+pw, :] (pw x n, ld PW) before the panel is eliminated, and Nz = M[:, p : p+pw]
// with the panel rows zeroed (n x pw, ld n) after it.
template <typename T>
__global__ void __launch_bounds__(256) k_panel_rows(const T* __restrict__ F, int64_t off, int n, int p, int pw,
                                                    T* __restrict__ R) {
  const int64_t f = blockIdx.y;
  const T* M = F + off + f * (int64_t)n * n;
  T* Rf = R + f * (int64_t)PW * n;
  const int r = threadIdx.x & (PW - 1);
  for (int c = blockIdx.x * (256 / PW) + threadIdx.x / PW; c < n; c += gridDim.x * (256 / PW))
    if (r < pw) Rf[r + (int64_t)c * PW] = M[(p + r) + (int64_t)c * n];
}

template <typename T>
__global__ void __launch_bounds__(256) k_panel_cols(const T* __restrict__ F, int64_t off, int n, int p, int pw,
                                                    T* __restrict__ Nz) {
  const int64_t f = blockIdx.y;
  const T* M = F + off + f * (int64_t)n * n;
  T* Nf = Nz + f * (int64_t)n * PW;
  for (int j = blockIdx.x; j < pw; j += gridDim.x)
    for (int i = threadIdx.x; i < n; i += blockDim.x)
      Nf[i + (int64_t)j * n] = (i >= p && i < p + pw) ? (T)0 : M[i + (int64_t)(p + j) * n];
}

// ------------------------------------------------------------------ solve kernels
__global__ void k_fwd_gather(const double* __restrict__ b, double* __restrict__ tsave, const int64_t* __restrict__ toff,
                             const int32_t* __restrict__ elim, const int64_t* __restrict__ elim_ptr,
                             const int32_t* __restrict__ f_ne, int64_t first, int E) {
  const int64_t f = first + blockIdx.x;
  const int ne = f_ne[f];
  const int32_t* el = elim + elim_ptr[f];
  double* t = tsave + toff[f];
  for (int i = threadIdx.x; i < E; i += blockDim.x) t[i] = i < ne ? b[el[i]] : 0.0;
}

// ---- accumulation of the sweeps
// FP32 factors: the vector entries are split into two floats (hi + lo) and the products
// are summed in float-float arithmetic (exact product error by FMA, Knuth's TwoSum for the
// sum), which keeps ~44 significant bits on FP32 pipes.  GB300 issues FP64 at a small
// fraction of its FP32 rate, so an FP64 convert + FMA per factor entry would bound the
// sweeps by FP64 issue instead of HBM; rounding the vectors to FP32 instead doubled the
// FGMRES iteration count at Ha = 500.  FP64 factors accumulate in FP64.
template <typename T>
struct SweepAcc;

template <>
struct SweepAcc<float> {
  using V = float2;
  float hi = 0.0f, lo = 0.0f;
  __device__ static V pack(double t) {
    const float h = (float)t;
    return make_float2(h, (float)(t - (double)h));
  }
  __device__ void add(float m, V v) {
    const float p = __fmul_rn(m, v.x);
    const float pe = fmaf(m, v.y, fmaf(m, v.x, -p));  // p + pe = m (v.x + v.y) to ~2^-48
    const float s = __fadd_rn(hi, p);
    const float bp = __fsub_rn(s, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(p, bp));
    hi = s;
    lo = __fadd_rn(lo, __fadd_rn(err, pe));
  }
  __device__ void merge(const SweepAcc<float>& o) { merge(o.hi, o.lo); }
  __device__ void merge(float ohi, float olo) {
    const float s = __fadd_rn(hi, ohi);
    const float bp = __fsub_rn(s, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(ohi, bp));
    hi = s;
    lo = __fadd_rn(lo, __fadd_rn(err, olo));
  }
  __device__ void warp_reduce() {
    for (int o = 16; o > 0; o >>= 1) {
      const float oh = __shfl_down_sync(0xffffffffu, hi, o), ol = __shfl_down_sync(0xffffffffu, lo, o);
      merge(oh, ol);
    }
  }
  __device__ double value() const { return (double)hi + (double)lo; }
};

template <>
struct SweepAcc<double> {
  using V = double;
  double a = 0.0;
  __device__ static V pack(double t) { return t; }
  __device__ void add(double m, V v) { a = fma(m, v, a); }
  __device__ void merge(const SweepAcc<double>& o) { a += o.a; }
  __device__ void warp_reduce() {
    for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
  }
  __device__ double value() const { return a; }
};

// 16-byte vectors of factor entries: a thread of the chunked sweeps owns R consecutive
// rows (column-major fronts: one vector load per column).
template <typename T>
struct RowVec;
template <>
struct RowVec<float> {
  using type = float4;
  static constexpr int R = 4;
};
template <>
struct RowVec<double> {
  using type = double2;
  static constexpr int R = 2;
};

// acc[r] += Σ_{k<len} col[k·ld + r] · v[k], r < R: eight 16-byte loads in flight per
// thread, R independent accumulators.  col must be 16-byte aligned and ld a multiple of R.
template <typename T>
__device__ __forceinline__ void strided_dot_rows(SweepAcc<T> (&acc)[RowVec<T>::R], const T* __restrict__ col,
                                                 int64_t ld, const typename SweepAcc<T>::V* __restrict__ v, int len) {
  using VT = typename RowVec<T>::type;
  constexpr int R = RowVec<T>::R;
  int k = 0;
  for (; k + 8 <= len; k += 8) {
    VT q[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) q[u] = __ldcs(reinterpret_cast<const VT*>(col + (int64_t)(k + u) * ld));
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const T* qa = reinterpret_cast<const T*>(&q[u]);
      const typename SweepAcc<T>::V vv = v[k + u];
#pragma unroll
      for (int r = 0; r < R; ++r) acc[r].add(qa[r], vv);
    }
  }
  for (; k < len; ++k) {
    const VT q = __ldcs(reinterpret_cast<const VT*>(col + (int64_t)k * ld));
    const T* qa = reinterpret_cast<const T*>(&q);
    const typename SweepAcc<T>::V vv = v[k];
#pragma unroll
    for (int r = 0; r < R; ++r) acc[r].add(qa[r], vv);
  }
}

// acc[c] += Σ_{i<len} col0[c·ld + i] v[i], c < ncols ≤ NC, for one warp: each lane takes
// 16-byte groups of four rows, loads the matching four packed vector entries once (two
// 16-byte loads) and reuses them for the NC columns.  A lane sums the products of four
// groups (16 terms per column) with FP32 FMAs, the vector's high and low parts separately,
// and folds those short sums into the float-float accumulators.  col0 and ld·4 bytes must
// be 16-byte aligned, v 16-byte aligned and zero-padded to a multiple of 4 entries.
template <int NC>
__device__ __forceinline__ void warp_cols_dot(SweepAcc<float> (&acc)[NC], const float* __restrict__ col0, int64_t ld,
                                              int ncols, const float2* __restrict__ v, int len, int lane) {
  const int len4 = (len + 3) >> 2;
  const float4* v4 = reinterpret_cast<const float4*>(v);  // two packed entries per float4
  for (int g0 = 0; g0 < len4; g0 += 128) {
    float h[NC], l[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) h[c] = l[c] = 0.0f;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int g = g0 + lane + 32 * u;
      if (g < len4) {
        const float4 va = v4[2 * g], vb = v4[2 * g + 1];
#pragma unroll
        for (int c = 0; c < NC; ++c) {
          if (c < ncols) {  // warp-uniform
            const float4 m = __ldcs(reinterpret_cast<const float4*>(col0 + c * ld) + g);
            h[c] = fmaf(m.x, va.x, h[c]); l[c] = fmaf(m.x, va.y, l[c]);
            h[c] = fmaf(m.y, va.z, h[c]); l[c] = fmaf(m.y, va.w, l[c]);
            h[c] = fmaf(m.z, vb.x, h[c]); l[c] = fmaf(m.z, vb.y, l[c]);
            h[c] = fmaf(m.w, vb.z, h[c]); l[c] = fmaf(m.w, vb.w, l[c]);
          }
        }
      }
    }
#pragma unroll
    for (int c = 0; c < NC; ++c) acc[c].merge(h[c], l[c]);
  }
}

// Transposed sweeps (adjoint solves): a warp takes NC adjacent columns of a front and runs
// down them together (each dot product is a contiguous column of the column-major front).
// FP32 factors read the level's packed vector segments (vpk); FP64 factors stage theirs in
// shared memory and use NC = 1.
// forward, transposed: b[bnd_j] −= Σ_{i<ne} TR[i, j] t_i   (TR = rows 0..E of column E+j)
template <typename T, int NC>
__global__ void __launch_bounds__(256) k_fwd_gemv_t(const T* __restrict__ F, const int64_t* __restrict__ f_off,
                                                    double* __restrict__ b, const double* __restrict__ tsave,
                                                    const int64_t* __restrict__ toff, const int32_t* __restrict__ bnd,
                                                    const int64_t* __restrict__ bnd_ptr, const int32_t* __restrict__ f_nb,
                                                    const int32_t* __restrict__ f_ne, int64_t first, int n, int E,
                                                    const float2* __restrict__ vpk) {
  using V = typename SweepAcc<T>::V;
  extern __shared__ __align__(16) unsigned char sm_raw[];
  V* ts = reinterpret_cast<V*>(sm_raw);
  const int64_t f = first + blockIdx.y;
  const int nb = f_nb[f], ne = f_ne[f];
  if constexpr (sizeof(T) != 4) {
    const double* t = tsave + toff[f];
    for (int i = threadIdx.x; i < ne; i += blockDim.x) ts[i] = SweepAcc<T>::pack(t[i]);
    __syncthreads();
  }
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int j = (blockIdx.x * (blockDim.x / 32) + warp) * NC;
  if (j >= nb) return;
  const int ncols = min(NC, nb - j);
  const T* colj = F + f_off[f] + (int64_t)(E + j) * n;
  SweepAcc<T> acc[NC];
  if constexpr (sizeof(T) == 4) {
    warp_cols_dot<NC>(acc, colj, n, ncols, vpk + (int64_t)blockIdx.y * n, ne, lane);  // packed t of this front
  } else {
    static_assert(sizeof(T) == 4 || NC == 1, "FP64 transposed sweeps take one column per warp");
    for (int i = lane; i < ne; i += 32) acc[0].add(colj[i], ts[i]);
  }
  const int32_t* bd = bnd + bnd_ptr[f];
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    acc[c].warp_reduce();
    if (lane == 0 && c < ncols) atomicAdd(&b[bd[j + c]], -acc[c].value());
  }
}

// backward, transposed: x[elim_i] = Σ_{c<ne} TL[c, i] t_c + Σ_{j<nb} BL[j, i] x_B[j]
// (column i of the front: rows 0..E are TL, rows E.. are BL)
template <typename T, int NC>
__global__ void __launch_bounds__(256) k_bwd_gemv_t(const T* __restrict__ F, const int64_t* __restrict__ f_off,
                                                    double* __restrict__ x, const double* __restrict__ tsave,
                                                    const int64_t* __restrict__ toff, const int32_t* __restrict__ elim,
                                                    const int64_t* __restrict__ elim_ptr, const int32_t* __restrict__ bnd,
                                                    const int64_t* __restrict__ bnd_ptr, const int32_t* __restrict__ f_ne,
                                                    const int32_t* __restrict__ f_nb, int64_t first, int n, int E,
                                                    const float2* __restrict__ vpk) {
  using V = typename SweepAcc<T>::V;
  extern __shared__ __align__(16) unsigned char sm_raw[];
  V* vs = reinterpret_cast<V*>(sm_raw);  // [E] t, then [n-E] x_B
  const int64_t f = first + blockIdx.y;
  const int ne = f_ne[f], nb = f_nb[f];
  if constexpr (sizeof(T) != 4) {
    const double* t = tsave + toff[f];
    const int32_t* bd = bnd + bnd_ptr[f];
    for (int i = threadIdx.x; i < ne; i += blockDim.x) vs[i] = SweepAcc<T>::pack(t[i]);
    for (int j = threadIdx.x; j < nb; j += blockDim.x) vs[E + j] = SweepAcc<T>::pack(x[bd[j]]);
    __syncthreads();
  }
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int i = (blockIdx.x * (blockDim.x / 32) + warp) * NC;
  if (i >= ne) return;
  const int ncols = min(NC, ne - i);
  const T* coli = F + f_off[f] + (int64_t)i * n;
  SweepAcc<T> acc[NC];
  if constexpr (sizeof(T) == 4) {
    const float2* v = vpk + (int64_t)blockIdx.y * n;  // packed [t ; x_B] of this front
    warp_cols_dot<NC>(acc, coli, n, ncols, v, ne, lane);
    warp_cols_dot<NC>(acc, coli + E, n, ncols, v + E, nb, lane);
  } else {
    static_assert(sizeof(T) == 4 || NC == 1, "FP64 transposed sweeps take one column per warp");
    for (int c = lane; c < ne; c += 32) acc[0].add(coli[c], vs[c]);
    for (int j = lane; j < nb; j += 32) acc[0].add(coli[E + j], vs[E + j]);
  }
  const int32_t* el = elim + elim_ptr[f];
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    acc[c].warp_reduce();
    if (lane == 0 && c < ncols) x[el[i + c]] = acc[c].value();
  }
}

// Packed (float-float) vector segments of a level's fronts for the transposed FP32 sweeps:
// vpk[front][0, E) = t (zero beyond ne), and with x given, vpk[front][E, n) = x_B (zero
// beyond nb).  One pass per level instead of every CTA staging its front's segment.
__global__ void k_pack_vec(const double* __restrict__ tsave, const int64_t* __restrict__ toff,
                           const double* __restrict__ x, const int32_t* __restrict__ bnd,
                           const int64_t* __restrict__ bnd_ptr, const int32_t* __restrict__ f_ne,
                           const int32_t* __restrict__ f_nb, int64_t first, int n, int E, float2* __restrict__ vpk) {
  const int64_t f = first + blockIdx.x;
  const int ne = f_ne[f], nb = f_nb[f];
  const double* t = tsave + toff[f];
  float2* v = vpk + (int64_t)blockIdx.x * n;
  for (int i = threadIdx.x; i < E; i += blockDim.x) v[i] = SweepAcc<float>::pack(i < ne ? t[i] : 0.0);
  if (x) {
    const int32_t* bd = bnd + bnd_ptr[f];
    for (int j = threadIdx.x; j < n - E; j += blockDim.x) v[E + j] = SweepAcc<float>::pack(j < nb ? x[bd[j]] : 0.0);
  }
}

// Chunked sweeps: grid (row tiles, column chunks, fronts); each thread owns R consecutive
// rows of its tile and reduces one chunk of `cols` columns, staged in shared memory; partial
// sums are added atomically.  Row accesses are coalesced 16-byte vectors (column-major
// fronts; E, B and n are multiples of 8, so every vector is aligned and rows up to the next
// multiple of R stay inside the padded front).  The chunk width is chosen per level so that
// levels with few fronts still fill the GPU.
constexpr int SW_THREADS = 128;

// forward: b[bnd_j] += Σ_{i<ne} M[E+j, i] t_i
template <typename T>
__global__ void __launch_bounds__(SW_THREADS) k_fwd_chunk(const T* __restrict__ F, const int64_t* __restrict__ f_off,
                                                          double* __restrict__ b, const double* __restrict__ tsave,
                                                          const int64_t* __restrict__ toff, const int32_t* __restrict__ bnd,
                                                          const int64_t* __restrict__ bnd_ptr,
                                                          const int32_t* __restrict__ f_nb,
                                                          const int32_t* __restrict__ f_ne, int64_t first, int n, int E,
                                                          int cols) {
  using V = typename SweepAcc<T>::V;
  constexpr int R = RowVec<T>::R;
  extern __shared__ __align__(16) unsigned char sm_raw[];
  V* ts = reinterpret_cast<V*>(sm_raw);
  const int64_t f = first + blockIdx.z;
  const int nb = f_nb[f];
  const int j0 = (blockIdx.x * SW_THREADS + threadIdx.x) * R;
  const int ne = f_ne[f];  // columns [ne, E) are padding
  const int c0 = blockIdx.y * cols, c1 = min(ne, c0 + cols);
  if (blockIdx.x * SW_THREADS * R >= nb || c0 >= ne) return;
  const double* t = tsave + toff[f];
  for (int c = c0 + threadIdx.x; c < c1; c += blockDim.x) ts[c - c0] = SweepAcc<T>::pack(t[c]);
  __syncthreads();
  if (j0 >= nb) return;
  SweepAcc<T> acc[R];
  strided_dot_rows<T>(acc, F + f_off[f] + E + j0 + (int64_t)c0 * n, n, ts, c1 - c0);
  const int32_t* bd = bnd + bnd_ptr[f];
#pragma unroll
  for (int r = 0; r < R; ++r)
    if (j0 + r < nb) atomicAdd(&b[bd[j0 + r]], acc[r].value());
}

// backward: y_i = Σ_c M[i, c] v_c with v = [t ; −x_B], accumulated into ybuf (then scattered)
template <typename T>
__global__ void __launch_bounds__(SW_THREADS) k_bwd_chunk(const T* __restrict__ F, const int64_t* __restrict__ f_off,
                                                          const double* __restrict__ x, const double* __restrict__ tsave,
                                                          const int64_t* __restrict__ toff, const int32_t* __restrict__ bnd,
                                                          const int64_t* __restrict__ bnd_ptr,
                                                          const int32_t* __restrict__ f_ne,
                                                          const int32_t* __restrict__ f_nb, double* __restrict__ ybuf,
                                                          int64_t first, int n, int E, int cols) {
  using V = typename SweepAcc<T>::V;
  constexpr int R = RowVec<T>::R;
  extern __shared__ __align__(16) unsigned char sm_raw[];
  V* vs = reinterpret_cast<V*>(sm_raw);
  const int64_t f = first + blockIdx.z;
  const int ne = f_ne[f], nb = f_nb[f];
  const int i0 = (blockIdx.x * SW_THREADS + threadIdx.x) * R;
  // virtual columns v in [0, ne + nb): v < ne -> column v, else column E + (v − ne)
  const int c0 = blockIdx.y * cols, c1 = min(ne + nb, c0 + cols);
  if (blockIdx.x * SW_THREADS * R >= ne || c0 >= ne + nb) return;
  const double* t = tsave + toff[f];
  const int32_t* bd = bnd + bnd_ptr[f];
  for (int v = c0 + threadIdx.x; v < c1; v += blockDim.x)
    vs[v - c0] = SweepAcc<T>::pack(v < ne ? t[v] : -x[bd[v - ne]]);
  __syncthreads();
  if (i0 >= ne) return;
  const T* M = F + f_off[f] + i0;
  SweepAcc<T> acc[R];
  const int va = min(c1, ne);
  if (va > c0) strided_dot_rows<T>(acc, M + (int64_t)c0 * n, n, vs, va - c0);
  const int vb = max(c0, ne);  // boundary columns: virtual v -> column E + (v − ne)
  if (c1 > vb) strided_dot_rows<T>(acc, M + (int64_t)(E - ne + vb) * n, n, vs + (vb - c0), c1 - vb);
#pragma unroll
  for (int r = 0; r < R; ++r)
    if (i0 + r < ne) atomicAdd(&ybuf[toff[f] + i0 + r], acc[r].value());
}

// ---- TMA-staged sweeps (FP32 factors)
// A CTA owns a tile of `rows` rows (at most TS_ROWS, sized per level so that the tiles cover
// the level's rows with little overhang) of one front and a chunk of its columns.  Thread 0
// streams the chunk through shared memory in stages of TS_COLS columns with
// cp.async.bulk.tensor (one 3-D tensor map per level: rows x columns x fronts), keeping
// TS_STAGES stages in flight behind mbarriers; every thread reduces two rows of each staged
// column in float-float arithmetic.  The forward sweep reads the boundary rows of the
// eliminated columns, the backward sweep the eliminated rows of the eliminated columns
// and of the boundary columns (two column segments, chunked separately).
constexpr int TS_ROWS = 256;
constexpr int TS_COLS = 16;
constexpr int TS_STAGES = 4;
constexpr int TS_THREADS = TS_ROWS / 2;   // launch bound; a level uses rows / 2 threads
constexpr long TS_WAIT_LIMIT = kSweepWaitDefault;  // bounded mbarrier waits (default; GBMHD_SWEEP_WAIT_LIMIT)

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(phase)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t phase, long limit = TS_WAIT_LIMIT) {
  for (long i = 0; i < limit; ++i)
    if (mbar_try_wait(bar, phase)) return true;
  return false;
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
      ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

// FWD: b[bnd_j] += Σ_{c<ne} M[E+j, c] t_c.   BWD: ybuf_i += Σ_v M[i, col(v)] w_v over v in this
// CTA's chunk, w = [t ; −x_B], col(v) = v (v < ne) or E + (v − ne).
//
// The level's vector gather and scatter are folded in.  FWD reads t_c = b[elim_c] itself (the
// level's eliminated dofs are not boundary dofs of any front of the level, so no CTA of the
// launch writes them) and the CTAs of the first row tile save t for the backward sweep.  BWD
// adds its partial sums straight into x[elim_i]; the solve zeroes x first.
template <bool FWD>
__global__ void __launch_bounds__(TS_THREADS) k_sweep_tma(const __grid_constant__ CUtensorMap map, int64_t first,
                                                          int E, int rows, int cw, int chunks_a,
                                                          double* __restrict__ b,
                                                          double* __restrict__ x,
                                                          double* __restrict__ tsave,
                                                          const int64_t* __restrict__ toff,
                                                          const int32_t* __restrict__ bnd,
                                                          const int64_t* __restrict__ bnd_ptr,
                                                          const int32_t* __restrict__ elim,
                                                          const int64_t* __restrict__ elim_ptr,
                                                          const int32_t* __restrict__ f_ne,
                                                          const int32_t* __restrict__ f_nb, int32_t* err,
                                                          long wait_limit) {
  extern __shared__ __align__(1024) unsigned char ts_raw[];
  float* tiles = reinterpret_cast<float*>(ts_raw);                  // [stage][column][row]
  float2* vs = reinterpret_cast<float2*>(ts_raw + (size_t)TS_STAGES * TS_COLS * rows * sizeof(float));  // [cw]
  __shared__ __align__(8) uint64_t full[TS_STAGES];
  __shared__ int abort_flag;
  const int fl = blockIdx.z;
  const int64_t f = first + fl;
  const int ne = f_ne[f], nb = f_nb[f];
  const int nrows = FWD ? nb : ne;
  const int row0 = blockIdx.x * rows;
  const bool seg_b = !FWD && (int)blockIdx.y >= chunks_a;
  const int c0 = (seg_b ? (int)blockIdx.y - chunks_a : (int)blockIdx.y) * cw;
  const int c1 = min(seg_b ? nb : ne, c0 + cw);
  const int32_t* el = elim + elim_ptr[f];
  if (FWD && blockIdx.x == 0) {  // save t for the backward sweep, also when the front has no rows here
    double* ts = tsave + toff[f];
    for (int c = c0 + (int)threadIdx.x; c < c1; c += blockDim.x) ts[c] = b[el[c]];
  }
  if (row0 >= nrows) return;
  if (c0 >= c1) return;
  const int ncol = c1 - c0;
  const int pcol0 = seg_b ? E + c0 : c0;
  const int prow0 = (FWD ? E : 0) + row0;
  const int nst = (ncol + TS_COLS - 1) / TS_COLS;
  const uint32_t stage_bytes = TS_COLS * rows * sizeof(float);
  if (threadIdx.x == 0) {
    for (int s = 0; s < TS_STAGES; ++s) mbar_init(&full[s], 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0)
    for (int s = 0; s < min(TS_STAGES, nst); ++s) {
      mbar_expect_tx(&full[s], stage_bytes);
      tma_load_3d(tiles + (size_t)s * TS_COLS * rows, &map, prow0, pcol0 + s * TS_COLS, fl, &full[s]);
    }
  const double* t = tsave + toff[f];
  const int32_t* bd = bnd + bnd_ptr[f];
  for (int c = threadIdx.x; c < ncol; c += blockDim.x)
    vs[c] = SweepAcc<float>::pack(FWD ? b[el[c0 + c]] : seg_b ? -x[bd[c0 + c]] : t[c0 + c]);
  __syncthreads();
  SweepAcc<float> a0, a1;
  const int r = 2 * threadIdx.x;
  for (int s = 0; s < nst; ++s) {
    const int buf = s % TS_STAGES;
    if (mbar_wait_bounded(&full[buf], (uint32_t)(s / TS_STAGES) & 1u, wait_limit)) {
      const float* tile = tiles + (size_t)buf * TS_COLS * rows;
      const float2* vv = vs + s * TS_COLS;
      const int cn = min(TS_COLS, ncol - s * TS_COLS);
      // a stage's (at most 16) products are summed with FP32 FMAs, the high and low parts of
      // the vector separately, and the two short sums are folded into the float-float
      // accumulators: ~3 instructions per factor entry instead of ~13 for float-float per
      // product, with the rounding of 16-term FP32 sums only
      float h0 = 0.0f, l0 = 0.0f, h1 = 0.0f, l1 = 0.0f;
#pragma unroll 4
      for (int c = 0; c < cn; ++c) {
        const float2 m = *reinterpret_cast<const float2*>(tile + c * rows + r);
        const float2 v = vv[c];
        h0 = fmaf(m.x, v.x, h0);
        l0 = fmaf(m.x, v.y, l0);
        h1 = fmaf(m.y, v.x, h1);
        l1 = fmaf(m.y, v.y, l1);
      }
      a0.merge(h0, l0);
      a1.merge(h1, l1);
    } else {
      abort_flag = 1;
    }
    __syncthreads();
    if (abort_flag) {
      if (threadIdx.x == 0) {  // let the copies in flight land before the CTA's shared memory is released
        // (with the full limit, whatever limit the stage wait had)
        for (int s2 = s; s2 < min(nst, s + TS_STAGES); ++s2)
          mbar_wait_bounded(&full[s2 % TS_STAGES], (uint32_t)(s2 / TS_STAGES) & 1u, TS_WAIT_LIMIT);
        atomicExch(err, 1);
      }
      return;
    }
    if (threadIdx.x == 0 && s + TS_STAGES < nst) {
      mbar_expect_tx(&full[buf], stage_bytes);
      tma_load_3d(tiles + (size_t)buf * TS_COLS * rows, &map, prow0, pcol0 + (s + TS_STAGES) * TS_COLS, fl,
                  &full[buf]);
    }
  }
  const int i0 = row0 + r;
  if (FWD) {
    if (i0 < nb) atomicAdd(&b[bd[i0]], a0.value());
    if (i0 + 1 < nb) atomicAdd(&b[bd[i0 + 1]], a1.value());
  } else {
    if (i0 < ne) atomicAdd(&x[el[i0]], a0.value());
    if (i0 + 1 < ne) atomicAdd(&x[el[i0 + 1]], a1.value());
  }
}

__global__ void k_zero_at(const int32_t* __restrict__ idx, int64_t cnt, double* __restrict__ x) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < cnt; i += (int64_t)gridDim.x * blockDim.x)
    x[idx[i]] = 0.0;
}

__global__ void k_bwd_scatter(double* __restrict__ x, double* __restrict__ ybuf, const int64_t* __restrict__ toff,
                              const int32_t* __restrict__ elim, const int64_t* __restrict__ elim_ptr,
                              const int32_t* __restrict__ f_ne, int64_t first) {
  const int64_t f = first + blockIdx.x;
  const int ne = f_ne[f];
  const int32_t* el = elim + elim_ptr[f];
  double* y = ybuf + toff[f];
  for (int i = threadIdx.x; i < ne; i += blockDim.x) {
    x[el[i]] = y[i];
    y[i] = 0.0;  // ready for the next solve
  }
}

// ------------------------------------------------------------------ host drivers
// ---- tensor maps of the TMA-staged sweeps
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_tiled_fn() {
  static EncodeTiledFn fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  return fn;
}

// Row tile of a sweep over `nrows` rows: the fewest tiles of at most TS_ROWS rows, each a
// multiple of 32 rows (16 threads), so that the TMA boxes overhang the rows little.
static int tma_rows(int nrows) {
  const int tiles = std::max(1, (nrows + TS_ROWS - 1) / TS_ROWS);
  const int per = (nrows + tiles - 1) / tiles;
  return std::min(TS_ROWS, std::max(32, (per + 31) / 32 * 32));
}

// Two maps per level over the FP32 fronts (forward: boundary rows, backward: eliminated
// rows): dims (n rows, n columns, count fronts), box (rows, TS_COLS, 1).  A level whose
// fronts are narrower than a box keeps the LDG sweeps.
static void build_sweep_maps(MFNumeric* M) {
  const MFSymbolic& S = M->S;
  const size_t nl = S.levels.size();
  M->maps.assign(2 * nl, CUtensorMap{});
  M->map_rows.assign(2 * nl, 0);
  M->map_ok.assign(nl, 0);
  M->maps_base = M->F;
  EncodeTiledFn enc = encode_tiled_fn();
  if (!enc) return;
  float* F = reinterpret_cast<float*>(M->F);
  for (size_t l = 0; l < nl; ++l) {
    const MFLevel& L = S.levels[l];
    if (L.n < TS_ROWS || L.count > (1 << 16)) continue;
    bool ok = true;
    for (int dir = 0; dir < 2; ++dir) {  // 0: forward (B rows), 1: backward (E rows)
      const int rows = tma_rows(dir == 0 ? std::max(L.B, 1) : L.E);
      const cuuint64_t dims[3] = {(cuuint64_t)L.n, (cuuint64_t)L.n, (cuuint64_t)L.count};
      const cuuint64_t strides[2] = {(cuuint64_t)L.n * sizeof(float), (cuuint64_t)L.n * L.n * sizeof(float)};
      const cuuint32_t box[3] = {(cuuint32_t)rows, TS_COLS, 1};
      const cuuint32_t estr[3] = {1, 1, 1};
      ok = ok && enc(&M->maps[2 * l + dir], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, F + L.off, dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
      M->map_rows[2 * l + dir] = rows;
    }
    M->map_ok[l] = ok ? 1 : 0;
  }
}

// Column chunk of the TMA sweeps: a multiple of TS_COLS, about two waves of three resident
// CTAs per SM for the level.
static int tma_cols(const gbmhd_ctx* ctx, int64_t rows, int tile_rows, int64_t ncols, int64_t fronts) {
  const int64_t per_chunk = std::max<int64_t>(1, (rows + tile_rows - 1) / tile_rows) * std::max<int64_t>(1, fronts);
  const int64_t want = (int64_t)ctx->num_sms * 6;
  const int64_t chunks = std::max<int64_t>(1, (want + per_chunk - 1) / per_chunk);
  int64_t cols = (ncols + chunks - 1) / chunks;
  cols = ((cols + TS_COLS - 1) / TS_COLS) * TS_COLS;
  return (int)std::max<int64_t>(TS_COLS, std::min<int64_t>(cols, 1024));
}

template <typename T>
static cublasStatus_t gemm_sb(MFNumeric* M, cublasOperation_t ta, cublasOperation_t tb, int m, int n, int k,
                              const T* alpha, const T* A, int lda, long long sA, const T* B, int ldb, long long sB,
                              const T* beta, T* C, int ldc, long long sC, int batch) {
  if constexpr (sizeof(T) == 8) {
    return cublasGemmStridedBatchedEx(M->blas, ta, tb, m, n, k, alpha, A, CUDA_R_64F, lda, sA, B, CUDA_R_64F, ldb, sB,
                                      beta, C, CUDA_R_64F, ldc, sC, batch, CUBLAS_COMPUTE_64F, CUBLAS_GEMM_DEFAULT);
  } else {
    cublasComputeType_t ct = M->fp32_gemm_mode == 0 ? CUBLAS_COMPUTE_32F_EMULATED_16BFX9 : CUBLAS_COMPUTE_32F;
    cublasStatus_t s = cublasGemmStridedBatchedEx(M->blas, ta, tb, m, n, k, alpha, A, CUDA_R_32F, lda, sA, B,
                                                  CUDA_R_32F, ldb, sB, beta, C, CUDA_R_32F, ldc, sC, batch, ct,
                                                  CUBLAS_GEMM_DEFAULT);
    if (s != CUBLAS_STATUS_SUCCESS && M->fp32_gemm_mode == 0) {
      M->fp32_gemm_mode = 1;  // emulation unavailable: plain FP32
      s = cublasGemmStridedBatchedEx(M->blas, ta, tb, m, n, k, alpha, A, CUDA_R_32F, lda, sA, B, CUDA_R_32F, ldb, sB,
                                     beta, C, CUDA_R_32F, ldc, sC, batch, CUBLAS_COMPUTE_32F, CUBLAS_GEMM_DEFAULT);
    }
    return s;
  }
}

template <typename T, typename V>
static int factor_impl(gbmhd_ctx* ctx, MFNumeric* M, const V* Aval, const double* d_reg) {
  const MFSymbolic& S = M->S;
  // buffers
  const size_t fbytes = sizeof(T) * (size_t)std::max<int64_t>(S.storage, 1);
  if (M->F_bytes != fbytes) {
    if (M->F) cudaFree(M->F);
    M->F = nullptr;
    MF_CUDA(cudaMalloc(&M->F, fbytes));
    M->F_bytes = fbytes;
  }
  size_t wmax = 0, pmax = 0;
  for (const MFLevel& L : S.levels) {
    wmax = std::max(wmax, (size_t)L.count * L.n * NB);
    pmax = std::max(pmax, (size_t)L.count * L.n * PW);
  }
  size_t pbytes = 0;
  for (const MFLevel& L : S.levels) pbytes = std::max(pbytes, (size_t)L.count * NB * NB);
  const size_t need = sizeof(T) * (3 * wmax + pbytes + 2 * pmax);
  if (M->work_bytes < need) {
    for (void* p : {M->Pbuf, M->Cbuf, M->Tbuf, M->T2buf, M->Rbuf, M->Nbuf})
      if (p) cudaFree(p);
    MF_CUDA(cudaMalloc(&M->Pbuf, sizeof(T) * std::max<size_t>(pbytes, 1)));
    MF_CUDA(cudaMalloc(&M->Cbuf, sizeof(T) * std::max<size_t>(wmax, 1)));
    MF_CUDA(cudaMalloc(&M->Tbuf, sizeof(T) * std::max<size_t>(wmax, 1)));
    MF_CUDA(cudaMalloc(&M->T2buf, sizeof(T) * std::max<size_t>(wmax, 1)));
    MF_CUDA(cudaMalloc(&M->Rbuf, sizeof(T) * std::max<size_t>(pmax, 1)));
    MF_CUDA(cudaMalloc(&M->Nbuf, sizeof(T) * std::max<size_t>(pmax, 1)));
    M->work_bytes = need;
  }
  T* F = reinterpret_cast<T*>(M->F);
  T* P = reinterpret_cast<T*>(M->Pbuf);
  T* C = reinterpret_cast<T*>(M->Cbuf);
  T* Tb = reinterpret_cast<T*>(M->Tbuf);
  T* T2 = reinterpret_cast<T*>(M->T2buf);
  T* R = reinterpret_cast<T*>(M->Rbuf);
  T* Nz = reinterpret_cast<T*>(M->Nbuf);
  MF_CUDA(cudaMemsetAsync(M->d_err, 0, sizeof(int32_t), ctx->stream));
  // level sizes on the device for the extend-add kernel
  std::vector<int> ln(S.levels.size()), le(S.levels.size());
  for (size_t l = 0; l < S.levels.size(); ++l) { ln[l] = S.levels[l].n; le[l] = S.levels[l].E; }
  int *d_ln = nullptr, *d_le = nullptr;
  MF_CUDA(cudaMallocAsync(&d_ln, sizeof(int) * ln.size(), ctx->stream));
  MF_CUDA(cudaMallocAsync(&d_le, sizeof(int) * le.size(), ctx->stream));
  MF_CUDA(cudaMemcpyAsync(d_ln, ln.data(), sizeof(int) * ln.size(), cudaMemcpyHostToDevice, ctx->stream));
  MF_CUDA(cudaMemcpyAsync(d_le, le.data(), sizeof(int) * le.size(), cudaMemcpyHostToDevice, ctx->stream));
  const T one = 1, mone = -1, zero = 0;
  for (size_t l = 0; l < S.levels.size(); ++l) {
    const MFLevel& L = S.levels[l];
    const int n = L.n, E = L.E;
    const int cnt = (int)L.count;
    MF_CUDA(cudaMemsetAsync(F + L.off, 0, sizeof(T) * (size_t)L.count * n * n, ctx->stream));
    { k_pad_diag<T><<<cnt, 128, 0, ctx->stream>>>(F, L.off, L.count, n, E, M->d.f_ne, L.first); gbmhd::count_launch(); }
    const int64_t nah = L.ah_end - L.ah_begin;
    if (nah > 0) {
      int64_t g = std::min<int64_t>((nah + 255) / 256, (int64_t)ctx->num_sms * 16);
      { k_arrowhead<T, V><<<(unsigned)g, 256, 0, ctx->stream>>>(Aval, M->d.ah_src, M->d.ah_dst, L.ah_begin, L.ah_end, F); gbmhd::count_launch(); }
    }
    if (l + 1 == S.levels.size() && d_reg && !S.reg_dst.empty()) {
      // the global p and φ representatives are eliminated in the root front
      const int64_t nr = (int64_t)S.reg_dst.size();
      { k_reg_add<T><<<(unsigned)std::min<int64_t>((nr + 255) / 256, 4096), 256, 0, ctx->stream>>>(F, M->d.reg_dst, M->d.reg_dof, d_reg, M->scaled ? M->d_dr : nullptr, M->d_dc, nr); gbmhd::count_launch(); }
    }
    const int64_t nch = L.ch_end - L.ch_begin;
    if (nch > 0) {
      int maxb = 0;
      for (int64_t c = L.ch_begin; c < L.ch_end; ++c) maxb = std::max(maxb, S.f_nb[S.child_list[c]]);
      const int gy = std::max(1, std::min(maxb, std::max(1, (int)(ctx->num_sms * 32 / nch))));
      dim3 grid((unsigned)nch, (unsigned)gy);
      { k_extend_add<T><<<grid, 256, 0, ctx->stream>>>(F, M->d.child_list, L.ch_begin, M->d.f_nb, M->d.f_off,
                                                     M->d.f_parent, M->d.f_level, M->d.ea_ptr, M->d.ea_pos, d_ln, d_le); gbmhd::count_launch(); }
    }
    MF_CUDA(cudaGetLastError());
    // Blocked in-place Gauss-Jordan over the eliminated pivots, by panels of PW pivots.
    // Inside a panel, each 64-pivot block is eliminated from the panel's columns only (its
    // inverse from k_pivot_inverse*, three small GEMMs); the rest of the front then takes the
    // whole panel's elimination in one rank-PW update: M[:, rest] += Nz·R, M[P, rest] = N[P]·R
    // (R = the panel rows before, N = the panel columns after).  Every pivot block still
    // updates the whole front before the next panel, so F12, F21 and S come from the same
    // progressive elimination as F11⁻¹.  (Forming them afterwards from the FP32 F11⁻¹ with
    // three large GEMMs multiplies the inverse's rounding by κ(F11): at Ha = 500 that tripled
    // the FGMRES iterations.)  One pass over a front per PW pivots instead of per 64 halves
    // the HBM traffic of these memory-bound updates.
    for (int p = 0; p < E; p += PW) {
      const int pw = std::min(PW, E - p);
      dim3 gr((unsigned)((n + 1) / 2), (unsigned)cnt);
      { k_panel_rows<T><<<gr, 256, 0, ctx->stream>>>(F, L.off, n, p, pw, R); gbmhd::count_launch(); }
      for (int k = p; k < p + pw; k += NB) {
        const int kb = std::min(NB, p + pw - k);
        if constexpr (sizeof(T) == 4)
          {
            if (cnt >= 2 * ctx->num_sms) k_pivot_inverse_df_smem<<<cnt, 256, 0, ctx->stream>>>(F, L.off, n, k, kb, P, M->d_err);
            else if (cnt >= ctx->num_sms) k_pivot_inverse_df<4><<<cnt, NB * 4, 0, ctx->stream>>>(F, L.off, n, k, kb, P, M->d_err);
            else k_pivot_inverse_df<16><<<cnt, NB * 16, 0, ctx->stream>>>(F, L.off, n, k, kb, P, M->d_err);
            gbmhd::count_launch();
          }
        else
          { k_pivot_inverse<T><<<cnt, 256, 0, ctx->stream>>>(F, L.off, n, k, kb, P, M->d_err); gbmhd::count_launch(); }
        dim3 gc((unsigned)std::max(kb, (pw + 3) / 4), (unsigned)cnt);
        { k_gj_copy<T><<<gc, 256, 0, ctx->stream>>>(F, L.off, n, k, kb, p, pw, C, Tb); gbmhd::count_launch(); }
        MF_CUDA(cudaGetLastError());
        // T2 = P · Tb  (kb x pw)
        gbmhd::count_gemm(); MF_BLAS(gemm_sb<T>(M, CUBLAS_OP_N, CUBLAS_OP_N, kb, pw, kb, &one, P, NB, (long long)NB * NB, Tb,
                           NB, (long long)NB * n, &zero, T2, NB, (long long)NB * n, cnt));
        // M[:, panel] -= C · T2   (n x pw)
        gbmhd::count_gemm(); MF_BLAS(gemm_sb<T>(M, CUBLAS_OP_N, CUBLAS_OP_N, n, pw, kb, &mone, C, n, (long long)n * NB, T2,
                           NB, (long long)NB * n, &one, F + L.off + (int64_t)p * n, n, (long long)n * n, cnt));
        // M[:, K] = −C · P  (n x kb)
        gbmhd::count_gemm(); MF_BLAS(gemm_sb<T>(M, CUBLAS_OP_N, CUBLAS_OP_N, n, kb, kb, &mone, C, n, (long long)n * NB, P,
                           NB, (long long)NB * NB, &zero, F + L.off + (int64_t)k * n, n, (long long)n * n, cnt));
        { k_gj_fix<T><<<gc, 256, 0, ctx->stream>>>(F, L.off, n, k, kb, p, pw, T2, P); gbmhd::count_launch(); }
        MF_CUDA(cudaGetLastError());
      }
      dim3 gn((unsigned)pw, (unsigned)cnt);
      { k_panel_cols<T><<<gn, 256, 0, ctx->stream>>>(F, L.off, n, p, pw, Nz); gbmhd::count_launch(); }
      MF_CUDA(cudaGetLastError());
      // rest = columns [0, p) and [p + pw, n)
      for (int side = 0; side < 2; ++side) {
        const int c0 = side == 0 ? 0 : p + pw, cw = side == 0 ? p : n - (p + pw);
        if (cw <= 0) continue;
        // M[:, rest] += Nz · R[:, rest]   (n x cw, inner pw)
        gbmhd::count_gemm(); MF_BLAS(gemm_sb<T>(M, CUBLAS_OP_N, CUBLAS_OP_N, n, cw, pw, &one, Nz, n, (long long)n * PW,
                           R + (int64_t)c0 * PW, PW, (long long)PW * n, &one, F + L.off + (int64_t)c0 * n, n,
                           (long long)n * n, cnt));
        // M[P, rest] = N[P, :] · R[:, rest]   (pw x cw; N[P, :] = the panel's pivot-block inverse)
        gbmhd::count_gemm(); MF_BLAS(gemm_sb<T>(M, CUBLAS_OP_N, CUBLAS_OP_N, pw, cw, pw, &one,
                           F + L.off + p + (int64_t)p * n, n, (long long)n * n, R + (int64_t)c0 * PW, PW,
                           (long long)PW * n, &zero, F + L.off + p + (int64_t)c0 * n, n, (long long)n * n, cnt));
      }
    }
  }
  MF_CUDA(cudaFreeAsync(d_ln, ctx->stream));
  MF_CUDA(cudaFreeAsync(d_le, ctx->stream));
  int32_t herr = 0;
  MF_CUDA(cudaMemcpyAsync(&herr, M->d_err, sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
  MF_CUDA(cudaStreamSynchronize(ctx->stream));
  if (herr) {
    ctx->err = "multifrontal: singular pivot block in the (u,j) factorization";
    return -3;
  }
  M->precision = sizeof(T) == 8 ? GBMHD_FP64 : GBMHD_MIXED;
  if (sizeof(T) == 4 && M->maps_base != M->F) build_sweep_maps(M);
  return 0;
}

// Ruiz equilibration of the Jacobian values (3 sweeps) into M->d_dr / M->d_dc and the scaled
// copy M->d_sval.
template <typename V>
static int equilibrate(gbmhd_ctx* ctx, MFNumeric* M, const V* val) {
  const int64_t n = ctx->ndofs, nnz = ctx->nnz;
  if (!M->d_dr) {
    MF_CUDA(cudaMalloc(&M->d_dr, sizeof(double) * std::max<int64_t>(n, 1)));
    MF_CUDA(cudaMalloc(&M->d_dc, sizeof(double) * std::max<int64_t>(n, 1)));
  }
  if (M->sval_bytes < sizeof(V) * (size_t)nnz) {
    if (M->d_sval) cudaFree(M->d_sval);
    MF_CUDA(cudaMalloc(&M->d_sval, sizeof(V) * std::max<int64_t>(nnz, 1)));
    M->sval_bytes = sizeof(V) * (size_t)nnz;
  }
  double* rmax = nullptr;
  unsigned long long* cmax = nullptr;
  MF_CUDA(cudaMallocAsync(&rmax, sizeof(double) * std::max<int64_t>(n, 1), ctx->stream));
  MF_CUDA(cudaMallocAsync(&cmax, sizeof(unsigned long long) * std::max<int64_t>(n, 1), ctx->stream));
  const unsigned gw = (unsigned)std::max<int64_t>(1, std::min<int64_t>((n * 32 + 255) / 256, (int64_t)ctx->num_sms * 16));
  const unsigned gv = (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)ctx->num_sms * 8));
  { k_fill<<<gv, 256, 0, ctx->stream>>>(n, 1.0, M->d_dr); gbmhd::count_launch(); }
  { k_fill<<<gv, 256, 0, ctx->stream>>>(n, 1.0, M->d_dc); gbmhd::count_launch(); }
  for (int it = 0; it < 3; ++it) {
    MF_CUDA(cudaMemsetAsync(cmax, 0, sizeof(unsigned long long) * n, ctx->stream));
    { k_ruiz_max<V><<<gw, 256, 0, ctx->stream>>>(n, ctx->d_rowptr, ctx->d_col, val, M->d_dr, M->d_dc, rmax, cmax); gbmhd::count_launch(); }
    { k_ruiz_update<<<gv, 256, 0, ctx->stream>>>(n, rmax, cmax, M->d_dr, M->d_dc); gbmhd::count_launch(); }
  }
  { k_scale_vals<V><<<gw, 256, 0, ctx->stream>>>(n, ctx->d_rowptr, ctx->d_col, val, M->d_dr, M->d_dc, reinterpret_cast<V*>(M->d_sval)); gbmhd::count_launch(); }
  MF_CUDA(cudaGetLastError());
  MF_CUDA(cudaFreeAsync(rmax, ctx->stream));
  MF_CUDA(cudaFreeAsync(cmax, ctx->stream));
  return 0;
}

template <typename T, typename V>
static int factor_scaled(gbmhd_ctx* ctx, MFNumeric* M, const V* val, const double* d_reg) {
  M->scaled = M->S.monolithic;
  if (M->scaled) {
    int rc = equilibrate<V>(ctx, M, val);
    if (rc) return rc;
    val = reinterpret_cast<const V*>(M->d_sval);
  }
  return factor_impl<T, V>(ctx, M, val, d_reg);
}

int mf_factor(gbmhd_ctx* ctx, MFNumeric* M, int precision, int values, const double* d_reg) {
  if (values == GBMHD_MIXED && !ctx->d_val32) { ctx->err = "multifrontal: no FP32 Jacobian assembled"; return -1; }
  // new factors: a sweep timeout of an earlier solve no longer applies
  MF_CUDA(cudaStreamSynchronize(ctx->stream));
  MF_CUDA(cudaMemset(M->d_sweep_err, 0, sizeof(int32_t)));
  *M->h_sweep_err = 0;
  if (values == GBMHD_FP64 && !ctx->d_val64) { ctx->err = "multifrontal: no FP64 Jacobian assembled"; return -1; }
  if (precision == GBMHD_MIXED) {
    if (values == GBMHD_MIXED) return factor_scaled<float, float>(ctx, M, ctx->d_val32, d_reg);
    return factor_scaled<float, double>(ctx, M, ctx->d_val64, d_reg);
  }
  if (values != GBMHD_FP64) { ctx->err = "multifrontal: FP64 factors need the FP64 Jacobian"; return -1; }
  return factor_scaled<double, double>(ctx, M, ctx->d_val64, d_reg);
}

// Column chunk of the chunked sweeps: wide enough that the partial-sum atomics stay a
// small fraction of the factor reads, narrow enough that a level with few fronts still
// launches about two waves of CTAs.
static int sweep_cols(const gbmhd_ctx* ctx, int64_t rows, int64_t ncols, int64_t fronts, int rows_per_cta) {
  const int64_t per_chunk = std::max<int64_t>(1, (rows + rows_per_cta - 1) / rows_per_cta) * std::max<int64_t>(1, fronts);
  const int64_t want = (int64_t)ctx->num_sms * 32;  // 2 waves of 16 resident 128-thread CTAs
  const int64_t chunks = std::max<int64_t>(1, (want + per_chunk - 1) / per_chunk);
  int64_t cols = (ncols + chunks - 1) / chunks;
  cols = ((cols + 31) / 32) * 32;
  return (int)std::max<int64_t>(64, std::min<int64_t>(cols, 1024));
}

// Columns per warp of the transposed FP32 sweeps: 4 while a level still gives at least two
// 256-thread CTAs per SM, else fewer (levels with few, large fronts).  FP64 factors: 1.
#define GT_NC(k) (sizeof(T) == 4 ? (k) : 1)
template <typename T>
static int gemv_t_cols(const gbmhd_ctx* ctx, int cols, int cnt) {
  if (sizeof(T) != 4) return 1;
  const int64_t want = 2LL * ctx->num_sms;
  for (int nc = 4; nc > 1; nc /= 2)
    if ((int64_t)cnt * ((cols + 8 * nc - 1) / (8 * nc)) >= want) return nc;
  return 1;
}

template <typename T>
static int solve_impl(gbmhd_ctx* ctx, MFNumeric* M, double* b, double* x, bool tr) {
  using V = typename SweepAcc<T>::V;
  const int rows_cta = SW_THREADS * RowVec<T>::R;
  const MFSymbolic& S = M->S;
  const T* F = reinterpret_cast<const T*>(M->F);
  // the TMA backward sweeps add their partial sums into x directly: zero x at the dofs this
  // factorization eliminates (the others, e.g. the p and φ blocks of the block-triangular
  // preconditioner, hold the caller's values)
  if (!tr && sizeof(T) == 4 && !S.elim.empty()) {
    const int64_t ne_all = (int64_t)S.elim.size();
    const unsigned gz = (unsigned)std::max<int64_t>(1, std::min<int64_t>((ne_all + 255) / 256, (int64_t)ctx->num_sms * 8));
    { k_zero_at<<<gz, 256, 0, ctx->stream>>>(M->d.elim, ne_all, x); gbmhd::count_launch(); }
  }
  for (size_t l = 0; l < S.levels.size(); ++l) {
    const MFLevel& L = S.levels[l];
    const int cnt = (int)L.count;
    const bool tma = !tr && sizeof(T) == 4 && M->map_ok[l];
    if (!(tma && L.B > 0))  // the TMA forward sweep gathers t itself
      { k_fwd_gather<<<cnt, 256, 0, ctx->stream>>>(b, M->tsave, M->tsave_off, M->d.elim, M->d.elim_ptr, M->d.f_ne, L.first, L.E); gbmhd::count_launch(); }
    if (L.B > 0) {
      if (tma) {
        const int rows = M->map_rows[2 * l];
        const int cw = tma_cols(ctx, L.B, rows, L.E, cnt);
        dim3 g((unsigned)((L.B + rows - 1) / rows), (unsigned)((L.E + cw - 1) / cw), (unsigned)cnt);
        const size_t sm = (size_t)TS_STAGES * TS_COLS * rows * sizeof(float) + sizeof(float2) * cw;
        MF_CUDA(cudaFuncSetAttribute(k_sweep_tma<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        { k_sweep_tma<true><<<g, rows / 2, sm, ctx->stream>>>(M->maps[2 * l], L.first, L.E, rows, cw, 0, b, x, M->tsave, M->tsave_off, M->d.bnd, M->d.bnd_ptr, M->d.elim, M->d.elim_ptr, M->d.f_ne, M->d.f_nb, M->d_sweep_err, M->wait_limit); gbmhd::count_launch(); }
      } else if (!tr) {
        const int cols = sweep_cols(ctx, L.B, L.E, cnt, rows_cta);
        dim3 g((unsigned)((L.B + rows_cta - 1) / rows_cta), (unsigned)((L.E + cols - 1) / cols), (unsigned)cnt);
        { k_fwd_chunk<T><<<g, SW_THREADS, sizeof(V) * cols, ctx->stream>>>(F, M->d.f_off, b, M->tsave, M->tsave_off, M->d.bnd, M->d.bnd_ptr, M->d.f_nb, M->d.f_ne, L.first, L.n, L.E, cols); gbmhd::count_launch(); }
      } else {
        const size_t sm = sizeof(T) == 4 ? 0 : sizeof(V) * L.E;
        const int nc = gemv_t_cols<T>(ctx, L.B, cnt);
        auto kf = nc == 4 ? k_fwd_gemv_t<T, GT_NC(4)> : nc == 2 ? k_fwd_gemv_t<T, GT_NC(2)> : k_fwd_gemv_t<T, 1>;
        MF_CUDA(cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)std::max<size_t>(sm, 1)));
        if (sizeof(T) == 4)
          { k_pack_vec<<<cnt, 256, 0, ctx->stream>>>(M->tsave, M->tsave_off, nullptr, M->d.bnd, M->d.bnd_ptr, M->d.f_ne, M->d.f_nb, L.first, L.n, L.E, M->vpk); gbmhd::count_launch(); }
        dim3 g((unsigned)((L.B + 8 * nc - 1) / (8 * nc)), (unsigned)cnt);
        { kf<<<g, 256, sm, ctx->stream>>>(F, M->d.f_off, b, M->tsave, M->tsave_off, M->d.bnd, M->d.bnd_ptr, M->d.f_nb, M->d.f_ne, L.first, L.n, L.E, M->vpk); gbmhd::count_launch(); }
      }
    }
    MF_CUDA(cudaGetLastError());
  }
  for (int l = (int)S.levels.size() - 1; l >= 0; --l) {
    const MFLevel& L = S.levels[l];
    const int cnt = (int)L.count;
    if (!tr && sizeof(T) == 4 && M->map_ok[l]) {
      const int rows = M->map_rows[2 * l + 1];
      const int cw = tma_cols(ctx, L.E, rows, L.n, cnt);
      const int ca = (L.E + cw - 1) / cw, cb = (L.B + cw - 1) / cw;
      dim3 g((unsigned)((L.E + rows - 1) / rows), (unsigned)(ca + cb), (unsigned)cnt);
      const size_t sm = (size_t)TS_STAGES * TS_COLS * rows * sizeof(float) + sizeof(float2) * cw;
      MF_CUDA(cudaFuncSetAttribute(k_sweep_tma<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
      { k_sweep_tma<false><<<g, rows / 2, sm, ctx->stream>>>(M->maps[2 * l + 1], L.first, L.E, rows, cw, ca, b, x, M->tsave, M->tsave_off, M->d.bnd, M->d.bnd_ptr, M->d.elim, M->d.elim_ptr, M->d.f_ne, M->d.f_nb, M->d_sweep_err, M->wait_limit); gbmhd::count_launch(); }
    } else if (!tr) {
      const int cols = sweep_cols(ctx, L.E, L.n, cnt, rows_cta);
      dim3 g((unsigned)((L.E + rows_cta - 1) / rows_cta), (unsigned)((L.n + cols - 1) / cols), (unsigned)cnt);
      { k_bwd_chunk<T><<<g, SW_THREADS, sizeof(V) * cols, ctx->stream>>>(F, M->d.f_off, x, M->tsave, M->tsave_off, M->d.bnd, M->d.bnd_ptr, M->d.f_ne, M->d.f_nb, M->ybuf, L.first, L.n, L.E, cols); gbmhd::count_launch(); }
      { k_bwd_scatter<<<cnt, 256, 0, ctx->stream>>>(x, M->ybuf, M->tsave_off, M->d.elim, M->d.elim_ptr, M->d.f_ne, L.first); gbmhd::count_launch(); }
    } else {
      const size_t sm = sizeof(T) == 4 ? 0 : sizeof(V) * L.n;
      const int nc = gemv_t_cols<T>(ctx, L.E, cnt);
      auto kb = nc == 4 ? k_bwd_gemv_t<T, GT_NC(4)> : nc == 2 ? k_bwd_gemv_t<T, GT_NC(2)> : k_bwd_gemv_t<T, 1>;
      MF_CUDA(cudaFuncSetAttribute(kb, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)std::max<size_t>(sm, 1)));
      if (sizeof(T) == 4)
        { k_pack_vec<<<cnt, 256, 0, ctx->stream>>>(M->tsave, M->tsave_off, x, M->d.bnd, M->d.bnd_ptr, M->d.f_ne, M->d.f_nb, L.first, L.n, L.E, M->vpk); gbmhd::count_launch(); }
      dim3 g((unsigned)((L.E + 8 * nc - 1) / (8 * nc)), (unsigned)cnt);
      { kb<<<g, 256, sm, ctx->stream>>>(F, M->d.f_off, x, M->tsave, M->tsave_off, M->d.elim, M->d.elim_ptr, M->d.bnd, M->d.bnd_ptr, M->d.f_ne, M->d.f_nb, L.first, L.n, L.E, M->vpk); gbmhd::count_launch(); }
    }
    MF_CUDA(cudaGetLastError());
  }
  return 0;
}

int mf_solve(gbmhd_ctx* ctx, MFNumeric* M, double* d_b, double* d_x, bool transpose) {
  if (M->precision != GBMHD_MIXED && M->precision != GBMHD_FP64) {
    ctx->err = "multifrontal: not factored";
    return -1;
  }
  if (*M->h_sweep_err) {  // set by an earlier solve whose copies arrived; this one cannot be trusted
    ctx->err = "multifrontal: a solve sweep's TMA wait timed out";
    return -3;
  }
  harvest_sweep_time(M, false);
  const bool timed = !M->ev_pending && M->ev0 && M->ev1;
  if (timed) MF_CUDA(cudaEventRecord(M->ev0, ctx->stream));
  const int64_t nd = ctx->ndofs;
  const unsigned gv = (unsigned)std::max<int64_t>(1, std::min<int64_t>((nd + 255) / 256, (int64_t)ctx->num_sms * 8));
  // (Dr A Dc)⁻¹ = Dc⁻¹ A⁻¹ Dr⁻¹, so A⁻¹ b = Dc (Dr A Dc)⁻¹ Dr b and A⁻ᵀ b = Dr (Dr A Dc)⁻ᵀ Dc b
  if (M->scaled) { k_scale_vec<<<gv, 256, 0, ctx->stream>>>(nd, transpose ? M->d_dc : M->d_dr, d_b); gbmhd::count_launch(); }
  const int rc = M->precision == GBMHD_MIXED ? solve_impl<float>(ctx, M, d_b, d_x, transpose)
                                             : solve_impl<double>(ctx, M, d_b, d_x, transpose);
  if (rc) return rc;
  if (M->scaled) { k_scale_vec<<<gv, 256, 0, ctx->stream>>>(nd, transpose ? M->d_dr : M->d_dc, d_x); gbmhd::count_launch(); }
  if (timed) {
    MF_CUDA(cudaEventRecord(M->ev1, ctx->stream));
    M->ev_pending = true;
  }
  MF_CUDA(cudaMemcpyAsync(M->h_sweep_err, M->d_sweep_err, sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
  return 0;
}

int mf_check_sweeps(gbmhd_ctx* ctx, MFNumeric* M) {
  MF_CUDA(cudaStreamSynchronize(ctx->stream));
  if (*M->h_sweep_err) {
    ctx->err = "multifrontal: a solve sweep's TMA wait timed out";
    return -3;
  }
  return 0;
}
