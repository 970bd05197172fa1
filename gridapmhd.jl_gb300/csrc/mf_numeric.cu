// Numeric multifrontal factorization and solves of the (u,j) block (see mf.h).
#include <cublas_v2.h>

#include <cstdlib>
#include <cstring>

#include "mf.h"

using namespace gbmhd;

namespace {

constexpr int NB = 64;  // Gauss-Jordan pivot block

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
  size_t work_bytes = 0;
  double* tsave = nullptr;     // forward-sweep values of the eliminated dofs
  double* ybuf = nullptr;      // backward-sweep accumulators (kept zero between solves)
  int64_t* tsave_off = nullptr;  // per front
  int64_t tsave_len = 0;
  int32_t* d_err = nullptr;    // device-side status (singular pivot block)
  int fp32_gemm_mode = 0;      // 0: BF16x9 emulated FP32, 1: plain FP32
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
  // the solve sweeps stage a front's vector segment in shared memory
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
  const char* mode = std::getenv("GBMHD_FP32_GEMM");
  M->fp32_gemm_mode = (mode && std::strcmp(mode, "fp32") == 0) ? 1 : 0;
  return 0;
}

void mf_destroy(MFNumeric* M) {
  if (!M) return;
  void* ptrs[] = {M->d.f_ne, M->d.f_nb, M->d.f_off, M->d.elim_ptr, M->d.bnd_ptr, M->d.elim, M->d.bnd,
                  M->d.ah_src, M->d.ah_dst, M->d.child_list, M->d.ea_ptr, M->d.ea_pos, M->d.f_parent,
                  M->d.f_level, M->d.reg_dst, M->d.reg_dof, M->F, M->Pbuf, M->Cbuf, M->Tbuf, M->T2buf, M->tsave, M->ybuf, M->tsave_off, M->d_err};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (M->blas) cublasDestroy(M->blas);
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
template <typename T>
__global__ void k_reg_add(T* F, const int64_t* __restrict__ dst, const int32_t* __restrict__ dof,
                          const double* __restrict__ reg, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    F[dst[i]] += (T)reg[dof[i]];
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

// Inverse of the kb x kb pivot block of every front (Gauss-Jordan with partial
// pivoting inside the block), computed in FP64 whatever the storage type and then
// rounded to it.  P[f] (NB x NB, column-major, ld NB).
template <typename T>
__global__ void __launch_bounds__(256) k_pivot_inverse(const T* __restrict__ F, int64_t off, int n, int k, int kb,
                                                       T* __restrict__ P, int32_t* err) {
  extern __shared__ __align__(16) unsigned char sm_raw[];
  double* A = reinterpret_cast<double*>(sm_raw);  // kb x 2kb, row-major [i][j]
  __shared__ int piv_row;
  __shared__ double piv_abs[256];
  __shared__ int piv_idx[256];
  const int64_t f = blockIdx.x;
  const T* M = F + off + f * (int64_t)n * n;
  const int w = 2 * kb;
  for (int idx = threadIdx.x; idx < kb * w; idx += blockDim.x) {
    const int i = idx / w, j = idx % w;
    A[idx] = j < kb ? (double)M[(k + i) + (int64_t)(k + j) * n] : ((j - kb) == i ? 1.0 : 0.0);
  }
  __syncthreads();
  for (int c = 0; c < kb; ++c) {
    // pivot search in column c, rows c..kb-1
    double best = -1.0;
    int bi = c;
    for (int i = c + threadIdx.x; i < kb; i += blockDim.x) {
      const double a = fabs((double)A[i * w + c]);
      if (a > best) { best = a; bi = i; }
    }
    piv_abs[threadIdx.x] = best;
    piv_idx[threadIdx.x] = bi;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s && piv_abs[threadIdx.x + s] > piv_abs[threadIdx.x]) {
        piv_abs[threadIdx.x] = piv_abs[threadIdx.x + s];
        piv_idx[threadIdx.x] = piv_idx[threadIdx.x + s];
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      piv_row = piv_idx[0];
      if (!(piv_abs[0] > 0.0)) atomicExch(err, 1);
    }
    __syncthreads();
    const int pr = piv_row;
    if (pr != c)
      for (int j = threadIdx.x; j < w; j += blockDim.x) {
        const double t = A[c * w + j];
        A[c * w + j] = A[pr * w + j];
        A[pr * w + j] = t;
      }
    __syncthreads();
    const double d = A[c * w + c];
    const double inv = d != 0.0 ? 1.0 / d : 0.0;
    __syncthreads();
    for (int j = threadIdx.x; j < w; j += blockDim.x) A[c * w + j] *= inv;
    __syncthreads();
    for (int idx = threadIdx.x; idx < kb * w; idx += blockDim.x) {
      const int i = idx / w, j = idx % w;
      if (i != c) {
        const double m = A[i * w + c];
        if (m != 0.0 && j != c) A[idx] -= m * A[c * w + j];
      }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kb; i += blockDim.x)
      if (i != c) A[i * w + c] = 0.0;
    __syncthreads();
  }
  T* Pf = P + f * (int64_t)NB * NB;
  for (int idx = threadIdx.x; idx < NB * NB; idx += blockDim.x) {
    const int i = idx % NB, j = idx / NB;  // column-major
    Pf[idx] = (i < kb && j < kb) ? (T)A[i * w + kb + j] : (T)0;
  }
}

// C = M[:, K] with the K rows zeroed; Tb = M[K, :]  (both per front).
template <typename T>
__global__ void k_gj_copy(const T* __restrict__ F, int64_t off, int n, int k, int kb, T* __restrict__ C,
                          T* __restrict__ Tb) {
  const int64_t f = blockIdx.y;
  const T* M = F + off + f * (int64_t)n * n;
  T* Cf = C + f * (int64_t)n * NB;
  T* Tf = Tb + f * (int64_t)NB * n;
  const int64_t tot = (int64_t)n * kb;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < tot; idx += (int64_t)gridDim.x * blockDim.x) {
    // column block: idx = i + j*n
    const int i = (int)(idx % n), j = (int)(idx / n);
    const T v = M[i + (int64_t)(k + j) * n];
    Cf[i + (int64_t)j * n] = (i >= k && i < k + kb) ? (T)0 : v;
    // row block: idx = r + c*kb
    const int r = (int)(idx % kb), c = (int)(idx / kb);
    Tf[r + (int64_t)c * NB] = M[(k + r) + (int64_t)c * n];
  }
}

// M[K, j] = T2[:, j] for j outside K; M[K, K] = P.
template <typename T>
__global__ void k_gj_fix(T* __restrict__ F, int64_t off, int n, int k, int kb, const T* __restrict__ T2,
                         const T* __restrict__ P) {
  const int64_t f = blockIdx.y;
  T* M = F + off + f * (int64_t)n * n;
  const T* T2f = T2 + f * (int64_t)NB * n;
  const T* Pf = P + f * (int64_t)NB * NB;
  const int64_t tot = (int64_t)n * kb;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < tot; idx += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(idx % kb), c = (int)(idx / kb);
    const bool inK = c >= k && c < k + kb;
    M[(k + r) + (int64_t)c * n] = inK ? Pf[r + (int64_t)(c - k) * NB] : T2f[r + (int64_t)c * NB];
  }
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
  __device__ void warp_reduce() {
    for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
  }
  __device__ double value() const { return a; }
};

// Transposed sweeps (adjoint solves), one warp per column: each dot product runs down a
// contiguous column of the column-major front.
// forward, transposed: b[bnd_j] −= Σ_{i<ne} TR[i, j] t_i   (TR = rows 0..E of column E+j)
template <typename T>
__global__ void __launch_bounds__(256) k_fwd_gemv_t(const T* __restrict__ F, const int64_t* __restrict__ f_off,
                                                    double* __restrict__ b, const double* __restrict__ tsave,
                                                    const int64_t* __restrict__ toff, const int32_t* __restrict__ bnd,
                                                    const int64_t* __restrict__ bnd_ptr, const int32_t* __restrict__ f_nb,
                                                    const int32_t* __restrict__ f_ne, int64_t first, int n, int E) {
  using V = typename SweepAcc<T>::V;
  extern __shared__ __align__(16) unsigned char sm_raw[];
  V* ts = reinterpret_cast<V*>(sm_raw);
  const int64_t f = first + blockIdx.y;
  const int nb = f_nb[f], ne = f_ne[f];
  const double* t = tsave + toff[f];
  for (int i = threadIdx.x; i < ne; i += blockDim.x) ts[i] = SweepAcc<T>::pack(t[i]);
  __syncthreads();
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int j = blockIdx.x * (blockDim.x / 32) + warp;
  if (j >= nb) return;
  const T* colj = F + f_off[f] + (int64_t)(E + j) * n;
  SweepAcc<T> acc;
  for (int i = lane; i < ne; i += 32) acc.add(colj[i], ts[i]);
  acc.warp_reduce();
  if (lane == 0) atomicAdd(&b[bnd[bnd_ptr[f] + j]], -acc.value());
}

// backward, transposed: x[elim_i] = Σ_{c<ne} TL[c, i] t_c + Σ_{j<nb} BL[j, i] x_B[j]
// (column i of the front: rows 0..E are TL, rows E.. are BL)
template <typename T>
__global__ void __launch_bounds__(256) k_bwd_gemv_t(const T* __restrict__ F, const int64_t* __restrict__ f_off,
                                                    double* __restrict__ x, const double* __restrict__ tsave,
                                                    const int64_t* __restrict__ toff, const int32_t* __restrict__ elim,
                                                    const int64_t* __restrict__ elim_ptr, const int32_t* __restrict__ bnd,
                                                    const int64_t* __restrict__ bnd_ptr, const int32_t* __restrict__ f_ne,
                                                    const int32_t* __restrict__ f_nb, int64_t first, int n, int E) {
  using V = typename SweepAcc<T>::V;
  extern __shared__ __align__(16) unsigned char sm_raw[];
  V* vs = reinterpret_cast<V*>(sm_raw);  // [E] t, then [n-E] x_B
  const int64_t f = first + blockIdx.y;
  const int ne = f_ne[f], nb = f_nb[f];
  const double* t = tsave + toff[f];
  const int32_t* bd = bnd + bnd_ptr[f];
  for (int i = threadIdx.x; i < ne; i += blockDim.x) vs[i] = SweepAcc<T>::pack(t[i]);
  for (int j = threadIdx.x; j < nb; j += blockDim.x) vs[E + j] = SweepAcc<T>::pack(x[bd[j]]);
  __syncthreads();
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int i = blockIdx.x * (blockDim.x / 32) + warp;
  if (i >= ne) return;
  const T* coli = F + f_off[f] + (int64_t)i * n;
  SweepAcc<T> acc;
  for (int c = lane; c < ne; c += 32) acc.add(coli[c], vs[c]);
  for (int j = lane; j < nb; j += 32) acc.add(coli[E + j], vs[E + j]);
  acc.warp_reduce();
  if (lane == 0) x[elim[elim_ptr[f] + i]] = acc.value();
}

// Chunked sweeps: grid (row tiles, column chunks, fronts); each thread owns one row of its
// tile and reduces one chunk of `cols` columns, staged in shared memory; partial sums are
// added atomically.  Row accesses are coalesced (column-major fronts).  The chunk width is
// chosen per level so that levels with few fronts still fill the GPU.
constexpr int SW_ROWS = 128;  // rows per CTA (one per thread)

// forward: b[bnd_j] += Σ_{i<ne} M[E+j, i] t_i
template <typename T>
__global__ void __launch_bounds__(SW_ROWS) k_fwd_chunk(const T* __restrict__ F, const int64_t* __restrict__ f_off,
                                                       double* __restrict__ b, const double* __restrict__ tsave,
                                                       const int64_t* __restrict__ toff, const int32_t* __restrict__ bnd,
                                                       const int64_t* __restrict__ bnd_ptr, const int32_t* __restrict__ f_nb,
                                                       const int32_t* __restrict__ f_ne, int64_t first, int n, int E,
                                                       int cols) {
  using V = typename SweepAcc<T>::V;
  extern __shared__ __align__(16) unsigned char sm_raw[];
  V* ts = reinterpret_cast<V*>(sm_raw);
  const int64_t f = first + blockIdx.z;
  const int nb = f_nb[f];
  const int j = blockIdx.x * SW_ROWS + threadIdx.x;
  const int ne = f_ne[f];  // columns [ne, E) are padding
  const int c0 = blockIdx.y * cols, c1 = min(ne, c0 + cols);
  if (blockIdx.x * SW_ROWS >= nb || c0 >= ne) return;
  const double* t = tsave + toff[f];
  for (int c = c0 + threadIdx.x; c < c1; c += blockDim.x) ts[c - c0] = SweepAcc<T>::pack(t[c]);
  __syncthreads();
  if (j >= nb) return;
  const T* M = F + f_off[f] + E + j;
  SweepAcc<T> acc;
#pragma unroll 8
  for (int c = c0; c < c1; ++c) acc.add(M[(int64_t)c * n], ts[c - c0]);
  atomicAdd(&b[bnd[bnd_ptr[f] + j]], acc.value());
}

// backward: y_i = Σ_c M[i, c] v_c with v = [t ; −x_B], accumulated into ybuf (then scattered)
template <typename T>
__global__ void __launch_bounds__(SW_ROWS) k_bwd_chunk(const T* __restrict__ F, const int64_t* __restrict__ f_off,
                                                       const double* __restrict__ x, const double* __restrict__ tsave,
                                                       const int64_t* __restrict__ toff, const int32_t* __restrict__ bnd,
                                                       const int64_t* __restrict__ bnd_ptr, const int32_t* __restrict__ f_ne,
                                                       const int32_t* __restrict__ f_nb, double* __restrict__ ybuf,
                                                       int64_t first, int n, int E, int cols) {
  using V = typename SweepAcc<T>::V;
  extern __shared__ __align__(16) unsigned char sm_raw[];
  V* vs = reinterpret_cast<V*>(sm_raw);
  const int64_t f = first + blockIdx.z;
  const int ne = f_ne[f], nb = f_nb[f];
  const int i = blockIdx.x * SW_ROWS + threadIdx.x;
  // virtual columns v in [0, ne + nb): v < ne -> column v, else column E + (v − ne)
  const int c0 = blockIdx.y * cols, c1 = min(ne + nb, c0 + cols);
  if (blockIdx.x * SW_ROWS >= ne || c0 >= ne + nb) return;
  const double* t = tsave + toff[f];
  const int32_t* bd = bnd + bnd_ptr[f];
  for (int v = c0 + threadIdx.x; v < c1; v += blockDim.x)
    vs[v - c0] = SweepAcc<T>::pack(v < ne ? t[v] : -x[bd[v - ne]]);
  __syncthreads();
  if (i >= ne) return;
  const T* M = F + f_off[f] + i;
  SweepAcc<T> acc;
  const int va = min(c1, ne);
#pragma unroll 8
  for (int v = c0; v < va; ++v) acc.add(M[(int64_t)v * n], vs[v - c0]);
  const T* MB = M + (int64_t)(E - ne) * n;
#pragma unroll 8
  for (int v = max(c0, ne); v < c1; ++v) acc.add(MB[(int64_t)v * n], vs[v - c0]);
  atomicAdd(&ybuf[toff[f] + i], acc.value());
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
  size_t wmax = 0;
  for (const MFLevel& L : S.levels) wmax = std::max(wmax, (size_t)L.count * L.n * NB);
  size_t pbytes = 0;
  for (const MFLevel& L : S.levels) pbytes = std::max(pbytes, (size_t)L.count * NB * NB);
  const size_t need = sizeof(T) * (3 * wmax + pbytes);
  if (M->work_bytes < need) {
    for (void* p : {M->Pbuf, M->Cbuf, M->Tbuf, M->T2buf})
      if (p) cudaFree(p);
    MF_CUDA(cudaMalloc(&M->Pbuf, sizeof(T) * std::max<size_t>(pbytes, 1)));
    MF_CUDA(cudaMalloc(&M->Cbuf, sizeof(T) * std::max<size_t>(wmax, 1)));
    MF_CUDA(cudaMalloc(&M->Tbuf, sizeof(T) * std::max<size_t>(wmax, 1)));
    MF_CUDA(cudaMalloc(&M->T2buf, sizeof(T) * std::max<size_t>(wmax, 1)));
    M->work_bytes = need;
  }
  T* F = reinterpret_cast<T*>(M->F);
  T* P = reinterpret_cast<T*>(M->Pbuf);
  T* C = reinterpret_cast<T*>(M->Cbuf);
  T* Tb = reinterpret_cast<T*>(M->Tbuf);
  T* T2 = reinterpret_cast<T*>(M->T2buf);
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
      { k_reg_add<T><<<(unsigned)std::min<int64_t>((nr + 255) / 256, 4096), 256, 0, ctx->stream>>>(F, M->d.reg_dst, M->d.reg_dof, d_reg, nr); gbmhd::count_launch(); }
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
    for (int k = 0; k < E; k += NB) {
      const int kb = std::min(NB, E - k);
      const size_t sm = sizeof(double) * (size_t)kb * 2 * kb;
      auto kinv = k_pivot_inverse<T>;
      MF_CUDA(cudaFuncSetAttribute(kinv, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(sizeof(double) * NB * 2 * NB)));
      { kinv<<<cnt, 256, sm, ctx->stream>>>(F, L.off, n, k, kb, P, M->d_err); gbmhd::count_launch(); }
      const int64_t tot = (int64_t)n * kb;
      dim3 gc((unsigned)std::min<int64_t>((tot + 255) / 256, 1024), (unsigned)cnt);
      { k_gj_copy<T><<<gc, 256, 0, ctx->stream>>>(F, L.off, n, k, kb, C, Tb); gbmhd::count_launch(); }
      MF_CUDA(cudaGetLastError());
      // T2 = P · Tb  (kb x n)
      gbmhd::count_gemm(); MF_BLAS(gemm_sb<T>(M, CUBLAS_OP_N, CUBLAS_OP_N, kb, n, kb, &one, P, NB, (long long)NB * NB, Tb, NB,
                         (long long)NB * n, &zero, T2, NB, (long long)NB * n, cnt));
      // M -= C · T2   (n x n)
      gbmhd::count_gemm(); MF_BLAS(gemm_sb<T>(M, CUBLAS_OP_N, CUBLAS_OP_N, n, n, kb, &mone, C, n, (long long)n * NB, T2, NB,
                         (long long)NB * n, &one, F + L.off, n, (long long)n * n, cnt));
      // M[:, K] = −C · P  (n x kb)
      gbmhd::count_gemm(); MF_BLAS(gemm_sb<T>(M, CUBLAS_OP_N, CUBLAS_OP_N, n, kb, kb, &mone, C, n, (long long)n * NB, P, NB,
                         (long long)NB * NB, &zero, F + L.off + (int64_t)k * n, n, (long long)n * n, cnt));
      { k_gj_fix<T><<<gc, 256, 0, ctx->stream>>>(F, L.off, n, k, kb, T2, P); gbmhd::count_launch(); }
      MF_CUDA(cudaGetLastError());
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
  return 0;
}

int mf_factor(gbmhd_ctx* ctx, MFNumeric* M, int precision, int values, const double* d_reg) {
  if (values == GBMHD_MIXED && !ctx->d_val32) { ctx->err = "multifrontal: no FP32 Jacobian assembled"; return -1; }
  if (values == GBMHD_FP64 && !ctx->d_val64) { ctx->err = "multifrontal: no FP64 Jacobian assembled"; return -1; }
  if (precision == GBMHD_MIXED) {
    if (values == GBMHD_MIXED) return factor_impl<float, float>(ctx, M, ctx->d_val32, d_reg);
    return factor_impl<float, double>(ctx, M, ctx->d_val64, d_reg);
  }
  if (values != GBMHD_FP64) { ctx->err = "multifrontal: FP64 factors need the FP64 Jacobian"; return -1; }
  return factor_impl<double, double>(ctx, M, ctx->d_val64, d_reg);
}

// Column chunk of the chunked sweeps: wide enough that the partial-sum atomics stay a
// small fraction of the factor reads, narrow enough that a level with few fronts still
// launches about two waves of CTAs.
static int sweep_cols(const gbmhd_ctx* ctx, int64_t rows, int64_t ncols, int64_t fronts) {
  const int64_t per_chunk = std::max<int64_t>(1, (rows + SW_ROWS - 1) / SW_ROWS) * std::max<int64_t>(1, fronts);
  const int64_t want = (int64_t)ctx->num_sms * 32;  // 2 waves of 16 resident 128-thread CTAs
  const int64_t chunks = std::max<int64_t>(1, (want + per_chunk - 1) / per_chunk);
  int64_t cols = (ncols + chunks - 1) / chunks;
  cols = ((cols + 31) / 32) * 32;
  return (int)std::max<int64_t>(64, std::min<int64_t>(cols, 1024));
}

template <typename T>
static int solve_impl(gbmhd_ctx* ctx, MFNumeric* M, double* b, double* x, bool tr) {
  using V = typename SweepAcc<T>::V;
  const MFSymbolic& S = M->S;
  const T* F = reinterpret_cast<const T*>(M->F);
  for (size_t l = 0; l < S.levels.size(); ++l) {
    const MFLevel& L = S.levels[l];
    const int cnt = (int)L.count;
    { k_fwd_gather<<<cnt, 256, 0, ctx->stream>>>(b, M->tsave, M->tsave_off, M->d.elim, M->d.elim_ptr, M->d.f_ne, L.first, L.E); gbmhd::count_launch(); }
    if (L.B > 0) {
      if (!tr) {
        const int cols = sweep_cols(ctx, L.B, L.E, cnt);
        dim3 g((unsigned)((L.B + SW_ROWS - 1) / SW_ROWS), (unsigned)((L.E + cols - 1) / cols), (unsigned)cnt);
        { k_fwd_chunk<T><<<g, SW_ROWS, sizeof(V) * cols, ctx->stream>>>(F, M->d.f_off, b, M->tsave, M->tsave_off, M->d.bnd, M->d.bnd_ptr, M->d.f_nb, M->d.f_ne, L.first, L.n, L.E, cols); gbmhd::count_launch(); }
      } else {
        const size_t sm = sizeof(V) * L.E;
        auto kf = k_fwd_gemv_t<T>;
        MF_CUDA(cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)std::max<size_t>(sm, 1)));
        dim3 g((unsigned)((L.B + 7) / 8), (unsigned)cnt);
        { kf<<<g, 256, sm, ctx->stream>>>(F, M->d.f_off, b, M->tsave, M->tsave_off, M->d.bnd, M->d.bnd_ptr, M->d.f_nb, M->d.f_ne, L.first, L.n, L.E); gbmhd::count_launch(); }
      }
    }
    MF_CUDA(cudaGetLastError());
  }
  for (int l = (int)S.levels.size() - 1; l >= 0; --l) {
    const MFLevel& L = S.levels[l];
    const int cnt = (int)L.count;
    if (!tr) {
      const int cols = sweep_cols(ctx, L.E, L.n, cnt);
      dim3 g((unsigned)((L.E + SW_ROWS - 1) / SW_ROWS), (unsigned)((L.n + cols - 1) / cols), (unsigned)cnt);
      { k_bwd_chunk<T><<<g, SW_ROWS, sizeof(V) * cols, ctx->stream>>>(F, M->d.f_off, x, M->tsave, M->tsave_off, M->d.bnd, M->d.bnd_ptr, M->d.f_ne, M->d.f_nb, M->ybuf, L.first, L.n, L.E, cols); gbmhd::count_launch(); }
      { k_bwd_scatter<<<cnt, 256, 0, ctx->stream>>>(x, M->ybuf, M->tsave_off, M->d.elim, M->d.elim_ptr, M->d.f_ne, L.first); gbmhd::count_launch(); }
    } else {
      const size_t sm = sizeof(V) * L.n;
      auto kb = k_bwd_gemv_t<T>;
      MF_CUDA(cudaFuncSetAttribute(kb, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
      dim3 g((unsigned)((L.E + 7) / 8), (unsigned)cnt);
      { kb<<<g, 256, sm, ctx->stream>>>(F, M->d.f_off, x, M->tsave, M->tsave_off, M->d.elim, M->d.elim_ptr, M->d.bnd, M->d.bnd_ptr, M->d.f_ne, M->d.f_nb, L.first, L.n, L.E); gbmhd::count_launch(); }
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
  harvest_sweep_time(M, false);
  const bool timed = !M->ev_pending && M->ev0 && M->ev1;
  if (timed) MF_CUDA(cudaEventRecord(M->ev0, ctx->stream));
  const int rc = M->precision == GBMHD_MIXED ? solve_impl<float>(ctx, M, d_b, d_x, transpose)
                                             : solve_impl<double>(ctx, M, d_b, d_x, transpose);
  if (rc) return rc;
  if (timed) {
    MF_CUDA(cudaEventRecord(M->ev1, ctx->stream));
    M->ev_pending = true;
  }
  return 0;
}
