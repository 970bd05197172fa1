// Numeric multifrontal factorization and solves of the (u,j) block (see mf.h).
#include <cublas_v2.h>
#include <cuda.h>  // CUtensorMap types; the encoder is reached through the runtime's driver entry point

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <utility>

#include "mf.h"
#include "tc_gemm.h"

using namespace gbmhd;

namespace {

constexpr int NB = 64;   // diagonal pivot block (inverted by one CTA)
constexpr long kSweepWaitDefault = 1L << 22;  // spin limit of the sweeps' mbarrier waits
// panel: the trailing submatrix of a front takes one rank-PW update per PW pivots.
constexpr int PW = 128;
static_assert(PW % NB == 0, "a panel holds whole pivot blocks");

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
  void* Pbuf = nullptr;        // diagonal-block inverses  [count][NB*NB]
  void* Cbuf = nullptr;        // column block below a pivot block [count][n*NB]
  void* gws = nullptr;         // split images of the FP32 GEMM operands (tc_gemm.cu)
  size_t gws_bytes = 0;
  size_t work_bytes = 0;
  double* tsave = nullptr;     // per front: E slots holding t, y and z of a solve
  int64_t* tsave_off = nullptr;  // per front
  int64_t tsave_len = 0;
  int32_t* d_err = nullptr;    // device-side status (singular pivot block)
  // TMA-staged sweeps (FP32 factors): one 3-D tensor map per level (rows x columns x fronts)
  std::vector<CUtensorMap> maps;
  std::vector<int> map_rows;      // row tile of each map
  std::vector<char> map_ok;
  std::vector<CUtensorMap> cmaps;  // per level: NB x NB boxes of the substitution chains
  std::vector<char> cmap_ok;
  const void* maps_base = nullptr;
  float2* vpk = nullptr;            // packed vector segments of one level (transposed GEMVs)
  bool scaled = false;              // factors are those of Dr A Dc (monolithic)
  double* d_dr = nullptr;           // [ndofs] row scales (powers of two)
  double* d_dc = nullptr;           // [ndofs] column scales
  void* d_sval = nullptr;           // scaled copy of the Jacobian values [nnz] (value precision)
  size_t sval_bytes = 0;
  int32_t* d_sweep_err = nullptr;   // set by a sweep whose TMA wait timed out
  int32_t* h_sweep_err = nullptr;   // pinned copy, read at the next solve and by mf_check_sweeps
  long wait_limit = 0;              // spin limit of the sweeps' mbarrier waits
  // one application of the monolithic factors as a CUDA graph per direction, on fixed buffers
  double* gb = nullptr;             // [ndofs] right-hand side copy
  double* gx = nullptr;             // [ndofs] solution
  cudaGraphExec_t gexec[2] = {nullptr, nullptr};
  const void* g_factors[2] = {nullptr, nullptr};  // front storage the graph was captured on
  int g_prec[2] = {-1, -1};
  int64_t g_kernels[2] = {0, 0};    // kernels in each graph (launch accounting)
  bool graphs_ok = true;            // capture failed once: launch directly
  // sweep timing: events around each solve, harvested when the next one starts
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // second stream of the sweeps: the GEMVs beyond the next super-block run beside the chains
  cudaStream_t s2 = nullptr;
  std::vector<cudaEvent_t> sev;      // a pool of events for the fork/join points of a solve
  // the level groups of one tree height run side by side in a solve: branch streams, their
  // fork/join events and the tree height of each level
  std::vector<cudaStream_t> bstreams;
  std::vector<cudaEvent_t> fev;
  std::vector<int32_t> lheight;
  // per factorization lane beyond the first: pivot-block, block-column and GEMM scratch
  std::vector<void*> lane_buf;
  std::vector<size_t> lane_bytes;
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
  // a solve reads L11 and L21 (forward), D⁻¹, U11 and U12 (backward): ne² + 2·ne·nb entries
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
  MF_CUDA(cudaStreamCreateWithFlags(&M->s2, cudaStreamNonBlocking));
  M->sev.assign(64, nullptr);
  for (cudaEvent_t& e : M->sev) MF_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  {
    // tree height of every front (a parent follows its children in the front order), and the
    // widest run of levels of one height
    std::vector<int32_t> fh(S.f_ne.size(), 0);
    for (size_t f = 0; f < fh.size(); ++f)
      if (S.f_parent[f] >= 0) fh[S.f_parent[f]] = std::max(fh[S.f_parent[f]], fh[f] + 1);
    M->lheight.resize(S.levels.size());
    size_t widest = 1, run = 0;
    for (size_t l = 0; l < S.levels.size(); ++l) {
      M->lheight[l] = S.levels[l].count > 0 ? fh[S.levels[l].first] : -1;
      run = (l > 0 && M->lheight[l] == M->lheight[l - 1]) ? run + 1 : 1;
      widest = std::max(widest, run);
    }
    if (const char* bs = std::getenv("GBMHD_SWEEP_BRANCHES"))  // 0: levels one by one
      if (std::atoi(bs) == 0) widest = 1;
    M->bstreams.assign(std::min<size_t>(widest - 1, 7), nullptr);
    for (cudaStream_t& st : M->bstreams) MF_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    M->fev.assign(16, nullptr);
    for (cudaEvent_t& e : M->fev) MF_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  if ((rc = upload(ctx, &M->tsave_off, toff))) return rc;
  MF_CUDA(cudaMalloc(&M->tsave, sizeof(double) * std::max<int64_t>(t, 1)));
  MF_CUDA(cudaMalloc(&M->d_err, sizeof(int32_t)));
  if (cublasCreate(&M->blas) != CUBLAS_STATUS_SUCCESS) {
    ctx->err = "multifrontal: cublasCreate failed";
    return -2;
  }
  MF_BLAS(cublasSetStream(M->blas, ctx->stream));
  M->wait_limit = kSweepWaitDefault;
  if (const char* gs = std::getenv("GBMHD_SWEEP_GRAPHS")) M->graphs_ok = std::atoi(gs) != 0;
  if (const char* wl = std::getenv("GBMHD_SWEEP_WAIT_LIMIT")) M->wait_limit = std::max(0L, std::atol(wl));
  return 0;
}

void mf_destroy(MFNumeric* M) {
  if (!M) return;
  void* ptrs[] = {M->d.f_ne, M->d.f_nb, M->d.f_off, M->d.elim_ptr, M->d.bnd_ptr, M->d.elim, M->d.bnd,
                  M->d.ah_src, M->d.ah_dst, M->d.child_list, M->d.ea_ptr, M->d.ea_pos, M->d.f_parent,
                  M->d.f_level, M->d.reg_dst, M->d.reg_dof, M->F, M->Pbuf, M->Cbuf, M->tsave, M->tsave_off, M->d_err};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (M->blas) cublasDestroy(M->blas);
  if (M->gws) cudaFree(M->gws);
  if (M->vpk) cudaFree(M->vpk);
  if (M->d_dr) cudaFree(M->d_dr);
  if (M->d_dc) cudaFree(M->d_dc);
  if (M->d_sval) cudaFree(M->d_sval);
  if (M->d_sweep_err) cudaFree(M->d_sweep_err);
  if (M->h_sweep_err) cudaFreeHost(M->h_sweep_err);
  for (int t = 0; t < 2; ++t)
    if (M->gexec[t]) cudaGraphExecDestroy(M->gexec[t]);
  if (M->gb) cudaFree(M->gb);
  if (M->gx) cudaFree(M->gx);
  if (M->ev0) cudaEventDestroy(M->ev0);
  if (M->ev1) cudaEventDestroy(M->ev1);
  for (cudaEvent_t e : M->sev)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : M->fev)
    if (e) cudaEventDestroy(e);
  for (cudaStream_t st : M->bstreams)
    if (st) cudaStreamDestroy(st);
  for (void* p : M->lane_buf)
    if (p) cudaFree(p);
  if (M->s2) cudaStreamDestroy(M->s2);
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
// The maxima run in the value precision: the scale factors are powers of two, so |a_ij|·r_i·c_j
// is exact in FP32 for the FP32 Jacobian (and only its power of two matters), and the 32-bit
// bit patterns of non-negative floats order like the floats.  GB300 issues FP64 at a small
// fraction of its FP32 rate: the FP64 version of this pass was FP64-issue bound.
template <typename V>
struct RuizBits;
template <>
struct RuizBits<float> {
  using U = unsigned int;
  __device__ static U bits(float a) { return __float_as_uint(a); }
  __device__ static float value(U u) { return __uint_as_float(u); }
};
template <>
struct RuizBits<double> {
  using U = unsigned long long;
  __device__ static U bits(double a) { return (unsigned long long)__double_as_longlong(a); }
  __device__ static double value(U u) { return __longlong_as_double((long long)u); }
};

template <typename V>
__global__ void k_ruiz_max(int64_t n, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                           const V* __restrict__ val, const V* __restrict__ dr, const V* __restrict__ dc,
                           V* __restrict__ rmax, typename RuizBits<V>::U* __restrict__ cmax) {
  const int lane = threadIdx.x & 31;
  for (int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; r < n;
       r += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const V sr = dr[r];
    V m = 0;
    for (int64_t t = rowptr[r] + lane; t < rowptr[r + 1]; t += 32) {
      const int32_t c = col[t];
      const V a = fabs(val[t] * sr * dc[c]);
      m = fmax(m, a);
      atomicMax(&cmax[c], RuizBits<V>::bits(a));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
    if (lane == 0) rmax[r] = m;
  }
}

__device__ __forceinline__ double pow2_rsqrt(double m) {  // 2^round(-log2(m)/2), 1 for m == 0
  if (!(m > 0.0)) return 1.0;
  return exp2(rint(-0.5 * log2(m)));
}

// dr, dc (FP64) and their copies in the value precision (drv, dcv) take the new factors
template <typename V>
__global__ void k_ruiz_update(int64_t n, const V* __restrict__ rmax, const typename RuizBits<V>::U* __restrict__ cmax,
                              double* __restrict__ dr, double* __restrict__ dc, V* __restrict__ drv,
                              V* __restrict__ dcv) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    dr[i] *= pow2_rsqrt((double)rmax[i]);
    dc[i] *= pow2_rsqrt((double)RuizBits<V>::value(cmax[i]));
    drv[i] = (V)dr[i];
    dcv[i] = (V)dc[i];
  }
}

template <typename V>
__global__ void k_scale_vals(int64_t n, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                             const V* __restrict__ val, const V* __restrict__ dr, const V* __restrict__ dc,
                             V* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  for (int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; r < n;
       r += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const V sr = dr[r];  // powers of two: exact in V
    for (int64_t t = rowptr[r] + lane; t < rowptr[r + 1]; t += 32) out[t] = val[t] * sr * dc[col[t]];
  }
}

template <typename T>
__global__ void k_fill_t(int64_t n, T a, T* __restrict__ v) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) v[i] = a;
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

// The same Gauss-Jordan steps with one barrier per column step.  Warp w holds columns w and
// w + 32 of the block, lane l rows l and l + 32 (four float-float entries per thread), so
// that a column lies in one warp and the pivot row's and row c's entries of a warp's columns
// lie in its own lanes.  The warp that holds column c + 1 updates it in step c, then at once
// searches its pivot and publishes (double-buffered in shared memory) the pivot row, the
// float-float reciprocal of the pivot and the multipliers m_i = A[i, c + 1] after the
// interchange; after the step's one barrier every warp forms its own entries of the scaled
// pivot row with warp shuffles.  Every entry goes through the same operations, in the same
// order, as in k_pivot_inverse_df, so the two kernels give the same bits.  Shared memory:
// ~2 KB (the multipliers and the interchanges), so the CTA fits on an SM beside a
// tensor-core GEMM CTA.
__global__ void __maxnreg__(40) k_pivot_inverse_dfw(const float* __restrict__ F, int64_t off, int n, int k,
                                                           int kb, float* __restrict__ P, int32_t* err) {
  __shared__ float mh[2][NB], ml[2][NB];
  __shared__ float sih[2], sil[2];
  __shared__ int spr[2];
  __shared__ int perm[NB], colsrc[NB], cdst[NB];
  const int64_t f = blockIdx.x;
  const float* M = F + off + f * (int64_t)n * n;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  constexpr unsigned FULL = 0xffffffffu;
  float h[2][2], l[2][2];  // [s][q]: column w + 32 s, row lane + 32 q
#pragma unroll
  for (int s = 0; s < 2; ++s)
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int i = lane + 32 * q, j = w + 32 * s;
      h[s][q] = (i < kb && j < kb) ? M[(k + i) + (int64_t)(k + j) * n] : 0.0f;
      l[s][q] = 0.0f;
    }
  // the warp holding column c: pivot row (argmax of the high parts over rows c..kb-1, ties:
  // the lower row), 1 / pivot and the multipliers into buffer c & 1
  auto publish = [&](int c) {
    const int sc = c >> 5, b = c & 1;
    float vh[2], vl[2];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      vh[q] = sc ? h[1][q] : h[0][q];
      vl[q] = sc ? l[1][q] : l[0][q];
    }
    float best = (lane >= c && lane < kb) ? fabsf(vh[0]) : -1.0f;
    int bi = lane;
    if (lane + 32 >= c && lane + 32 < kb && fabsf(vh[1]) > best) { best = fabsf(vh[1]); bi = lane + 32; }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float ob = __shfl_xor_sync(FULL, best, o);
      const int oi = __shfl_xor_sync(FULL, bi, o);
      if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
    }
    const int pr = best > 0.0f ? bi : c;  // singular block: keep going, the error flag is set
    const float dh = __shfl_sync(FULL, (pr >> 5) ? vh[1] : vh[0], pr & 31);
    const float dl = __shfl_sync(FULL, (pr >> 5) ? vl[1] : vl[0], pr & 31);
    const float ch_ = __shfl_sync(FULL, (c >> 5) ? vh[1] : vh[0], c & 31);  // A[c, c]
    const float cl_ = __shfl_sync(FULL, (c >> 5) ? vl[1] : vl[0], c & 31);
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int i = lane + 32 * q;
      float m_h = vh[q], m_l = vl[q];
      if (i == pr) { m_h = ch_; m_l = cl_; }  // row pr now holds the old row c
      if (i == c) { m_h = 0.0f; m_l = 0.0f; }
      mh[b][i] = m_h;
      ml[b][i] = m_l;
    }
    if (lane == 0) {
      float ih = 0.0f, il = 0.0f;
      if (dh != 0.0f) df_rcp(dh, dl, ih, il);
      sih[b] = ih;
      sil[b] = il;
      spr[b] = pr;
      perm[c] = pr;
      if (!(best > 0.0f)) atomicExch(err, 1);
    }
  };
  if (w == 0 && kb > 0) publish(0);
  __syncthreads();
  for (int c = 0; c < kb; ++c) {
    const int b = c & 1;
    const int pr = spr[b];
    const float ih = sih[b], il = sil[b];
    const bool swap = pr != c;
    float m_h[2], m_l[2];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      m_h[q] = mh[b][lane + 32 * q];
      m_l[q] = ml[b][lane + 32 * q];
    }
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const int j = w + 32 * s;
      // the pivot row's and the old row c's entries of column j
      const float ah_p = __shfl_sync(FULL, (pr >> 5) ? h[s][1] : h[s][0], pr & 31);
      const float al_p = __shfl_sync(FULL, (pr >> 5) ? l[s][1] : l[s][0], pr & 31);
      const float ah_c = __shfl_sync(FULL, (c >> 5) ? h[s][1] : h[s][0], c & 31);
      const float al_c = __shfl_sync(FULL, (c >> 5) ? l[s][1] : l[s][0], c & 31);
      float r_h, r_l;
      if (j == c) { r_h = ih; r_l = il; }
      else df_mul(ah_p, al_p, ih, il, r_h, r_l);
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const int i = lane + 32 * q;
        if (i == c) {
          h[s][q] = r_h;
          l[s][q] = r_l;
        } else {
          const bool from_c = swap && i == pr;
          float ah = from_c ? ah_c : h[s][q], al = from_c ? al_c : l[s][q];
          if (j == c) { ah = 0.0f; al = 0.0f; }
          df_sub_prod(ah, al, m_h[q], m_l[q], r_h, r_l, h[s][q], l[s][q]);
        }
      }
    }
    if (c + 1 < kb && w == ((c + 1) & 31)) publish(c + 1);
    __syncthreads();
  }
  if (threadIdx.x == 0) {  // undo the row interchanges as column interchanges, last first
    for (int j = 0; j < NB; ++j) colsrc[j] = j;
    for (int c = kb - 1; c >= 0; --c) {
      const int p = perm[c];
      const int t = colsrc[c];
      colsrc[c] = colsrc[p];
      colsrc[p] = t;
    }
    for (int j = 0; j < NB; ++j) cdst[colsrc[j]] = j;
  }
  __syncthreads();
  // each warp stores its two columns where the interchanges put them (column-major, zero
  // outside kb x kb); the block needs no staging buffer, so its CTA fits beside a
  // tensor-core GEMM CTA on one SM
  float* Pf = P + f * (int64_t)NB * NB;
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    const int cs = w + 32 * s, j = cdst[cs];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int i = lane + 32 * q;
      Pf[i + j * NB] = (i < kb && cs < kb) ? __fadd_rn(h[s][q], l[s][q]) : 0.0f;
    }
  }
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

// ---- LU factorization helpers (the GEMMs of a panel step are strided-batched over the fronts)
// dst[i + j·n] = M[r0 + i, c0 + j], i < nr, j < nc (per front; dst stride n·NB).
template <typename T>
__global__ void __launch_bounds__(256) k_copy_block(const T* __restrict__ F, int64_t off, int n, int r0, int nr,
                                                    int c0, int nc, T* __restrict__ dst) {
  const int64_t f = blockIdx.y;
  const T* M = F + off + f * (int64_t)n * n;
  T* D = dst + f * (int64_t)n * NB;
  for (int j = blockIdx.x; j < nc; j += gridDim.x)
    for (int i = threadIdx.x; i < nr; i += blockDim.x) D[i + (int64_t)j * n] = M[(r0 + i) + (int64_t)(c0 + j) * n];
}

// M[k + i, k + j] = P[i + j·NB], i, j < kb: the diagonal block's inverse goes into the front.
template <typename T>
__global__ void __launch_bounds__(256) k_put_inverse(T* __restrict__ F, int64_t off, int n, int k, int kb,
                                                     const T* __restrict__ P) {
  const int64_t f = blockIdx.x;
  T* M = F + off + f * (int64_t)n * n;
  const T* Pf = P + f * (int64_t)NB * NB;
  for (int e = threadIdx.x; e < kb * kb; e += blockDim.x) {
    const int i = e % kb, j = e / kb;
    M[(k + i) + (int64_t)(k + j) * n] = Pf[i + j * NB];
  }
}

// ------------------------------------------------------------------ solve kernels
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
  __device__ void warp_reduce8() {  // over aligned groups of 8 lanes
    for (int o = 4; o > 0; o >>= 1) {
      const float oh = __shfl_xor_sync(0xffffffffu, hi, o, 8), ol = __shfl_xor_sync(0xffffffffu, lo, o, 8);
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
  __device__ void warp_reduce8() {
    for (int o = 4; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o, 8);
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

// ---- LU-form sweeps
// A front holds [D⁻¹\L11 , U11 ; L21 , S].  A solve runs over the eliminated block in
// super-blocks of SB rows: a substitution chain over the NB-blocks inside a super-block
// (k_tri_*), then a GEMV for the rows (forward) or the columns (backward) beyond it (k_rect*),
// which for the last super-block is the coupling with the boundary.  Front index i < E
// addresses the front's E slots of tsave (t, y and z of the sweeps) or x[elim[i]] (i < ne);
// i ≥ E addresses b[bnd[i − E]] or x[bnd[i − E]] (i − E < nb).
constexpr int SB = 512;
static_assert(SB % NB == 0, "super-blocks hold whole NB-blocks");

template <typename T>
__device__ __forceinline__ double dsub(double a, const SweepAcc<T>& acc) { return a - acc.value(); }

// acc += Σ_{u<cnt} m[u] v[u].  FP32 factors: the products with the vector's high and low
// parts are summed with FP32 FMAs (at most 16 terms), then folded into the float-float
// accumulator, as in the GEMV sweeps.
template <typename T>
__device__ __forceinline__ void acc_add_block(SweepAcc<T>& acc, const T* m, const typename SweepAcc<T>::V* v, int cnt);
template <>
__device__ __forceinline__ void acc_add_block<float>(SweepAcc<float>& acc, const float* m, const float2* v, int cnt) {
  float h = 0.0f, l = 0.0f;
  for (int u = 0; u < cnt; ++u) {
    h = fmaf(m[u], v[u].x, h);
    l = fmaf(m[u], v[u].y, l);
  }
  acc.merge(h, l);
}
template <>
__device__ __forceinline__ void acc_add_block<double>(SweepAcc<double>& acc, const double* m, const double* v, int cnt) {
  for (int u = 0; u < cnt; ++u) acc.a = fma(m[u], v[u], acc.a);
}

template <typename VT>
__device__ __forceinline__ VT vzero();
template <>
__device__ __forceinline__ float4 vzero<float4>() { return make_float4(0.f, 0.f, 0.f, 0.f); }
template <>
__device__ __forceinline__ double2 vzero<double2>() { return make_double2(0.0, 0.0); }

// acc[q] += Σ_u m[u][q] · vs[idx[u]] over the (at most 16) terms with ok[u].  FP32 factors: the
// products with the vector's high and low parts are summed with FP32 FMAs and then folded into
// the float-float accumulators (as in the GEMV sweeps); FP64 factors: FMAs.  vs is in shared
// memory and read here, after the loads of m have been issued.
template <typename T, int R, int N>
__device__ __forceinline__ void fold_rows(SweepAcc<T> (&acc)[R], const typename RowVec<T>::type (&m)[N],
                                          const typename SweepAcc<T>::V* vs, const int (&idx)[N],
                                          const bool (&ok)[N]) {
  static_assert(N <= 16, "at most 16 FP32 products per fold");
  if constexpr (sizeof(T) == 4) {
#pragma unroll
    for (int q = 0; q < R; ++q) {
      float h = 0.0f, l = 0.0f;
#pragma unroll
      for (int u = 0; u < N; ++u)
        if (ok[u]) {
          const float mq = reinterpret_cast<const float*>(&m[u])[q];
          const float2 v = vs[idx[u]];
          h = fmaf(mq, v.x, h);
          l = fmaf(mq, v.y, l);
        }
      acc[q].merge(h, l);
    }
  } else {
#pragma unroll
    for (int q = 0; q < R; ++q)
#pragma unroll
      for (int u = 0; u < N; ++u)
        if (ok[u]) acc[q].a = fma(reinterpret_cast<const double*>(&m[u])[q], vs[idx[u]], acc[q].a);
  }
}

// float-float partial sums of a row, merged across the `width` lanes of an aligned group
// (xor shuffles, FP32 arithmetic: GB300 issues FP64 at a small fraction of its FP32 rate)
__device__ __forceinline__ void group_merge(SweepAcc<float>& a, int width) {
  for (int o = width / 2; o > 0; o >>= 1) a.merge(__shfl_xor_sync(0xffffffffu, a.hi, o), __shfl_xor_sync(0xffffffffu, a.lo, o));
}
__device__ __forceinline__ void group_merge(SweepAcc<double>& a, int width) {
  for (int o = width / 2; o > 0; o >>= 1) a.a += __shfl_xor_sync(0xffffffffu, a.a, o);
}

// An accumulator's value in the packed vector format (float-float, or FP64)
__device__ __forceinline__ float2 acc_packed(const SweepAcc<float>& a) { return make_float2(a.hi, a.lo); }
__device__ __forceinline__ double acc_packed(const SweepAcc<double>& a) { return a.a; }

// Packed vector values (float-float, or FP64): p − a, and the FP64 value
__device__ __forceinline__ float2 vsub(float2 p, const SweepAcc<float>& a) {
  SweepAcc<float> s;
  s.hi = p.x;
  s.lo = p.y;
  s.merge(-a.hi, -a.lo);
  return make_float2(s.hi, s.lo);
}
__device__ __forceinline__ double vsub(double p, const SweepAcc<double>& a) { return p - a.a; }
__device__ __forceinline__ double vto(float2 p) { return (double)p.x + (double)p.y; }
__device__ __forceinline__ double vto(double p) { return p; }

// Vector values inside the chain kernels: float-float for FP32 factors (FP32 arithmetic in
// every step; FP64 only where a value is read from or written to the FP64 vectors), FP64 for
// FP64 factors.
template <typename T>
struct ChainVal;
template <>
struct ChainVal<float> {
  SweepAcc<float> v;
  __device__ void set(double d) {
    v.hi = (float)d;
    v.lo = (float)(d - (double)v.hi);
  }
  __device__ void sub(const SweepAcc<float>& a) { v.merge(-a.hi, -a.lo); }
  __device__ float2 packed() const { return make_float2(v.hi, v.lo); }
  __device__ double value() const { return v.value(); }
};
template <>
struct ChainVal<double> {
  double v = 0.0;
  __device__ void set(double d) { v = d; }
  __device__ void sub(const SweepAcc<double>& a) { v -= a.a; }
  __device__ double packed() const { return v; }
  __device__ double value() const { return v; }
};

// Forward chain, unit lower: for the NB-blocks [k, k1) of [s0, s1) in order,
//   t[k1:s1] −= M[k1:s1, k:k1] t[k:k1]      (t = the front's tsave slots, in place).
// A thread owns R consecutive rows (16-byte loads along the column-major front) and every
// G-th column of a block, so that its loads of one step are issued together (one memory round
// trip per step).  The G column groups of a row quad are adjacent lanes of one warp and merge
// their float-float partial sums by shuffles.  Levels with many fronts use G = 1 (small CTAs,
// many per SM), levels with few fronts G = 4.  With gather (the first super-block of a level)
// t is read from b[elim] for the whole front first.
template <typename T, int G>
__global__ void __launch_bounds__(SB / RowVec<T>::R * G, 512 / (SB / RowVec<T>::R * G)) k_tri_fwd(
    const T* __restrict__ F, const int64_t* __restrict__ f_off, double* __restrict__ tsave,
    const int64_t* __restrict__ toff, const double* __restrict__ b, const int32_t* __restrict__ elim,
    const int64_t* __restrict__ elim_ptr, const int32_t* __restrict__ f_ne, int64_t first, int n, int E, int s0,
    int s1, int gather) {
  using V = typename SweepAcc<T>::V;
  using VT = typename RowVec<T>::type;
  constexpr int R = RowVec<T>::R, CPG = NB / G, CU = CPG < 16 ? CPG : 16;
  static_assert(32 % G == 0, "the column groups of a row quad share a warp");
  __shared__ V vb[NB];
  const int64_t f = first + blockIdx.x;
  const T* M = F + f_off[f];
  double* t = tsave + toff[f];
  const int ne = f_ne[f];
  const int32_t* el = elim + elim_ptr[f];
  const int g = threadIdx.x % G, rq = threadIdx.x / G;  // column group (adjacent lanes), row quad
  const int r0 = s0 + R * rq;
  if (gather)
    for (int i = threadIdx.x; i < E; i += blockDim.x)
      if (i < s0 || i >= s1) t[i] = i < ne ? b[el[i]] : 0.0;
  ChainVal<T> tr[R];
#pragma unroll
  for (int q = 0; q < R; ++q) {
    const int r = r0 + q;
    tr[q].set(r < s1 ? (gather ? (r < ne ? b[el[r]] : 0.0) : t[r]) : 0.0);
  }
  for (int k = s0; k < s1; k += NB) {
    const int k1 = min(k + NB, s1);
    __syncthreads();  // the previous step's readers of vb are done
    if (g == 0 && r0 >= k && r0 < k1)
#pragma unroll
      for (int q = 0; q < R; ++q) vb[r0 + q - k] = tr[q].packed();
    __syncthreads();
    const bool active = r0 >= k1 && r0 < s1;  // k1 and s1 are multiples of R
    SweepAcc<T> acc[R];
    if (active)
#pragma unroll 1
      for (int u0 = 0; u0 < CPG; u0 += CU) {  // chunks of at most 16 vector loads per thread
        VT m[CU];
        int idx[CU];
        bool ok[CU];
#pragma unroll
        for (int u = 0; u < CU; ++u) {
          const int c = k + g + G * (u0 + u);
          ok[u] = u0 + u < CPG && c < k1;
          idx[u] = ok[u] ? c - k : 0;
          m[u] = ok[u] ? __ldcs(reinterpret_cast<const VT*>(M + r0 + (int64_t)c * n)) : vzero<VT>();
        }
        fold_rows<T, R, CU>(acc, m, vb, idx, ok);
      }
    if constexpr (G > 1)
#pragma unroll
      for (int q = 0; q < R; ++q) group_merge(acc[q], G);  // every lane of the warp takes part
    if (active)
#pragma unroll
      for (int q = 0; q < R; ++q) tr[q].sub(acc[q]);
  }
  if (g == 0)
#pragma unroll
    for (int q = 0; q < R; ++q)
      if (r0 + q < s1) t[r0 + q] = tr[q].value();
}

// Backward chain, block upper with the stored block inverses: for the NB-blocks [k, k1) of
// [s0, s1) in reverse,  x_k = D_k⁻¹ (z_k − M[k:k1, k1:s1] x[k1:s1]),  z = the tsave slots.
// Writes x[elim[i]] for i < ne.  A thread owns R consecutive rows of the block and every G-th
// column; the U loads and the D⁻¹ loads of a step are issued together.  Column groups: 8 in
// adjacent lanes (shuffle merges) times GH warps (merged through shared memory), G = 8·GH.
template <typename T, int GH>
__global__ void __launch_bounds__(32 * NB / RowVec<T>::R / 4 * GH, 512 / (32 * NB / RowVec<T>::R / 4 * GH)) k_tri_bwd(
    const T* __restrict__ F, const int64_t* __restrict__ f_off, const double* __restrict__ tsave,
    const int64_t* __restrict__ toff, double* __restrict__ x, const int32_t* __restrict__ elim,
    const int64_t* __restrict__ elim_ptr, const int32_t* __restrict__ f_ne, int64_t first, int n, int s0, int s1) {
  using V = typename SweepAcc<T>::V;
  using VT = typename RowVec<T>::type;
  constexpr int R = RowVec<T>::R, RQ = NB / R;  // row quads of a block
  constexpr int RQW = 4;                         // row quads per warp (lanes: 8 column groups x 4)
  constexpr int WPG = RQ / RQW;                  // warps per column-group set
  constexpr int G = 8 * GH, CU = 16, CD = (NB + G - 1) / G;
  __shared__ V xv[SB];              // the solved x of this super-block (packed)
  __shared__ V rhs[NB];
  __shared__ float2 part[GH][NB];   // cross-warp partial sums (float-float)
  const int64_t f = first + blockIdx.x;
  const T* M = F + f_off[f];
  const double* z = tsave + toff[f];
  const int ne = f_ne[f];
  const int32_t* el = elim + elim_ptr[f];
  const int lane = threadIdx.x % 32, w = threadIdx.x / 32;
  const int g = (lane % 8) + 8 * (w / WPG);             // column group
  const int gh = w / WPG;
  const int rq = (lane / 8) + RQW * (w % WPG);          // row quad
  const int i0 = R * rq;
  const int nblk = (s1 - s0 + NB - 1) / NB;
  auto merge_rows = [&](SweepAcc<T> (&a)[R]) {
    // 8 adjacent lanes by shuffles, then the GH warp sets through shared memory; the row sums
    // end in a (all lanes of a column-group set hold them)
#pragma unroll
    for (int q = 0; q < R; ++q) group_merge(a[q], 8);
    if constexpr (GH > 1 && sizeof(T) == 4) {
      if (lane % 8 == 0)
#pragma unroll
        for (int q = 0; q < R; ++q) part[gh][i0 + q] = make_float2(a[q].hi, a[q].lo);
      __syncthreads();
#pragma unroll
      for (int q = 0; q < R; ++q) {
        SweepAcc<T> s;
#pragma unroll
        for (int h = 0; h < GH; ++h) s.merge(part[h][i0 + q].x, part[h][i0 + q].y);
        a[q] = s;
      }
    }
  };
  static_assert(sizeof(T) == 4 || GH == 1, "FP64 factors use one warp set of column groups");
  for (int bk = nblk - 1; bk >= 0; --bk) {
    const int k = s0 + bk * NB, k1 = min(k + NB, s1), kb = k1 - k;
    const bool live = i0 < kb;  // kb is a multiple of R
    const T* rows = M + k + i0;
    // D⁻¹ columns of this thread (independent of the chain: loaded with the U loads)
    VT dm[CD];
    int didx[CD];
    bool dok[CD];
#pragma unroll
    for (int u = 0; u < CD; ++u) {
      const int c = g + G * u;
      dok[u] = live && c < kb;
      didx[u] = dok[u] ? c : 0;
      dm[u] = dok[u] ? *reinterpret_cast<const VT*>(rows + (int64_t)(k + c) * n) : vzero<VT>();
    }
    // (1) r = z_k − M[k:k1, k1:s1] x[k1:s1], by chunks of CU columns per thread
    SweepAcc<T> acc[R];
    if (live)
#pragma unroll 1
      for (int cb = k1 + g; cb < s1; cb += CU * G) {
        VT m[CU];
        int idx[CU];
        bool ok[CU];
#pragma unroll
        for (int u = 0; u < CU; ++u) {
          const int c = cb + G * u;
          ok[u] = c < s1;
          idx[u] = ok[u] ? c - s0 : 0;
          m[u] = ok[u] ? __ldcs(reinterpret_cast<const VT*>(rows + (int64_t)c * n)) : vzero<VT>();
        }
        fold_rows<T, R, CU>(acc, m, xv, idx, ok);
      }
    merge_rows(acc);
    if (g == 0 && live)
#pragma unroll
      for (int q = 0; q < R; ++q) {
        ChainVal<T> r;
        r.set(z[k + i0 + q]);
        r.sub(acc[q]);
        rhs[i0 + q] = r.packed();
      }
    __syncthreads();
    // (2) x_k = D⁻¹ r
    SweepAcc<T> a2[R];
    if (live) fold_rows<T, R, CD>(a2, dm, rhs, didx, dok);
    merge_rows(a2);
    if (g == 0 && live)
#pragma unroll
      for (int q = 0; q < R; ++q) {
        xv[k + i0 + q - s0] = acc_packed(a2[q]);
        if (k + i0 + q < ne) x[el[k + i0 + q]] = a2[q].value();
      }
    __syncthreads();
  }
}

// Transposed forward chain (Uᵀ: block lower with D⁻ᵀ): for the NB-blocks [k, k1) of [s0, s1)
// in order,  y_k = D_k⁻ᵀ t_k,  then t[k1:s1] −= M[k:k1, k1:s1]ᵀ y_k.  Column dot products over
// the block's NB rows: eight lanes per column (NB / 8 rows each, 16-byte loads), reduced with
// shuffles; a CTA of 512 threads takes 64 columns per pass and issues the loads of all its
// passes of a step together.  With gather, t is read from b[elim] for the whole front first.
constexpr int TT_THREADS = 512;
template <typename T>
__global__ void __launch_bounds__(TT_THREADS) k_tri_fwd_t(const T* __restrict__ F, const int64_t* __restrict__ f_off,
                                                          double* __restrict__ tsave, const int64_t* __restrict__ toff,
                                                          const double* __restrict__ b,
                                                          const int32_t* __restrict__ elim,
                                                          const int64_t* __restrict__ elim_ptr,
                                                          const int32_t* __restrict__ f_ne, int64_t first, int n,
                                                          int E, int s0, int s1, int gather) {
  using V = typename SweepAcc<T>::V;
  using VT = typename RowVec<T>::type;
  constexpr int R = RowVec<T>::R, LV = NB / 8 / R;  // vector loads per lane and column
  constexpr int NP = SB / (TT_THREADS / 8);          // passes of 64 columns over a super-block
  __shared__ V tt[SB];  // packed (FP32 arithmetic on float-float for FP32 factors)
  __shared__ V yb[NB];
  const int64_t f = first + blockIdx.x;
  const T* M = F + f_off[f];
  double* t = tsave + toff[f];
  const int ne = f_ne[f];
  const int32_t* el = elim + elim_ptr[f];
  const int j = threadIdx.x % 8, cs = threadIdx.x / 8;  // lane in the column, column slot
  if (gather) {
    for (int i = threadIdx.x; i < E; i += blockDim.x) {
      const double v = i < ne ? b[el[i]] : 0.0;
      if (i >= s0 && i < s1) tt[i - s0] = SweepAcc<T>::pack(v);
      else t[i] = v;
    }
  } else {
    for (int i = threadIdx.x; i < s1 - s0; i += blockDim.x) tt[i] = SweepAcc<T>::pack(t[s0 + i]);
  }
  __syncthreads();
  for (int k = s0; k < s1; k += NB) {
    const int k1 = min(k + NB, s1), kb = k1 - k;
    // (a) y_c = Σ_r D⁻¹[r, c] t_r, c = cs < kb
    {
      SweepAcc<T> acc;
      if (cs < kb) {
        const T* col = M + k + (int64_t)(k + cs) * n;
#pragma unroll
        for (int u = 0; u < LV; ++u) {
          const int r = R * (j + 8 * u);
          if (r < kb) {
            const VT m = *reinterpret_cast<const VT*>(col + r);
#pragma unroll
            for (int q = 0; q < R; ++q) acc.add(reinterpret_cast<const T*>(&m)[q], tt[k - s0 + r + q]);
          }
        }
      }
      acc.warp_reduce8();
      __syncthreads();  // every lane has read tt[k..k1)
      if (j == 0 && cs < kb) {
        tt[k - s0 + cs] = acc_packed(acc);
        yb[cs] = acc_packed(acc);
      }
      __syncthreads();
    }
    // (b) t_c −= Σ_{r ∈ [k, k1)} M[r, c] y_r, c ∈ [k1, s1): all passes' loads first
    VT m[NP][LV];
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      const int c = k1 + cs + 64 * p;
#pragma unroll
      for (int u = 0; u < LV; ++u) {
        const int r = R * (j + 8 * u);
        m[p][u] = (c < s1 && r < kb) ? __ldcs(reinterpret_cast<const VT*>(M + k + r + (int64_t)c * n)) : vzero<VT>();
      }
    }
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      const int c = k1 + cs + 64 * p;
      SweepAcc<T> acc;
#pragma unroll
      for (int u = 0; u < LV; ++u) {
        const int r = R * (j + 8 * u);
        if (r < kb)
#pragma unroll
          for (int q = 0; q < R; ++q) acc.add(reinterpret_cast<const T*>(&m[p][u])[q], yb[r + q]);
      }
      acc.warp_reduce8();
      if (j == 0 && c < s1) tt[c - s0] = vsub(tt[c - s0], acc);
    }
    __syncthreads();
  }
  for (int i = threadIdx.x; i < s1 - s0; i += blockDim.x) t[s0 + i] = vto(tt[i]);
}

// Transposed backward chain (Lᵀ: unit upper): for the NB-blocks [k, k1) of [s0, s1) in
// reverse,  x_k = z_k − M[k1:s1, k:k1]ᵀ x[k1:s1];  writes x[elim[i]] for i < ne.  Eight lanes per
// column, each taking every eighth 16-byte row group below the block; all loads of a step are
// issued together.
template <typename T>
__global__ void __launch_bounds__(TT_THREADS) k_tri_bwd_t(const T* __restrict__ F, const int64_t* __restrict__ f_off,
                                                          const double* __restrict__ tsave,
                                                          const int64_t* __restrict__ toff, double* __restrict__ x,
                                                          const int32_t* __restrict__ elim,
                                                          const int64_t* __restrict__ elim_ptr,
                                                          const int32_t* __restrict__ f_ne, int64_t first, int n,
                                                          int s0, int s1) {
  using V = typename SweepAcc<T>::V;
  using VT = typename RowVec<T>::type;
  constexpr int R = RowVec<T>::R, NL = (SB - NB) / (8 * R);  // row groups per lane, at most
  __shared__ V xv[SB];
  const int64_t f = first + blockIdx.x;
  const T* M = F + f_off[f];
  const double* z = tsave + toff[f];
  const int ne = f_ne[f];
  const int32_t* el = elim + elim_ptr[f];
  const int j = threadIdx.x % 8, cs = threadIdx.x / 8;
  const int nblk = (s1 - s0 + NB - 1) / NB;
  for (int bk = nblk - 1; bk >= 0; --bk) {
    const int k = s0 + bk * NB, k1 = min(k + NB, s1), kb = k1 - k;
    SweepAcc<T> acc;
    if (cs < kb) {
      const T* col = M + (int64_t)(k + cs) * n;
      VT m[NL];
#pragma unroll
      for (int u = 0; u < NL; ++u) {
        const int r = k1 + R * (j + 8 * u);
        m[u] = r < s1 ? __ldcs(reinterpret_cast<const VT*>(col + r)) : vzero<VT>();
      }
#pragma unroll
      for (int u = 0; u < NL; ++u) {
        const int r = k1 + R * (j + 8 * u);
        if (r < s1)
#pragma unroll
          for (int q = 0; q < R; ++q) acc.add(reinterpret_cast<const T*>(&m[u])[q], xv[r + q - s0]);
      }
    }
    acc.warp_reduce8();
    if (j == 0 && cs < kb) {
      const V v = vsub(SweepAcc<T>::pack(z[k + cs]), acc);
      xv[k + cs - s0] = v;
      if (k + cs < ne) x[el[k + cs]] = vto(v);
    }
    __syncthreads();
  }
}

// Vector value at front index i: the E part from tsave (from_x = 0) or x[elim[i]] (from_x = 1,
// zero for i ≥ ne); the boundary part from x[bnd[i − E]] (zero for i − E ≥ nb or x null).
__device__ __forceinline__ double front_vec(int i, int E, int ne, int nb, const double* t, const double* x,
                                            const int32_t* el, const int32_t* bd, int from_x) {
  if (i < E) return from_x ? (i < ne ? x[el[i]] : 0.0) : t[i];
  return (x && i - E < nb) ? x[bd[i - E]] : 0.0;
}

// out −= v at front index i: the E part into tsave, the boundary part into b[bnd[i − E]].
__device__ __forceinline__ void front_sub(int i, int E, int nb, double* t, double* b, const int32_t* bd, double v) {
  if (i < E) atomicAdd(&t[i], -v);
  else if (i - E < nb) atomicAdd(&b[bd[i - E]], -v);
}

// Rectangular GEMV of the sweeps: out[r] −= Σ_{c ∈ [c0, c1)} M[r, c] v[c] for r ∈ [r0, r1).
// Grid (row tiles, column chunks, fronts); a thread owns R consecutive rows (16-byte vector
// loads of the column-major front; r0 a multiple of R) and reduces one chunk of `cols`
// columns staged in shared memory; partial sums are added atomically.  The TMA-staged
// version (k_rect_tma) takes the FP32 levels whose fronts are at least a box wide.
constexpr int SW_THREADS = 128;
template <typename T>
__global__ void __launch_bounds__(SW_THREADS) k_rect(const T* __restrict__ F, const int64_t* __restrict__ f_off,
                                                     double* __restrict__ tsave, const int64_t* __restrict__ toff,
                                                     const double* __restrict__ x, double* __restrict__ b,
                                                     const int32_t* __restrict__ elim,
                                                     const int64_t* __restrict__ elim_ptr,
                                                     const int32_t* __restrict__ bnd, const int64_t* __restrict__ bnd_ptr,
                                                     const int32_t* __restrict__ f_ne, const int32_t* __restrict__ f_nb,
                                                     int64_t first, int n, int E, int r0, int r1, int c0, int c1,
                                                     int cols, int from_x) {
  using V = typename SweepAcc<T>::V;
  constexpr int R = RowVec<T>::R;
  extern __shared__ __align__(16) unsigned char sm_raw[];
  V* vs = reinterpret_cast<V*>(sm_raw);
  const int64_t f = first + blockIdx.z;
  const int ne = f_ne[f], nb = f_nb[f];
  const int j0 = r0 + (int)(blockIdx.x * SW_THREADS + threadIdx.x) * R;
  const int ca = c0 + (int)blockIdx.y * cols, cb = min(c1, ca + cols);
  if (r0 + (int)blockIdx.x * SW_THREADS * R >= r1 || ca >= cb) return;
  double* t = tsave + toff[f];
  const int32_t* el = elim + elim_ptr[f];
  const int32_t* bd = bnd + bnd_ptr[f];
  for (int c = ca + threadIdx.x; c < cb; c += blockDim.x)
    vs[c - ca] = SweepAcc<T>::pack(front_vec(c, E, ne, nb, t, x, el, bd, from_x));
  __syncthreads();
  if (j0 >= r1) return;
  SweepAcc<T> acc[R];
  strided_dot_rows<T>(acc, F + f_off[f] + j0 + (int64_t)ca * n, n, vs, cb - ca);
#pragma unroll
  for (int q = 0; q < R; ++q)
    if (j0 + q < r1) front_sub(j0 + q, E, nb, t, b, bd, acc[q].value());
}

// Packed vector of front indices [r0, r1) for the transposed FP32 GEMVs: vpk[front][i − r0],
// zero-padded to ld entries.
__global__ void k_pack_front(const double* __restrict__ tsave, const int64_t* __restrict__ toff,
                             const double* __restrict__ x, const int32_t* __restrict__ elim,
                             const int64_t* __restrict__ elim_ptr, const int32_t* __restrict__ bnd,
                             const int64_t* __restrict__ bnd_ptr, const int32_t* __restrict__ f_ne,
                             const int32_t* __restrict__ f_nb, int64_t first, int E, int r0, int r1, int ld,
                             int from_x, float2* __restrict__ vpk) {
  const int64_t f = first + blockIdx.x;
  const int ne = f_ne[f], nb = f_nb[f];
  const double* t = tsave + toff[f];
  const int32_t* el = elim + elim_ptr[f];
  const int32_t* bd = bnd + bnd_ptr[f];
  float2* v = vpk + (int64_t)blockIdx.x * ld;
  for (int i = r0 + threadIdx.x; i < r0 + ld; i += blockDim.x)
    v[i - r0] = SweepAcc<float>::pack(i < r1 ? front_vec(i, E, ne, nb, t, x, el, bd, from_x) : 0.0);
}

// Transposed rectangular GEMV: out[c] −= Σ_{r ∈ [r0, r1)} M[r, c] v[r] for c ∈ [c0, c1).  A warp
// takes NC adjacent columns and runs down them together (each a contiguous column segment);
// FP32 factors read the packed vector (vpk, ld entries per front), FP64 factors gather theirs
// into shared memory.
template <typename T, int NC>
__global__ void __launch_bounds__(256) k_rect_t(const T* __restrict__ F, const int64_t* __restrict__ f_off,
                                                double* __restrict__ tsave, const int64_t* __restrict__ toff,
                                                const double* __restrict__ x, double* __restrict__ b,
                                                const int32_t* __restrict__ elim, const int64_t* __restrict__ elim_ptr,
                                                const int32_t* __restrict__ bnd, const int64_t* __restrict__ bnd_ptr,
                                                const int32_t* __restrict__ f_ne, const int32_t* __restrict__ f_nb,
                                                int64_t first, int n, int E, int r0, int r1, int c0, int c1, int ld,
                                                int from_x, const float2* __restrict__ vpk) {
  extern __shared__ __align__(16) unsigned char sm_raw[];
  const int64_t f = first + blockIdx.y;
  const int ne = f_ne[f], nb = f_nb[f];
  double* t = tsave + toff[f];
  const int32_t* el = elim + elim_ptr[f];
  const int32_t* bd = bnd + bnd_ptr[f];
  double* vd = reinterpret_cast<double*>(sm_raw);
  if constexpr (sizeof(T) != 4) {
    for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) vd[i - r0] = front_vec(i, E, ne, nb, t, x, el, bd, from_x);
    __syncthreads();
  }
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int c = c0 + (int)(blockIdx.x * (blockDim.x / 32) + warp) * NC;
  if (c >= c1) return;
  const int ncols = min(NC, c1 - c);
  const T* col = F + f_off[f] + r0 + (int64_t)c * n;
  SweepAcc<T> acc[NC];
  if constexpr (sizeof(T) == 4) {
    warp_cols_dot<NC>(acc, col, n, ncols, vpk + (int64_t)blockIdx.y * ld, r1 - r0, lane);
  } else {
    static_assert(sizeof(T) == 4 || NC == 1, "FP64 transposed sweeps take one column per warp");
    for (int r = lane; r < r1 - r0; r += 32) acc[0].add(col[r], vd[r]);
  }
#pragma unroll
  for (int q = 0; q < NC; ++q) {
    acc[q].warp_reduce();
    if (lane == 0 && q < ncols) front_sub(c + q, E, nb, t, b, bd, acc[q].value());
  }
}

// ---- TMA-staged GEMVs of the sweeps (FP32 factors)
// A CTA owns a tile of `rows` rows (at most TS_ROWS, sized per level so that the tiles cover
// the rows with little overhang) of one front and a chunk of its columns.  Thread 0 streams
// the chunk through shared memory in stages of TS_COLS columns with cp.async.bulk.tensor (one
// 3-D tensor map per level and direction: rows x columns x fronts), keeping TS_STAGES stages in
// flight behind mbarriers; every thread reduces two rows of each staged column in float-float
// arithmetic.
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

// Programmatic dependent launch: the sweep kernels are launched so that they may start while
// the kernel before them finishes.  Everything before pdl_wait() (barrier set-up and the TMA
// copies of factor blocks, which no kernel of a solve writes) overlaps that kernel's tail;
// pdl_wait() returns once the previous kernel has completed and its writes are visible, and
// only then are the solve's vectors read or written.  pdl_trigger() after it lets the next
// kernel start its own set-up.  Launched without the attribute, both are no-ops.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// out[r] −= Σ_{c ∈ [c0, c1)} M[r, c] v[c] for r ∈ [r0, r1) (the semantics of k_rect) with the
// front's columns streamed through shared memory by TMA.  CTA (row tile, column chunk,
// front): thread 0 issues the stage copies; every wait is bounded (wait_limit spins), and a
// wait that runs out makes the CTA wait (with the full limit) for its copies in flight, set
// the error flag and return.
__global__ void __launch_bounds__(TS_THREADS) k_rect_tma(const __grid_constant__ CUtensorMap map, int64_t first,
                                                         int E, int r0, int r1, int c0, int c1, int rows, int cw,
                                                         double* __restrict__ tsave, const int64_t* __restrict__ toff,
                                                         const double* __restrict__ x, double* __restrict__ b,
                                                         const int32_t* __restrict__ elim,
                                                         const int64_t* __restrict__ elim_ptr,
                                                         const int32_t* __restrict__ bnd,
                                                         const int64_t* __restrict__ bnd_ptr,
                                                         const int32_t* __restrict__ f_ne,
                                                         const int32_t* __restrict__ f_nb, int from_x, int32_t* err,
                                                         long wait_limit) {
  extern __shared__ __align__(1024) unsigned char ts_raw[];
  float* tiles = reinterpret_cast<float*>(ts_raw);                  // [stage][column][row]
  float2* vs = reinterpret_cast<float2*>(ts_raw + (size_t)TS_STAGES * TS_COLS * rows * sizeof(float));  // [cw]
  __shared__ __align__(8) uint64_t full[TS_STAGES];
  __shared__ int abort_flag;
  const int fl = blockIdx.z;
  const int64_t f = first + fl;
  const int ne = f_ne[f], nb = f_nb[f];
  const int row0 = r0 + (int)blockIdx.x * rows;
  const int ca = c0 + (int)blockIdx.y * cw, cb = min(c1, ca + cw);
  if (row0 >= r1 || ca >= cb) return;
  const int ncol = cb - ca;
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
      tma_load_3d(tiles + (size_t)s * TS_COLS * rows, &map, row0, ca + s * TS_COLS, fl, &full[s]);
    }
  double* t = tsave + toff[f];
  const int32_t* el = elim + elim_ptr[f];
  const int32_t* bd = bnd + bnd_ptr[f];
  pdl_wait();
  pdl_trigger();
  for (int c = threadIdx.x; c < ncol; c += blockDim.x)
    vs[c] = SweepAcc<float>::pack(front_vec(ca + c, E, ne, nb, t, x, el, bd, from_x));
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
      // accumulators: ~3 instructions per factor entry
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
        for (int s2 = s; s2 < min(nst, s + TS_STAGES); ++s2)
          mbar_wait_bounded(&full[s2 % TS_STAGES], (uint32_t)(s2 / TS_STAGES) & 1u, TS_WAIT_LIMIT);
        atomicExch(err, 1);
      }
      return;
    }
    if (threadIdx.x == 0 && s + TS_STAGES < nst) {
      mbar_expect_tx(&full[buf], stage_bytes);
      tma_load_3d(tiles + (size_t)buf * TS_COLS * rows, &map, row0, ca + (s + TS_STAGES) * TS_COLS, fl, &full[buf]);
    }
  }
  const int i0 = row0 + r;
  if (i0 < r1) front_sub(i0, E, nb, t, b, bd, a0.value());
  if (i0 + 1 < r1) front_sub(i0 + 1, E, nb, t, b, bd, a1.value());
}

// ---- substitution chains with TMA-staged blocks (FP32 factors)
// Every NB x NB block a chain reads is one TMA box (NB rows x NB columns of one front, 16 KB),
// copied into a ring of NSLOT shared-memory slots by thread 0 ahead of the step that uses
// it; a step waits only for its own blocks, and the ring is refilled after each step.  A step
// reads at most nb ≤ NSLOT blocks (checked on the host), so the ring never waits on itself.
// Thread layout: R = 4 consecutive rows of the super-block (one 16-byte shared-memory load
// per column) times G column groups; the G lanes of a row quad are LPR = 32 / G lanes apart
// in one warp (conflict-free shared-memory rows, xor-shuffle merges).  Waits are bounded: one
// that runs out makes the CTA wait (with the full limit) for its copies in flight, set the
// error flag and return.
constexpr int CH_BOX_BYTES = NB * NB * (int)sizeof(float);

template <int NSLOT>
__device__ __forceinline__ void chain_drain(uint64_t* full, int q0, int q1, int32_t* err) {
  for (int q = q0; q < q1; ++q) mbar_wait_bounded(&full[q % NSLOT], (uint32_t)(q / NSLOT) & 1u, TS_WAIT_LIMIT);
  atomicExch(err, 1);
}

// acc[q] += Σ_c box[c][rl + q] · v[c] over the columns c = g, g + G, … of a box (FP32
// products of the vector's high and low parts summed in chunks of 16, folded into the
// float-float accumulators)
template <int G>
__device__ __forceinline__ void box_rows(SweepAcc<float> (&acc)[4], const float* __restrict__ box, int rl, int g,
                                         const float2* __restrict__ v) {
  constexpr int CPG = NB / G, CU = CPG < 16 ? CPG : 16;
#pragma unroll
  for (int c0 = 0; c0 < CPG; c0 += CU) {
    float h[4] = {0.f, 0.f, 0.f, 0.f}, l[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int u = 0; u < CU; ++u) {
      const int c = g + G * (c0 + u);
      const float4 m = *reinterpret_cast<const float4*>(box + c * NB + rl);
      const float2 vv = v[c];
      h[0] = fmaf(m.x, vv.x, h[0]); l[0] = fmaf(m.x, vv.y, l[0]);
      h[1] = fmaf(m.y, vv.x, h[1]); l[1] = fmaf(m.y, vv.y, l[1]);
      h[2] = fmaf(m.z, vv.x, h[2]); l[2] = fmaf(m.z, vv.y, l[2]);
      h[3] = fmaf(m.w, vv.x, h[3]); l[3] = fmaf(m.w, vv.y, l[3]);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[q].merge(h[q], l[q]);
  }
}

template <int G>
__device__ __forceinline__ void merge_groups(SweepAcc<float> (&acc)[4]) {
  constexpr int LPR = 32 / G;
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int o = LPR; o < 32; o <<= 1)
      acc[q].merge(__shfl_xor_sync(0xffffffffu, acc[q].hi, o), __shfl_xor_sync(0xffffffffu, acc[q].lo, o));
}

// Forward chain (unit lower), the semantics of k_tri_fwd: for the NB-blocks k of [s0, s1) in
// order, t[block j] −= M[block j, block k] t[block k] for the blocks j > k of the
// super-block.  Boxes in step order: (k, j) for j = k+1 … nb−1.
template <int G, int NSLOT>
__global__ void __launch_bounds__(128 * G) k_chain_fwd(const __grid_constant__ CUtensorMap map, int64_t first,
                                                       double* __restrict__ tsave, const int64_t* __restrict__ toff,
                                                       const double* __restrict__ b, const int32_t* __restrict__ elim,
                                                       const int64_t* __restrict__ elim_ptr,
                                                       const int32_t* __restrict__ f_ne, int E, int s0, int s1,
                                                       int gather, int32_t* err, long wait_limit) {
  constexpr int LPR = 32 / G;
  extern __shared__ __align__(1024) unsigned char ch_raw[];
  float* slots = reinterpret_cast<float*>(ch_raw);  // [NSLOT][NB columns][NB rows]
  __shared__ __align__(8) uint64_t full[NSLOT];
  __shared__ float2 vb[2][NB];
  __shared__ int abort_flag;
  const int fl = blockIdx.x;
  const int64_t f = first + fl;
  double* t = tsave + toff[f];
  const int ne = f_ne[f];
  const int32_t* el = elim + elim_ptr[f];
  const int lane = threadIdx.x & 31, g = lane / LPR;
  const int rq = (threadIdx.x >> 5) * LPR + lane % LPR;  // row quad of the super-block
  const int r0 = s0 + 4 * rq, jb = rq / (NB / 4), rl = 4 * (rq % (NB / 4));
  const int nb = (s1 - s0 + NB - 1) / NB, nbox = nb * (nb - 1) / 2;
  if (threadIdx.x == 0) {
    for (int s = 0; s < NSLOT; ++s) mbar_init(&full[s], 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  int qi = 0, ik = 0, ij = 1;  // next box to issue and its (column block, row block): thread 0
  auto issue = [&](int qend) {
    for (; qi < qend; ++qi) {
      const int s = qi % NSLOT;
      mbar_expect_tx(&full[s], CH_BOX_BYTES);
      tma_load_3d(slots + (size_t)s * NB * NB, &map, s0 + NB * ij, s0 + NB * ik, fl, &full[s]);
      if (++ij == nb) { ++ik; ij = ik + 1; }
    }
  };
  if (threadIdx.x == 0) issue(min(nbox, NSLOT));
  pdl_wait();
  pdl_trigger();
  if (gather)
    for (int i = threadIdx.x; i < E; i += blockDim.x)
      if (i < s0 || i >= s1) t[i] = i < ne ? b[el[i]] : 0.0;
  ChainVal<float> tr[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int r = r0 + q;
    tr[q].set(r < s1 ? (gather ? (r < ne ? b[el[r]] : 0.0) : t[r]) : 0.0);
  }
  // One barrier per step: at its top t_k is in vb[k & 1] (published by the threads of block k
  // at the end of the step before) and the boxes of the step before are consumed.
  if (g == 0 && jb == 0)
#pragma unroll
    for (int q = 0; q < 4; ++q) vb[0][rl + q] = tr[q].packed();
  int qc = 0, qprev = 0;  // first box of the current and of the previous step
  for (int k = 0; k + 1 < nb; ++k) {
    __syncthreads();
    if (abort_flag) {
      if (threadIdx.x == 0) chain_drain<NSLOT>(full, qprev, qi, err);
      return;
    }
    if (threadIdx.x == 0 && k > 0) issue(min(nbox, qc + NSLOT));
    SweepAcc<float> acc[4];
    const bool active = jb > k && r0 < s1;
    if (active) {
      const int q = qc + (jb - k - 1);
      if (mbar_wait_bounded(&full[q % NSLOT], (uint32_t)(q / NSLOT) & 1u, wait_limit))
        box_rows<G>(acc, slots + (size_t)(q % NSLOT) * NB * NB, rl, g, vb[k & 1]);
      else
        abort_flag = 1;
    }
    if constexpr (G > 1) merge_groups<G>(acc);
    if (active)
#pragma unroll
      for (int q = 0; q < 4; ++q) tr[q].sub(acc[q]);
    qprev = qc;
    qc += nb - 1 - k;
    if (g == 0 && jb == k + 1)  // block k + 1 is final: publish it for the next step
#pragma unroll
      for (int q = 0; q < 4; ++q) vb[(k + 1) & 1][rl + q] = tr[q].packed();
  }
  __syncthreads();  // the last step's boxes are consumed
  if (abort_flag) {
    if (threadIdx.x == 0) chain_drain<NSLOT>(full, qprev, qi, err);
    return;
  }
  if (g == 0)
#pragma unroll
    for (int q = 0; q < 4; ++q)
      if (r0 + q < s1) t[r0 + q] = tr[q].value();
}

// Backward chain (block upper with the stored block inverses), right-looking, the semantics
// of k_tri_bwd: for the NB-blocks k of [s0, s1) in reverse, x_k = D_k⁻¹ z_k, then
// z[block j] −= M[block j, block k] x_k for the blocks j < k.  Writes x[elim[i]] for i < ne.
// Boxes in step order: (k, k) (the inverse), then (j, k) for j = 0 … k−1.
template <int G, int NSLOT>
__global__ void __launch_bounds__(128 * G) k_chain_bwd(const __grid_constant__ CUtensorMap map, int64_t first,
                                                       const double* __restrict__ tsave,
                                                       const int64_t* __restrict__ toff, double* __restrict__ x,
                                                       const int32_t* __restrict__ elim,
                                                       const int64_t* __restrict__ elim_ptr,
                                                       const int32_t* __restrict__ f_ne, int s0, int s1,
                                                       int32_t* err, long wait_limit) {
  constexpr int LPR = 32 / G;
  extern __shared__ __align__(1024) unsigned char ch_raw[];
  float* slots = reinterpret_cast<float*>(ch_raw);
  __shared__ __align__(8) uint64_t full[NSLOT];
  __shared__ float2 vb[NB], xb[NB];
  __shared__ int abort_flag;
  const int fl = blockIdx.x;
  const int64_t f = first + fl;
  const double* z = tsave + toff[f];
  const int ne = f_ne[f];
  const int32_t* el = elim + elim_ptr[f];
  const int lane = threadIdx.x & 31, g = lane / LPR;
  const int rq = (threadIdx.x >> 5) * LPR + lane % LPR;
  const int r0 = s0 + 4 * rq, jb = rq / (NB / 4), rl = 4 * (rq % (NB / 4));
  const int nb = (s1 - s0 + NB - 1) / NB, nbox = nb * (nb + 1) / 2;
  if (threadIdx.x == 0) {
    for (int s = 0; s < NSLOT; ++s) mbar_init(&full[s], 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  int qi = 0, ik = nb - 1, ij = -1;  // ij = −1: the inverse block of step ik
  auto issue = [&](int qend) {
    for (; qi < qend; ++qi) {
      const int s = qi % NSLOT;
      const int row = ij < 0 ? ik : ij;
      mbar_expect_tx(&full[s], CH_BOX_BYTES);
      tma_load_3d(slots + (size_t)s * NB * NB, &map, s0 + NB * row, s0 + NB * ik, fl, &full[s]);
      if (++ij == ik) { --ik; ij = -1; }
    }
  };
  if (threadIdx.x == 0) issue(min(nbox, NSLOT));
  pdl_wait();
  pdl_trigger();
  ChainVal<float> tr[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) tr[q].set(r0 + q < s1 ? z[r0 + q] : 0.0);
  // Two barriers per step: at the top of step k, z_k is in vb (published by the threads of block
  // k at the end of the step before) and the boxes of the step before are consumed; the second
  // publishes x_k.
  const float2 zero2 = make_float2(0.f, 0.f);
  if (g == 0 && jb == nb - 1)
#pragma unroll
    for (int q = 0; q < 4; ++q) vb[rl + q] = r0 + q < s1 ? tr[q].packed() : zero2;
  int qc = 0, qprev = 0;
  for (int k = nb - 1; k >= 0; --k) {
    __syncthreads();
    if (abort_flag) {
      if (threadIdx.x == 0) chain_drain<NSLOT>(full, qprev, qi, err);
      return;
    }
    if (threadIdx.x == 0 && k < nb - 1) issue(min(nbox, qc + NSLOT));
    // x_k = D_k⁻¹ z_k (the threads of row block k)
    SweepAcc<float> acc[4];
    if (jb == k) {
      if (mbar_wait_bounded(&full[qc % NSLOT], (uint32_t)(qc / NSLOT) & 1u, wait_limit))
        box_rows<G>(acc, slots + (size_t)(qc % NSLOT) * NB * NB, rl, g, vb);
      else
        abort_flag = 1;
    }
    if constexpr (G > 1) merge_groups<G>(acc);
    if (jb == k && g == 0)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int r = r0 + q;
        xb[rl + q] = r < s1 ? acc_packed(acc[q]) : zero2;
        if (r < ne) x[el[r]] = acc[q].value();
      }
    __syncthreads();
    // z_j −= M[block j, block k] x_k (the threads of the row blocks j < k)
    SweepAcc<float> a2[4];
    if (jb < k) {
      const int q = qc + 1 + jb;
      if (mbar_wait_bounded(&full[q % NSLOT], (uint32_t)(q / NSLOT) & 1u, wait_limit))
        box_rows<G>(a2, slots + (size_t)(q % NSLOT) * NB * NB, rl, g, xb);
      else
        abort_flag = 1;
    }
    if constexpr (G > 1) merge_groups<G>(a2);
    if (jb < k)
#pragma unroll
      for (int q = 0; q < 4; ++q) tr[q].sub(a2[q]);
    qprev = qc;
    qc += k + 1;
    if (g == 0 && jb == k - 1)  // block k − 1 is final: publish it for the next step
#pragma unroll
      for (int q = 0; q < 4; ++q) vb[rl + q] = r0 + q < s1 ? tr[q].packed() : zero2;
  }
  __syncthreads();  // the last step's boxes are consumed
  if (abort_flag && threadIdx.x == 0) chain_drain<NSLOT>(full, qprev, qi, err);
}

// Transposed chains (the adjoint's solves) on the same boxes.  A column of a box is 64
// contiguous floats in shared memory: eight lanes per column (rows 4j + 32u, u = 0, 1: 16-byte
// loads, conflict-free), partial sums of 8 products per lane folded into float-float and
// reduced over the eight lanes with shuffles; 512 threads take the 64 columns of a box per
// pass.  The super-block's vector segment lives in shared memory (float-float).
constexpr int CT_THREADS = 512;

// Σ_r box[c][r] v[r] over this lane's 8 rows, added to acc
__device__ __forceinline__ void box_col8(SweepAcc<float>& acc, const float* __restrict__ box, int c, int j,
                                         const float2* __restrict__ v) {
  float h = 0.0f, l = 0.0f;
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int r = 4 * j + 32 * u;
    const float4 m = *reinterpret_cast<const float4*>(box + c * NB + r);
    const float2 v0 = v[r], v1 = v[r + 1], v2 = v[r + 2], v3 = v[r + 3];
    h = fmaf(m.x, v0.x, h); l = fmaf(m.x, v0.y, l);
    h = fmaf(m.y, v1.x, h); l = fmaf(m.y, v1.y, l);
    h = fmaf(m.z, v2.x, h); l = fmaf(m.z, v2.y, l);
    h = fmaf(m.w, v3.x, h); l = fmaf(m.w, v3.y, l);
  }
  acc.merge(h, l);
}

// Transposed forward chain (Uᵀ: block lower with D⁻ᵀ), the semantics of k_tri_fwd_t: for the
// NB-blocks k of [s0, s1) in order, y_k = D_k⁻ᵀ t_k, then t[block j] −= M[block k, block j]ᵀ y_k
// for j > k.  Boxes in step order: (k, k), then (k, j) for j = k+1 … nb−1.
template <int NSLOT>
__global__ void __launch_bounds__(CT_THREADS) k_chain_fwd_t(const __grid_constant__ CUtensorMap map, int64_t first,
                                                            double* __restrict__ tsave,
                                                            const int64_t* __restrict__ toff,
                                                            const double* __restrict__ b,
                                                            const int32_t* __restrict__ elim,
                                                            const int64_t* __restrict__ elim_ptr,
                                                            const int32_t* __restrict__ f_ne, int E, int s0, int s1,
                                                            int gather, int32_t* err, long wait_limit) {
  extern __shared__ __align__(1024) unsigned char ch_raw[];
  float* slots = reinterpret_cast<float*>(ch_raw);
  __shared__ __align__(8) uint64_t full[NSLOT];
  __shared__ float2 tt[SB], yb[NB];
  __shared__ int abort_flag;
  const int fl = blockIdx.x;
  const int64_t f = first + fl;
  double* t = tsave + toff[f];
  const int ne = f_ne[f];
  const int32_t* el = elim + elim_ptr[f];
  const int j = threadIdx.x % 8, cs = threadIdx.x / 8;  // lane in the column, column of a box
  const int len = s1 - s0, nb = (len + NB - 1) / NB, nbox = nb * (nb + 1) / 2;
  if (threadIdx.x == 0) {
    for (int s = 0; s < NSLOT; ++s) mbar_init(&full[s], 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  int qi = 0, ik = 0, ij = -1;  // ij = −1: the inverse block of step ik
  auto issue = [&](int qend) {
    for (; qi < qend; ++qi) {
      const int s = qi % NSLOT;
      mbar_expect_tx(&full[s], CH_BOX_BYTES);
      tma_load_3d(slots + (size_t)s * NB * NB, &map, s0 + NB * ik, s0 + NB * (ij < 0 ? ik : ij), fl, &full[s]);
      ij = ij < 0 ? ik + 1 : ij + 1;
      if (ij == nb) { ++ik; ij = -1; }
    }
  };
  if (threadIdx.x == 0) issue(min(nbox, NSLOT));
  for (int i = threadIdx.x; i < SB; i += blockDim.x) tt[i] = make_float2(0.f, 0.f);
  __syncthreads();
  pdl_wait();
  pdl_trigger();
  if (gather) {
    for (int i = threadIdx.x; i < E; i += blockDim.x) {
      const double v = i < ne ? b[el[i]] : 0.0;
      if (i >= s0 && i < s1) tt[i - s0] = SweepAcc<float>::pack(v);
      else t[i] = v;
    }
  } else {
    for (int i = threadIdx.x; i < len; i += blockDim.x) tt[i] = SweepAcc<float>::pack(t[s0 + i]);
  }
  __syncthreads();
  int qc = 0;
  for (int k = 0; k < nb; ++k) {
    const int kb = min(NB, len - NB * k);
    // (a) y_c = Σ_r D⁻¹[r, c] t_r
    SweepAcc<float> acc;
    if (mbar_wait_bounded(&full[qc % NSLOT], (uint32_t)(qc / NSLOT) & 1u, wait_limit))
      box_col8(acc, slots + (size_t)(qc % NSLOT) * NB * NB, cs, j, tt + NB * k);
    else
      abort_flag = 1;
    acc.warp_reduce8();
    __syncthreads();  // every lane has read t of block k
    if (j == 0 && cs < kb) {
      tt[NB * k + cs] = acc_packed(acc);
      yb[cs] = acc_packed(acc);
    }
    if (j == 0 && cs >= kb) yb[cs] = make_float2(0.f, 0.f);
    __syncthreads();
    // (b) t[block jj] −= M[block k, block jj]ᵀ y_k
    for (int jj = k + 1; jj < nb; ++jj) {
      const int q = qc + (jj - k);
      SweepAcc<float> a2;
      if (mbar_wait_bounded(&full[q % NSLOT], (uint32_t)(q / NSLOT) & 1u, wait_limit))
        box_col8(a2, slots + (size_t)(q % NSLOT) * NB * NB, cs, j, yb);
      else
        abort_flag = 1;
      a2.warp_reduce8();
      const int c = NB * jj + cs;
      if (j == 0 && c < len) tt[c] = vsub(tt[c], a2);
    }
    __syncthreads();  // the step's boxes are consumed
    if (abort_flag) {
      if (threadIdx.x == 0) chain_drain<NSLOT>(full, qc, qi, err);
      return;
    }
    qc += nb - k;
    if (threadIdx.x == 0) issue(min(nbox, qc + NSLOT));
  }
  for (int i = threadIdx.x; i < len; i += blockDim.x) t[s0 + i] = vto(tt[i]);
}

// Transposed backward chain (Lᵀ: unit upper), the semantics of k_tri_bwd_t: for the NB-blocks k
// of [s0, s1) in reverse, x_k = z_k − Σ_{j>k} M[block j, block k]ᵀ x_j; writes x[elim[i]] for
// i < ne.  Boxes in step order: (j, k) for j = k+1 … nb−1.
template <int NSLOT>
__global__ void __launch_bounds__(CT_THREADS) k_chain_bwd_t(const __grid_constant__ CUtensorMap map, int64_t first,
                                                            const double* __restrict__ tsave,
                                                            const int64_t* __restrict__ toff, double* __restrict__ x,
                                                            const int32_t* __restrict__ elim,
                                                            const int64_t* __restrict__ elim_ptr,
                                                            const int32_t* __restrict__ f_ne, int s0, int s1,
                                                            int32_t* err, long wait_limit) {
  extern __shared__ __align__(1024) unsigned char ch_raw[];
  float* slots = reinterpret_cast<float*>(ch_raw);
  __shared__ __align__(8) uint64_t full[NSLOT];
  __shared__ float2 xv[SB];
  __shared__ int abort_flag;
  const int fl = blockIdx.x;
  const int64_t f = first + fl;
  const double* z = tsave + toff[f];
  const int ne = f_ne[f];
  const int32_t* el = elim + elim_ptr[f];
  const int j = threadIdx.x % 8, cs = threadIdx.x / 8;
  const int len = s1 - s0, nb = (len + NB - 1) / NB, nbox = nb * (nb - 1) / 2;
  if (threadIdx.x == 0) {
    for (int s = 0; s < NSLOT; ++s) mbar_init(&full[s], 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  int qi = 0, ik = nb - 2, ij = nb - 1;  // step ik reads the boxes (ij, ik), ij = ik+1 … nb−1
  auto issue = [&](int qend) {
    for (; qi < qend; ++qi) {
      const int s = qi % NSLOT;
      mbar_expect_tx(&full[s], CH_BOX_BYTES);
      tma_load_3d(slots + (size_t)s * NB * NB, &map, s0 + NB * ij, s0 + NB * ik, fl, &full[s]);
      if (++ij == nb) { --ik; ij = ik + 1; }
    }
  };
  if (threadIdx.x == 0) issue(min(nbox, NSLOT));
  for (int i = threadIdx.x; i < SB; i += blockDim.x) xv[i] = make_float2(0.f, 0.f);
  __syncthreads();
  pdl_wait();
  pdl_trigger();
  int qc = 0;
  for (int k = nb - 1; k >= 0; --k) {
    const int kb = min(NB, len - NB * k);
    SweepAcc<float> acc;
    for (int jj = k + 1; jj < nb; ++jj) {
      const int q = qc + (jj - k - 1);
      if (mbar_wait_bounded(&full[q % NSLOT], (uint32_t)(q / NSLOT) & 1u, wait_limit))
        box_col8(acc, slots + (size_t)(q % NSLOT) * NB * NB, cs, j, xv + NB * jj);
      else
        abort_flag = 1;
    }
    acc.warp_reduce8();
    if (j == 0 && cs < kb) {
      const int r = s0 + NB * k + cs;
      const float2 v = vsub(SweepAcc<float>::pack(z[r]), acc);
      xv[NB * k + cs] = v;
      if (r < ne) x[el[r]] = vto(v);
    }
    __syncthreads();  // x of block k is visible, the step's boxes are consumed
    if (abort_flag) {
      if (threadIdx.x == 0) chain_drain<NSLOT>(full, qc, qi, err);
      return;
    }
    qc += nb - 1 - k;
    if (threadIdx.x == 0) issue(min(nbox, qc + NSLOT));
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

// Two maps per level over the FP32 fronts (forward and backward GEMVs of the sweeps): dims
// (n rows, n columns, count fronts), box (rows, TS_COLS, 1).  A level whose fronts are
// narrower than a box keeps the LDG GEMVs.
static void build_sweep_maps(MFNumeric* M) {
  const MFSymbolic& S = M->S;
  const size_t nl = S.levels.size();
  M->maps.assign(2 * nl, CUtensorMap{});
  M->map_rows.assign(2 * nl, 0);
  M->map_ok.assign(nl, 0);
  M->cmaps.assign(nl, CUtensorMap{});
  M->cmap_ok.assign(nl, 0);
  M->maps_base = M->F;
  EncodeTiledFn enc = encode_tiled_fn();
  if (!enc) return;
  float* F = reinterpret_cast<float*>(M->F);
  for (size_t l = 0; l < nl; ++l) {
    const MFLevel& L = S.levels[l];
    // chain boxes: NB rows x NB columns of one front (16-byte row coordinates: NB-aligned)
    if (L.n >= NB && L.n % 4 == 0 && L.off % 4 == 0 && L.count <= (1LL << 31) - 1) {
      const cuuint64_t dims[3] = {(cuuint64_t)L.n, (cuuint64_t)L.n, (cuuint64_t)L.count};
      const cuuint64_t strides[2] = {(cuuint64_t)L.n * sizeof(float), (cuuint64_t)L.n * L.n * sizeof(float)};
      const cuuint32_t box[3] = {NB, NB, 1};
      const cuuint32_t estr[3] = {1, 1, 1};
      M->cmap_ok[l] = enc(&M->cmaps[l], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, F + L.off, dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
    }
    if (L.n < TS_ROWS || L.count > (1 << 16)) continue;
    bool ok = true;
    for (int dir = 0; dir < 2; ++dir) {  // 0: forward (B rows), 1: backward (E rows)
      // forward: the rows beyond a super-block (the boundary rows when E ≤ SB);
      // backward: the rows of a super-block
      const int rows = dir == 0 ? (L.E <= SB ? tma_rows(std::max(L.B, 1)) : TS_ROWS) : tma_rows(std::min(L.E, SB));
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

// C = α·A·B + β·C for the fronts of a level (strided-batched, column-major).  FP32 factors use
// the library's tensor-core GEMM (tc_gemm.cu); FP64 factors (the plain FP64 path) use cuBLAS
// DGEMM.
// One factorization lane: a stream and the scratch of the levels it factors.
template <typename T>
struct FactorLane {
  cudaStream_t st = nullptr;
  T* P = nullptr;        // diagonal-block inverses  [count][NB*NB]
  T* C = nullptr;        // column block below a pivot block [count][n*NB]
  void* gws = nullptr;   // split images of the FP32 GEMM operands
  size_t gws_bytes = 0;
};

template <typename T>
static int gemm(gbmhd_ctx* ctx, MFNumeric* M, const FactorLane<T>& lane, int m, int n, int k, T alpha, const T* A,
                int lda, long long sA, const T* B, int ldb, long long sB, T beta, T* C, int ldc, long long sC,
                int batch) {
  if (m <= 0 || n <= 0 || k <= 0) return 0;
  if constexpr (sizeof(T) == 4) {
    std::string msg;
    const int rc = gbmhd::tc_gemm_f32(lane.st, m, n, k, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, batch,
                                      lane.gws, lane.gws_bytes, M->d_err, &msg);
    if (rc) ctx->err = "multifrontal: " + msg;
    return rc;
  } else {
    gbmhd::count_gemm();
    MF_BLAS(cublasGemmStridedBatchedEx(M->blas, CUBLAS_OP_N, CUBLAS_OP_N, m, n, k, &alpha, A, CUDA_R_64F, lda, sA,
                                       B, CUDA_R_64F, ldb, sB, &beta, C, CUDA_R_64F, ldc, sC, batch,
                                       CUBLAS_COMPUTE_64F, CUBLAS_GEMM_DEFAULT));
    return 0;
  }
}

// Pivot-block inverse of the FP32 factors: 0 = k_pivot_inverse_df<16>, 1 = k_pivot_inverse_df<4>,
// 2 = k_pivot_inverse_df_smem, 3 = k_pivot_inverse_dfw.  All four give the same bits.
static void launch_pivot_inverse(int variant, int cnt, cudaStream_t st, const float* F, int64_t off, int n, int k,
                                 int kb, float* P, int32_t* err) {
  switch (variant) {
    case 0: k_pivot_inverse_df<16><<<cnt, NB * 16, 0, st>>>(F, off, n, k, kb, P, err); break;
    case 1: k_pivot_inverse_df<4><<<cnt, NB * 4, 0, st>>>(F, off, n, k, kb, P, err); break;
    case 2: k_pivot_inverse_df_smem<<<cnt, 256, 0, st>>>(F, off, n, k, kb, P, err); break;
    default: k_pivot_inverse_dfw<<<cnt, 1024, 0, st>>>(F, off, n, k, kb, P, err); break;
  }
}

// forced: the GBMHD_PIVOT_KERNEL override (-1: none).  Measured on one GB300 (64 x 64 blocks,
// per launch): 1–152 blocks 98 µs (0), 156 µs (1), 133 µs (2), 84 µs (3); 256 blocks 193, 177,
// 150, 142 µs; 2048 blocks 1333, 964, 666, 907 µs.
static int pivot_variant(const gbmhd_ctx* ctx, int cnt, int forced) {
  if (forced >= 0 && forced <= 3) return forced;
  return cnt >= 2 * ctx->num_sms ? 2 : 3;
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
  size_t wmax = 0, pbytes = 0;
  for (const MFLevel& L : S.levels) {
    wmax = std::max(wmax, (size_t)L.count * L.n * NB);
    pbytes = std::max(pbytes, (size_t)L.count * NB * NB);
  }
  const size_t need = sizeof(T) * (wmax + pbytes);
  if (M->work_bytes < need) {
    for (void* p : {M->Pbuf, M->Cbuf})
      if (p) cudaFree(p);
    MF_CUDA(cudaMalloc(&M->Pbuf, sizeof(T) * std::max<size_t>(pbytes, 1)));
    MF_CUDA(cudaMalloc(&M->Cbuf, sizeof(T) * std::max<size_t>(wmax, 1)));
    M->work_bytes = need;
  }
  if constexpr (sizeof(T) == 4) {
    // the largest split workspace of the level's GEMMs: the first panel's L products
    // (rb x kb x kb), U rows (kb x rest x ≤ PW) and trailing update (rest x rest x pw)
    size_t gws = 0;
    for (const MFLevel& L : S.levels) {
      const int pw = std::min(PW, L.E), kb = std::min(NB, L.E), cnt = (int)L.count;
      gws = std::max(gws, gbmhd::tc_gemm_workspace(L.n - kb, kb, kb, cnt));
      gws = std::max(gws, gbmhd::tc_gemm_workspace(kb, L.n - pw, pw, cnt));
      gws = std::max(gws, gbmhd::tc_gemm_workspace(L.n - pw, L.n - pw, pw, cnt));
    }
    if (M->gws_bytes < gws) {
      if (M->gws) cudaFree(M->gws);
      M->gws = nullptr;
      M->gws_bytes = 0;
      MF_CUDA(cudaMalloc(&M->gws, gws));
      M->gws_bytes = gws;
    }
  }
  T* F = reinterpret_cast<T*>(M->F);
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
  const char* pks = std::getenv("GBMHD_PIVOT_KERNEL");
  const int pk = pks ? std::atoi(pks) : -1;
  // GBMHD_MF_LEVEL_TIMES: device time of each level (CUDA events) and the host's time to
  // issue it, printed to stderr (the levels then run one after another)
  const bool ltimes = std::getenv("GBMHD_MF_LEVEL_TIMES") != nullptr;
  std::vector<cudaEvent_t> lev_ev;
  std::vector<double> lev_host;
  if (ltimes) {
    lev_ev.resize(S.levels.size() + 1);
    for (cudaEvent_t& e : lev_ev) MF_CUDA(cudaEventCreate(&e));
    lev_host.resize(S.levels.size() + 1);
  }
  // Lanes: the level groups of one tree height are independent (each assembles, extend-adds
  // and eliminates its own fronts; their children are lower), so with FP32 factors they run
  // side by side, the first group on the context stream and the others on the branch
  // streams, each lane with its own pivot-block, block-column and GEMM scratch.
  const size_t nlev = S.levels.size();
  std::vector<int> lane_of(nlev, 0);
  int nlanes = 1;
  if (sizeof(T) == 4 && !ltimes && !M->bstreams.empty()) {
    nlanes = 1 + (int)M->bstreams.size();
    for (size_t la = 0; la < nlev;) {
      size_t lb = la + 1;
      while (lb < nlev && M->lheight[lb] == M->lheight[la]) ++lb;
      for (size_t i = 1; i < lb - la; ++i) lane_of[la + i] = 1 + (int)((i - 1) % (nlanes - 1));
      la = lb;
    }
  }
  auto level_scratch = [&](const MFLevel& L, size_t* pb, size_t* cb, size_t* gb) {
    const int pw = std::min(PW, L.E), kb = std::min(NB, L.E), cnt = (int)L.count;
    *pb = sizeof(T) * (size_t)L.count * NB * NB;
    *cb = sizeof(T) * (size_t)L.count * L.n * NB;
    *gb = 0;
    if (sizeof(T) == 4) {
      *gb = std::max(*gb, gbmhd::tc_gemm_workspace(L.n - kb, kb, kb, cnt));
      *gb = std::max(*gb, gbmhd::tc_gemm_workspace(kb, L.n - pw, pw, cnt));
      *gb = std::max(*gb, gbmhd::tc_gemm_workspace(L.n - pw, L.n - pw, pw, cnt));
    }
  };
  if (nlanes > 1) {
    std::vector<size_t> need(3 * nlanes, 0);
    for (size_t l = 0; l < nlev; ++l) {
      if (!lane_of[l]) continue;
      size_t pb, cb, gb;
      level_scratch(S.levels[l], &pb, &cb, &gb);
      const int i = lane_of[l];
      need[3 * i] = std::max(need[3 * i], pb);
      need[3 * i + 1] = std::max(need[3 * i + 1], cb);
      need[3 * i + 2] = std::max(need[3 * i + 2], gb);
    }
    size_t more = 0;
    for (int i = 1; i < nlanes; ++i)
      for (int q = 0; q < 3; ++q)
        if (M->lane_bytes.size() <= (size_t)(3 * i + q) || M->lane_bytes[3 * i + q] < need[3 * i + q]) more += need[3 * i + q];
    size_t free_b = 0, total_b = 0;
    MF_CUDA(cudaMemGetInfo(&free_b, &total_b));
    if (more + ((size_t)2 << 30) > free_b) {
      nlanes = 1;  // not worth the memory: the levels run in sequence
      std::fill(lane_of.begin(), lane_of.end(), 0);
    } else {
      M->lane_buf.resize(3 * nlanes, nullptr);
      M->lane_bytes.resize(3 * nlanes, 0);
      for (int i = 1; i < nlanes; ++i)
        for (int q = 0; q < 3; ++q) {
          const int j = 3 * i + q;
          if (M->lane_bytes[j] >= need[j]) continue;
          if (M->lane_buf[j]) cudaFree(M->lane_buf[j]);
          M->lane_buf[j] = nullptr;
          M->lane_bytes[j] = 0;
          MF_CUDA(cudaMalloc(&M->lane_buf[j], std::max<size_t>(need[j], 16)));
          M->lane_bytes[j] = std::max<size_t>(need[j], 16);
        }
    }
  }
  std::vector<FactorLane<T>> lanes(nlanes);
  lanes[0] = FactorLane<T>{ctx->stream, reinterpret_cast<T*>(M->Pbuf), reinterpret_cast<T*>(M->Cbuf), M->gws,
                           M->gws_bytes};
  for (int i = 1; i < nlanes; ++i)
    lanes[i] = FactorLane<T>{M->bstreams[i - 1], reinterpret_cast<T*>(M->lane_buf[3 * i]),
                             reinterpret_cast<T*>(M->lane_buf[3 * i + 1]), M->lane_buf[3 * i + 2],
                             M->lane_bytes[3 * i + 2]};
  auto factor_level = [&](size_t l, const FactorLane<T>& lane) -> int {
    const MFLevel& L = S.levels[l];
    const int n = L.n, E = L.E;
    const int cnt = (int)L.count;
    const long long sn = (long long)n * n;  // front stride
    T* F0 = F + L.off;
    MF_CUDA(cudaMemsetAsync(F0, 0, sizeof(T) * (size_t)L.count * n * n, lane.st));
    { k_pad_diag<T><<<cnt, 128, 0, lane.st>>>(F, L.off, L.count, n, E, M->d.f_ne, L.first); gbmhd::count_launch(); }
    const int64_t nah = L.ah_end - L.ah_begin;
    if (nah > 0) {
      int64_t g = std::min<int64_t>((nah + 255) / 256, (int64_t)ctx->num_sms * 16);
      { k_arrowhead<T, V><<<(unsigned)g, 256, 0, lane.st>>>(Aval, M->d.ah_src, M->d.ah_dst, L.ah_begin, L.ah_end, F); gbmhd::count_launch(); }
    }
    if (l + 1 == S.levels.size() && d_reg && !S.reg_dst.empty()) {
      // the global p and φ representatives are eliminated in the root front
      const int64_t nr = (int64_t)S.reg_dst.size();
      { k_reg_add<T><<<(unsigned)std::min<int64_t>((nr + 255) / 256, 4096), 256, 0, lane.st>>>(F, M->d.reg_dst, M->d.reg_dof, d_reg, M->scaled ? M->d_dr : nullptr, M->d_dc, nr); gbmhd::count_launch(); }
    }
    const int64_t nch = L.ch_end - L.ch_begin;
    if (nch > 0) {
      int maxb = 0;
      for (int64_t c = L.ch_begin; c < L.ch_end; ++c) maxb = std::max(maxb, S.f_nb[S.child_list[c]]);
      const int gy = std::max(1, std::min(maxb, std::max(1, (int)(ctx->num_sms * 32 / nch))));
      dim3 grid((unsigned)nch, (unsigned)gy);
      { k_extend_add<T><<<grid, 256, 0, lane.st>>>(F, M->d.child_list, L.ch_begin, M->d.f_nb, M->d.f_off,
                                                     M->d.f_parent, M->d.f_level, M->d.ea_ptr, M->d.ea_pos, d_ln, d_le); gbmhd::count_launch(); }
    }
    MF_CUDA(cudaGetLastError());
    // Blocked right-looking LU of the eliminated block, by panels of PW pivots.  For each
    // NB-pivot block K of the panel: D_K⁻¹ (k_pivot_inverse*, partial pivoting inside the
    // block), L = M[below K, K]·D_K⁻¹, and the panel's later columns take L·M[K, ...].  The
    // panel's later blocks then update their rows beyond the panel (U), and the trailing
    // submatrix takes the whole panel in one rank-PW update.  D_K⁻¹ replaces M[K, K].
    for (int p = 0; p < E; p += PW) {
      const int pw = std::min(PW, E - p);
      for (int k = p; k < p + pw; k += NB) {
        const int kb = std::min(NB, p + pw - k);
        if constexpr (sizeof(T) == 4)
          {
            launch_pivot_inverse(pivot_variant(ctx, cnt, pk), cnt, lane.st, F, L.off, n, k, kb, lane.P, M->d_err);
            gbmhd::count_launch();
          }
        else
          { k_pivot_inverse<T><<<cnt, 256, 0, lane.st>>>(F, L.off, n, k, kb, lane.P, M->d_err); gbmhd::count_launch(); }
        const int rb = n - (k + kb);  // rows below the block (eliminated and boundary)
        if (rb > 0) {
          dim3 gc((unsigned)kb, (unsigned)cnt);
          { k_copy_block<T><<<gc, 256, 0, lane.st>>>(F, L.off, n, k + kb, rb, k, kb, lane.C); gbmhd::count_launch(); }
          MF_CUDA(cudaGetLastError());
          T* Lk = F0 + (k + kb) + (int64_t)k * n;  // M[below, K]
          const T* Dk = F0 + k + (int64_t)k * n;   // M[K, K], still the block itself
          const long long sC = (long long)n * NB, sP = (long long)NB * NB;
          int rc = 0;
          // L = A·D⁻¹ with one refinement step for FP32 factors:  L₀ = A·D⁻¹,  R = A − L₀·D,
          // L = L₀ + R·D⁻¹.  The FP32 inverse carries errors of κ(D)·2⁻²⁴; without the step they
          // enter the Schur complements (FP32 emulation, 24x24x4 at Ha = 500: 15 → 5 FGMRES
          // iterations to 1e-10 on the first Newton system).
          if ((rc = gemm<T>(ctx, M, lane, rb, kb, kb, one, lane.C, n, sC, lane.P, NB, sP, zero, Lk, n, sn, cnt))) return rc;
          if constexpr (sizeof(T) == 4) {
            if ((rc = gemm<T>(ctx, M, lane, rb, kb, kb, mone, Lk, n, sn, Dk, n, sn, one, lane.C, n, sC, cnt))) return rc;
            if ((rc = gemm<T>(ctx, M, lane, rb, kb, kb, one, lane.C, n, sC, lane.P, NB, sP, one, Lk, n, sn, cnt))) return rc;
          }
          const int cr = p + pw - (k + kb);  // the panel's later columns
          if (cr > 0 && (rc = gemm<T>(ctx, M, lane, rb, cr, kb, mone, Lk, n, sn, F0 + k + (int64_t)(k + kb) * n, n, sn,
                                      one, F0 + (k + kb) + (int64_t)(k + kb) * n, n, sn, cnt)))
            return rc;
        }
        { k_put_inverse<T><<<cnt, 256, 0, lane.st>>>(F, L.off, n, k, kb, lane.P); gbmhd::count_launch(); }
        MF_CUDA(cudaGetLastError());
      }
      const int c0 = p + pw, rest = n - c0;
      if (rest > 0) {
        int rc = 0;
        for (int k = p + NB; k < p + pw; k += NB) {  // U rows of the panel's later blocks
          const int kb = std::min(NB, p + pw - k);
          if ((rc = gemm<T>(ctx, M, lane, kb, rest, k - p, mone, F0 + k + (int64_t)p * n, n, sn, F0 + p + (int64_t)c0 * n, n,
                            sn, one, F0 + k + (int64_t)c0 * n, n, sn, cnt)))
            return rc;
        }
        // trailing update: M[c0:, c0:] −= M[c0:, panel] · M[panel, c0:]
        if ((rc = gemm<T>(ctx, M, lane, rest, rest, pw, mone, F0 + c0 + (int64_t)p * n, n, sn, F0 + p + (int64_t)c0 * n, n,
                          sn, one, F0 + c0 + (int64_t)c0 * n, n, sn, cnt)))
          return rc;
      }
    }
    return 0;
  };
  size_t fvn = 0;
  auto next_fev = [&]() { return M->fev[fvn++ % M->fev.size()]; };
  for (size_t la = 0; la < nlev;) {
    size_t lb = la + 1;
    while (lb < nlev && M->lheight[lb] == M->lheight[la]) ++lb;
    int used = 0;
    for (size_t l = la; l < lb; ++l) used = std::max(used, lane_of[l]);
    if (used > 0) {
      cudaEvent_t fork = next_fev();
      MF_CUDA(cudaEventRecord(fork, ctx->stream));
      for (int i = 1; i <= used; ++i) MF_CUDA(cudaStreamWaitEvent(lanes[i].st, fork, 0));
    }
    for (size_t l = la; l < lb; ++l) {
      if (ltimes) {
        MF_CUDA(cudaEventRecord(lev_ev[l], ctx->stream));
        lev_host[l] = std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
      }
      int rc = factor_level(l, lanes[lane_of[l]]);
      if (rc) return rc;
    }
    for (int i = 1; i <= used; ++i) {
      cudaEvent_t join = next_fev();
      MF_CUDA(cudaEventRecord(join, lanes[i].st));
      MF_CUDA(cudaStreamWaitEvent(ctx->stream, join, 0));
    }
    la = lb;
  }
  if (ltimes) {
    MF_CUDA(cudaEventRecord(lev_ev.back(), ctx->stream));
    lev_host.back() = std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
  }
  MF_CUDA(cudaFreeAsync(d_ln, ctx->stream));
  MF_CUDA(cudaFreeAsync(d_le, ctx->stream));
  int32_t herr = 0;
  MF_CUDA(cudaMemcpyAsync(&herr, M->d_err, sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
  MF_CUDA(cudaStreamSynchronize(ctx->stream));
  if (ltimes) {
    double dev_total = 0.0;
    for (size_t l = 0; l < S.levels.size(); ++l) {
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, lev_ev[l], lev_ev[l + 1]);
      dev_total += ms;
      std::fprintf(stderr, "mf level %2zu: fronts %6lld E %5d n %5d  device %8.3f ms  host issue %8.3f ms\n", l,
                   (long long)S.levels[l].count, S.levels[l].E, S.levels[l].n, ms,
                   1e3 * (lev_host[l + 1] - lev_host[l]));
    }
    std::fprintf(stderr, "mf levels: device %.3f ms (precision %d, pivot kernel %d)\n", dev_total, (int)sizeof(T), pk);
    for (cudaEvent_t e : lev_ev) cudaEventDestroy(e);
  }
  if (herr) {
    ctx->err = herr == 2 ? "multifrontal: a tensor-core GEMM wait timed out"
                         : "multifrontal: singular pivot block in the factorization";
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
  using U = typename RuizBits<V>::U;
  V* rmax = nullptr;
  U* cmax = nullptr;
  V *drv = nullptr, *dcv = nullptr;  // the factors in the value precision
  MF_CUDA(cudaMallocAsync(&rmax, sizeof(V) * std::max<int64_t>(n, 1), ctx->stream));
  MF_CUDA(cudaMallocAsync(&cmax, sizeof(U) * std::max<int64_t>(n, 1), ctx->stream));
  MF_CUDA(cudaMallocAsync(&drv, sizeof(V) * std::max<int64_t>(n, 1), ctx->stream));
  MF_CUDA(cudaMallocAsync(&dcv, sizeof(V) * std::max<int64_t>(n, 1), ctx->stream));
  const unsigned gw = (unsigned)std::max<int64_t>(1, std::min<int64_t>((n * 32 + 255) / 256, (int64_t)ctx->num_sms * 16));
  const unsigned gv = (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)ctx->num_sms * 8));
  { k_fill<<<gv, 256, 0, ctx->stream>>>(n, 1.0, M->d_dr); gbmhd::count_launch(); }
  { k_fill<<<gv, 256, 0, ctx->stream>>>(n, 1.0, M->d_dc); gbmhd::count_launch(); }
  { k_fill_t<V><<<gv, 256, 0, ctx->stream>>>(n, (V)1, drv); gbmhd::count_launch(); }
  { k_fill_t<V><<<gv, 256, 0, ctx->stream>>>(n, (V)1, dcv); gbmhd::count_launch(); }
  for (int it = 0; it < 3; ++it) {
    MF_CUDA(cudaMemsetAsync(cmax, 0, sizeof(U) * n, ctx->stream));
    { k_ruiz_max<V><<<gw, 256, 0, ctx->stream>>>(n, ctx->d_rowptr, ctx->d_col, val, drv, dcv, rmax, cmax); gbmhd::count_launch(); }
    { k_ruiz_update<V><<<gv, 256, 0, ctx->stream>>>(n, rmax, cmax, M->d_dr, M->d_dc, drv, dcv); gbmhd::count_launch(); }
  }
  { k_scale_vals<V><<<gw, 256, 0, ctx->stream>>>(n, ctx->d_rowptr, ctx->d_col, val, drv, dcv, reinterpret_cast<V*>(M->d_sval)); gbmhd::count_launch(); }
  MF_CUDA(cudaGetLastError());
  MF_CUDA(cudaFreeAsync(rmax, ctx->stream));
  MF_CUDA(cudaFreeAsync(cmax, ctx->stream));
  MF_CUDA(cudaFreeAsync(drv, ctx->stream));
  MF_CUDA(cudaFreeAsync(dcv, ctx->stream));
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

// Column chunk of the LDG GEMVs: wide enough that the partial-sum atomics stay a small
// fraction of the factor reads, narrow enough that a level with few fronts still launches
// about two waves of CTAs.
static int sweep_cols(const gbmhd_ctx* ctx, int64_t rows, int64_t ncols, int64_t fronts, int rows_per_cta) {
  const int64_t per_chunk = std::max<int64_t>(1, (rows + rows_per_cta - 1) / rows_per_cta) * std::max<int64_t>(1, fronts);
  const int64_t want = (int64_t)ctx->num_sms * 32;  // 2 waves of 16 resident 128-thread CTAs
  const int64_t chunks = std::max<int64_t>(1, (want + per_chunk - 1) / per_chunk);
  int64_t cols = (ncols + chunks - 1) / chunks;
  cols = ((cols + 31) / 32) * 32;
  return (int)std::max<int64_t>(64, std::min<int64_t>(cols, 1024));
}

// Columns per warp of the transposed FP32 GEMVs: 4 while a level still gives at least two
// 256-thread CTAs per SM, else fewer (levels with few, large fronts).  FP64 factors: 1.
#define GT_NC(k) (sizeof(T) == 4 ? (k) : 1)
// column groups of the chain kernels: FP64 factors (two rows per thread) use half as many,
// so that a CTA keeps at most 512 threads
#define TRI_G(k) (sizeof(T) == 4 ? (k) : 1)
#define TRI_GH(k) (sizeof(T) == 4 ? (k) : 1)
template <typename T>
static int gemv_t_cols(const gbmhd_ctx* ctx, int cols, int cnt) {
  if (sizeof(T) != 4) return 1;
  const int64_t want = 2LL * ctx->num_sms;
  for (int nc = 4; nc > 1; nc /= 2)
    if ((int64_t)cnt * ((cols + 8 * nc - 1) / (8 * nc)) >= want) return nc;
  return 1;
}

// Launch with programmatic stream serialization (the kernel's pdl_wait() orders it after the
// previous kernel of the stream; see pdl_wait).  Captured into the application's graph as a
// programmatic edge.
template <typename... KArgs, typename... Args>
static cudaError_t launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                              Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}

// TMA-staged chain of one super-block [s0, s1) of level l (FP32 factors with a chain map).
// Levels with many fronts: 128-thread CTAs and a ring of just enough slots for one step
// (several CTAs per SM); levels with few fronts: 512 threads and 12 slots (one CTA per SM,
// the ring a step and a half ahead).
template <int G, int NS>
static int chain_launch(gbmhd_ctx* ctx, MFNumeric* M, size_t l, bool fwd, int s0, int s1, int gather,
                        const double* b, double* x, cudaStream_t st) {
  const MFLevel& L = M->S.levels[l];
  const DevSym& d = M->d;
  const int sm = NS * CH_BOX_BYTES;
  if (fwd) {
    MF_CUDA(cudaFuncSetAttribute(k_chain_fwd<G, NS>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
    MF_CUDA(cudaFuncSetAttribute(k_chain_fwd<G, NS>, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    MF_CUDA(launch_pdl(k_chain_fwd<G, NS>, dim3((unsigned)L.count), dim3(128 * G), sm, st, M->cmaps[l],
                       L.first, M->tsave, (const int64_t*)M->tsave_off, b, (const int32_t*)d.elim,
                       (const int64_t*)d.elim_ptr, (const int32_t*)d.f_ne, L.E, s0, s1, gather, M->d_sweep_err,
                       M->wait_limit));
  } else {
    MF_CUDA(cudaFuncSetAttribute(k_chain_bwd<G, NS>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
    MF_CUDA(cudaFuncSetAttribute(k_chain_bwd<G, NS>, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    MF_CUDA(launch_pdl(k_chain_bwd<G, NS>, dim3((unsigned)L.count), dim3(128 * G), sm, st, M->cmaps[l],
                       L.first, (const double*)M->tsave, (const int64_t*)M->tsave_off, x, (const int32_t*)d.elim,
                       (const int64_t*)d.elim_ptr, (const int32_t*)d.f_ne, s0, s1, M->d_sweep_err,
                       M->wait_limit));
  }
  gbmhd::count_launch();
  MF_CUDA(cudaGetLastError());
  return 0;
}

template <int NS>
static int chain_launch_t(gbmhd_ctx* ctx, MFNumeric* M, size_t l, bool fwd, int s0, int s1, int gather,
                          const double* b, double* x) {
  const MFLevel& L = M->S.levels[l];
  const DevSym& d = M->d;
  const int sm = NS * CH_BOX_BYTES;
  if (fwd) {
    MF_CUDA(cudaFuncSetAttribute(k_chain_fwd_t<NS>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
    MF_CUDA(cudaFuncSetAttribute(k_chain_fwd_t<NS>, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    MF_CUDA(launch_pdl(k_chain_fwd_t<NS>, dim3((unsigned)L.count), dim3(CT_THREADS), sm, ctx->stream, M->cmaps[l],
                       L.first, M->tsave, (const int64_t*)M->tsave_off, b, (const int32_t*)d.elim,
                       (const int64_t*)d.elim_ptr, (const int32_t*)d.f_ne, L.E, s0, s1, gather, M->d_sweep_err,
                       M->wait_limit));
  } else {
    MF_CUDA(cudaFuncSetAttribute(k_chain_bwd_t<NS>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
    MF_CUDA(cudaFuncSetAttribute(k_chain_bwd_t<NS>, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    MF_CUDA(launch_pdl(k_chain_bwd_t<NS>, dim3((unsigned)L.count), dim3(CT_THREADS), sm, ctx->stream, M->cmaps[l],
                       L.first, (const double*)M->tsave, (const int64_t*)M->tsave_off, x, (const int32_t*)d.elim,
                       (const int64_t*)d.elim_ptr, (const int32_t*)d.f_ne, s0, s1, M->d_sweep_err,
                       M->wait_limit));
  }
  gbmhd::count_launch();
  MF_CUDA(cudaGetLastError());
  return 0;
}

static_assert(SB / NB <= 8, "the ring variants below hold the blocks of one step (nb <= 8)");
static int chain_tma_t(gbmhd_ctx* ctx, MFNumeric* M, size_t l, bool fwd, int s0, int s1, int gather,
                       const double* b, double* x) {
  const int nb = (s1 - s0 + NB - 1) / NB;
  if (M->S.levels[l].count >= 2 * ctx->num_sms) {
    if (nb <= 4) return chain_launch_t<4>(ctx, M, l, fwd, s0, s1, gather, b, x);
    if (nb <= 6) return chain_launch_t<6>(ctx, M, l, fwd, s0, s1, gather, b, x);
    return chain_launch_t<8>(ctx, M, l, fwd, s0, s1, gather, b, x);
  }
  return chain_launch_t<12>(ctx, M, l, fwd, s0, s1, gather, b, x);
}

static int chain_tma(gbmhd_ctx* ctx, MFNumeric* M, size_t l, bool fwd, int s0, int s1, int gather, const double* b,
                     double* x, cudaStream_t st) {
  const int nb = (s1 - s0 + NB - 1) / NB;
  if (M->S.levels[l].count >= 2 * ctx->num_sms) {
    if (nb <= 4) return chain_launch<1, 4>(ctx, M, l, fwd, s0, s1, gather, b, x, st);
    if (nb <= 6) return chain_launch<1, 6>(ctx, M, l, fwd, s0, s1, gather, b, x, st);
    return chain_launch<1, 8>(ctx, M, l, fwd, s0, s1, gather, b, x, st);
  }
  return chain_launch<4, 12>(ctx, M, l, fwd, s0, s1, gather, b, x, st);
}

// One application of the factors: x = A⁻¹ b (or A⁻ᵀ b when tr) on the factorized dofs.  Per
// level (forward bottom-up, backward top-down) and per super-block: the substitution chain
// (k_tri_*), then the GEMV beyond the super-block (k_rect / k_rect_tma, or k_rect_t for the
// transposed solve).  b is overwritten at the factorized dofs.
template <typename T>
static int solve_impl(gbmhd_ctx* ctx, MFNumeric* M, double* b, double* x, bool tr) {
  using V = typename SweepAcc<T>::V;
  const int rows_cta = SW_THREADS * RowVec<T>::R;
  const MFSymbolic& S = M->S;
  const T* F = reinterpret_cast<const T*>(M->F);
  const DevSym& d = M->d;
  // out[r] −= M[r0:r1, c0:c1] v   (dir: 0 forward map, 1 backward map)
  auto rect = [&](size_t l, int dir, int r0, int r1, int c0, int c1, int from_x,
                  cudaStream_t st = nullptr) -> int {
    if (!st) st = ctx->stream;
    const MFLevel& L = S.levels[l];
    if (r1 <= r0 || c1 <= c0) return 0;
    const int cnt = (int)L.count;
    if (sizeof(T) == 4 && M->map_ok[l]) {
      const int rows = M->map_rows[2 * l + dir];
      const int cw = tma_cols(ctx, r1 - r0, rows, c1 - c0, cnt);
      dim3 g((unsigned)((r1 - r0 + rows - 1) / rows), (unsigned)((c1 - c0 + cw - 1) / cw), (unsigned)cnt);
      const size_t sm = (size_t)TS_STAGES * TS_COLS * rows * sizeof(float) + sizeof(float2) * cw;
      MF_CUDA(cudaFuncSetAttribute(k_rect_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
      MF_CUDA(cudaFuncSetAttribute(k_rect_tma, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
      MF_CUDA(launch_pdl(k_rect_tma, g, dim3(rows / 2), sm, st, M->maps[2 * l + dir], L.first, L.E, r0, r1, c0,
                         c1, rows, cw, M->tsave, (const int64_t*)M->tsave_off, (const double*)x, b,
                         (const int32_t*)d.elim, (const int64_t*)d.elim_ptr, (const int32_t*)d.bnd,
                         (const int64_t*)d.bnd_ptr, (const int32_t*)d.f_ne, (const int32_t*)d.f_nb, from_x,
                         M->d_sweep_err, M->wait_limit));
      gbmhd::count_launch();
    } else {
      const int cols = sweep_cols(ctx, r1 - r0, c1 - c0, cnt, rows_cta);
      dim3 g((unsigned)((r1 - r0 + rows_cta - 1) / rows_cta), (unsigned)((c1 - c0 + cols - 1) / cols), (unsigned)cnt);
      { k_rect<T><<<g, SW_THREADS, sizeof(V) * cols, st>>>(F, d.f_off, M->tsave, M->tsave_off, x, b, d.elim,
            d.elim_ptr, d.bnd, d.bnd_ptr, d.f_ne, d.f_nb, L.first, L.n, L.E, r0, r1, c0, c1, cols, from_x); gbmhd::count_launch(); }
    }
    MF_CUDA(cudaGetLastError());
    return 0;
  };
  // out[c] −= M[r0:r1, c0:c1]ᵀ v
  auto rect_t = [&](size_t l, int r0, int r1, int c0, int c1, int from_x) -> int {
    const MFLevel& L = S.levels[l];
    if (r1 <= r0 || c1 <= c0) return 0;
    const int cnt = (int)L.count;
    const int ld = (r1 - r0 + 3) / 4 * 4;
    if (sizeof(T) == 4)
      { k_pack_front<<<cnt, 256, 0, ctx->stream>>>(M->tsave, M->tsave_off, x, d.elim, d.elim_ptr, d.bnd, d.bnd_ptr,
            d.f_ne, d.f_nb, L.first, L.E, r0, r1, ld, from_x, M->vpk); gbmhd::count_launch(); }
    const size_t sm = sizeof(T) == 4 ? 0 : sizeof(double) * (size_t)(r1 - r0);
    const int nc = gemv_t_cols<T>(ctx, c1 - c0, cnt);
    auto kf = nc == 4 ? k_rect_t<T, GT_NC(4)> : nc == 2 ? k_rect_t<T, GT_NC(2)> : k_rect_t<T, 1>;
    MF_CUDA(cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)std::max<size_t>(sm, 1)));
    dim3 g((unsigned)((c1 - c0 + 8 * nc - 1) / (8 * nc)), (unsigned)cnt);
    { kf<<<g, 256, sm, ctx->stream>>>(F, d.f_off, M->tsave, M->tsave_off, x, b, d.elim, d.elim_ptr, d.bnd, d.bnd_ptr,
          d.f_ne, d.f_nb, L.first, L.n, L.E, r0, r1, c0, c1, ld, from_x, M->vpk); gbmhd::count_launch(); }
    MF_CUDA(cudaGetLastError());
    return 0;
  };
  int rc = 0;
  // Levels of several super-blocks (FP32 factors with TMA maps): the GEMV of super-block j is
  // split into the next super-block's rows, which the next chain needs, and the rows beyond,
  // which run on the second stream beside that chain and join before chain j + 2.  (Their
  // partial sums are added atomically, so the two may overlap in their output rows.)
  size_t evn = 0;
  auto next_ev = [&]() { return M->sev[evn++ % M->sev.size()]; };
  // forward substitution of level l on stream st (the split GEMVs only on the context stream)
  auto fwd_level = [&](size_t l, cudaStream_t st) -> int {
    const MFLevel& L = S.levels[l];
    const int cnt = (int)L.count, n = L.n, E = L.E;
    const bool wide = cnt >= 2 * ctx->num_sms;  // many fronts: small CTAs, one wave
    const bool split = st == ctx->stream && !tr && sizeof(T) == 4 && M->map_ok[l] && M->cmap_ok[l] && E > SB;
    cudaEvent_t rest_done[2] = {nullptr, nullptr};  // the row GEMVs beyond of super-blocks j − 2, j − 1
    for (int s0 = 0, j = 0; s0 < E; s0 += SB, ++j) {
      const int s1 = std::min(E, s0 + SB);
      const int gather = s0 == 0;  // the first chain reads t = b[elim] for the whole front
      if (!tr) {
        constexpr int R = RowVec<T>::R;
        if (split && rest_done[j & 1]) MF_CUDA(cudaStreamWaitEvent(st, rest_done[j & 1], 0));
        if (sizeof(T) == 4 && M->cmap_ok[l]) {
          if ((rc = chain_tma(ctx, M, l, true, s0, s1, gather, b, x, st))) return rc;
        } else if (sizeof(T) == 8 || wide)
          { k_tri_fwd<T, 1><<<cnt, SB / R, 0, st>>>(F, d.f_off, M->tsave, M->tsave_off, b, d.elim, d.elim_ptr, d.f_ne, L.first, n, E, s0, s1, gather); gbmhd::count_launch(); }
        else
          { k_tri_fwd<T, TRI_G(4)><<<cnt, SB / R * TRI_G(4), 0, st>>>(F, d.f_off, M->tsave, M->tsave_off, b, d.elim, d.elim_ptr, d.f_ne, L.first, n, E, s0, s1, gather); gbmhd::count_launch(); }
        if (split && s1 < E) {
          const int s1n = std::min(E, s1 + SB);
          cudaEvent_t ec = next_ev(), eb = next_ev();
          MF_CUDA(cudaEventRecord(ec, st));
          MF_CUDA(cudaStreamWaitEvent(M->s2, ec, 0));
          if ((rc = rect(l, 0, s1n, n, s0, s1, 0, M->s2))) return rc;
          MF_CUDA(cudaEventRecord(eb, M->s2));
          rest_done[j & 1] = eb;
          if ((rc = rect(l, 0, s1, s1n, s0, s1, 0, st))) return rc;
        } else {
          if ((rc = rect(l, 0, s1, n, s0, s1, 0, st))) return rc;
        }
      } else {
        if (sizeof(T) == 4 && M->cmap_ok[l]) {
          if ((rc = chain_tma_t(ctx, M, l, true, s0, s1, gather, b, x))) return rc;
        } else
        { k_tri_fwd_t<T><<<cnt, TT_THREADS, 0, ctx->stream>>>(F, d.f_off, M->tsave, M->tsave_off, b, d.elim, d.elim_ptr, d.f_ne, L.first, n, E, s0, s1, gather); gbmhd::count_launch(); }
        if ((rc = rect_t(l, s0, s1, s1, n, 0))) return rc;
      }
    }
    for (cudaEvent_t e : rest_done)  // join the second stream before the next level
      if (e) MF_CUDA(cudaStreamWaitEvent(st, e, 0));
    MF_CUDA(cudaGetLastError());
    return 0;
  };
  // backward substitution of level l on stream st
  auto bwd_level = [&](size_t l, cudaStream_t st) -> int {
    const MFLevel& L = S.levels[l];
    const int cnt = (int)L.count, n = L.n, E = L.E;
    const int nsb = (E + SB - 1) / SB;
    // Backward split (as forward): the GEMV of super-block sb over the columns beyond
    // super-block sb + 1 needs the x of super-blocks ≥ sb + 2 only, so it runs on the second
    // stream after chain sb + 2 (the boundary columns: from the start of the level); the
    // columns of super-block sb + 1 follow chain sb + 1 on the main stream.
    const bool split = st == ctx->stream && !tr && sizeof(T) == 4 && M->map_ok[l] && M->cmap_ok[l] && nsb >= 2;
    std::vector<cudaEvent_t> rest_done(split ? nsb : 0, nullptr);
    auto launch_rest = [&](int sb) -> int {  // columns [start of super-block sb + 2, n) of the rows of sb
      const int r0 = sb * SB, r1 = std::min(E, r0 + SB), c0 = std::min(E, r1 + SB);
      cudaEvent_t ec = next_ev(), eb = next_ev();
      MF_CUDA(cudaEventRecord(ec, st));
      MF_CUDA(cudaStreamWaitEvent(M->s2, ec, 0));
      const int rc2 = rect(l, 1, r0, r1, c0, n, 1, M->s2);
      if (rc2) return rc2;
      MF_CUDA(cudaEventRecord(eb, M->s2));
      rest_done[sb] = eb;
      return 0;
    };
    if (split && (rc = launch_rest(nsb - 2))) return rc;
    for (int sb = nsb - 1; sb >= 0; --sb) {
      const int s0 = sb * SB, s1 = std::min(E, s0 + SB);
      if (!tr) {
        if (split && sb < nsb - 1) {
          if ((rc = rect(l, 1, s0, s1, s1, std::min(E, s1 + SB), 1, st))) return rc;
          MF_CUDA(cudaStreamWaitEvent(st, rest_done[sb], 0));
        } else {
          if ((rc = rect(l, 1, s0, s1, s1, n, 1, st))) return rc;
        }
        constexpr int W1 = 32 * NB / RowVec<T>::R / 4;  // threads of one column-group set
        if (sizeof(T) == 4 && M->cmap_ok[l]) {
          if ((rc = chain_tma(ctx, M, l, false, s0, s1, 0, b, x, st))) return rc;
        } else if (cnt >= ctx->num_sms || sizeof(T) == 8)
          { k_tri_bwd<T, 1><<<cnt, W1, 0, st>>>(F, d.f_off, M->tsave, M->tsave_off, x, d.elim, d.elim_ptr, d.f_ne, L.first, n, s0, s1); gbmhd::count_launch(); }
        else
          { k_tri_bwd<T, TRI_GH(4)><<<cnt, W1 * TRI_GH(4), 0, st>>>(F, d.f_off, M->tsave, M->tsave_off, x, d.elim, d.elim_ptr, d.f_ne, L.first, n, s0, s1); gbmhd::count_launch(); }
        if (split && sb >= 2 && (rc = launch_rest(sb - 2))) return rc;
      } else {
        if ((rc = rect_t(l, s1, n, s0, s1, 1))) return rc;
        if (sizeof(T) == 4 && M->cmap_ok[l]) {
          if ((rc = chain_tma_t(ctx, M, l, false, s0, s1, 0, b, x))) return rc;
        } else
        { k_tri_bwd_t<T><<<cnt, TT_THREADS, 0, ctx->stream>>>(F, d.f_off, M->tsave, M->tsave_off, x, d.elim, d.elim_ptr,
              d.f_ne, L.first, n, s0, s1); gbmhd::count_launch(); }
      }
    }
    MF_CUDA(cudaGetLastError());
    return 0;
  };
  // The level groups of one tree height are independent in both substitutions: a group reads
  // only the dofs its descendants (forward) or ancestors (backward) produce, writes its own
  // eliminated dofs, and adds into its ancestors' boundary dofs atomically.  So the groups of
  // one height run side by side: the first (the largest fronts) on the context stream, the
  // others on the branch streams, joined before the next height.  The transposed solve
  // shares one packing buffer between levels and keeps them in sequence.
  size_t fvn = 0;
  auto next_fev = [&]() { return M->fev[fvn++ % M->fev.size()]; };
  auto run_height = [&](size_t la, size_t lb, bool fwd) -> int {  // levels [la, lb), one height
    const bool conc = !tr && lb - la > 1 && !M->bstreams.empty();
    if (!conc) {
      for (size_t i = 0; i < lb - la; ++i) {
        const size_t l = fwd ? la + i : lb - 1 - i;
        if ((rc = fwd ? fwd_level(l, ctx->stream) : bwd_level(l, ctx->stream))) return rc;
      }
      return 0;
    }
    const size_t nbs = M->bstreams.size();
    cudaEvent_t fork = next_fev();
    MF_CUDA(cudaEventRecord(fork, ctx->stream));
    for (size_t i = 1; i < lb - la && i <= nbs; ++i) MF_CUDA(cudaStreamWaitEvent(M->bstreams[i - 1], fork, 0));
    for (size_t i = 0; i < lb - la; ++i) {
      const cudaStream_t st = i == 0 ? ctx->stream : M->bstreams[(i - 1) % nbs];
      if ((rc = fwd ? fwd_level(la + i, st) : bwd_level(la + i, st))) return rc;
    }
    for (size_t i = 1; i < lb - la && i <= nbs; ++i) {
      cudaEvent_t join = next_fev();
      MF_CUDA(cudaEventRecord(join, M->bstreams[i - 1]));
      MF_CUDA(cudaStreamWaitEvent(ctx->stream, join, 0));
    }
    return 0;
  };
  const size_t nlev = S.levels.size();
  for (size_t la = 0; la < nlev;) {  // forward, bottom-up
    size_t lb = la + 1;
    while (lb < nlev && M->lheight[lb] == M->lheight[la]) ++lb;
    if ((rc = run_height(la, lb, true))) return rc;
    la = lb;
  }
  for (size_t lb = nlev; lb > 0;) {  // backward, top-down
    size_t la = lb - 1;
    while (la > 0 && M->lheight[la - 1] == M->lheight[lb - 1]) --la;
    if ((rc = run_height(la, lb, false))) return rc;
    lb = la;
  }
  return 0;
}

// The scaled solve: x = Dc (Dr A Dc)⁻¹ Dr b, or Dr (Dr A Dc)⁻ᵀ Dc b; b is overwritten.
static int solve_scaled(gbmhd_ctx* ctx, MFNumeric* M, double* d_b, double* d_x, bool transpose) {
  const int64_t nd = ctx->ndofs;
  const unsigned gv = (unsigned)std::max<int64_t>(1, std::min<int64_t>((nd + 255) / 256, (int64_t)ctx->num_sms * 8));
  if (M->scaled) { k_scale_vec<<<gv, 256, 0, ctx->stream>>>(nd, transpose ? M->d_dc : M->d_dr, d_b); gbmhd::count_launch(); }
  const int rc = M->precision == GBMHD_MIXED ? solve_impl<float>(ctx, M, d_b, d_x, transpose)
                                             : solve_impl<double>(ctx, M, d_b, d_x, transpose);
  if (rc) return rc;
  if (M->scaled) { k_scale_vec<<<gv, 256, 0, ctx->stream>>>(nd, transpose ? M->d_dr : M->d_dc, d_x); gbmhd::count_launch(); }
  return 0;
}

// Graph of one application on the fixed buffers gb → gx (monolithic factors: every dof of
// x is written, so x's previous contents do not matter).  About 120 short kernels per
// application at 64x64x4; replaying them as one graph removes the launch gaps between them.
static int solve_graph(gbmhd_ctx* ctx, MFNumeric* M, double* d_b, double* d_x, bool tr) {
  const int64_t nd = ctx->ndofs;
  const int t = tr ? 1 : 0;
  if (!M->gb) {
    MF_CUDA(cudaMalloc(&M->gb, sizeof(double) * std::max<int64_t>(nd, 1)));
    MF_CUDA(cudaMalloc(&M->gx, sizeof(double) * std::max<int64_t>(nd, 1)));
  }
  MF_CUDA(cudaMemcpyAsync(M->gb, d_b, sizeof(double) * nd, cudaMemcpyDeviceToDevice, ctx->stream));
  if (!M->gexec[t] || M->g_factors[t] != M->F || M->g_prec[t] != M->precision) {
    if (M->gexec[t]) cudaGraphExecDestroy(M->gexec[t]);
    M->gexec[t] = nullptr;
    const int64_t k0 = gbmhd::launch_count();
    cudaGraph_t g = nullptr;
    MF_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    const int rc = solve_scaled(ctx, M, M->gb, M->gx, tr);
    const cudaError_t ec = cudaStreamEndCapture(ctx->stream, &g);
    if (rc || ec != cudaSuccess || !g) {
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();
      M->graphs_ok = false;  // launch directly from now on
      if (rc) return rc;
      return solve_scaled(ctx, M, d_b, d_x, tr);
    }
    const cudaError_t ei = cudaGraphInstantiate(&M->gexec[t], g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) {
      cudaGetLastError();
      M->gexec[t] = nullptr;
      M->graphs_ok = false;
      return solve_scaled(ctx, M, d_b, d_x, tr);
    }
    M->g_kernels[t] = gbmhd::launch_count() - k0;
    M->g_factors[t] = M->F;
    M->g_prec[t] = M->precision;
  } else {
    gbmhd::count_launch(M->g_kernels[t]);
  }
  MF_CUDA(cudaGraphLaunch(M->gexec[t], ctx->stream));
  MF_CUDA(cudaMemcpyAsync(d_x, M->gx, sizeof(double) * nd, cudaMemcpyDeviceToDevice, ctx->stream));
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
  const int rc = (M->S.monolithic && M->graphs_ok) ? solve_graph(ctx, M, d_b, d_x, transpose)
                                                   : solve_scaled(ctx, M, d_b, d_x, transpose);
  if (rc) return rc;
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

extern "C" int gbmhd_diag_pivot_inverse(int32_t variant, int32_t count, int32_t n, int32_t kb, const float* F, float* P,
                                        int32_t reps, double* ms_per_launch, int32_t* status) {
  if (variant < 0 || variant > 3 || count < 1 || n < 1 || kb < 1 || kb > NB || kb > n || !F || !P || reps < 0)
    return -1;
  int32_t* d_err = nullptr;
  if (cudaMalloc(&d_err, sizeof(int32_t)) != cudaSuccess) return -2;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = 0;
  if (cudaMemset(d_err, 0, sizeof(int32_t)) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
      cudaEventCreate(&e1) != cudaSuccess)
    rc = -2;
  if (!rc) {
    launch_pivot_inverse(variant, count, nullptr, F, 0, n, 0, kb, P, d_err);
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) rc = -2;
  }
  int32_t h = 0;
  if (!rc && cudaMemcpy(&h, d_err, sizeof(int32_t), cudaMemcpyDeviceToHost) != cudaSuccess) rc = -2;
  if (!rc && reps > 0) {
    cudaEventRecord(e0, nullptr);
    for (int r = 0; r < reps; ++r) launch_pivot_inverse(variant, count, nullptr, F, 0, n, 0, kb, P, d_err);
    cudaEventRecord(e1, nullptr);
    float ms = 0.0f;
    if (cudaGetLastError() != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
        cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
      rc = -2;
    if (ms_per_launch) *ms_per_launch = ms / reps;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(d_err);
  if (status) *status = h;
  return rc;
}
