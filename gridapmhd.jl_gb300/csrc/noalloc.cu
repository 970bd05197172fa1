// Allocation-free evaluation of the parameter gradient of the discrete adjoint.
//
// gbmhd_adjoint allocates device buffers on every call (the state, the objective
// gradient, the adjoint vector, dR/dθ work vectors).  Some hosts cannot allocate device
// memory while they iterate: an optimisation or uncertainty-quantification driver that
// runs the gradient inside a loop whose device memory was reserved up front by its own
// pool (CUDA.jl or a PyTorch caching allocator holding the device), or an embedded
// solver that is not allowed to call cudaMalloc/cudaFree after initialisation.  Once
// such a host has the adjoint vector λ (from its own solve, or from gbmhd_adjoint
// called during set-up), this entry point turns λ into dJ/dγ and dJ/dcw without
// allocating: its scratch lives in a file-scope device array of fixed size.
//
// Scratch: g_noalloc_scratch holds one partial product per cell (dJ/dγ) and one per
// thin-wall facet (dJ/dcw); 262,144 cells + 65,536 facets, 2.5 MiB, held on every device
// that loads the library until the process exits.  Each call writes every slot it later
// reads, so nothing needs to be cleared between calls; calls that overlap on the GPU
// (two streams, or two contexts on one device) share the array and race.
//
// The device address of the array is looked up (cudaGetSymbolAddress) on the first call
// made on a device, with that device current (the call checks that it is the context's
// device); make that first call before any stream capture on the device.  The address is
// cached per device for the life of the process: a cudaDeviceReset unloads the module and
// invalidates it, so do not call this entry point after resetting a device.
#include <mutex>

#include "internal.h"

namespace gbmhd {
namespace {

constexpr int64_t kNoAllocMaxCells = 1 << 18;
constexpr int64_t kNoAllocMaxFacets = 1 << 16;
__device__ __align__(256) double g_noalloc_scratch[kNoAllocMaxCells + kNoAllocMaxFacets];

std::mutex g_noalloc_mutex;
constexpr int kMaxDevices = 64;
double* g_noalloc_ptr[kMaxDevices] = {nullptr};

// ∂R/∂γ = −∫(j×B)·v on the u rows; slot[cell] = Σ_a λ_row(a) ∂R_a/∂γ.
__global__ void __launch_bounds__(128) k_noalloc_gamma(int64_t ncells, int64_t ndofs, const double* __restrict__ cellX,
                                                       const int32_t* __restrict__ gidx, const int32_t* __restrict__ row,
                                                       const unsigned long long* __restrict__ sign,
                                                       const double* __restrict__ x, const double* __restrict__ xfull,
                                                       const DevTables<double>* __restrict__ tb, DevParams P, const double* __restrict__ lam,
                                                       double* __restrict__ slot) {
  __shared__ double X[24], vj[36], wdet[NQ], jxB[NQ][3], red[4];
  const int tid = threadIdx.x;
  for (int64_t cell = blockIdx.x; cell < ncells; cell += gridDim.x) {
    __syncthreads();
    const unsigned long long sgn = sign ? sign[cell] : 0ull;
    if (tid < 24) X[tid] = cellX[cell * 24 + tid];
    if (tid < 36) {
      const int32_t gi = gidx[cell * ND + OJ + tid];
      const double v = gi < ndofs ? x[gi] : xfull[gi];  // free values from x, Dirichlet values from the context
      vj[tid] = v * (((sgn >> tid) & 1ull) ? -1.0 : 1.0);
    }
    __syncthreads();
    if (tid < NQ) {
      const int q = tid;
      double J[3][3];
      for (int i = 0; i < 3; ++i)
        for (int a = 0; a < 3; ++a) {
          double s = 0.0;
          for (int v = 0; v < 8; ++v) s += X[3 * v + i] * tb->gq1[q][v][a];
          J[i][a] = s;
        }
      const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                         J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                         J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
      wdet[q] = tb->w[q] * det;
      double j[3] = {0, 0, 0};
      for (int b = 0; b < 36; ++b) {
        const int d = b / 12;
        for (int i = 0; i < 3; ++i) j[i] += vj[b] * J[i][d] / det * tb->rt[q][b];
      }
      jxB[q][0] = j[1] * P.B[2] - j[2] * P.B[1];
      jxB[q][1] = j[2] * P.B[0] - j[0] * P.B[2];
      jxB[q][2] = j[0] * P.B[1] - j[1] * P.B[0];
    }
    __syncthreads();
    double acc = 0.0;
    if (tid < 81) {
      const int c = tid / 27, n = tid % 27;
      const int32_t r = row[cell * ND + tid];
      if (r >= 0) {
        double s = 0.0;
        for (int q = 0; q < NQ; ++q) s += wdet[q] * (-jxB[q][c] * tb->n2[q][n]);
        acc = lam[r] * s;
      }
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((tid & 31) == 0) red[tid >> 5] = acc;
    __syncthreads();
    if (tid == 0) slot[cell] = red[0] + red[1] + red[2] + red[3];
  }
}
// ∂R/∂cw = τ∫(s·n)(n·∇j·n) on thin-wall facets; slot[e] = Σ_a λ_row(a) ∂R_a/∂cw.
__global__ void __launch_bounds__(64) k_noalloc_cw(int64_t nfacets, int64_t ndofs, const int32_t* __restrict__ fcell,
                                                   const int8_t* __restrict__ flface, const double* __restrict__ fprm,
                                                   const double* __restrict__ cellX, const int32_t* __restrict__ gidx,
                                                   const int32_t* __restrict__ row,
                                                   const unsigned long long* __restrict__ sign,
                                                   const double* __restrict__ x, const double* __restrict__ xfull,
                                                   const FacetTables* __restrict__ ft, const double* __restrict__ lam,
                                                   double* __restrict__ slot) {
  __shared__ double X[24], vj[36], gnn[NQF][36], sn[NQF][36], dA[NQF], red[2];
  __shared__ int32_t rw[36];
  const int tid = threadIdx.x;
  for (int64_t e = blockIdx.x; e < nfacets; e += gridDim.x) {
    __syncthreads();
    const int64_t cell = fcell[e];
    const int f = flface[e];
    const int ax = f / 2, side = f % 2;
    const unsigned long long sgn = sign ? sign[cell] : 0ull;
    if (tid < 24) X[tid] = cellX[cell * 24 + tid];
    if (tid < 36) {
      const int32_t gi = gidx[cell * ND + OJ + tid];
      vj[tid] = gi < ndofs ? x[gi] : xfull[gi];
      rw[tid] = row[cell * ND + OJ + tid];
    }
    __syncthreads();
    if (tid < NQF) {
      const int t = tid;
      double J[3][3];
      for (int i = 0; i < 3; ++i)
        for (int a = 0; a < 3; ++a) {
          double s = 0.0;
          for (int v = 0; v < 8; ++v) s += X[3 * v + i] * ft->fgq1[f][t][v][a];
          J[i][a] = s;
        }
      const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                         J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                         J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
      const double id = 1.0 / det;
      double Ji[3][3];
      Ji[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) * id;
      Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
      Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
      Ji[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) * id;
      Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
      Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
      Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) * id;
      Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
      Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
      double n[3];
      for (int i = 0; i < 3; ++i) n[i] = Ji[ax][i] * (side ? 1.0 : -1.0);
      const double nl = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
      for (int i = 0; i < 3; ++i) n[i] /= nl;
      dA[t] = ft->fw[t] * fabs(det) * nl;
      double nJinv[3];
      for (int a = 0; a < 3; ++a) nJinv[a] = n[0] * Ji[a][0] + n[1] * Ji[a][1] + n[2] * Ji[a][2];
      for (int b = 0; b < 36; ++b) {
        const int d = b / 12;
        const double sg = ((sgn >> b) & 1ull) ? -1.0 : 1.0;
        const double nJd = n[0] * J[0][d] + n[1] * J[1][d] + n[2] * J[2][d];
        sn[t][b] = sg * nJd * id * ft->frt[f][t][b];
        const double* g = ft->frtg[f][t][b];
        gnn[t][b] = sg * id * (nJinv[0] * g[0] + nJinv[1] * g[1] + nJinv[2] * g[2]) * nJd;
      }
    }
    __syncthreads();
    const double tau = fprm[4 * e + 0];
    double acc = 0.0;
    if (tid < 36 && rw[tid] >= 0) {
      double s = 0.0;
      for (int t = 0; t < NQF; ++t) {
        double jnn = 0.0;
        for (int b = 0; b < 36; ++b) jnn += vj[b] * gnn[t][b];
        s += dA[t] * tau * sn[t][tid] * jnn;
      }
      acc = lam[rw[tid]] * s;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((tid & 31) == 0) red[tid >> 5] = acc;
    __syncthreads();
    if (tid == 0) slot[e] = red[0] + red[1];
  }
}

// out[k] = −Σ slot_k (one CTA per output; fixed summation order, so repeated calls agree bit for bit).
__global__ void __launch_bounds__(256) k_noalloc_sum(const double* __restrict__ cells, int64_t ncells,
                                                    const double* __restrict__ facets, int64_t nfacets,
                                                    double* __restrict__ out) {
  __shared__ double red[256];
  const double* src = blockIdx.x == 0 ? cells : facets;
  const int64_t n = blockIdx.x == 0 ? ncells : nfacets;
  double acc = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) acc += src[i];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = -red[0];
}

}  // namespace
}  // namespace gbmhd

using namespace gbmhd;

extern "C" int gbmhd_param_gradient_noalloc(gbmhd_ctx* ctx, const double* d_x, const double* d_lambda,
                                            double* d_out) {
  if (!ctx) return -1;
  if (!d_x || !d_lambda || !d_out) { ctx->err = "param_gradient_noalloc: NULL argument"; return -1; }
  if (ctx->ncells > kNoAllocMaxCells) {
    ctx->err = "param_gradient_noalloc: " + std::to_string(ctx->ncells) + " cells exceed the scratch limit of " +
               std::to_string(kNoAllocMaxCells);
    return -1;
  }
  if (ctx->nfacets > kNoAllocMaxFacets) {
    ctx->err = "param_gradient_noalloc: " + std::to_string(ctx->nfacets) + " facets exceed the scratch limit of " +
               std::to_string(kNoAllocMaxFacets);
    return -1;
  }
  // The address is looked up with the context's device current: the kernels run on the
  // context's stream, which belongs to that device.
  int cur = 0;
  GB_CUDA(cudaGetDevice(&cur));
  if (cur != ctx->device) {
    ctx->err = "param_gradient_noalloc: device " + std::to_string(cur) + " is current but the context lives on device " +
               std::to_string(ctx->device) + "; make the context's device current first";
    return -1;
  }
  const int dev = ctx->device;
  if (dev < 0 || dev >= kMaxDevices) { ctx->err = "param_gradient_noalloc: device id out of range"; return -1; }
  double* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
      // host code may not use &g_noalloc_scratch: ask the runtime for its device address
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess) {
        ctx->err = std::string("param_gradient_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e);
        return -2;
      }
      g_noalloc_ptr[dev] = static_cast<double*>(p);
    }
    scratch = g_noalloc_ptr[dev];
  }
  double* cell_slots = scratch;
  double* facet_slots = scratch + kNoAllocMaxCells;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(ctx->ncells, (int64_t)ctx->num_sms * 8));
  { k_noalloc_gamma<<<grid, 128, 0, ctx->stream>>>(ctx->ncells, ctx->ndofs, ctx->d_cellX, ctx->d_gidx, ctx->d_row,
        reinterpret_cast<const unsigned long long*>(ctx->d_sign), d_x, ctx->d_xfull,
        reinterpret_cast<const DevTables<double>*>(ctx->d_tab64), ctx->prm, d_lambda,
        cell_slots); gbmhd::count_launch(); }
  if (ctx->nfacets > 0) {
    const int gf = (int)std::min<int64_t>(ctx->nfacets, (int64_t)ctx->num_sms * 8);
    { k_noalloc_cw<<<gf, 64, 0, ctx->stream>>>(ctx->nfacets, ctx->ndofs, ctx->d_fcellid, ctx->d_flface, ctx->d_fprm,
          ctx->d_cellX, ctx->d_gidx, ctx->d_row, reinterpret_cast<const unsigned long long*>(ctx->d_sign), d_x,
          ctx->d_xfull, reinterpret_cast<const FacetTables*>(ctx->d_ftab), d_lambda, facet_slots); gbmhd::count_launch(); }
  }
  { k_noalloc_sum<<<2, 256, 0, ctx->stream>>>(cell_slots, ctx->ncells, facet_slots, ctx->nfacets, d_out); gbmhd::count_launch(); }
  GB_CUDA(cudaGetLastError());
  return 0;
}
