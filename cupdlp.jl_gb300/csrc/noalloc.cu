// noalloc.cu — gpdhg_convergence_noalloc: termination statistics of a candidate solution
// computed without allocating any memory.
//
// Who needs it: callers that may not allocate on the GPU at the moment they want a
// solution checked — code inside a host that owns all device memory through its own pool
// (a Julia CUDA.jl or PyTorch caching allocator that must not be bypassed), a serving path
// with a fixed memory budget, or a process whose device memory is exhausted by design. They
// pass device pointers to the problem vectors, the candidate and its two products, and get
// back the reference's ConvergenceInformation.
//
// The call is synchronous: it ends by copying the statistics to the host and waiting for its
// stream. It therefore cannot run on a stream that is being captured into a CUDA graph; such a
// call is refused with GPDHG_ERR_NOT_SUPPORTED before any other CUDA call, which leaves the
// caller's capture intact.
//
// Scratch: one file-scope device array (kScratchDoubles doubles, 608.3 KiB), which every GPU
// that loads the library holds until the process exits. Its device address is looked up with
// cudaGetSymbolAddress, with the device current, on the first call in each CUDA context (once
// per device, again only if that device's context was destroyed and re-created, since the
// module and its symbol are reloaded then). Every call reuses the same array: each call
// overwrites all partials it reads, so nothing needs clearing, and calls that overlap on the
// GPU (two streams, or two host threads) race on it.
#include <cmath>
#include <cstring>
#include <mutex>

#include "eval_kernels.cuh"
#include "host_logic.h"

namespace gpdhg {
namespace {

constexpr int kNoallocItem = 4096;                                     // elements per CTA
constexpr long long kNoallocMaxLength = 1LL << 24;                     // n and m at most
constexpr int kNoallocMaxItems = (int)(kNoallocMaxLength / kNoallocItem);
constexpr int kQn = 10, kQm = 9;
constexpr int kScratchDoubles = (kQn + kQm) * kNoallocMaxItems + 32;

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

enum { kA_LuSq = 0, kA_LuMax, kA_Cx, kA_XMax, kA_XSq, kA_RcvSq, kA_RcvMax, kA_Contrib, kA_CSq, kA_CMax };
constexpr unsigned kAMax = (1u << kA_LuMax) | (1u << kA_XMax) | (1u << kA_RcvMax) | (1u << kA_CMax);
enum { kB_CvSq = 0, kB_CvMax, kB_DrSq, kB_DrMax, kB_By, kB_YMax, kB_YSq, kB_BSq, kB_BMax };
constexpr unsigned kBMax = (1u << kB_CvMax) | (1u << kB_DrMax) | (1u << kB_YMax) | (1u << kB_BMax);

// Column side: bound violations, objective, reduced costs of g = c - A'y (the statistics of
// compute_primal_residual!, primal_obj and compute_dual_stats!, src/iteration_stats_utils_gpu.jl:71-238).
struct ColumnStats {
  const double *l, *u, *c, *x, *aty;
  __device__ __forceinline__ void operator()(long long j, double* a) const {
    const double xv = x[j], lv_ = l[j], uv_ = u[j], cv = c[j];
    const bool fl = isfinite(lv_), fu = isfinite(uv_);
    const double lv = jmax(lv_ - xv, 0.0), uv = jmax(xv - uv_, 0.0);
    a[kA_LuSq] += lv * lv + uv * uv;
    a[kA_LuMax] = nan_max(a[kA_LuMax], nan_max(lv, uv));
    a[kA_Cx] += cv * xv;
    a[kA_XMax] = nan_max(a[kA_XMax], fabs(xv));
    a[kA_XSq] += xv * xv;
    const double g = cv - aty[j];
    const double rc = reduced_cost(g, fl, fu);
    const double rcv = g - rc;
    a[kA_RcvSq] += rcv * rcv;
    a[kA_RcvMax] = nan_max(a[kA_RcvMax], fabs(rcv));
    a[kA_Contrib] += rc_contribution(rc, lv_, uv_);
    a[kA_CSq] += cv * cv;
    a[kA_CMax] = nan_max(a[kA_CMax], fabs(cv));
  }
};

// Row side: constraint violations of A x, dual sign violations, b'y.
struct RowStats {
  const double *b, *y, *ax;
  int neq;
  __device__ __forceinline__ void operator()(long long i, double* a) const {
    const double bv = b[i], yv = y[i];
    const bool ineq = i >= neq;
    double cv = bv - ax[i];
    if (ineq) cv = jmax(cv, 0.0);
    a[kB_CvSq] += cv * cv;
    a[kB_CvMax] = nan_max(a[kB_CvMax], fabs(cv));
    if (ineq) {
      const double dr = jmax(-yv, 0.0);
      a[kB_DrSq] += dr * dr;
      a[kB_DrMax] = nan_max(a[kB_DrMax], dr);
    }
    a[kB_By] += bv * yv;
    a[kB_YMax] = nan_max(a[kB_YMax], fabs(yv));
    a[kB_YSq] += yv * yv;
    a[kB_BSq] += bv * bv;
    a[kB_BMax] = nan_max(a[kB_BMax], fabs(bv));
  }
};

// The segmented reduction of the solver with its item list implied by the block index
// (item k = [k * 4096, (k + 1) * 4096)) and its partials in the caller-free scratch.
template <int Q, unsigned MAXMASK, class F>
__global__ void __launch_bounds__(kBlock) noalloc_reduce_kernel(long long len, F f, double* partials, int nitems) {
  __shared__ double sh[32];
  double acc[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) acc[q] = 0.0;
  const long long b = (long long)blockIdx.x * kNoallocItem;
  const long long e = b + kNoallocItem < len ? b + kNoallocItem : len;
  for (long long i = b + threadIdx.x; i < e; i += kBlock) f(i, acc);
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const double r = ((MAXMASK >> q) & 1u) ? block_nan_max(acc[q], sh) : block_sum(acc[q], sh);
    if (threadIdx.x == 0) partials[(size_t)q * nitems + blockIdx.x] = r;
  }
}

template <int Q, unsigned MAXMASK>
__global__ void __launch_bounds__(kBlock) noalloc_finalize_kernel(const double* partials, int nitems, double* out) {
  __shared__ double sh[32];
  for (int q = 0; q < Q; ++q) {
    const bool is_max = (MAXMASK >> q) & 1u;
    double a = 0.0;
    for (int k = threadIdx.x; k < nitems; k += kBlock) {
      const double v = partials[(size_t)q * nitems + k];
      a = is_max ? nan_max(a, v) : a + v;
    }
    a = is_max ? block_nan_max(a, sh) : block_sum(a, sh);
    if (threadIdx.x == 0) out[q] = a;
  }
}

using CtxGetIdFn = int (*)(void* ctx, unsigned long long* id);   // cuCtxGetId

// Id of the current CUDA context through the driver entry point (cudart is linked statically,
// libcuda is not); 0 when there is none yet.
unsigned long long current_context_id() {
  static CtxGetIdFn fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      f = nullptr;
    }
    return reinterpret_cast<CtxGetIdFn>(f);
  }();
  if (!fn) throw Error(GPDHG_ERR_CUDA, "cuCtxGetId is not available from the driver");
  unsigned long long id = 0;
  return fn(nullptr, &id) == 0 ? id : 0ULL;
}

struct ScratchAddress {
  unsigned long long context = 0;
  double* ptr = nullptr;
};
std::mutex g_addr_mutex;
ScratchAddress g_addr[256];

// Device address of the scratch array in the current device's current context: looked up
// once per context, so a device whose context was reset gets the reloaded module's address.
double* scratch_address() {
  int dev = 0;
  CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 256) throw Error(GPDHG_ERR_CUDA, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_addr_mutex);
  ScratchAddress& a = g_addr[dev];
  const unsigned long long ctx = current_context_id();
  if (!a.ptr || ctx == 0 || ctx != a.context) {
    void* p = nullptr;
    CK(cudaGetSymbolAddress(&p, g_noalloc_scratch));   // makes the device's primary context current
    a.ptr = static_cast<double*>(p);
    a.context = current_context_id();
    if (a.context == 0) throw Error(GPDHG_ERR_CUDA, "no current CUDA context after the symbol lookup");
  }
  return a.ptr;
}

}  // namespace
}  // namespace gpdhg

namespace gpdhg {

void convergence_noalloc(int32_t n, int32_t m, int32_t neq, double obj_const, const double* l, const double* u,
                         const double* c, const double* b, const double* x, const double* y, const double* ax,
                         const double* aty, double eps_abs, double eps_rel, void* stream,
                         gpdhg_convergence_information* out) {
  if (!out || !l || !u || !c || !x || !aty) throw Error(GPDHG_ERR_INVALID_ARGUMENT, "required pointer is NULL");
  if (n <= 0 || m < 0 || neq < 0 || neq > m)
    throw Error(GPDHG_ERR_INVALID_ARGUMENT, "need n > 0 and 0 <= num_equalities <= m");
  if (m > 0 && (!b || !y || !ax)) throw Error(GPDHG_ERR_INVALID_ARGUMENT, "row-side pointer is NULL");
  if ((long long)n > kNoallocMaxLength || (long long)m > kNoallocMaxLength)
    throw Error(GPDHG_ERR_INVALID_ARGUMENT,
                "gpdhg_convergence_noalloc handles at most 16,777,216 variables and constraints");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // A capturing stream cannot take the synchronous read-back at the end; refuse before any
  // other CUDA call so that the caller's capture is left valid.
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  const cudaError_t ce = cudaStreamIsCapturing(s, &cap);
  if (ce != cudaSuccess || cap != cudaStreamCaptureStatusNone) {
    if (ce != cudaSuccess) cudaGetLastError();
    throw Error(GPDHG_ERR_NOT_SUPPORTED,
                "gpdhg_convergence_noalloc is synchronous and cannot run on a stream that is being captured");
  }
  double* base = scratch_address();
  double* part_n = base;
  double* part_m = base + (size_t)kQn * kNoallocMaxItems;
  double* outs = base + (size_t)(kQn + kQm) * kNoallocMaxItems;
  const int in = (int)((n + kNoallocItem - 1) / kNoallocItem);
  const int im = (int)((m + kNoallocItem - 1) / kNoallocItem);
  noalloc_reduce_kernel<kQn, kAMax><<<in, kBlock, 0, s>>>(n, ColumnStats{l, u, c, x, aty}, part_n, in);
  CK_LAUNCH();
  if (im > 0) {
    noalloc_reduce_kernel<kQm, kBMax><<<im, kBlock, 0, s>>>(m, RowStats{b, y, ax, neq}, part_m, im);
    CK_LAUNCH();
  }
  noalloc_finalize_kernel<kQn, kAMax><<<1, kBlock, 0, s>>>(part_n, in, outs);
  CK_LAUNCH();
  noalloc_finalize_kernel<kQm, kBMax><<<1, kBlock, 0, s>>>(part_m, im, outs + 16);
  CK_LAUNCH();
  double h[32];
  CK(cudaMemcpyAsync(h, outs, sizeof(h), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  const double* A = h;
  const double* B = h + 16;
  // compute_convergence_information (src/iteration_stats_utils_gpu.jl:251-309) with the
  // CachedQuadraticProgramInfo norms of this problem (src/termination.jl:130-137)
  const double linf_c = A[kA_CMax], l2_c = std::sqrt(A[kA_CSq]);
  const double linf_b = B[kB_BMax], l2_b = std::sqrt(B[kB_BSq]);
  const double eps_ratio = eps_abs / eps_rel;
  gpdhg_convergence_information ci;
  std::memset(&ci, 0, sizeof(ci));
  ci.candidate_type = GPDHG_POINT_TYPE_CURRENT_ITERATE;
  ci.primal_objective = obj_const + A[kA_Cx];
  ci.l_inf_primal_residual = jmax_h(B[kB_CvMax], A[kA_LuMax]);
  ci.l2_primal_residual = std::sqrt(B[kB_CvSq] + A[kA_LuSq]);
  ci.relative_l_inf_primal_residual = ci.l_inf_primal_residual / (eps_ratio + linf_b);
  ci.relative_l2_primal_residual = ci.l2_primal_residual / (eps_ratio + l2_b);
  ci.l_inf_primal_variable = A[kA_XMax];
  ci.l2_primal_variable = std::sqrt(A[kA_XSq]);
  const double dual_res_inf = jmax_h(B[kB_DrMax], A[kA_RcvMax]);
  ci.dual_objective = B[kB_By] + obj_const + A[kA_Contrib];
  ci.l_inf_dual_residual = dual_res_inf;
  ci.l2_dual_residual = std::sqrt(B[kB_DrSq] + A[kA_RcvSq]);
  ci.relative_l_inf_dual_residual = ci.l_inf_dual_residual / (eps_ratio + linf_c);
  ci.relative_l2_dual_residual = ci.l2_dual_residual / (eps_ratio + l2_c);
  ci.l_inf_dual_variable = B[kB_YMax];
  ci.l2_dual_variable = std::sqrt(B[kB_YSq]);
  ci.corrected_dual_objective = dual_res_inf == 0.0 ? ci.dual_objective : -INFINITY;
  const double gap = std::fabs(ci.primal_objective - ci.dual_objective);
  ci.relative_optimality_gap = gap / (eps_ratio + std::fabs(ci.primal_objective) + std::fabs(ci.dual_objective));
  *out = ci;
}

}  // namespace gpdhg
