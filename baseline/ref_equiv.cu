// ref_equiv.cu — the reference's solve loop on the GPU in the reference's own form: a
// baseline to measure the library against on the same GPU, never linked by the product.
//
// cuPDLP.jl (Julia, CUDA.jl) cannot be installed where this is built or run, so this file
// makes the calls its solve loop makes, in its order and with its synchronisation:
//   * one kernel per reference kernel or fused broadcast (`.=`, `.+=`), FP64 throughout;
//     the step kernels are followed by a device synchronisation (`CUDA.@sync`,
//     src/primal_dual_hybrid_gradient_gpu.jl:213,277);
//   * cuSPARSE SpMV with CUSPARSE_SPMV_CSR_ALG2 on CSR(A) and on an explicit CSR(A')
//     (`CUDA.CUSPARSE.mv!`, :225 and :307), int32 indices;
//   * `CUDA.dot` / `CUDA.norm` as cuBLAS ddot / dnrm2 with their results returned to the
//     host (:329-333), `norm(., Inf)` and `sum` as a device reduction read back by the host;
//   * weighted sums `s .+= v * w` as two kernels (the product allocates a temporary in
//     CUDA.jl; here it is preallocated), src/saddle_point_gpu.jl:131-221;
//   * evaluation (src/iteration_stats_utils_gpu.jl:71-502): violation vectors written by
//     kernels, concatenations copied into one buffer, then one reduction each.
// The host logic (take_step!, run_restart_scheme, compute_new_primal_weight,
// check_termination_criteria) follows src/primal_dual_hybrid_gradient_gpu.jl:343-798,
// src/saddle_point_gpu.jl:419-692 and src/termination.jl:142-246 step for step.
// Device memory is allocated once up front (CUDA.jl's pool makes its per-step temporaries
// cheap; allocating them here per step would penalise the baseline).
#include <cublas_v2.h>
#include <cuda_runtime.h>
#include <cusparse.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>

#include "gpdhg.h"

namespace {

constexpr int kThreads = 128;   // ThreadPerBlock of the reference
constexpr double kInf = std::numeric_limits<double>::infinity();

struct Fail : std::runtime_error {
  using std::runtime_error::runtime_error;
};
#define RQ(x)                                                                                 \
  do {                                                                                        \
    cudaError_t e_ = (x);                                                                     \
    if (e_ != cudaSuccess) throw Fail(std::string(#x) + ": " + cudaGetErrorString(e_));       \
  } while (0)
#define RQS(x)                                                                                \
  do {                                                                                        \
    cusparseStatus_t e_ = (x);                                                                \
    if (e_ != CUSPARSE_STATUS_SUCCESS) throw Fail(std::string(#x) + " failed");              \
  } while (0)
#define RQB(x)                                                                                \
  do {                                                                                        \
    cublasStatus_t e_ = (x);                                                                  \
    if (e_ != CUBLAS_STATUS_SUCCESS) throw Fail(std::string(#x) + " failed");                \
  } while (0)

inline double jmax(double a, double b) { return (a != a || b != b) ? NAN : (a > b ? a : b); }
inline double jmin(double a, double b) { return (a != a || b != b) ? NAN : (a < b ? a : b); }
__device__ __forceinline__ double dmax(double a, double b) { return (a != a || b != b) ? NAN : (a > b ? a : b); }
__device__ __forceinline__ double dmin(double a, double b) { return (a != a || b != b) ? NAN : (a < b ? a : b); }

inline unsigned blocks(long long n) { return (unsigned)std::max<long long>(1, (n + kThreads - 1) / kThreads); }

template <class T>
struct Dev {
  T* p = nullptr;
  long long n = 0;
  void alloc(long long k) {
    n = k;
    RQ(cudaMalloc(&p, sizeof(T) * std::max<long long>(k, 1)));
  }
  ~Dev() {
    if (p) cudaFree(p);
  }
  operator T*() const { return p; }
};

// ---- kernels of the step (src/primal_dual_hybrid_gradient_gpu.jl:177-292) --------------------

__global__ void next_primal_kernel(const double* c, const double* l, const double* u, const double* x,
                                   const double* kty, double step, double pw, long long n, double* dx) {
  const long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (j < n) {
    double v = x[j] - (step / pw) * (c[j] - kty[j]);
    v = dmin(u[j], dmax(l[j], v));
    dx[j] = v - x[j];
  }
}

__global__ void next_dual_kernel(const double* b, const double* y, const double* kx, const double* dkx, double step,
                                 double pw, long long neq, long long m, double* dy) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < m) {
    double v = y[i] + (pw * step) * (b[i] - 2.0 * dkx[i] - 1.0 * kx[i]);
    if (i >= neq) v = dmax(v, 0.0);
    dy[i] = v - y[i];
  }
}

// ---- broadcasts (one CUDA.jl kernel each) ---------------------------------------------------

__global__ void add_kernel(double* a, const double* b, long long n) {   // a .+= b
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) a[i] += b[i];
}
__global__ void scale_kernel(double* out, const double* a, double w, long long n) {   // out = a * w
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) out[i] = a[i] * w;
}
__global__ void div_kernel(double* out, const double* a, double w, long long n) {   // out .= a ./ w
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) out[i] = a[i] / w;
}
__global__ void neg_div_kernel(double* out, const double* a, double w, long long n) {   // out .= -a ./ w
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) out[i] = -a[i] / w;
}
__global__ void sub_kernel(double* out, const double* a, const double* b, long long n) {   // out .= a .- b
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) out[i] = a[i] - b[i];
}
__global__ void vdiv_kernel(double* out, const double* a, const double* b, long long n) {   // out .= a ./ b
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) out[i] = a[i] / b[i];
}
__global__ void vmul_kernel(double* out, const double* a, const double* b, long long n) {   // out .= a .* b
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) out[i] = a[i] * b[i];
}
__global__ void fill_kernel(double* out, double v, long long n) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) out[i] = v;
}

// ---- evaluation kernels (src/iteration_stats_utils_gpu.jl:23-238) ---------------------------

__global__ void variable_violation_kernel(const double* x, const double* l, const double* u, long long n,
                                          double* lv, double* uv) {
  const long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (j < n) {
    lv[j] = dmax(l[j] - x[j], 0.0);
    uv[j] = dmax(x[j] - u[j], 0.0);
  }
}
__global__ void constraint_violation_kernel(const double* kx, const double* b, long long neq, long long m,
                                            double* cv) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < m) {
    const double v = (b ? b[i] : 0.0) - kx[i];
    cv[i] = i < neq ? v : dmax(v, 0.0);
  }
}
__global__ void reduced_costs_kernel(const double* g, const unsigned char* fl, const unsigned char* fu, long long n,
                                     double* rc, double* rcv) {
  const long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (j < n) {
    rc[j] = dmax(g[j], 0.0) * (double)fl[j] + dmin(g[j], 0.0) * (double)fu[j];
    rcv[j] = g[j] - rc[j];
  }
}
__global__ void dual_residual_kernel(const double* y, long long neq, long long nineq, double* dr) {
  const long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (k < nineq) dr[k] = dmax(-y[k + neq], 0.0);
}
__global__ void contribution_kernel(const double* l, const double* u, const double* rc, long long n, double* out) {
  const long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (j < n) {
    const double r = rc[j];
    out[j] = r > 0.0 ? l[j] * r : (r < 0.0 ? u[j] * r : 0.0);
  }
}
__global__ void ray_bounds_kernel(const unsigned char* fl, const unsigned char* fu, long long n, double* lr,
                                  double* ur) {
  const long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (j < n) {
    lr[j] = fl[j] ? 0.0 : -INFINITY;
    ur[j] = fu[j] ? 0.0 : INFINITY;
  }
}
__global__ void finite_kernel(const double* v, long long n, unsigned char* out) {
  const long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (j < n) out[j] = isfinite(v[j]) ? 1 : 0;
}

// mapreduce(abs, max) and sum: one block-level tree per CTA, then one CTA over the partials
template <bool MAXABS>
__global__ void reduce_kernel(const double* a, long long n, double* part) {
  __shared__ double sh[256];
  double acc = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    acc = MAXABS ? dmax(acc, fabs(a[i])) : acc + a[i];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] = MAXABS ? dmax(sh[threadIdx.x], sh[threadIdx.x + s]) : sh[threadIdx.x] + sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// ---- the solver ------------------------------------------------------------------------------

struct Csr {
  int32_t rows = 0, cols = 0;
  long long nnz = 0;
  Dev<int32_t> rp, ci;
  Dev<double> v;
  cusparseSpMatDescr_t d = nullptr;
};

struct Solver {
  gpdhg_params P;
  cudaStream_t st = nullptr;
  cublasHandle_t cb = nullptr;
  cusparseHandle_t cs = nullptr;
  long long n = 0, m = 0, neq = 0;
  double obj_const = 0.0;
  Csr A, At;
  // scaled problem, original problem, rescaling vectors
  Dev<double> c, l, u, b, oc, ol, ou, ob, con, var;
  Dev<unsigned char> fl, fu, ofl, ofu;
  // CuPdhgSolverState / CuBufferState / CuBufferAvgState / CuSolutionWeightedAverage
  Dev<double> x, y, Kx, Kty, dx, dy, dKx, sx, sy, sKx, sKty, tmpn, tmpm, ax, ay, aKx, agrad, grad;
  // restart info (CuRestartInfo)
  Dev<double> rx, ry, rKx, rgrad;
  // evaluation buffers (BufferOriginalSol, BufferKKTState)
  Dev<double> xo, yo, Kxo, go, lv, uv, cv, rc, rcv, dr, contrib, cat, lr, ur, xr, Kxr, gr, part;
  double step = 0.0, pw = 1.0, kkt_passes = 0.0, wx = 0.0, wy = 0.0;
  long long cxn = 0, cyn = 0, total_iters = 0, accepted = 0, rejected = 0;
  bool numerical_error = false;
  long long last_len = 1;
  double pdist = 0.0, ddist = 0.0, ratio_last = 1.0;
  double qc_linf_c = 0, qc_linf_b = 0, qc_l2_c = 0, qc_l2_b = 0;
  // cuSPARSE SpMV buffers, dense vector descriptors
  void* spbuf_a = nullptr;
  void* spbuf_t = nullptr;
  size_t spbuf_a_size = 0, spbuf_t_size = 0;
  long long launches = 0;

  ~Solver() {
    if (A.d) cusparseDestroySpMat(A.d);
    if (At.d) cusparseDestroySpMat(At.d);
    if (spbuf_a) cudaFree(spbuf_a);
    if (spbuf_t) cudaFree(spbuf_t);
    if (cb) cublasDestroy(cb);
    if (cs) cusparseDestroy(cs);
    if (st) cudaStreamDestroy(st);
  }

  void sync() { RQ(cudaStreamSynchronize(st)); }
  void check_launch() {
    RQ(cudaGetLastError());
    ++launches;
  }

  // CUDA.CUSPARSE.mv!('N', 1, M, xin, 0, yout, 'O', CUSPARSE_SPMV_CSR_ALG2)
  void spmv(Csr& M, void* buf, const double* xin, double* yout) {
    cusparseDnVecDescr_t vx, vy;
    RQS(cusparseCreateDnVec(&vx, M.cols, const_cast<double*>(xin), CUDA_R_64F));
    RQS(cusparseCreateDnVec(&vy, M.rows, yout, CUDA_R_64F));
    const double one = 1.0, zero = 0.0;
    RQS(cusparseSpMV(cs, CUSPARSE_OPERATION_NON_TRANSPOSE, &one, M.d, vx, &zero, vy, CUDA_R_64F,
                     CUSPARSE_SPMV_CSR_ALG2, buf));
    cusparseDestroyDnVec(vx);
    cusparseDestroyDnVec(vy);
    ++launches;
  }
  void spmv_a(const double* xin, double* yout) { spmv(A, spbuf_a, xin, yout); }
  void spmv_t(const double* yin, double* xout) { spmv(At, spbuf_t, yin, xout); }

  double dot(const double* a, const double* b2, long long k) {
    if (k == 0) return 0.0;
    double r = 0.0;
    RQB(cublasDdot(cb, (int)k, a, 1, b2, 1, &r));
    ++launches;
    return r;
  }
  double nrm2(const double* a, long long k) {
    if (k == 0) return 0.0;
    double r = 0.0;
    RQB(cublasDnrm2(cb, (int)k, a, 1, &r));
    ++launches;
    return r;
  }
  template <bool MAXABS>
  double reduce(const double* a, long long k) {
    if (k == 0) return 0.0;
    const int g = (int)std::min<long long>(1024, (k + 255) / 256);
    reduce_kernel<MAXABS><<<g, 256, 0, st>>>(a, k, part);
    check_launch();
    reduce_kernel<MAXABS><<<1, 256, 0, st>>>(part, g, part.p + 1024);
    check_launch();
    double h = 0.0;
    RQ(cudaMemcpyAsync(&h, part.p + 1024, sizeof(double), cudaMemcpyDeviceToHost, st));
    sync();
    return h;
  }
  double norm_inf(const double* a, long long k) { return reduce<true>(a, k); }
  double sum(const double* a, long long k) { return reduce<false>(a, k); }

  // [a; b; c] copied into the concatenation buffer (CUDA.jl allocates and copies)
  long long concat(std::initializer_list<std::pair<const double*, long long>> parts) {
    long long off = 0;
    for (auto& pr : parts) {
      if (pr.second) RQ(cudaMemcpyAsync(cat.p + off, pr.first, sizeof(double) * pr.second, cudaMemcpyDeviceToDevice, st));
      off += pr.second;
    }
    return off;
  }

  void copy(double* d, const double* s, long long k) {
    if (k) RQ(cudaMemcpyAsync(d, s, sizeof(double) * k, cudaMemcpyDeviceToDevice, st));
  }
  void fill0(double* d, long long k) {
    if (!k) return;
    fill_kernel<<<blocks(k), kThreads, 0, st>>>(d, 0.0, k);   // .= CUDA.zeros(...)
    check_launch();
  }

  // ---- take_step! ----------------------------------------------------------------------------
  void next_primal(double tau) {
    next_primal_kernel<<<blocks(n), kThreads, 0, st>>>(c, l, u, x, Kty, tau, pw, n, dx);
    check_launch();
    sync();                                      // CUDA.@sync (:213)
    if (m) spmv_a(dx, dKx);                      // :225
  }
  void next_dual(double tau) {
    if (!m) return;
    next_dual_kernel<<<blocks(m), kThreads, 0, st>>>(b, y, Kx, dKx, tau, pw, neq, m, dy);
    check_launch();
    sync();                                      // CUDA.@sync (:277)
  }
  void axpy_w(double* s, const double* v, double w, double* tmp, long long k) {   // s .+= v * w
    if (!k) return;
    scale_kernel<<<blocks(k), kThreads, 0, st>>>(tmp, v, w, k);
    check_launch();
    add_kernel<<<blocks(k), kThreads, 0, st>>>(s, tmp, k);
    check_launch();
  }
  void update_solution() {                       // :297-319
    add_kernel<<<blocks(n), kThreads, 0, st>>>(x, dx, n);
    check_launch();
    if (m) {
      add_kernel<<<blocks(m), kThreads, 0, st>>>(Kx, dKx, m);
      check_launch();
      add_kernel<<<blocks(m), kThreads, 0, st>>>(y, dy, m);
      check_launch();
      spmv_t(y, Kty);                            // :307
    }
    const double w = step;
    axpy_w(sx, x, w, tmpn, n);
    ++cxn;
    wx += w;
    axpy_w(sy, y, w, tmpm, m);
    ++cyn;
    wy += w;
    axpy_w(sKx, Kx, w, tmpm, m);
    axpy_w(sKty, Kty, w, tmpn, n);
  }
  void take_step_adaptive() {                    // :343-413
    double tau = step;
    bool done = false;
    while (!done) {
      ++total_iters;
      next_primal(tau);
      next_dual(tau);
      const double inter = std::fabs(dot(dKx, dy, m));
      const double ndx = nrm2(dx, n), ndy = nrm2(dy, m);
      const double movement = 0.5 * pw * ndx * ndx + (0.5 / pw) * ndy * ndy;
      kkt_passes += 1.0;
      double limit;
      if (inter > 0.0) {
        limit = movement / inter;
        if (movement == 0.0) {
          numerical_error = true;
          break;
        }
      } else {
        limit = kInf;
      }
      if (tau <= limit) {
        update_solution();
        done = true;
        ++accepted;
      } else {
        ++rejected;
      }
      const double k1 = (double)(total_iters + 1);
      const double first = (1.0 - 1.0 / std::pow(k1, P.reduction_exponent)) * limit;
      const double second = (1.0 + 1.0 / std::pow(k1, P.growth_exponent)) * tau;
      tau = jmin(first, second);
    }
    step = tau;
  }

  // ---- evaluation ----------------------------------------------------------------------------
  struct PrimalRes {
    double linf, l2;
  };
  // compute_primal_residual! + the norms of [cv; lv; uv] (:71-94, :271-272)
  PrimalRes primal_residual(const double* xv, const double* kxv, const double* lb, const double* ub,
                            const double* rhs, bool want_inf) {
    variable_violation_kernel<<<blocks(n), kThreads, 0, st>>>(xv, lb, ub, n, lv, uv);
    check_launch();
    sync();
    if (m) {
      constraint_violation_kernel<<<blocks(m), kThreads, 0, st>>>(kxv, rhs, neq, m, cv);
      check_launch();
      sync();
    }
    PrimalRes r{0.0, 0.0};
    long long k = concat({{cv, m}, {lv, n}, {uv, n}});
    if (want_inf) r.linf = norm_inf(cat, k);
    k = concat({{cv, m}, {lv, n}, {uv, n}});
    r.l2 = nrm2(cat, k);
    return r;
  }
  struct DualStats {
    double obj, res_inf, res_l2, rc_inf;
  };
  // compute_dual_stats! (:216-238) with the 2-norm of [dr; rcv] (:288)
  DualStats dual_stats(const double* yv, const double* g, const double* lb, const double* ub,
                       const unsigned char* finl, const unsigned char* finu, const double* rhs, double c0,
                       bool want_rc_inf) {
    reduced_costs_kernel<<<blocks(n), kThreads, 0, st>>>(g, finl, finu, n, rc, rcv);
    check_launch();
    sync();
    const long long nineq = m - neq;
    if (nineq > 0) {
      dual_residual_kernel<<<blocks(nineq), kThreads, 0, st>>>(yv, neq, nineq, dr);
      check_launch();
      sync();
    }
    DualStats s{};
    long long k = concat({{dr, nineq}, {rcv, n}});
    s.res_inf = norm_inf(cat, k);
    const double base = dot(rhs, yv, m) + c0;
    contribution_kernel<<<blocks(n), kThreads, 0, st>>>(lb, ub, rc, n, contrib);
    check_launch();
    sync();
    s.obj = base + sum(contrib, n);
    k = concat({{dr, nineq}, {rcv, n}});
    s.res_l2 = nrm2(cat, k);
    if (want_rc_inf) s.rc_inf = norm_inf(rc, n);
    return s;
  }

  gpdhg_convergence_information convergence_info(double eps_ratio) {   // :251-309 (original problem)
    gpdhg_convergence_information ci;
    std::memset(&ci, 0, sizeof(ci));
    PrimalRes pr = primal_residual(xo, Kxo, ol, ou, ob, true);
    ci.primal_objective = obj_const + dot(oc, xo, n);
    ci.l_inf_primal_residual = pr.linf;
    ci.l2_primal_residual = pr.l2;
    ci.relative_l_inf_primal_residual = pr.linf / (eps_ratio + qc_linf_b);
    ci.relative_l2_primal_residual = pr.l2 / (eps_ratio + qc_l2_b);
    ci.l_inf_primal_variable = norm_inf(xo, n);
    ci.l2_primal_variable = nrm2(xo, n);
    DualStats ds = dual_stats(yo, go, ol, ou, ofl, ofu, ob, obj_const, false);
    ci.dual_objective = ds.obj;
    ci.l_inf_dual_residual = ds.res_inf;
    ci.l2_dual_residual = ds.res_l2;
    ci.relative_l_inf_dual_residual = ds.res_inf / (eps_ratio + qc_linf_c);
    ci.relative_l2_dual_residual = ds.res_l2 / (eps_ratio + qc_l2_c);
    ci.l_inf_dual_variable = norm_inf(yo, m);
    ci.l2_dual_variable = nrm2(yo, m);
    ci.corrected_dual_objective = ds.res_inf == 0.0 ? ds.obj : -kInf;
    const double gap = std::fabs(ci.primal_objective - ci.dual_objective);
    ci.relative_optimality_gap = gap / (eps_ratio + std::fabs(ci.primal_objective) + std::fabs(ci.dual_objective));
    ci.candidate_type = GPDHG_POINT_TYPE_AVERAGE_ITERATE;
    return ci;
  }

  gpdhg_infeasibility_information infeasibility_info() {   // :314-372
    gpdhg_infeasibility_information ii;
    std::memset(&ii, 0, sizeof(ii));
    const double s = norm_inf(xo, n);
    copy(xr, xo, n);
    copy(Kxr, Kxo, m);
    if (s != 0.0) {
      div_kernel<<<blocks(n), kThreads, 0, st>>>(xr, xo, s, n);
      check_launch();
      if (m) {
        div_kernel<<<blocks(m), kThreads, 0, st>>>(Kxr, Kxo, s, m);
        check_launch();
      }
    }
    ray_bounds_kernel<<<blocks(n), kThreads, 0, st>>>(ofl, ofu, n, lr, ur);
    check_launch();
    PrimalRes pr = primal_residual(xr, Kxr, lr, ur, nullptr, true);
    ii.max_primal_ray_infeasibility = pr.linf;
    ii.primal_ray_linear_objective = dot(oc, xr, n);
    sub_kernel<<<blocks(n), kThreads, 0, st>>>(gr, go, oc, n);
    check_launch();
    DualStats ds = dual_stats(yo, gr, ol, ou, ofl, ofu, ob, obj_const, true);
    const double sf = jmax(norm_inf(yo, m), ds.rc_inf);
    if (sf != 0.0) {
      ii.max_dual_ray_infeasibility = ds.res_inf / sf;
      ii.dual_ray_objective = ds.obj / sf;
    }
    ii.candidate_type = GPDHG_POINT_TYPE_AVERAGE_ITERATE;
    return ii;
  }

  gpdhg_iteration_stats evaluate(long long iteration, double t) {   // :447-502
    vdiv_kernel<<<blocks(n), kThreads, 0, st>>>(xo, ax, var, n);
    check_launch();
    vmul_kernel<<<blocks(n), kThreads, 0, st>>>(go, agrad, var, n);
    check_launch();
    if (m) {
      vdiv_kernel<<<blocks(m), kThreads, 0, st>>>(yo, ay, con, m);
      check_launch();
      vmul_kernel<<<blocks(m), kThreads, 0, st>>>(Kxo, aKx, con, m);
      check_launch();
    }
    gpdhg_iteration_stats s;
    std::memset(&s, 0, sizeof(s));
    s.iteration_number = (int32_t)(iteration - 1);
    s.cumulative_kkt_matrix_passes = kkt_passes;
    s.cumulative_time_sec = t;
    s.convergence_information = convergence_info(P.eps_optimal_absolute / P.eps_optimal_relative);
    s.infeasibility_information = infeasibility_info();
    s.step_size = step;
    s.primal_weight = pw;
    s.precision = GPDHG_PRECISION_FP64;
    return s;
  }

  void compute_average() {   // src/saddle_point_gpu.jl:226-240
    div_kernel<<<blocks(n), kThreads, 0, st>>>(ax, sx, wx, n);
    check_launch();
    if (m) {
      div_kernel<<<blocks(m), kThreads, 0, st>>>(ay, sy, wy, m);
      check_launch();
      div_kernel<<<blocks(m), kThreads, 0, st>>>(aKx, sKx, wx, m);
      check_launch();
    }
    neg_div_kernel<<<blocks(n), kThreads, 0, st>>>(agrad, sKty, wy, n);
    check_launch();
    add_kernel<<<blocks(n), kThreads, 0, st>>>(agrad, c, n);
    check_launch();
  }

  // compute_weight_kkt_residual, src/saddle_point_gpu.jl:250-278 (scaled problem)
  double weighted_kkt(const double* xv, const double* yv, const double* kxv, const double* gv) {
    PrimalRes pr = primal_residual(xv, kxv, l, u, b, false);
    const double pobj = obj_const + dot(c, xv, n);
    DualStats ds = dual_stats(yv, gv, l, u, fl, fu, b, obj_const, false);
    const double g = std::fabs(pobj - ds.obj);
    return std::sqrt(pw * pr.l2 * pr.l2 + 1.0 / pw * ds.res_l2 * ds.res_l2 + g * g);
  }

  double dist(const double* a, const double* b2, double* tmp, long long k) {   // norm(a - b)
    if (!k) return 0.0;
    sub_kernel<<<blocks(k), kThreads, 0, st>>>(tmp, a, b2, k);
    check_launch();
    return nrm2(tmp, k);
  }

  int run_restart_scheme(long long iterations_completed, double pnp, double dnp) {   // :479-622
    if (!(cxn > 0 && cyn > 0)) return GPDHG_RESTART_CHOICE_NO_RESTART;
    const long long restart_length = cxn;
    bool do_restart = (double)restart_length >= P.artificial_restart_threshold * (double)iterations_completed;
    bool reset_to_average;
    double candidate = std::numeric_limits<double>::quiet_NaN();
    if (P.restart_scheme == GPDHG_NO_RESTARTS) {
      reset_to_average = false;
    } else {
      const double cur = weighted_kkt(x, y, Kx, grad);
      const double av = weighted_kkt(ax, ay, aKx, agrad);
      reset_to_average = P.restart_to_current_metric == GPDHG_KKT_GREEDY ? (cur >= av) : true;
      candidate = reset_to_average ? av : cur;
    }
    if (!do_restart) {
      if (P.restart_scheme == GPDHG_ADAPTIVE_KKT) {
        const double last = weighted_kkt(rx, ry, rKx, rgrad);
        const double ratio = candidate / last;
        if (ratio < P.necessary_reduction_for_restart) {
          if (ratio < P.sufficient_reduction_for_restart)
            do_restart = true;
          else if (ratio > ratio_last)
            do_restart = true;
        }
        ratio_last = ratio;
      } else if (P.restart_scheme == GPDHG_FIXED_FREQUENCY && P.restart_frequency_if_fixed <= restart_length) {
        do_restart = true;
      }
    }
    if (!do_restart) return GPDHG_RESTART_CHOICE_NO_RESTART;
    if (reset_to_average) {
      copy(x, ax, n);
      copy(y, ay, m);
      copy(Kx, aKx, m);
      sub_kernel<<<blocks(n), kThreads, 0, st>>>(Kty, c, agrad, n);
      check_launch();
      copy(grad, agrad, n);
    }
    fill0(sx, n);
    fill0(sy, m);
    cxn = cyn = 0;
    wx = wy = 0.0;
    fill0(sKx, m);
    fill0(sKty, n);
    const double dxn = dist(ax, rx, tmpn, n), dyn = dist(ay, ry, tmpm, m);   // update_last_restart_info!
    pdist = std::sqrt(pnp) * dxn / std::sqrt(pw);
    ddist = std::sqrt(dnp) * dyn * std::sqrt(pw);
    copy(rx, x, n);
    copy(ry, y, m);
    last_len = restart_length;
    copy(rKx, Kx, m);
    copy(rgrad, grad, n);
    return reset_to_average ? GPDHG_RESTART_CHOICE_RESTART_TO_AVERAGE : GPDHG_RESTART_CHOICE_WEIGHTED_AVERAGE_RESET;
  }

  double new_primal_weight() {   // src/saddle_point_gpu.jl:627-654
    const double eps = std::numeric_limits<double>::epsilon();
    if (pdist > eps && ddist > eps) {
      const double th = P.primal_weight_update_smoothing;
      return std::exp(th * std::log(ddist / pdist) + (1.0 - th) * std::log(pw));
    }
    return pw;
  }

  int check_termination(const gpdhg_iteration_stats& s) {   // src/termination.jl:142-246
    const auto& ci = s.convergence_information;
    const double abs_obj = std::fabs(ci.primal_objective) + std::fabs(ci.dual_objective);
    const double gap = std::fabs(ci.primal_objective - ci.dual_objective);
    const bool linf = P.optimality_norm == GPDHG_L_INF;
    const double pe = linf ? ci.l_inf_primal_residual : ci.l2_primal_residual;
    const double pb = linf ? qc_linf_b : qc_l2_b;
    const double de = linf ? ci.l_inf_dual_residual : ci.l2_dual_residual;
    const double db = linf ? qc_linf_c : qc_l2_c;
    const double a = P.eps_optimal_absolute, r = P.eps_optimal_relative;
    if (de < a + r * db && pe < a + r * pb && gap < a + r * abs_obj) return GPDHG_TERMINATION_REASON_OPTIMAL;
    const auto& ii = s.infeasibility_information;
    if (ii.dual_ray_objective > 0.0 && ii.max_dual_ray_infeasibility / ii.dual_ray_objective <= P.eps_primal_infeasible)
      return GPDHG_TERMINATION_REASON_PRIMAL_INFEASIBLE;
    if (ii.primal_ray_linear_objective < 0.0 &&
        ii.max_primal_ray_infeasibility / (-ii.primal_ray_linear_objective) <= P.eps_dual_infeasible)
      return GPDHG_TERMINATION_REASON_DUAL_INFEASIBLE;
    if (s.iteration_number >= P.iteration_limit) return GPDHG_TERMINATION_REASON_ITERATION_LIMIT;
    if (s.cumulative_kkt_matrix_passes >= P.kkt_matrix_pass_limit) return GPDHG_TERMINATION_REASON_KKT_MATRIX_PASS_LIMIT;
    if (s.cumulative_time_sec >= P.time_sec_limit) return GPDHG_TERMINATION_REASON_TIME_LIMIT;
    return 0;
  }

  // ---- set-up (src/cpu_to_gpu.jl) --------------------------------------------------------------
  void setup(const gpdhg_lp_desc* d) {
    n = d->num_variables;
    m = d->num_constraints;
    neq = d->num_equalities;
    obj_const = d->objective_constant;
    RQ(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    RQB(cublasCreate(&cb));
    RQB(cublasSetStream(cb, st));
    RQB(cublasSetPointerMode(cb, CUBLAS_POINTER_MODE_HOST));
    RQS(cusparseCreate(&cs));
    RQS(cusparseSetStream(cs, st));
    // CSR(A) from the descriptor, CSR(A') by a host counting sort (the reference builds
    // CuSparseMatrixCSR(A') on the host side of cpu_to_gpu.jl)
    const long long nnz = d->nnz;
    std::vector<int32_t> trp(n + 1, 0), tci(std::max<long long>(nnz, 1));
    std::vector<double> tv(std::max<long long>(nnz, 1));
    for (long long k = 0; k < nnz; ++k) ++trp[d->col_idx[k] + 1];
    for (long long j = 0; j < n; ++j) trp[j + 1] += trp[j];
    std::vector<int32_t> pos(trp.begin(), trp.end() - 1);
    for (long long i = 0; i < m; ++i)
      for (int32_t k = d->row_ptr[i]; k < d->row_ptr[i + 1]; ++k) {
        const int32_t q = pos[d->col_idx[k]]++;
        tci[q] = (int32_t)i;
        tv[q] = d->values[k];
      }
    auto up_csr = [&](Csr& M, int32_t rows, int32_t cols, const int32_t* rp, const int32_t* ci, const double* v) {
      M.rows = rows;
      M.cols = cols;
      M.nnz = nnz;
      M.rp.alloc(rows + 1);
      M.ci.alloc(nnz);
      M.v.alloc(nnz);
      RQ(cudaMemcpy(M.rp, rp, sizeof(int32_t) * (rows + 1), cudaMemcpyHostToDevice));
      if (nnz) {
        RQ(cudaMemcpy(M.ci, ci, sizeof(int32_t) * nnz, cudaMemcpyHostToDevice));
        RQ(cudaMemcpy(M.v, v, sizeof(double) * nnz, cudaMemcpyHostToDevice));
      }
      RQS(cusparseCreateCsr(&M.d, rows, cols, nnz, M.rp.p, M.ci.p, M.v.p, CUSPARSE_INDEX_32I, CUSPARSE_INDEX_32I,
                            CUSPARSE_INDEX_BASE_ZERO, CUDA_R_64F));
    };
    up_csr(A, (int32_t)m, (int32_t)n, d->row_ptr, d->col_idx, d->values);
    up_csr(At, (int32_t)n, (int32_t)m, trp.data(), tci.data(), tv.data());
    auto up = [&](Dev<double>& v, const double* h, long long k) {
      v.alloc(k);
      if (k) RQ(cudaMemcpy(v, h, sizeof(double) * k, cudaMemcpyHostToDevice));
    };
    up(c, d->objective_vector, n);
    up(l, d->variable_lower_bound, n);
    up(u, d->variable_upper_bound, n);
    up(b, d->right_hand_side, m);
    const bool has_orig = d->original_objective_vector != nullptr;
    up(oc, has_orig ? d->original_objective_vector : d->objective_vector, n);
    up(ol, has_orig ? d->original_variable_lower_bound : d->variable_lower_bound, n);
    up(ou, has_orig ? d->original_variable_upper_bound : d->variable_upper_bound, n);
    up(ob, has_orig ? d->original_right_hand_side : d->right_hand_side, m);
    std::vector<double> ones(std::max(n, m), 1.0);
    up(con, d->constraint_rescaling ? d->constraint_rescaling : ones.data(), m);
    up(var, d->variable_rescaling ? d->variable_rescaling : ones.data(), n);
    for (Dev<unsigned char>* f : {&fl, &fu, &ofl, &ofu}) f->alloc(n);
    finite_kernel<<<blocks(n), kThreads, 0, st>>>(l, n, fl);
    finite_kernel<<<blocks(n), kThreads, 0, st>>>(u, n, fu);
    finite_kernel<<<blocks(n), kThreads, 0, st>>>(ol, n, ofl);
    finite_kernel<<<blocks(n), kThreads, 0, st>>>(ou, n, ofu);
    RQ(cudaGetLastError());
    for (Dev<double>* v : {&x, &Kty, &dx, &sx, &sKty, &tmpn, &ax, &agrad, &grad, &rx, &rgrad, &xo, &go, &lv, &uv, &rc,
                           &rcv, &contrib, &lr, &ur, &xr, &gr})
      v->alloc(n);
    for (Dev<double>* v : {&y, &Kx, &dy, &dKx, &sy, &sKx, &tmpm, &ay, &aKx, &ry, &rKx, &yo, &Kxo, &cv, &dr, &Kxr})
      v->alloc(m);
    cat.alloc(m + 2 * n);
    part.alloc(2048);
    for (Dev<double>* v : {&x, &Kty, &sx, &sKty, &ax, &agrad, &rx, &rgrad}) RQ(cudaMemsetAsync(*v, 0, sizeof(double) * n, st));
    for (Dev<double>* v : {&y, &Kx, &sy, &sKx, &ay, &aKx, &ry, &rKx}) RQ(cudaMemsetAsync(*v, 0, sizeof(double) * std::max(m, 1LL), st));
    // SpMV workspaces
    {
      cusparseDnVecDescr_t vx, vy;
      const double one = 1.0, zero = 0.0;
      RQS(cusparseCreateDnVec(&vx, n, dx.p, CUDA_R_64F));
      RQS(cusparseCreateDnVec(&vy, std::max(m, 1LL), dKx.p, CUDA_R_64F));
      if (m) {
        RQS(cusparseSpMV_bufferSize(cs, CUSPARSE_OPERATION_NON_TRANSPOSE, &one, A.d, vx, &zero, vy, CUDA_R_64F,
                                    CUSPARSE_SPMV_CSR_ALG2, &spbuf_a_size));
        RQS(cusparseSpMV_bufferSize(cs, CUSPARSE_OPERATION_NON_TRANSPOSE, &one, At.d, vy, &zero, vx, CUDA_R_64F,
                                    CUSPARSE_SPMV_CSR_ALG2, &spbuf_t_size));
      }
      cusparseDestroyDnVec(vx);
      cusparseDestroyDnVec(vy);
      RQ(cudaMalloc(&spbuf_a, std::max<size_t>(spbuf_a_size, 16)));
      RQ(cudaMalloc(&spbuf_t, std::max<size_t>(spbuf_t_size, 16)));
    }
    sync();
  }

  int run(gpdhg_result* res, double* x_avg_out, double* y_avg_out) {   // :457-798
    // cached_quadratic_program_info (original problem)
    qc_linf_c = norm_inf(oc, n);
    qc_linf_b = norm_inf(ob, m);
    qc_l2_c = nrm2(oc, n);
    qc_l2_b = nrm2(ob, m);
    sub_kernel<<<blocks(n), kThreads, 0, st>>>(grad, c, Kty, n);   // buffer_primal_gradient
    check_launch();
    if (P.step_size_policy != GPDHG_STEPSIZE_ADAPTIVE) throw Fail("only the adaptive step-size policy is provided");
    kkt_passes += 0.5;
    {
      const double amax = norm_inf(A.v, A.nnz);   // norm(A, Inf) of the scaled matrix (entrywise)
      step = amax > 0.0 ? 1.0 / amax : 1.0;
    }
    if (P.scale_invariant_initial_primal_weight) {   // select_initial_primal_weight
      const double rhs = nrm2(b, m), obj = nrm2(c, n);
      pw = (obj > 0.0 && rhs > 0.0) ? P.primal_importance * (obj / rhs) : P.primal_importance;
    } else {
      pw = P.primal_importance;
    }
    copy(rgrad, grad, n);   // create_last_restart_info
    sync();
    const auto t0 = std::chrono::steady_clock::now();
    auto now = [&] { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); };
    long long iteration = 0;
    const long long freq = P.termination_evaluation_frequency;
    int nstats = 0;
    while (true) {
      ++iteration;
      if ((iteration - 1) % freq == 0 || iteration == (long long)P.iteration_limit + 1 || iteration <= 10 ||
          numerical_error) {
        kkt_passes += 2.0;
        if (numerical_error || cxn == 0 || cyn == 0) {
          copy(ax, x, n);
          copy(ay, y, m);
          copy(aKx, Kx, m);
          copy(agrad, grad, n);
        } else {
          compute_average();
        }
        gpdhg_iteration_stats s = evaluate(iteration, now());
        int reason = check_termination(s);
        if (numerical_error && reason == 0) reason = GPDHG_TERMINATION_REASON_NUMERICAL_ERROR;
        if (iteration < 10 && (reason == GPDHG_TERMINATION_REASON_PRIMAL_INFEASIBLE ||
                               reason == GPDHG_TERMINATION_REASON_DUAL_INFEASIBLE))
          reason = 0;
        ++nstats;
        if (reason != 0) {
          if (x_avg_out) RQ(cudaMemcpy(x_avg_out, ax, sizeof(double) * n, cudaMemcpyDeviceToHost));
          if (y_avg_out && m) RQ(cudaMemcpy(y_avg_out, ay, sizeof(double) * m, cudaMemcpyDeviceToHost));
          std::memset(res, 0, sizeof(*res));
          res->termination_reason = reason;
          res->iteration_count = (int32_t)(iteration - 1);
          res->total_number_iterations = total_iters;
          res->cumulative_kkt_matrix_passes = kkt_passes;
          res->solve_time_sec = now();
          res->num_iteration_stats = nstats;
          res->fp64_handoff_iteration = -1;
          s.restart_used = GPDHG_RESTART_CHOICE_UNSPECIFIED;
          res->last_iteration_stats = s;
          res->accepted_steps = accepted;
          res->rejected_steps = rejected;
          res->kernels_launched = launches;
          return GPDHG_OK;
        }
        sub_kernel<<<blocks(n), kThreads, 0, st>>>(grad, c, Kty, n);
        check_launch();
        const double pnp = 1.0 / step * pw, dnp = 1.0 / step / pw;   // define_norms
        const int rcu = run_restart_scheme(iteration - 1, pnp, dnp);
        if (rcu != GPDHG_RESTART_CHOICE_NO_RESTART) pw = new_primal_weight();
      }
      take_step_adaptive();
    }
  }
};

thread_local std::string g_err;

}  // namespace

extern "C" {

// Solves a scaled LP (gpdhg_lp_desc with its original vectors and rescaling, as given to
// gpdhg_problem_create) with the reference's GPU call pattern; x_avg / y_avg receive the
// scaled averaged iterate (may be NULL). Returns 0 or an error code (refeq_last_error).
int refeq_solve(const gpdhg_lp_desc* desc, const gpdhg_params* params, gpdhg_result* res, double* x_avg,
                double* y_avg) {
  try {
    if (!desc || !params || !res) throw Fail("NULL argument");
    if (desc->num_variables <= 0 || desc->num_constraints < 0) throw Fail("need n > 0 and m >= 0");
    Solver s;
    s.P = *params;
    s.setup(desc);
    return s.run(res, x_avg, y_avg);
  } catch (const std::exception& e) {
    g_err = e.what();
    return GPDHG_ERR_CUDA;
  }
}

const char* refeq_last_error(void) { return g_err.c_str(); }

}  // extern "C"
