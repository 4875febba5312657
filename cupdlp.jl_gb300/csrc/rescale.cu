// rescale.cu — rescale_problem (src/preprocess.jl:619-675) on the GPU, for
// gpdhg_problem_create_unscaled: Ruiz L-inf iterations (:398-463), the optional L2-norm
// rescaling, and Pock-Chambolle (:494-525), each applied in place to both CSR copies of A,
// to l, u, c, b, and accumulated into the constraint / variable rescaling vectors.
//
// Every operation follows the host restatement (cupdlp/preprocess.py) in kind and order:
// maxima, square roots and divisions are correctly rounded on both sides, a scaled entry is
// ((1 / E_i) a_ij) (1 / D_j) in both CSR copies, c ./= D, bounds .*= D, b ./= E, and the
// cumulative vectors are multiplied in the reference's order, so Ruiz scaling is bitwise the
// host's. Row sums (Pock-Chambolle, L2) add in a fixed warp-tree order, which differs from
// the host's sequential order by rounding only.
#include <algorithm>
#include <cmath>
#include <vector>

#include "problem.h"

namespace gpdhg {

namespace {

enum RowOp : int { kRowAbsMax = 0, kRowPowSum = 1, kRowScaledSq = 2 };

// One warp per row of a CSR matrix: max |a| (exact in any order), sum |a|^alpha, or
// sum (a / sf_row)^2 (fixed shuffle-tree order).
__global__ void __launch_bounds__(kBlock) row_reduce_kernel(int nrows, const int32_t* __restrict__ rp,
                                                            const double* __restrict__ val, int op, double alpha,
                                                            const double* __restrict__ sf, double* out) {
  const int lane = threadIdx.x & 31;
  const long long warps = (long long)gridDim.x * (kBlock / 32);
  for (long long r = (long long)blockIdx.x * (kBlock / 32) + (threadIdx.x >> 5); r < nrows; r += warps) {
    const int b = rp[r], e = rp[r + 1];
    double acc = 0.0;
    const double inv = op == kRowScaledSq ? 1.0 / sf[r] : 0.0;
    for (int k = b + lane; k < e; k += 32) {
      const double a = fabs(val[k]);
      if (op == kRowAbsMax) acc = fmax(acc, a);
      else if (op == kRowPowSum) acc += pow(a, alpha);
      else {
        const double t = val[k] * inv;
        acc += t * t;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double v = __shfl_down_sync(0xffffffffu, acc, o);
      acc = op == kRowAbsMax ? fmax(acc, v) : acc + v;
    }
    if (lane == 0) out[r] = acc;
  }
}

enum FactorOp : int { kFactorSqrt = 0, kFactorL2 = 1 };

// Per entry: f = sqrt(x) (Ruiz, Pock-Chambolle) or f = sqrt(sf * sqrt(x)) (L2); f == 0 -> 1;
// cum *= f; inv = 1 / f.
__global__ void factor_kernel(long long len, int op, const double* __restrict__ x, const double* __restrict__ sf,
                              double* __restrict__ f, double* __restrict__ inv, double* __restrict__ cum) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x) {
    double v;
    if (op == kFactorSqrt) {
      v = sqrt(x[i]);
    } else {
      const double s = sf[i] == 0.0 ? 1.0 : sf[i];
      double norm = s * sqrt(x[i]);
      if (norm == 0.0) norm = 1.0;
      v = sqrt(norm);
    }
    if (v == 0.0) v = 1.0;
    f[i] = v;
    inv[i] = 1.0 / v;
    cum[i] *= v;
  }
}

// sf == 0 -> 1 (the L2 pre-scale of an empty row or column).
__global__ void unit_if_zero_kernel(long long len, double* x) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x)
    if (x[i] == 0.0) x[i] = 1.0;
}

// a_ij <- ((1 / E_i) a_ij) (1 / D_j) in a CSR whose rows are A's rows (transposed = 0) or
// A's columns (transposed = 1).
__global__ void scale_matrix_kernel(int nrows, const int32_t* __restrict__ rp, const int32_t* __restrict__ col,
                                    double* __restrict__ val, const double* __restrict__ inv_con,
                                    const double* __restrict__ inv_var, int transposed) {
  const int lane = threadIdx.x & 31;
  const long long warps = (long long)gridDim.x * (kBlock / 32);
  for (long long r = (long long)blockIdx.x * (kBlock / 32) + (threadIdx.x >> 5); r < nrows; r += warps) {
    const int b = rp[r], e = rp[r + 1];
    for (int k = b + lane; k < e; k += 32) {
      const double ic = transposed ? inv_con[col[k]] : inv_con[r];
      const double iv = transposed ? inv_var[r] : inv_var[col[k]];
      val[k] = (ic * val[k]) * iv;
    }
  }
}

// c ./= D, l .*= D, u .*= D (n entries); b ./= E (m entries).
__global__ void scale_vectors_kernel(int n, int m, const double* __restrict__ var, const double* __restrict__ con,
                                     double* c, double* l, double* u, double* b) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    c[i] = c[i] / var[i];
    u[i] = u[i] * var[i];
    l[i] = l[i] * var[i];
  }
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += stride) b[i] = b[i] / con[i];
}

__global__ void fill_kernel(long long len, double v, double* x) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x)
    x[i] = v;
}

int grid_of(long long work, int per_block) {
  return (int)std::max<long long>(1, std::min<long long>((work + per_block - 1) / per_block, 8192));
}

}  // namespace

void rescale_on_device(gpdhg_problem* p, const gpdhg_params& prm) {
  cudaStream_t s = p->stream;
  const int n = p->n, m = p->m;
  const size_t N = std::max(n, 1), M = std::max(m, 1);
  DBuf<double> rx(N), cx(M), rsf(N), csf(M), fv(N), fc(M), iv(N), ic(M), cum_v(N), cum_c(M);
  const int gw_n = grid_of(n, kBlock / 32), gw_m = grid_of(m, kBlock / 32);
  const int ge_n = grid_of(n, kBlock), ge_m = grid_of(m, kBlock);
  // p->var / p->con start at ones (problem_init with no rescaling vectors)
  auto apply = [&]() {
    if (m) scale_matrix_kernel<<<gw_m, kBlock, 0, s>>>(m, p->A.row_ptr.get(), p->A.col.get(), p->A.val64.get(),
                                                       ic.get(), iv.get(), 0);
    scale_matrix_kernel<<<gw_n, kBlock, 0, s>>>(n, p->At.row_ptr.get(), p->At.col.get(), p->At.val64.get(), ic.get(),
                                                iv.get(), 1);
    scale_vectors_kernel<<<std::max(ge_n, ge_m), kBlock, 0, s>>>(n, m, fv.get(), fc.get(), p->c.get(), p->l.get(),
                                                                 p->u.get(), p->b.get());
    CK_LAUNCH();
  };
  auto stage_total = [&](DBuf<double>& cum, DBuf<double>& total, long long len) {
    // total *= cum (the reference multiplies each stage's cumulative vector in)
    if (len == 0) return;
    std::vector<double> h1(len), h2(len);
    CK(cudaMemcpyAsync(h1.data(), cum.get(), sizeof(double) * len, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(h2.data(), total.get(), sizeof(double) * len, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    for (long long i = 0; i < len; ++i) h2[i] *= h1[i];
    CK(cudaMemcpyAsync(total.get(), h2.data(), sizeof(double) * len, cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));
  };
  auto reset_cum = [&]() {
    fill_kernel<<<ge_n, kBlock, 0, s>>>(n, 1.0, cum_v.get());
    if (m) fill_kernel<<<ge_m, kBlock, 0, s>>>(m, 1.0, cum_c.get());
    CK_LAUNCH();
  };
  // ruiz_rescaling with p = Inf (:398-463): D_j = sqrt(max_i |a_ij|), E_i = sqrt(max_j |a_ij|)
  if (prm.l_inf_ruiz_iterations > 0) {
    reset_cum();
    for (int it = 0; it < prm.l_inf_ruiz_iterations; ++it) {
      row_reduce_kernel<<<gw_n, kBlock, 0, s>>>(n, p->At.row_ptr.get(), p->At.val64.get(), kRowAbsMax, 0.0, nullptr,
                                                rx.get());
      if (m) row_reduce_kernel<<<gw_m, kBlock, 0, s>>>(m, p->A.row_ptr.get(), p->A.val64.get(), kRowAbsMax, 0.0,
                                                       nullptr, cx.get());
      factor_kernel<<<ge_n, kBlock, 0, s>>>(n, kFactorSqrt, rx.get(), nullptr, fv.get(), iv.get(), cum_v.get());
      if (m) factor_kernel<<<ge_m, kBlock, 0, s>>>(m, kFactorSqrt, cx.get(), nullptr, fc.get(), ic.get(), cum_c.get());
      CK_LAUNCH();
      apply();
    }
    stage_total(cum_v, p->var, n);
    stage_total(cum_c, p->con, m);
  }
  // l2_norm_rescaling: rows and columns scaled by sqrt of their 2-norms
  if (prm.l2_norm_rescaling) {
    reset_cum();
    row_reduce_kernel<<<gw_n, kBlock, 0, s>>>(n, p->At.row_ptr.get(), p->At.val64.get(), kRowAbsMax, 0.0, nullptr,
                                              rsf.get());
    if (m) row_reduce_kernel<<<gw_m, kBlock, 0, s>>>(m, p->A.row_ptr.get(), p->A.val64.get(), kRowAbsMax, 0.0,
                                                     nullptr, csf.get());
    unit_if_zero_kernel<<<ge_n, kBlock, 0, s>>>(n, rsf.get());
    if (m) unit_if_zero_kernel<<<ge_m, kBlock, 0, s>>>(m, csf.get());
    row_reduce_kernel<<<gw_n, kBlock, 0, s>>>(n, p->At.row_ptr.get(), p->At.val64.get(), kRowScaledSq, 0.0,
                                              rsf.get(), rx.get());
    if (m) row_reduce_kernel<<<gw_m, kBlock, 0, s>>>(m, p->A.row_ptr.get(), p->A.val64.get(), kRowScaledSq, 0.0,
                                                     csf.get(), cx.get());
    factor_kernel<<<ge_n, kBlock, 0, s>>>(n, kFactorL2, rx.get(), rsf.get(), fv.get(), iv.get(), cum_v.get());
    if (m) factor_kernel<<<ge_m, kBlock, 0, s>>>(m, kFactorL2, cx.get(), csf.get(), fc.get(), ic.get(), cum_c.get());
    CK_LAUNCH();
    apply();
    stage_total(cum_v, p->var, n);
    stage_total(cum_c, p->con, m);
  }
  // pock_chambolle_rescaling (:494-525): D_j = sqrt(sum_i |a_ij|^(2-alpha)), E_i = sqrt(sum_j |a_ij|^alpha)
  if (!std::isnan(prm.pock_chambolle_alpha)) {
    const double alpha = prm.pock_chambolle_alpha;
    if (!(alpha >= 0.0 && alpha <= 2.0))
      throw Error(GPDHG_ERR_INVALID_ARGUMENT, "pock_chambolle_alpha must lie in [0, 2]");
    reset_cum();
    row_reduce_kernel<<<gw_n, kBlock, 0, s>>>(n, p->At.row_ptr.get(), p->At.val64.get(), kRowPowSum, 2.0 - alpha,
                                              nullptr, rx.get());
    if (m) row_reduce_kernel<<<gw_m, kBlock, 0, s>>>(m, p->A.row_ptr.get(), p->A.val64.get(), kRowPowSum, alpha,
                                                     nullptr, cx.get());
    factor_kernel<<<ge_n, kBlock, 0, s>>>(n, kFactorSqrt, rx.get(), nullptr, fv.get(), iv.get(), cum_v.get());
    if (m) factor_kernel<<<ge_m, kBlock, 0, s>>>(m, kFactorSqrt, cx.get(), nullptr, fc.get(), ic.get(), cum_c.get());
    CK_LAUNCH();
    apply();
    stage_total(cum_v, p->var, n);
    stage_total(cum_c, p->con, m);
  }
  CK(cudaStreamSynchronize(s));
  // host scalars of the scaled problem, as problem_init derives them from a scaled descriptor:
  // tau_0 = 1 / max|a_ij| (:571) and the norms of select_initial_primal_weight
  std::vector<double> hv((size_t)std::max<long long>(p->nnz, 1)), hc(N), hb(M);
  if (p->nnz) CK(cudaMemcpyAsync(hv.data(), p->A.val64.get(), sizeof(double) * p->nnz, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(hc.data(), p->c.get(), sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  if (m) CK(cudaMemcpyAsync(hb.data(), p->b.get(), sizeof(double) * m, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  double amax = 0.0, sc = 0.0, sb = 0.0;
  for (long long k = 0; k < p->nnz; ++k) amax = std::max(amax, std::fabs(hv[k]));
  for (int j = 0; j < n; ++j) sc += hc[j] * hc[j];
  for (int i = 0; i < m; ++i) sb += hb[i] * hb[i];
  p->amax = amax;
  p->norm2_c_scaled = std::sqrt(sc);
  p->norm2_b_scaled = m ? std::sqrt(sb) : 0.0;
}

void get_rescaling(const gpdhg_problem* p, double* con, double* var) {
  if (con && p->m)
    CK(cudaMemcpyAsync(con, p->con.get(), sizeof(double) * p->m, cudaMemcpyDeviceToHost, p->stream));
  if (var) CK(cudaMemcpyAsync(var, p->var.get(), sizeof(double) * p->n, cudaMemcpyDeviceToHost, p->stream));
  CK(cudaStreamSynchronize(p->stream));
}

}  // namespace gpdhg
