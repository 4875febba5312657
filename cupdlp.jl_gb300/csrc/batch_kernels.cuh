// batch_kernels.cuh — step and evaluation kernels for many LPs packed into one
// block-diagonal ("segmented") CSR.
//
// Every row-block item of the packed A and A' belongs to exactly one instance, and an
// instance's items are built exactly as for a lone solve, so each instance sees the same
// per-CTA sums in the same order as when solved alone: results are bitwise identical
// alone and in a batch. Per-instance scalars live in a StepState array; the last CTA of
// an instance's dual pass (a per-instance arrival counter) takes that instance's
// accept/reject decision. A finished or retired instance's CTAs exit at once.
#pragma once

#include "eval_kernels.cuh"
#include "step_kernels.cuh"

namespace gpdhg {

// Per-instance ranges of the packed layout.
struct BatchIndex {
  const int32_t* item_inst_p;  // instance of each A' item
  const int32_t* item_inst_d;  // instance of each A item
  const int32_t* p_item_begin; // first A' item of each instance (count + 1 entries)
  const int32_t* d_item_begin; // first A item of each instance (count + 1 entries)
  const int32_t* row_off;      // first packed row of each instance (count + 1)
  const int32_t* neq;          // equality rows of each instance
};

template <class T>
struct BatchPrimalArgs {
  CsrView<T> At;
  BatchIndex bi;
  const T* c;
  const T* l;
  const T* u;
  T* x;
  T* dx;
  T* kty;
  T* sx;
  T* skty;
  const T* y0;
  const T* y1;
  const StepState* st;  // one per instance
  double* part_p;
  int mode;
  int direct;
};

template <class T>
__global__ void __launch_bounds__(kBlock) batch_primal_kernel(BatchPrimalArgs<T> a) {
  __shared__ T prod[kItemNnz];
  __shared__ T rowsum[kBlock];
  __shared__ double red[32];
  const int item = blockIdx.x;
  const int inst = a.bi.item_inst_p[item];
  const StepState* st = a.st + inst;
  if (st->done) return;
  const bool pending = st->pending_commit != 0;
  const bool commit_only = a.mode == kStepCommitOnly;
  if (commit_only && !pending) return;
  const T w = (T)st->commit_weight;
  const T tto = (T)(st->tau / st->omega);
  const T* ycur = st->parity ? a.y1 : a.y0;
  T acc = T(0);
  const bool direct = a.direct != 0;
  auto candidate = [&](int j, T xv, T ktyv) {
    T v = xv - tto * (a.c[j] - ktyv);
    v = jmin(a.u[j], jmax(a.l[j], v));
    const T d = v - xv;
    a.dx[j] = direct ? v : d;
    acc += d * d;
  };
  if (pending) {
    auto epi = [&](int j, T ktyv) {
      const T xv = direct ? a.dx[j] : a.x[j] + a.dx[j];
      a.x[j] = xv;
      a.kty[j] = ktyv;
      a.sx[j] += xv * w;
      a.skty[j] += ktyv * w;
      if (!commit_only) candidate(j, xv, ktyv);
    };
    row_block_spmv(a.At, ycur, item, prod, rowsum, red, epi);
  } else {
    const RowItem it = a.At.items[item];
    const int j = it.row_begin + threadIdx.x;
    if (j < it.row_end) candidate(j, a.x[j], a.kty[j]);
  }
  if (commit_only) return;
  const double s = block_sum_mixed(acc, red);
  if (threadIdx.x == 0) a.part_p[item] = s;
}

template <class T>
struct BatchDualArgs {
  CsrView<T> A;
  BatchIndex bi;
  const T* dx;
  const T* b;
  T* y0;
  T* y1;
  T* kx0;
  T* kx1;
  T* sy;
  T* skx;
  StepState* st;
  const double* part_p;
  double* part_d;  // [interaction | ||dy||^2], num_items each
  int num_items;
  int mode;
  int direct;
};

template <class T>
__global__ void __launch_bounds__(kBlock) batch_dual_kernel(BatchDualArgs<T> a) {
  __shared__ T prod[kItemNnz];
  __shared__ T rowsum[kBlock];
  __shared__ double red[32];
  __shared__ int is_last;
  const int item = blockIdx.x;
  const int inst = a.bi.item_inst_d[item];
  StepState* st = a.st + inst;
  if (st->done) return;
  const bool pending = st->pending_commit != 0;
  const bool commit_only = a.mode == kStepCommitOnly;
  if (commit_only && !pending) return;
  const T w = (T)st->commit_weight;
  const T od = (T)(st->omega * st->tau);
  const int p = st->parity;
  const T* ycur = p ? a.y1 : a.y0;
  T* ynew = p ? a.y0 : a.y1;
  const T* kxcur = p ? a.kx1 : a.kx0;
  T* kxnew = p ? a.kx0 : a.kx1;
  const int ineq_from = a.bi.row_off[inst] + a.bi.neq[inst];
  T acc_i = T(0), acc_d = T(0);
  if (commit_only) {
    const RowItem it = a.A.items[item];
    const int i = it.row_begin + threadIdx.x;
    if (i < it.row_end) {
      a.sy[i] += ycur[i] * w;
      a.skx[i] += kxcur[i] * w;
    }
  } else {
    const bool direct = a.direct != 0;
    auto epi = [&](int i, T rs) {
      const T yv = ycur[i], kxv = kxcur[i];
      if (pending) {
        a.sy[i] += yv * w;
        a.skx[i] += kxv * w;
      }
      const T kdx = direct ? rs - kxv : rs;
      T v = yv + od * ((a.b[i] - T(2) * kdx) - kxv);
      if (i >= ineq_from) v = jmax(v, T(0));
      const T d = v - yv;
      ynew[i] = yv + d;
      kxnew[i] = direct ? rs : kxv + kdx;
      acc_i += kdx * d;
      acc_d += d * d;
    };
    row_block_spmv(a.A, a.dx, item, prod, rowsum, red, epi);
  }
  if (!commit_only) {
    const double bi = block_sum_mixed(acc_i, red);
    const double bd = block_sum_mixed(acc_d, red);
    if (threadIdx.x == 0) {
      a.part_d[item] = bi;
      a.part_d[a.num_items + item] = bd;
    }
  }
  const int d0 = a.bi.d_item_begin[inst], d1 = a.bi.d_item_begin[inst + 1];
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned prev = atomicAdd(&st->arrive, 1u);
    is_last = (prev == (unsigned)(d1 - d0 - 1)) ? 1 : 0;
  }
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  if (commit_only) {
    if (threadIdx.x == 0) {
      st->pending_commit = 0;
      st->arrive = 0;
    }
    return;
  }
  // the instance's last CTA: its partials in item order (same order as a lone solve)
  double si = 0.0, sd = 0.0, sx = 0.0;
  for (int k = d0 + threadIdx.x; k < d1; k += kBlock) {
    si += __ldcg(a.part_d + k);
    sd += __ldcg(a.part_d + a.num_items + k);
  }
  const int p0 = a.bi.p_item_begin[inst], p1 = a.bi.p_item_begin[inst + 1];
  for (int k = p0 + threadIdx.x; k < p1; k += kBlock) sx += __ldcg(a.part_p + k);
  si = block_sum(si, red);
  sd = block_sum(sd, red);
  sx = block_sum(sx, red);
  if (threadIdx.x == 0) {
    st->arrive = 0;
    if (pending) st->primal_spmv += 1;
    st->pending_commit = 0;
    step_decision(st, si, sx, sd);
  }
}

// ---- segmented FP64 reductions --------------------------------------------------
// A segment item is a contiguous element range of one instance; partials are written
// per item, and one CTA per instance reduces its items in order.
template <int Q, unsigned MAXMASK, class F>
__global__ void __launch_bounds__(kBlock) seg_reduce_kernel(const SegItem* items, const uint8_t* active, F f,
                                                            double* partials, int num_items) {
  __shared__ double sh[32];
  const SegItem it = items[blockIdx.x];
  if (!active[it.inst]) return;
  double acc[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) acc[q] = 0.0;
  for (int i = it.begin + threadIdx.x; i < it.end; i += kBlock) f((long long)i, acc);
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const double r = ((MAXMASK >> q) & 1u) ? block_nan_max(acc[q], sh) : block_sum(acc[q], sh);
    if (threadIdx.x == 0) partials[(size_t)q * num_items + blockIdx.x] = r;
  }
}

template <int Q, unsigned MAXMASK>
__global__ void __launch_bounds__(kBlock) seg_finalize_kernel(const int32_t* inst_item_begin, const uint8_t* active,
                                                              const double* partials, int num_items, double* out,
                                                              int out_stride) {
  __shared__ double sh[32];
  const int inst = blockIdx.x;
  if (!active[inst]) return;
  const int k0 = inst_item_begin[inst], k1 = inst_item_begin[inst + 1];
  for (int q = 0; q < Q; ++q) {
    const bool is_max = (MAXMASK >> q) & 1u;
    double a = 0.0;
    for (int k = k0 + threadIdx.x; k < k1; k += kBlock) {
      const double v = partials[(size_t)q * num_items + k];
      a = is_max ? nan_max(a, v) : a + v;
    }
    a = is_max ? block_nan_max(a, sh) : block_sum(a, sh);
    if (threadIdx.x == 0) out[(size_t)inst * out_stride + q] = a;
  }
}

// Per-element helpers driven by per-instance flags / weights.
template <class T>
struct BatchVecArgs {
  const int32_t* inst_of;   // instance of each element
  const uint8_t* flag;      // per-instance selector
  const StepState* st;
  int len;
};

// compute_average! (or the current point when the instance has no average yet)
template <class T>
__global__ void batch_average_n_kernel(BatchVecArgs<T> v, const uint8_t* use_current, const T* sx, const T* skty,
                                       const T* c, const T* x, const T* grad, T* ax, T* agrad) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < v.len; j += gridDim.x * blockDim.x) {
    const int k = v.inst_of[j];
    if (!v.flag[k]) continue;
    if (use_current[k]) {
      ax[j] = x[j];
      agrad[j] = grad[j];
    } else {
      const double wx = v.st[k].sum_w_primal, wy = v.st[k].sum_w_dual;
      ax[j] = (T)((double)sx[j] / wx);
      const T g = (T)(-(double)skty[j] / wy);
      agrad[j] = g + c[j];
    }
  }
}

template <class T>
__global__ void batch_average_m_kernel(BatchVecArgs<T> v, const uint8_t* use_current, const T* sy, const T* skx,
                                       const T* y0, const T* y1, const T* kx0, const T* kx1, T* ay, T* akx) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < v.len; i += gridDim.x * blockDim.x) {
    const int k = v.inst_of[i];
    if (!v.flag[k]) continue;
    if (use_current[k]) {
      const int p = v.st[k].parity;
      ay[i] = p ? y1[i] : y0[i];
      akx[i] = p ? kx1[i] : kx0[i];
    } else {
      const double wx = v.st[k].sum_w_primal, wy = v.st[k].sum_w_dual;
      ay[i] = (T)((double)sy[i] / wy);
      akx[i] = (T)((double)skx[i] / wx);
    }
  }
}

template <class T>
__global__ void batch_grad_kernel(BatchVecArgs<T> v, const T* c, const T* kty, T* grad) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < v.len; j += gridDim.x * blockDim.x) {
    if (!v.flag[v.inst_of[j]]) continue;
    grad[j] = c[j] - kty[j];
  }
}

// Restart actions (src/saddle_point_gpu.jl:575-614) for the instances with flag set:
// to_avg[k] selects reset-to-average; sums are cleared; the restart point is stored.
template <class T>
__global__ void batch_restart_n_kernel(BatchVecArgs<T> v, const uint8_t* to_avg, const T* ax, const T* agrad,
                                       const T* c, T* x, T* kty, T* grad, T* sx, T* skty, T* rx, T* rgrad) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < v.len; j += gridDim.x * blockDim.x) {
    const int k = v.inst_of[j];
    if (!v.flag[k]) continue;
    if (to_avg[k]) {
      x[j] = ax[j];
      kty[j] = c[j] - agrad[j];
      grad[j] = agrad[j];
    }
    sx[j] = T(0);
    skty[j] = T(0);
    rx[j] = x[j];
    rgrad[j] = grad[j];
  }
}

template <class T>
__global__ void batch_restart_m_kernel(BatchVecArgs<T> v, const uint8_t* to_avg, const T* ay, const T* akx, T* y0,
                                       T* y1, T* kx0, T* kx1, T* sy, T* skx, T* ry, T* rkx) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < v.len; i += gridDim.x * blockDim.x) {
    const int k = v.inst_of[i];
    if (!v.flag[k]) continue;
    const int p = v.st[k].parity;
    T* yc = p ? y1 : y0;
    T* kc = p ? kx1 : kx0;
    if (to_avg[k]) {
      yc[i] = ay[i];
      kc[i] = akx[i];
    }
    sy[i] = T(0);
    skx[i] = T(0);
    ry[i] = yc[i];
    rkx[i] = kc[i];
  }
}

}  // namespace gpdhg
