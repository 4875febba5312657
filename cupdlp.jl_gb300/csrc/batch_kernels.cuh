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

// ---- segmented FP64 reductions --------------------------------------------------
// A segment item is a contiguous element range of one instance; partials are written
// per item, and one CTA per instance reduces its items in order.
template <int Q, unsigned MAXMASK, class F>
__global__ void __launch_bounds__(kBlock) seg_reduce_kernel(const SegItem* items, const uint8_t* active, F f,
                                                            double* partials, int num_items) {
  __shared__ double sh[(Q < kRedChunk ? Q : kRedChunk) * kBlock];
  __shared__ double res[Q];
  const SegItem it = items[blockIdx.x];
  if (!active[it.inst]) return;
  double acc[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) acc[q] = 0.0;
  for (int i = it.begin + threadIdx.x; i < it.end; i += kBlock) f((long long)i, acc);
  const double r = block_reduce_q<Q, MAXMASK>(acc, sh, res);
  if ((int)threadIdx.x < Q) partials[(size_t)threadIdx.x * num_items + blockIdx.x] = r;
}

template <int Q, unsigned MAXMASK>
__global__ void __launch_bounds__(kBlock) seg_finalize_kernel(const int32_t* inst_item_begin, const uint8_t* active,
                                                              const double* partials, int num_items, double* out,
                                                              int out_stride) {
  __shared__ double sh[(Q < kRedChunk ? Q : kRedChunk) * kBlock];
  __shared__ double res[Q];
  const int inst = blockIdx.x;
  if (!active[inst]) return;
  const int k0 = inst_item_begin[inst], k1 = inst_item_begin[inst + 1];
  double acc[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) acc[q] = 0.0;
  for (int k = k0 + threadIdx.x; k < k1; k += kBlock) {
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const double v = partials[(size_t)q * num_items + k];
      acc[q] = ((MAXMASK >> q) & 1u) ? nan_max(acc[q], v) : acc[q] + v;
    }
  }
  const double r = block_reduce_q<Q, MAXMASK>(acc, sh, res);
  if ((int)threadIdx.x < Q) out[(size_t)inst * out_stride + threadIdx.x] = r;
}

// Per-element helpers driven by per-instance flags / weights.
template <class T>
struct BatchVecArgs {
  const int32_t* inst_of;   // instance of each element
  const uint8_t* flag;      // per-instance selector
  const StepState* st;
  int len;
};

// compute_average! (or the current point when the instance has no average yet), the average's
// K'y given as aty = A' y-bar
template <class T>
__global__ void batch_average_n_kernel(BatchVecArgs<T> v, const uint8_t* use_current, const T* sx, const T* aty,
                                       const T* c, const T* x, const T* grad, T* ax, T* agrad) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < v.len; j += gridDim.x * blockDim.x) {
    const int k = v.inst_of[j];
    if (!v.flag[k]) continue;
    if (use_current[k]) {
      ax[j] = x[j];
      agrad[j] = grad[j];
    } else {
      const StepState& q = v.st[k];
      ax[j] = (T)div_rcp((double)sx[j], q.sum_w_primal, q.rcp_w_primal);
      agrad[j] = c[j] - aty[j];  // aty = A' y-bar
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
      const StepState& q = v.st[k];
      ay[i] = (T)div_rcp((double)sy[i], q.sum_w_dual, q.rcp_w_dual);
      akx[i] = (T)div_rcp((double)skx[i], q.sum_w_primal, q.rcp_w_primal);
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
                                       const T* c, T* x, T* kty, T* grad, T* sx, T* rx, T* rgrad) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < v.len; j += gridDim.x * blockDim.x) {
    const int k = v.inst_of[j];
    if (!v.flag[k]) continue;
    if (to_avg[k]) {
      x[j] = ax[j];
      kty[j] = c[j] - agrad[j];
      grad[j] = agrad[j];
    }
    sx[j] = T(0);
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
