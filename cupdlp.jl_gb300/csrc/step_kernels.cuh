// step_kernels.cuh — the two fused kernels of one PDHG step attempt.
//
// Reference step (src/primal_dual_hybrid_gradient_gpu.jl:177-413) per attempt:
//   x^ = proj_[l,u](x - (tau/omega)(c - K'y));  dx = x^ - x            (:177-197)
//   K dx                                                               (:225, cuSPARSE)
//   y^ = y + omega tau (b - 2 K dx - K x);  y^[ineq] >= 0;  dy = y^ - y (:232-260)
//   |dy . K dx|, ||dx||, ||dy||                                        (:324-338)
//   accept if tau <= movement / interaction; then x += dx, Kx += K dx, y += dy,
//   K'y = A' y and the four weighted sums (:297-319, src/saddle_point_gpu.jl:131-221);
//   tau <- min((1-(k+1)^-0.3) limit, (1+(k+1)^-0.6) tau)                (:405-409)
//
// Here one attempt is two kernels and no host round trip:
//   primal_step_kernel: [if the previous attempt was accepted] K'y = A' y (CSR of A'),
//       x += dx, and the x / K'y weighted sums; then the next dx, and per-CTA ||dx||^2.
//   dual_step_kernel:   [if the previous attempt was accepted] the y / Kx weighted sums;
//       then K dx (CSR of A), the projected dual candidate, Kx + K dx into the other half of
//       the double-buffered y / Kx, per-CTA interaction and ||dy||^2 partials; the last CTA
//       to finish reduces all partials in a fixed order and takes the accept/reject and
//       step-size decision, flipping the buffer parity on accept.
// So an accepted step costs exactly one pass over A and one over A'; a rejected attempt
// costs one pass over A plus a streaming pass over the n-vectors.
//
// `direct` mode (the FP32 bulk phase): the primal kernel stores the candidate x^ itself
// (in the dx buffer) and the dual kernel forms K x^ = A x^ from scratch, K dx = K x^ - K x,
// and stores K x^ as the next K x. The reference's incremental K x += K dx (:304) is kept
// in FP64 for parity; in FP32 it drifts by ~1e-6 relative, which this mode removes.
#pragma once

#include "common.cuh"

namespace gpdhg {

enum StepMode : int { kStepNormal = 0, kStepCommitOnly = 1 };

// Per-thread accumulators in T, warp tree in T, across warps in FP64.
template <class T>
__device__ __forceinline__ double block_sum_mixed(T v, double* sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) sh[wid] = (double)v;
  __syncthreads();
  double r = 0.0;
  if (wid == 0) {
    r = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0.0;
    r = warp_sum(r);
  }
  return r;
}

__device__ __forceinline__ int floor_pow2(int v) { return 1 << (31 - __clz(v)); }

// Row block of item `item` of M times xg; calls epi(row, row_sum) once per row.
// Every thread of the CTA must call this (it synchronises).
template <class T, class Epi>
__device__ __forceinline__ void row_block_spmv(const CsrView<T>& M, const T* __restrict__ xg, int item,
                                               T* prod, T* rowsum, double* red, Epi& epi) {
  const int tid = threadIdx.x;
  const RowItem it = M.items[item];
  const int r0 = it.row_begin, r1 = it.row_end;
  const int rows = r1 - r0;
  const int s0 = M.row_ptr[r0];
  const int s1 = M.row_ptr[r1];
  const int cnt = s1 - s0;
  if (cnt > kItemNnz) {
    // long row: the whole CTA strides over it, then a fixed-order tree
    T acc = T(0);
    for (int e = s0 + tid; e < s1; e += kBlock) acc += M.val[e] * xg[M.col[e]];
    acc = warp_sum(acc);
    __syncthreads();
    T* wsum = rowsum;  // reuse: 8 warp sums
    if ((tid & 31) == 0) wsum[tid >> 5] = acc;
    __syncthreads();
    if (tid == 0) {
      T s = T(0);
      for (int w = 0; w < kBlock / 32; ++w) s += wsum[w];
      epi(r0, s);
    }
    return;
  }
  for (int e = tid; e < cnt; e += kBlock) prod[e] = M.val[s0 + e] * xg[M.col[s0 + e]];
  __syncthreads();
  const int g = min(32, floor_pow2(kBlock / (rows > 0 ? rows : 1)));
  const int grp = tid / g, lane = tid % g;
  T acc = T(0);
  if (grp < rows) {
    const int a = M.row_ptr[r0 + grp] - s0, b = M.row_ptr[r0 + grp + 1] - s0;
    for (int e = a + lane; e < b; e += g) acc += prod[e];
  }
  for (int o = g >> 1; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o, g);
  if (lane == 0 && grp < rows) rowsum[grp] = acc;
  __syncthreads();
  if (tid < rows) epi(r0 + tid, rowsum[tid]);
  (void)red;
}

template <class T>
struct PrimalArgs {
  CsrView<T> At;   // CSR of A' (n rows)
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
  const StepState* st;
  double* part_p;  // one ||dx||^2 partial per CTA
  int mode;
  int direct;
};

template <class T>
__global__ void __launch_bounds__(kBlock) primal_step_kernel(PrimalArgs<T> a) {
  __shared__ T prod[kItemNnz];
  __shared__ T rowsum[kBlock];
  __shared__ double red[32];
  const StepState* st = a.st;
  if (st->done) return;
  const bool pending = st->pending_commit != 0;
  const bool commit_only = a.mode == kStepCommitOnly;
  if (commit_only && !pending) return;
  const T w = (T)st->commit_weight;
  const T tto = (T)(st->tau / st->omega);  // step_size / primal_weight
  const T* ycur = st->parity ? a.y1 : a.y0;
  const int item = blockIdx.x;
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
struct DualArgs {
  CsrView<T> A;    // CSR of A (m rows)
  const T* dx;
  const T* b;
  T* y0;
  T* y1;
  T* kx0;
  T* kx1;
  T* sy;
  T* skx;
  int neq;
  int num_p_blocks;
  StepState* st;
  const double* part_p;
  double* part_d;  // [interaction | ||dy||^2], gridDim.x each
  int mode;
  int direct;      // dx holds x^ and the row sums are K x^ (see above)
};

// Decision of take_step! for one attempt (thread 0 of the last CTA).
__device__ __forceinline__ void step_decision(StepState* st, double inter_signed, double dx2, double dy2) {
  st->total_iters += st->constant_step ? 0 : 1;
  st->kkt_passes += 1.0;
  st->attempts_in_chunk += 1;
  const double omega = st->omega;
  const double tau = st->tau;
  const double inter = fabs(inter_signed);
  const double ndx = sqrt(dx2), ndy = sqrt(dy2);
  const double movement = 0.5 * omega * ndx * ndx + (0.5 / omega) * ndy * ndy;
  double limit;
  bool accept;
  if (st->constant_step) {
    limit = __longlong_as_double(0x7ff0000000000000LL);
    accept = true;
  } else {
    if (inter > 0.0) {
      limit = movement / inter;
      if (movement == 0.0) {
        // :384-390: terminate at the next evaluation; tau is left as it is
        st->numerical_error = 1;
        st->done = 1;
        st->pending_commit = 0;
        return;
      }
    } else {
      limit = __longlong_as_double(0x7ff0000000000000LL);
    }
    accept = tau <= limit;
  }
  st->last_limit = limit;
  if (accept) {
    st->parity ^= 1;
    st->pending_commit = 1;
    st->commit_weight = st->iter_start_tau;
    st->count_primal += 1;
    st->count_dual += 1;
    st->sum_w_primal += st->iter_start_tau;
    st->sum_w_dual += st->iter_start_tau;
    st->accepted += 1;
    st->accepted_in_chunk += 1;
  } else {
    st->pending_commit = 0;
    st->rejected += 1;
  }
  if (!st->constant_step) {
    // (1 - (k+1)^-r) and (1 + (k+1)^-g): from the host-computed table while it lasts
    const long long k = st->total_iters;
    double f1, f2;
    if (st->pow_table && k < st->pow_table_len) {
      f1 = st->pow_table[2 * k];
      f2 = st->pow_table[2 * k + 1];
    } else {
      const double k1 = (double)(k + 1);
      f1 = 1.0 - 1.0 / pow(k1, st->reduction_exponent);
      f2 = 1.0 + 1.0 / pow(k1, st->growth_exponent);
    }
    const double first = f1 * limit;
    const double second = f2 * tau;
    st->tau = jmin(first, second);
  }
  if (accept) st->iter_start_tau = st->tau;
  if (st->accepted_in_chunk >= st->target_in_chunk || st->attempts_in_chunk >= st->max_attempts_in_chunk)
    st->done = 1;
}

template <class T>
__global__ void __launch_bounds__(kBlock) dual_step_kernel(DualArgs<T> a) {
  __shared__ T prod[kItemNnz];
  __shared__ T rowsum[kBlock];
  __shared__ double red[32];
  __shared__ int is_last;
  StepState* st = a.st;
  if (st->done) return;
  const bool pending = st->pending_commit != 0;
  const bool commit_only = a.mode == kStepCommitOnly;
  if (commit_only && !pending) {
    // nothing to commit; the flag is already clear
    return;
  }
  const T w = (T)st->commit_weight;
  const T od = (T)(st->omega * st->tau);  // primal_weight * step_size
  const int p = st->parity;
  const T* ycur = p ? a.y1 : a.y0;
  T* ynew = p ? a.y0 : a.y1;
  const T* kxcur = p ? a.kx1 : a.kx0;
  T* kxnew = p ? a.kx0 : a.kx1;
  const int item = blockIdx.x;
  T acc_i = T(0), acc_d = T(0);
  if (item < a.A.num_items) {
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
        if (i >= a.neq) v = jmax(v, T(0));
        const T d = v - yv;
        ynew[i] = yv + d;
        kxnew[i] = direct ? rs : kxv + kdx;
        acc_i += kdx * d;
        acc_d += d * d;
      };
      row_block_spmv(a.A, a.dx, item, prod, rowsum, red, epi);
    }
  }
  double bi = 0.0, bd = 0.0;
  if (!commit_only) {
    bi = block_sum_mixed(acc_i, red);
    bd = block_sum_mixed(acc_d, red);
    if (threadIdx.x == 0) {
      a.part_d[item] = bi;
      a.part_d[gridDim.x + item] = bd;
    }
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned prev = atomicAdd(&st->arrive, 1u);
    is_last = (prev == gridDim.x - 1) ? 1 : 0;
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
  // last CTA: fixed-order reduction of every CTA's partials
  double si = 0.0, sd = 0.0, sx = 0.0;
  for (int k = threadIdx.x; k < (int)gridDim.x; k += kBlock) {
    si += __ldcg(a.part_d + k);
    sd += __ldcg(a.part_d + gridDim.x + k);
  }
  for (int k = threadIdx.x; k < a.num_p_blocks; k += kBlock) sx += __ldcg(a.part_p + k);
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

}  // namespace gpdhg
