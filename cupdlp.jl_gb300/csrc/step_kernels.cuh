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
#include "spmv.cuh"

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

// Per-instance ranges of the packed layout (a lone LP is a batch of one).
struct BatchIndex {
  const int32_t* item_inst_p;  // instance of each A' item
  const int32_t* item_inst_d;  // instance of each A item
  const int32_t* p_item_begin; // first A' item of each instance (count + 1 entries)
  const int32_t* d_item_begin; // first A item of each instance (count + 1 entries)
  const int32_t* row_off;      // first packed row of each instance (count + 1)
  const int32_t* neq;          // equality rows of each instance
};

template <class T>
struct PrimalArgs {
  CsrView<T> At;   // CSR of A' (n rows)
  BatchIndex bi;
  const T* c;
  const T* l;
  const T* u;
  T* x;
  T* dx;           // dx, or x^ in direct mode
  T* kty;
  T* sx;
  T* skty;
  const T* y0;
  const T* y1;
  const StepState* st;  // one per instance
  double* part_p;       // one ||dx||^2 partial per CTA
  int mode;
  int direct;
};

template <class T>
struct PrimalPre {
  T x, dx, sx, skty, c, l, u;
};

template <class T>
__global__ void __launch_bounds__(kBlock, 4) primal_step_kernel(PrimalArgs<T> a) {
  __shared__ T stage[kStage];
  __shared__ T wsum[kBlock / 32];
  __shared__ double red[32];
  const int item = blockIdx.x;
  const StepState* st = a.st + a.bi.item_inst_p[item];
  if (st->done) return;
  const bool pending = st->pending_commit != 0;
  const bool commit_only = a.mode == kStepCommitOnly;
  if (commit_only && !pending) return;
  const bool direct = a.direct != 0;
  const T w = (T)st->commit_weight;
  const T tto = (T)(st->tau / st->omega);  // step_size / primal_weight
  const T* ycur = st->parity ? a.y1 : a.y0;
  T acc = T(0);
  auto candidate = [&](int j, T xv, T ktyv, T c, T l, T u) {
    T v = xv - tto * (c - ktyv);
    v = imin(u, imax(l, v));   // min(u, max(l, .)) (:192); NaN-free data is validated on entry
    const T d = v - xv;
    a.dx[j] = direct ? v : d;  // gathered by the dual kernel next: a normal (L2-resident) store
    acc += d * d;
  };
  if (pending) {
    auto pre = [&](int j) {
      PrimalPre<T> p;
      p.x = direct ? T(0) : lds(a.x + j);
      p.dx = lds(a.dx + j);
      p.sx = lds(a.sx + j);
      p.skty = lds(a.skty + j);
      if (!commit_only) {
        p.c = lds(a.c + j);
        p.l = lds(a.l + j);
        p.u = lds(a.u + j);
      }
      return p;
    };
    auto post = [&](int j, T ktyv, const PrimalPre<T>& p) {
      const T xv = direct ? p.dx : p.x + p.dx;   // x += dx (:303)
      sts(a.x + j, xv);
      sts(a.kty + j, ktyv);                      // K'y = A'y (:307)
      sts(a.sx + j, p.sx + xv * w);              // weighted sums (src/saddle_point_gpu.jl:137,182)
      sts(a.skty + j, p.skty + ktyv * w);
      if (!commit_only) candidate(j, xv, ktyv, p.c, p.l, p.u);
    };
    spmv_item(a.At, ycur, item, stage, wsum, pre, post);
  } else {
    const RowItem it = a.At.items[item];
    for (int j = it.row_begin + threadIdx.x; j < it.row_end; j += kBlock)
      candidate(j, lds(a.x + j), lds(a.kty + j), lds(a.c + j), lds(a.l + j), lds(a.u + j));
  }
  if (commit_only) return;
  const double s = block_sum_mixed(acc, red);
  if (threadIdx.x == 0) a.part_p[item] = s;
}

template <class T>
struct DualArgs {
  CsrView<T> A;    // CSR of A (m rows)
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
  int direct;      // dx holds x^ and the row sums are K x^ (see above)
};

template <class T>
struct DualPre {
  T y, kx, b, sy, skx;
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
__global__ void __launch_bounds__(kBlock, 4) dual_step_kernel(DualArgs<T> a) {
  __shared__ T stage[kStage];
  __shared__ T wsum[kBlock / 32];
  __shared__ double red[32];
  __shared__ int is_last;
  const int item = blockIdx.x;
  const int inst = a.bi.item_inst_d[item];
  StepState* st = a.st + inst;
  if (st->done) return;
  const bool pending = st->pending_commit != 0;
  const bool commit_only = a.mode == kStepCommitOnly;
  if (commit_only && !pending) return;
  const bool direct = a.direct != 0;
  const T w = (T)st->commit_weight;
  const T od = (T)(st->omega * st->tau);  // primal_weight * step_size
  const int p = st->parity;
  const T* ycur = p ? a.y1 : a.y0;
  T* ynew = p ? a.y0 : a.y1;
  const T* kxcur = p ? a.kx1 : a.kx0;
  T* kxnew = p ? a.kx0 : a.kx1;
  const int ineq_from = a.bi.row_off[inst] + a.bi.neq[inst];
  T acc_i = T(0), acc_d = T(0);
  if (commit_only) {
    const RowItem it = a.A.items[item];
    for (int i = it.row_begin + threadIdx.x; i < it.row_end; i += kBlock) {
      a.sy[i] += ycur[i] * w;
      a.skx[i] += kxcur[i] * w;
    }
  } else {
    auto pre = [&](int i) {
      DualPre<T> q;
      q.y = lds(ycur + i);
      q.kx = lds(kxcur + i);
      q.b = lds(a.b + i);
      if (pending) {
        q.sy = lds(a.sy + i);
        q.skx = lds(a.skx + i);
      }
      return q;
    };
    auto post = [&](int i, T rs, const DualPre<T>& q) {
      if (pending) {
        sts(a.sy + i, q.sy + q.y * w);
        sts(a.skx + i, q.skx + q.kx * w);
      }
      const T kdx = direct ? rs - q.kx : rs;
      T v = q.y + od * ((q.b - T(2) * kdx) - q.kx);   // (:247), extrapolation coefficient 1
      if (i >= ineq_from) v = imax(v, T(0));          // (:254)
      const T d = v - q.y;
      ynew[i] = q.y + d;                              // y += dy (:306); gathered by the next primal kernel
      sts(kxnew + i, direct ? rs : q.kx + kdx);       // Kx += K dx (:304)
      acc_i += kdx * d;
      acc_d += d * d;
    };
    spmv_item(a.A, a.dx, item, stage, wsum, pre, post);
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
  // the instance's last CTA: its partials in item order, then take_step!'s decision
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

}  // namespace gpdhg
