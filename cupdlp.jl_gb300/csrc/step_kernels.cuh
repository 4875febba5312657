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
// Here one attempt is two persistent kernels (pipe.cuh) and no host round trip:
//   primal_step_kernel: [if the previous attempt was accepted] K'y = A' y (chunks of A'),
//       x += dx, and the x / K'y weighted sums; then the next dx, and per-chunk ||dx||^2.
//   dual_step_kernel:   [if the previous attempt was accepted] the y / Kx weighted sums;
//       then K dx (chunks of A), the projected dual candidate, Kx + K dx into the other half
//       of the double-buffered y / Kx, per-chunk interaction and ||dy||^2 partials; the CTA
//       that finishes an instance's last chunk reduces that instance's partials in chunk
//       order and takes the accept/reject and step-size decision, flipping the buffer
//       parity on accept.
// So an accepted step costs exactly one pass over A and one over A'; a rejected attempt
// costs one pass over A plus a streaming pass over the n-vectors.
//
// `direct` mode (the FP32 bulk phase): the primal kernel stores the candidate x^ itself
// (in the dx buffer) and the dual kernel forms K x^ = A x^ from scratch, K dx = K x^ - K x,
// and stores K x^ as the next K x. The reference's incremental K x += K dx (:304) is kept
// in FP64 for parity; in FP32 it drifts by ~1e-6 relative, which this mode removes.
#pragma once

#include "common.cuh"
#include "pipe.cuh"

namespace gpdhg {

enum StepMode : int { kStepNormal = 0, kStepCommitOnly = 1 };

// Per-instance ranges of the packed layout (a lone LP is a batch of one).
struct BatchIndex {
  const int32_t* p_chunk_begin;  // first A' chunk of each instance (count + 1 entries)
  const int32_t* d_chunk_begin;  // first A chunk of each instance (count + 1 entries)
  const int32_t* row_off;        // first packed row of each instance (count + 1)
  const int32_t* neq;            // equality rows of each instance
};

// Vector slots of the primal stage: pending commit / no pending commit.
enum PrimalSlot { kPX = 0, kPDX = 1, kPKTY = 1, kPSX = 2, kPSKTY = 3, kPC = 4, kPL = 5, kPU = 6, kPrimalSlots = 7 };
// Vector slots of the dual stage.
enum DualSlot { kDY = 0, kDKX = 1, kDB = 2, kDSY = 3, kDSKX = 4, kDualSlots = 5 };

template <class T>
struct PrimalArgs {
  ChunkView<T> plan;   // chunks of A' (rows = variables)
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
  StepState* st;   // one per instance
  double* part_p;  // one ||dx||^2 partial per chunk
  int mode;
  int direct;
  int single;      // one instance: a finished solve returns at once
};

template <class T>
struct DualArgs {
  ChunkView<T> plan;   // chunks of A (rows = constraints)
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
  double* part_d;  // [interaction | ||dy||^2], one pair per chunk
  int mode;
  int direct;      // dx holds x^ and the row sums are K x^ (see above)
  int single;
};

// Shared memory beyond the dynamic stage ring.
template <class T>
struct StepSmem {
  uint64_t bars[kPipeStages];
  StageHdr hdr[kPipeStages];
  ScanSmem<T> scan;
  double red[2 * (kBlock / 32)];
  double red2[32];
  int flag;
};

template <class T>
__global__ void __launch_bounds__(kBlock, 2) primal_step_kernel(PrimalArgs<T> a) {
  using L = StageLayout<T, kPrimalSlots>;
  extern __shared__ __align__(128) uint8_t ring_raw[];
  __shared__ StepSmem<T> sm;
  // StageLayout::kTotal has 128 spare bytes so the ring can start on a 128-byte boundary
  uint8_t* ring = ring_raw + ((128u - (smem_addr(ring_raw) & 127u)) & 127u);
  if (a.single && a.st->done) return;
  const bool commit_only = a.mode == kStepCommitOnly;
  const bool direct = a.direct != 0;
  const int tid = threadIdx.x;
  auto stage = [&](int s) { return ring + (size_t)s * L::kBytes; };
  auto vec = [&](int s, int slot) { return reinterpret_cast<T*>(stage(s) + L::off_vec + slot * L::kVec); };

  auto issue = [&](int, int s, const Chunk& ch, const StepScalars& v) {
    StageHdr& h = sm.hdr[s];
    h.ch = ch;
    h.issued = 0;
    if (v.done) return;
    const int pending = v.pending;
    if (commit_only && !pending) return;
    h.pending = pending;
    h.parity = v.parity;
    h.s0 = v.w;
    h.s1 = v.tau / v.omega;  // step_size / primal_weight
    const int al = ch.row_begin & ~(L::V - 1);
    const int cnt = ch.rows ? ((ch.row_begin + ch.rows + L::V - 1) & ~(L::V - 1)) - al : 0;
    h.voff = ch.row_begin - al;
    uint64_t* bar = &sm.bars[s];
    const uint32_t vb = (uint32_t)(cnt * (int)sizeof(T));
    const uint32_t mb = pending ? (uint32_t)blob_bytes<T>(ch.rows, ch.nnz) : 0u;
    int nv;
    if (pending) nv = (direct ? 3 : 4) + (commit_only ? 0 : 3);
    else nv = 5;
    mbar_arrive_expect_tx(bar, mb + (uint32_t)nv * vb);
    if (mb) bulk_load_stream(stage(s), a.plan.blob + ch.blob, mb, bar, policy_evict_first());
    if (pending) {
      if (!direct) issue_vec(vec(s, kPX), a.x, al, cnt, bar);
      issue_vec(vec(s, kPDX), a.dx, al, cnt, bar);
      issue_vec(vec(s, kPSX), a.sx, al, cnt, bar);
      issue_vec(vec(s, kPSKTY), a.skty, al, cnt, bar);
    } else {
      issue_vec(vec(s, kPX), a.x, al, cnt, bar);
      issue_vec(vec(s, kPKTY), a.kty, al, cnt, bar);
    }
    if (!commit_only) {
      issue_vec(vec(s, kPC), a.c, al, cnt, bar);
      issue_vec(vec(s, kPL), a.l, al, cnt, bar);
      issue_vec(vec(s, kPU), a.u, al, cnt, bar);
    }
    h.issued = 1;
  };

  auto gather = [&](int s) {
    const StageHdr& h = sm.hdr[s];
    if (!h.issued || !h.pending) return;
    const int32_t* col = reinterpret_cast<const int32_t*>(stage(s) + blob_rp_bytes<T>(h.ch.rows));
    T* xs = reinterpret_cast<T*>(stage(s) + L::off_xs);
    const T* yg = h.parity ? a.y1 : a.y0;
    for (int k = tid; k < h.ch.nnz; k += kBlock) gather_async(xs + pad_index(k, PipeTraits<T>::kPadShift), yg + col[k]);
  };

  auto compute = [&](int c, int s) {
    const StageHdr& h = sm.hdr[s];
    if (!h.issued) return;
    const Chunk& ch = h.ch;
    const T w = (T)h.s0;
    const T tto = (T)h.s1;
    T acc = T(0);
    int slot = c;  // partial slot of this chunk's rows
    auto candidate = [&](int j, T xv, T ktyv, T cv, T lv, T uv) {
      T v = xv - tto * (cv - ktyv);
      v = imin(uv, imax(lv, v));   // min(u, max(l, .)) (:192); NaN-free data is validated on entry
      const T d = v - xv;
      a.dx[j] = direct ? v : d;    // gathered by the dual kernel next: a normal (L2-resident) store
      acc += d * d;
    };
    int rows = ch.rows;
    if (h.pending) {
      uint8_t* base = stage(s);
      const int32_t* rp = reinterpret_cast<const int32_t*>(base);
      const T* val = reinterpret_cast<const T*>(base + blob_rp_bytes<T>(ch.rows) + blob_col_bytes<T>(ch.nnz));
      const T* xs = reinterpret_cast<const T*>(base + L::off_xs);
      T* rs = reinterpret_cast<T*>(base + L::off_rs);
      chunk_row_sums<T>(rp, val, xs, ch.rows, ch.nnz, ch.e_log2, rs, sm.scan);
      __syncthreads();
      if (ch.split >= 0) {
        // a split row's contribution always lands in its first piece's slot, whichever
        // piece finishes it, so the decision's reduction order does not depend on timing
        if (tid == 0 && !commit_only) a.part_p[c] = 0.0;
        if (!split_combine<T>(ch, a.plan, rs, &sm.flag)) return;
        slot = c - ch.piece;
      }
      const T* vx = vec(s, kPX);
      const T* vdx = vec(s, kPDX);
      const T* vsx = vec(s, kPSX);
      const T* vsk = vec(s, kPSKTY);
      for (int r = tid; r < rows; r += kBlock) {
        const int j = ch.row_begin + r, q = h.voff + r;
        const T ktyv = rs[r];
        const T xv = direct ? vdx[q] : vx[q] + vdx[q];   // x += dx (:303)
        sts(a.x + j, xv);
        sts(a.kty + j, ktyv);                            // K'y = A'y (:307)
        sts(a.sx + j, vsx[q] + xv * w);                  // weighted sums (src/saddle_point_gpu.jl:137,182)
        sts(a.skty + j, vsk[q] + ktyv * w);
        if (!commit_only) candidate(j, xv, ktyv, vec(s, kPC)[q], vec(s, kPL)[q], vec(s, kPU)[q]);
      }
    } else {
      if (ch.split >= 0 && ch.piece != ch.pieces - 1) rows = 0;
      for (int r = tid; r < rows; r += kBlock) {
        const int q = h.voff + r;
        candidate(ch.row_begin + r, vec(s, kPX)[q], vec(s, kPKTY)[q], vec(s, kPC)[q], vec(s, kPL)[q], vec(s, kPU)[q]);
      }
    }
    if (commit_only) return;
    const double p = block_sum_1(acc, sm.red);
    if (tid == 0) a.part_p[slot] = p;
  };

  if (!run_pipeline(a.plan.chunks, a.plan.num, a.st, sm.bars, sm.hdr, issue, gather, compute) && tid == 0)
    atomicOr(&a.st->pipe_fault, 1);
}

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
__global__ void __launch_bounds__(kBlock, 2) dual_step_kernel(DualArgs<T> a) {
  using L = StageLayout<T, kDualSlots>;
  extern __shared__ __align__(128) uint8_t ring_raw[];
  __shared__ StepSmem<T> sm;
  // StageLayout::kTotal has 128 spare bytes so the ring can start on a 128-byte boundary
  uint8_t* ring = ring_raw + ((128u - (smem_addr(ring_raw) & 127u)) & 127u);
  if (a.single && a.st->done) return;
  const bool commit_only = a.mode == kStepCommitOnly;
  const bool direct = a.direct != 0;
  const int tid = threadIdx.x;
  auto stage = [&](int s) { return ring + (size_t)s * L::kBytes; };
  auto vec = [&](int s, int slot) { return reinterpret_cast<T*>(stage(s) + L::off_vec + slot * L::kVec); };

  auto issue = [&](int, int s, const Chunk& ch, const StepScalars& v) {
    StageHdr& h = sm.hdr[s];
    h.ch = ch;
    h.issued = 0;
    if (v.done) return;
    const int pending = v.pending;
    if (commit_only && !pending) return;
    h.pending = pending;
    h.parity = v.parity;
    h.s0 = v.w;
    h.s1 = v.omega * v.tau;  // primal_weight * step_size
    const int al = ch.row_begin & ~(L::V - 1);
    const int cnt = ch.rows ? ((ch.row_begin + ch.rows + L::V - 1) & ~(L::V - 1)) - al : 0;
    h.voff = ch.row_begin - al;
    uint64_t* bar = &sm.bars[s];
    const uint32_t vb = (uint32_t)(cnt * (int)sizeof(T));
    const uint32_t mb = commit_only ? 0u : (uint32_t)blob_bytes<T>(ch.rows, ch.nnz);
    const int nv = 2 + (commit_only ? 0 : 1) + (pending ? 2 : 0);
    mbar_arrive_expect_tx(bar, mb + (uint32_t)nv * vb);
    if (mb) bulk_load_stream(stage(s), a.plan.blob + ch.blob, mb, bar, policy_evict_first());
    issue_vec(vec(s, kDY), h.parity ? a.y1 : a.y0, al, cnt, bar);
    issue_vec(vec(s, kDKX), h.parity ? a.kx1 : a.kx0, al, cnt, bar);
    if (!commit_only) issue_vec(vec(s, kDB), a.b, al, cnt, bar);
    if (pending) {
      issue_vec(vec(s, kDSY), a.sy, al, cnt, bar);
      issue_vec(vec(s, kDSKX), a.skx, al, cnt, bar);
    }
    h.issued = 1;
  };

  auto gather = [&](int s) {
    const StageHdr& h = sm.hdr[s];
    if (!h.issued || commit_only) return;
    const int32_t* col = reinterpret_cast<const int32_t*>(stage(s) + blob_rp_bytes<T>(h.ch.rows));
    T* xs = reinterpret_cast<T*>(stage(s) + L::off_xs);
    for (int k = tid; k < h.ch.nnz; k += kBlock) gather_async(xs + pad_index(k, PipeTraits<T>::kPadShift), a.dx + col[k]);
  };

  // Arrivals are counted per CTA and instance: the CTA flushes its count when its chunk
  // sequence moves to another instance and at the end, and the flush that completes the
  // instance's chunk count takes take_step!'s decision for it.
  int cur_inst = -1, cur_count = 0, cur_pending = 0;  // uniform across the CTA
  auto flush = [&]() {
    if (cur_count == 0) return;
    const int inst = cur_inst;
    StepState* st = a.st + inst;
    const int d0 = a.bi.d_chunk_begin[inst], d1 = a.bi.d_chunk_begin[inst + 1];
    if (tid == 0) {
      __threadfence();
      const unsigned prev = atomicAdd(&st->arrive, (unsigned)cur_count);
      sm.flag = (prev + (unsigned)cur_count == (unsigned)(d1 - d0)) ? 1 : 0;
    }
    cur_count = 0;
    __syncthreads();
    if (!sm.flag) return;
    __threadfence();
    if (commit_only) {
      if (tid == 0) {
        st->pending_commit = 0;
        st->arrive = 0;
      }
      return;
    }
    // the instance's partials in chunk order
    double si = 0.0, sd = 0.0, sx = 0.0;
    for (int k = d0 + tid; k < d1; k += kBlock) {
      si += __ldcg(a.part_d + k);
      sd += __ldcg(a.part_d + a.plan.num + k);
    }
    const int p0 = a.bi.p_chunk_begin[inst], p1 = a.bi.p_chunk_begin[inst + 1];
    for (int k = p0 + tid; k < p1; k += kBlock) sx += __ldcg(a.part_p + k);
    si = block_sum(si, sm.red2);
    sd = block_sum(sd, sm.red2);
    sx = block_sum(sx, sm.red2);
    if (tid == 0) {
      st->arrive = 0;
      if (cur_pending) st->primal_spmv += 1;
      st->pending_commit = 0;
      step_decision(st, si, sx, sd);
    }
  };

  auto compute = [&](int c, int s) {
    const StageHdr& h = sm.hdr[s];
    if (!h.issued) return;
    const Chunk& ch = h.ch;
    if (ch.inst != cur_inst) {
      flush();
      cur_inst = ch.inst;
      cur_pending = h.pending;
    }
    ++cur_count;
    const T w = (T)h.s0;
    const T od = (T)h.s1;
    const int p = h.parity;
    T* ynew = p ? a.y0 : a.y1;
    T* kxnew = p ? a.kx0 : a.kx1;
    const T* vy = vec(s, kDY);
    const T* vkx = vec(s, kDKX);
    int rows = ch.rows;
    if (commit_only) {
      if (ch.split >= 0 && ch.piece != ch.pieces - 1) rows = 0;
      for (int r = tid; r < rows; r += kBlock) {
        const int i = ch.row_begin + r, q = h.voff + r;
        sts(a.sy + i, vec(s, kDSY)[q] + vy[q] * w);
        sts(a.skx + i, vec(s, kDSKX)[q] + vkx[q] * w);
      }
      return;
    }
    const int ineq_from = ch.aux;
    uint8_t* base = stage(s);
    const int32_t* rp = reinterpret_cast<const int32_t*>(base);
    const T* val = reinterpret_cast<const T*>(base + blob_rp_bytes<T>(ch.rows) + blob_col_bytes<T>(ch.nnz));
    const T* xs = reinterpret_cast<const T*>(base + L::off_xs);
    T* rs = reinterpret_cast<T*>(base + L::off_rs);
    chunk_row_sums<T>(rp, val, xs, ch.rows, ch.nnz, ch.e_log2, rs, sm.scan);
    __syncthreads();
    int slot = c;
    if (ch.split >= 0) {  // as in the primal kernel: the first piece's slot holds the row
      if (tid == 0) {
        a.part_d[c] = 0.0;
        a.part_d[a.plan.num + c] = 0.0;
      }
      if (!split_combine<T>(ch, a.plan, rs, &sm.flag)) return;
      slot = c - ch.piece;
    }
    T acc_i = T(0), acc_d = T(0);
    const T* vb = vec(s, kDB);
    for (int r = tid; r < rows; r += kBlock) {
      const int i = ch.row_begin + r, q = h.voff + r;
      const T y = vy[q], kx = vkx[q], rsum = rs[r];
      if (h.pending) {
        sts(a.sy + i, vec(s, kDSY)[q] + y * w);
        sts(a.skx + i, vec(s, kDSKX)[q] + kx * w);
      }
      const T kdx = direct ? rsum - kx : rsum;
      T v = y + od * ((vb[q] - T(2) * kdx) - kx);   // (:247), extrapolation coefficient 1
      if (i >= ineq_from) v = imax(v, T(0));        // (:254)
      const T d = v - y;
      ynew[i] = y + d;                              // y += dy (:306); gathered by the next primal kernel
      sts(kxnew + i, direct ? rsum : kx + kdx);     // Kx += K dx (:304)
      acc_i += kdx * d;
      acc_d += d * d;
    }
    double bi, bd;
    block_sum_2(acc_i, acc_d, sm.red, bi, bd);
    if (tid == 0) {
      a.part_d[slot] = bi;
      a.part_d[a.plan.num + slot] = bd;
    }
  };

  if (!run_pipeline(a.plan.chunks, a.plan.num, a.st, sm.bars, sm.hdr, issue, gather, compute)) {
    if (tid == 0) atomicOr(&a.st->pipe_fault, 1);
    return;
  }
  flush();
}

}  // namespace gpdhg
