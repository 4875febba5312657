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
// Here one attempt is two kernels over warp tiles (tiles.h, tile_spmv.cuh) and no host
// round trip:
//   primal_step_kernel: [if the previous attempt was accepted] K'y = A' y (tiles of A'),
//       x += dx, and the x weighted sum; then the next dx, and per-CTA ||dx||^2. (The
//       average's K'y is formed at evaluation time as A' y-bar, not summed here.)
//   dual_step_kernel:   [if the previous attempt was accepted] the y / Kx weighted sums;
//       then K dx (tiles of A), the projected dual candidate, Kx + K dx into the other half
//       of the double-buffered y / Kx, per-CTA interaction and ||dy||^2 partials; the
//       instance's first CTA also sums the primal kernel's ||dx||^2 partials and prepares
//       the decision's inputs that need no dual partial; the last CTA of an instance to
//       finish reduces that instance's dual partials in a fixed order and takes the
//       accept/reject and step-size decision, flipping the buffer parity on accept.
//       (A separate decision kernel measured slower: one more kernel boundary per attempt
//       costs more than this CTA's serial tail.)
// Every CTA belongs to one instance; each warp owns whole tiles (row sums in registers,
// the fused epilogue on its rows), so no barrier sits between a warp's loads and its
// arithmetic, and latency is hidden by the many warps resident per SM. A split row's
// contribution to the partials is written to a per-split-row slot by the one warp that
// completes it, so all reductions keep a fixed order.
// So an accepted step costs exactly one pass over A and one over A'; a rejected attempt
// costs one pass over A plus a streaming pass over the n-vectors.
//
// `direct` mode (the FP32 bulk phase): the primal kernel stores the candidate x^ itself
// (in the dx buffer) and the dual kernel forms K x^ = A x^ from scratch, K dx = K x^ - K x,
// and stores K x^ as the next K x. The reference's incremental K x += K dx (:304) is kept
// in FP64 for parity; in FP32 it drifts by ~1e-6 relative, which this mode removes.
#pragma once

#include "common.cuh"
#include "tile_spmv.cuh"
#include "tiles.h"

namespace gpdhg {

enum StepMode : int { kStepNormal = 0, kStepCommitOnly = 1 };

// Programmatic dependent launch (sm_90+): the step kernels are launched with the
// programmatic-serialization attribute, so a kernel's CTAs may start while the previous
// kernel finishes. Everything before pdl_wait() must read only constant data (the tile
// plan); pdl_wait() returns once the previous kernel has completed and its writes are
// visible (immediately when it was launched without the attribute).
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" :::); }

template <class T>
struct PrimalArgs {
  CsrView<T> At;         // CSR of A' (rows = variables)
  TileView<T> plan;      // tiles of A'
  const T* c;
  const T* l;
  const T* u;
  T* x;
  T* dx;                 // dx, or x^ in direct mode
  T* kty;
  T* sx;
  const T* y0;
  const T* y1;
  StepState* st;         // one per instance
  double* part_p;        // ||dx||^2 per CTA
  double* part_p_split;  // ||dx||^2 of each split row
  int mode;
  int direct;
};

template <class T>
struct DualArgs {
  CsrView<T> A;          // CSR of A (rows = constraints)
  TileView<T> plan;      // tiles of A
  const int32_t* p_cta_begin;    // primal plan: first CTA of each instance
  const int32_t* p_split_begin;  // primal plan: first split row of each instance
  const T* dx;
  const T* b;
  T* y0;
  T* y1;
  T* kx0;
  T* kx1;
  T* sy;
  T* skx;
  StepState* st_mut;     // one per instance; the instance's last CTA updates it
  const double* part_p;
  const double* part_p_split;
  double* part_d;        // [interaction | ||dy||^2] per CTA (num_ctas each)
  double* part_d_split;  // (interaction, ||dy||^2) of each split row
  int mode;
  int direct;            // dx holds x^ and the row sums are K x^ (see above)
};

// Sums over the CTA of Q per-thread partials in a fixed order, valid in thread 0; `sh`
// holds Q * kBlock doubles and may be reused by consecutive calls. FP64 partials go through
// shared memory: lane l of warp 0 adds entry l of every warp in warp order, then one shuffle
// tree finishes (12 warp-wide FP64 adds per quantity, where a shuffle tree in every warp
// takes 40: GB300 issues FP64 at 2 lanes per SM and cycle). FP32 partials: a shuffle tree
// per warp in FP32, the warp sums added in FP64.
template <int Q, class T>
__device__ __forceinline__ void cta_sums(const T (&v)[Q], double (&out)[Q], double* sh) {
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  __syncthreads();  // a previous call's readers are done with sh
  if constexpr (sizeof(T) == 8) {
#pragma unroll
    for (int q = 0; q < Q; ++q) sh[q * kBlock + t] = v[q];
    __syncthreads();
    if (t < 32) {
#pragma unroll
      for (int q = 0; q < Q; ++q) {
        double s = sh[q * kBlock + lane];
#pragma unroll
        for (int w = 1; w < kBlock / 32; ++w) s += sh[q * kBlock + w * 32 + lane];
        out[q] = warp_sum(s);
      }
    }
  } else {
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const T ws = warp_sum(v[q]);
      if (lane == 0) sh[q * 32 + warp] = (double)ws;
    }
    __syncthreads();
    if (t == 0) {
#pragma unroll
      for (int q = 0; q < Q; ++q) {
        double s = 0.0;
        for (int w = 0; w < kBlock / 32; ++w) s += sh[q * 32 + w];
        out[q] = s;
      }
    }
  }
}

// One lane's epilogue inputs for its row of a tile (issued with the tile's matrix loads).
template <class T>
struct PrimalIn {
  T dx;  // dx (x^ in direct mode); K'y when no commit is pending
  T x;
  T sx;
  T c;
  T l;
  T u;
};

// FP64 step kernels run row epilogues after the CTA's row sums are in shared memory, one row
// per thread (the dual kernel for its warp tiles, the primal kernel for its warp-streamed
// rows). Summed tile by tile, a tile's epilogue (about a dozen FP64 instructions per row) runs
// on only the lanes that own its rows (a handful when rows are longer than a lane's run, one
// for a streamed row), yet every warp-wide FP64 instruction occupies GB300's narrow FP64 pipe
// for the whole warp: on the power-law LP that made the pipe, not memory, the dual's bound
// (79% busy). FP32 keeps the per-tile epilogue (its pipe is wide, and the shared-memory row
// buffer would take L1 from the gathers).
template <class T>
constexpr bool kDenseEpilogue = sizeof(T) == 8;
template <class T>
constexpr int kDenseSlots = kDenseEpilogue<T> ? kTilesPerCtaMax * kTileRows : 1;

template <class T>
__global__ void __launch_bounds__(kBlock, kPrimalCtasPerSm<T>) primal_step_kernel(PrimalArgs<T> a) {
  __shared__ T rs_all[kBlock / 32][32];
  __shared__ double red[kBlock];
  __shared__ T wlane[kBlock];
  __shared__ Tile tl[kTilesPerCtaMax];
  const int b = a.plan.cta_map ? a.plan.cta_map[blockIdx.x] : (int)blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // programmatic dependent launch: stage the constant tile descriptors, wait for the previous
  // kernel, and only then let the next (dual) kernel's CTAs launch: once all of ours have
  // passed this point, the state the previous dual kernel wrote is complete, so the dual
  // kernel may read it before its own wait (this kernel never writes it)
  const int nt = stage_tiles(a.plan.tiles, a.plan.cta_tile_begin[b], a.plan.cta_tile_begin[b + 1], tl);
  pdl_wait();
  pdl_launch_dependents();
  const StepState* st = a.st + a.plan.cta_inst[b];
  if (st->done) return;
  const int pending = st->pending_commit;
  const bool commit_only = a.mode == kStepCommitOnly;
  if (commit_only && !pending) return;
  const bool direct = a.direct != 0;
  // step_size / primal_weight: one FP64 division per CTA (GB300's FP64 pipe is narrow)
  __shared__ double s_tto;
  if (threadIdx.x == 0) s_tto = st->tau / st->omega;
  __syncthreads();
  const T w = (T)st->commit_weight;
  const T tto = (T)s_tto;
  const T* yg = st->parity ? a.y1 : a.y0;
  T* rs = rs_all[warp];
  T acc = T(0);
  auto load_in = [&](const Tile& t, PrimalIn<T>& e) {
    e = PrimalIn<T>{};
    if (lane >= t.rows) return;
    const int j = t.row_begin + lane;
    if (!commit_only) {
      e.c = lds(a.c + j);
      e.l = lds(a.l + j);
      e.u = lds(a.u + j);
    }
    if (pending) {
      e.dx = lds(a.dx + j);
      if (!direct) e.x = lds(a.x + j);
      e.sx = lds(a.sx + j);
    } else {
      e.x = lds(a.x + j);
      e.dx = lds(a.kty + j);
    }
  };
  // x^ = proj(x - (tau/omega)(c - K'y)) and dx (:177-197); its ||dx||^2 term goes into the
  // CTA's sum with one FMA, or into the split row's own slot
  auto candidate = [&](int j, T xv, T ktyv, const PrimalIn<T>& e, const Tile& t, bool split) {
    T v = xv - tto * (e.c - ktyv);
    v = imin(e.u, imax(e.l, v));   // min(u, max(l, .)) (:192)
    const T d = v - xv;
    a.dx[j] = direct ? v : d;      // gathered by the dual kernel next: a normal (L2-resident) store
    if (split) {
      a.part_p_split[t.split] = (double)(d * d);
      __threadfence();
    } else {
      acc = fma(d, d, acc);
    }
  };
  // split handling and the fused epilogue of tile t, once its row sums are in rs
  auto finish = [&](const Tile& t, const PrimalIn<T>& e) {
    const bool split = t.split >= 0;
    const int j = t.row_begin + lane;
    if (pending) {
      int rows = t.rows;
      if (split) rows = split_finish(t, a.plan, rs) ? 1 : 0;
      if (lane < rows) {
        const T ktyv = rs[lane];
        const T xv = direct ? e.dx : e.x + e.dx;   // x += dx (:303)
        sts(a.x + j, xv);
        sts(a.kty + j, ktyv);                       // K'y = A'y (:307)
        sts(a.sx + j, e.sx + xv * w);               // weighted sum (src/saddle_point_gpu.jl:137)
        if (!commit_only) candidate(j, xv, ktyv, e, t, split);
      }
      __syncwarp();
    } else {
      // previous attempt rejected: K'y is unchanged, only the candidate is recomputed
      const int rows = (split && t.piece != t.pieces - 1) ? 0 : t.rows;
      if (lane < rows) candidate(j, e.x, e.dx, e, t, split);
    }
  };
  TileLoad<T> L0;
  PrimalIn<T> E0;
  if (nt > 0 && tl[0].e_log2 <= group_code(1)) {
    // group tiles: 8 / W long rows, W warps each; the group's first warp finishes its row
    const int W = 1 << group_log2(tl[0].e_log2);
    const int q = warp / W, sub = warp % W;
    const bool has = q < nt;
    Tile t{};
    if (has) t = tl[q];
    if (has && sub == 0) load_in(t, E0);
    if (pending) group_row_sum(a.At.col, a.At.val, yg, t, has, W, sub, wlane, rs);
    if (has && sub == 0) finish(t, E0);
  } else if (kDenseEpilogue<T> && nt > 0 && tl[0].e_log2 == kWarpLong) {
    // FP64 CTAs of warp-streamed rows (one row per tile): the warps stream their rows' sums
    // into shared memory, then thread q runs the epilogue of tile q's row, so the FP64
    // instructions of the epilogue run on full warps instead of on each warp's lane 0
    __shared__ T lsum[kDenseEpilogue<T> ? kTilesPerCtaMax : 1];
    if (pending)
      for (int q = warp; q < nt; q += kBlock / 32) {
        const T sum = long_row_sum(a.At.col, a.At.val, yg, tl[q]);
        if (lane == 0) lsum[q] = sum;
      }
    __syncthreads();
    for (int q = threadIdx.x; q < nt; q += kBlock) {
      const Tile& t = tl[q];
      const int j = t.row_begin;
      PrimalIn<T> e{};
      if (!commit_only) {
        e.c = lds(a.c + j);
        e.l = lds(a.l + j);
        e.u = lds(a.u + j);
      }
      if (pending) {
        e.dx = lds(a.dx + j);
        if (!direct) e.x = lds(a.x + j);
        e.sx = lds(a.sx + j);
        const T ktyv = lsum[q];
        const T xv = direct ? e.dx : e.x + e.dx;   // x += dx (:303)
        sts(a.x + j, xv);
        sts(a.kty + j, ktyv);                       // K'y = A'y (:307)
        sts(a.sx + j, e.sx + xv * w);               // weighted sum (src/saddle_point_gpu.jl:137)
        if (!commit_only) candidate(j, xv, ktyv, e, t, false);
      } else {
        e.x = lds(a.x + j);
        e.dx = lds(a.kty + j);
        candidate(j, e.x, e.dx, e, t, false);
      }
    }
  } else {
    // each warp walks its tiles q = warp, warp + 8, ...: a tile's epilogue inputs, row
    // offsets, columns and values are all issued before any of them is used
    for (int q = warp; q < nt; q += kBlock / 32) {
      const Tile t = tl[q];
      load_in(t, E0);
      if (pending) {
        tile_load(a.At.row_ptr, a.plan.icol, a.plan.ival, t, L0);
        tile_sums(a.At.col, a.At.val, yg, t, L0, rs);
      }
      finish(t, E0);
    }
  }
  if (commit_only) return;
  const T v[1] = {acc};
  double o[1];
  cta_sums<1>(v, o, red);
  if (threadIdx.x == 0) a.part_p[b] = o[0];
}

// Primal part of take_step!'s movement (:324-333), 0.5 * omega * ||dx||^2 evaluated as the
// reference does (the norm squared again).
__device__ __forceinline__ double half_w_dx2(double omega, double dx2) {
  const double ndx = sqrt(dx2);
  return 0.5 * omega * ndx * ndx;
}

// Decision of take_step! for one attempt, on a copy of the instance's state (the caller
// writes it back). f1 / f2 are the step-size factors (1 - (k+1)^-r), (1 + (k+1)^-g)
// for the attempt counter after this attempt, hw_dx2 = half_w_dx2(omega, ||dx||^2) and
// hoo = 0.5 / omega, all prepared by the instance's first dual CTA while the others still run.
__device__ __forceinline__ void step_decision(StepState& s, double f1, double f2, double inter_signed, double hw_dx2,
                                              double hoo, double dy2) {
  s.total_iters += s.constant_step ? 0 : 1;
  s.kkt_passes += 1.0;
  s.attempts_in_chunk += 1;
  const double tau = s.tau;
  const double inter = fabs(inter_signed);
  const double ndy = sqrt(dy2);
  const double movement = hw_dx2 + hoo * ndy * ndy;
  double limit;
  bool accept;
  if (s.constant_step) {
    limit = __longlong_as_double(0x7ff0000000000000LL);
    accept = true;
  } else {
    if (inter > 0.0) {
      limit = movement / inter;
      if (movement == 0.0) {
        // :384-390: terminate at the next evaluation; tau is left as it is
        s.numerical_error = 1;
        s.done = 1;
        s.pending_commit = 0;
        return;
      }
    } else {
      limit = __longlong_as_double(0x7ff0000000000000LL);
    }
    accept = tau <= limit;
  }
  s.last_limit = limit;
  if (accept) {
    s.parity ^= 1;
    s.pending_commit = 1;
    s.commit_weight = s.iter_start_tau;
    s.count_primal += 1;
    s.count_dual += 1;
    s.sum_w_primal += s.iter_start_tau;
    s.sum_w_dual += s.iter_start_tau;
    s.accepted += 1;
    s.accepted_in_chunk += 1;
  } else {
    s.pending_commit = 0;
    s.rejected += 1;
  }
  if (!s.constant_step) {
    const double first = f1 * limit;
    const double second = f2 * tau;
    s.tau = jmin(first, second);
  }
  if (accept) s.iter_start_tau = s.tau;
  if (s.accepted_in_chunk >= s.target_in_chunk || s.attempts_in_chunk >= s.max_attempts_in_chunk) s.done = 1;
}

// Step-size factors for attempt counter k (take_step!, :405-407): the host table while it
// lasts, else the same formula on the device.
__device__ __forceinline__ void step_factors(const StepState& s, long long k, double& f1, double& f2) {
  if (s.pow_table && k < s.pow_table_len) {
    f1 = __ldcg(s.pow_table + 2 * k);
    f2 = __ldcg(s.pow_table + 2 * k + 1);
  } else {
    const double k1 = (double)(k + 1);
    f1 = 1.0 - 1.0 / pow(k1, s.reduction_exponent);
    f2 = 1.0 + 1.0 / pow(k1, s.growth_exponent);
  }
}

// One lane's epilogue inputs for its row of a tile of A (issued with the tile's matrix loads).
template <class T>
struct DualIn {
  T y;
  T kx;
  T b;
  T sy;
  T sk;
};

// The dual kernel's FP64 tiles stop their segmented scan at the longest lane span of a
// crossing row (tile_sums); FP32 adds are cheap and keep the full scan.
template <class T>
constexpr bool kSpanScan = sizeof(T) == 8;

template <class T>
__global__ void __launch_bounds__(kBlock, kDualCtasPerSm) dual_step_kernel(DualArgs<T> a) {
  __shared__ T rs_all[kBlock / 32][32];
  __shared__ T wlane[kBlock];
  __shared__ T ipart[kBlock / 32][kBlock / 32];
  __shared__ Tile tl[kTilesPerCtaMax];
  __shared__ double red[2 * kBlock];
  __shared__ int is_last;
  const int b = a.plan.cta_map ? a.plan.cta_map[blockIdx.x] : (int)blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  pdl_launch_dependents();  // the next primal kernel reads the state only after its wait
  const int nt = stage_tiles(a.plan.tiles, a.plan.cta_tile_begin[b], a.plan.cta_tile_begin[b + 1], tl);
  // The state this kernel reads was written by the previous dual kernel, which completed
  // before the primal kernel let this one launch (see there): read it now, from L2 (a line in
  // this SM's L1 may predate it), so the loads overlap the primal kernel's last CTAs.
  const StepState* st = a.st_mut + a.plan.cta_inst[b];
  const int done = __ldcg(&st->done);
  const int pending = __ldcg(&st->pending_commit);
  const int p = __ldcg(&st->parity);
  const double commit_weight = __ldcg(&st->commit_weight);
  const double od64 = __ldcg(&st->omega) * __ldcg(&st->tau);  // primal_weight * step_size
  pdl_wait();
  if (done) return;
  const bool commit_only = a.mode == kStepCommitOnly;
  if (commit_only && !pending) return;
  const bool direct = a.direct != 0;
  const T w = (T)commit_weight;
  const T od = (T)od64;
  const T* ycur = p ? a.y1 : a.y0;
  T* ynew = p ? a.y0 : a.y1;
  const T* kxcur = p ? a.kx1 : a.kx0;
  T* kxnew = p ? a.kx0 : a.kx1;
  T* rs = rs_all[warp];
  T acc_i = T(0), acc_d = T(0);
  auto load_in = [&](const Tile& t, DualIn<T>& e) {
    e = DualIn<T>{};
    if (lane >= t.rows) return;
    const int i = t.row_begin + lane;
    e.y = lds(ycur + i);
    e.kx = lds(kxcur + i);
    if (!commit_only) e.b = lds(a.b + i);
    if (pending) {
      e.sy = lds(a.sy + i);
      e.sk = lds(a.skx + i);
    }
  };
  auto finish = [&](const Tile& t, const DualIn<T>& e) {
    const bool split = t.split >= 0;
    const int i = t.row_begin + lane;
    if (commit_only) {
      const int rows = (split && t.piece != t.pieces - 1) ? 0 : t.rows;
      if (lane < rows) {
        sts(a.sy + i, e.sy + e.y * w);
        sts(a.skx + i, e.sk + e.kx * w);
      }
      return;
    }
    int rows = t.rows;
    if (split) rows = split_finish(t, a.plan, rs) ? 1 : 0;
    if (lane < rows) {
      const T rsum = rs[lane];
      const T y = e.y, kx = e.kx;
      if (pending) {
        sts(a.sy + i, e.sy + y * w);
        sts(a.skx + i, e.sk + kx * w);
      }
      const T kdx = direct ? rsum - kx : rsum;
      T v = y + od * ((e.b - T(2) * kdx) - kx);   // (:247), extrapolation coefficient 1
      if (i >= t.aux) v = imax(v, T(0));          // (:254)
      const T d = v - y;
      ynew[i] = y + d;                            // y += dy (:306); gathered by the next primal kernel
      sts(kxnew + i, direct ? rsum : kx + kdx);   // Kx += K dx (:304)
      if (split) {
        a.part_d_split[2 * t.split] = (double)(kdx * d);
        a.part_d_split[2 * t.split + 1] = (double)(d * d);
        __threadfence();
      } else {
        acc_i = fma(kdx, d, acc_i);
        acc_d = fma(d, d, acc_d);
      }
    }
    __syncwarp();
  };
  TileLoad<T> L0;
  DualIn<T> E0;
  bool interleave = nt == kBlock / 32;
  for (int q = 0; q < nt && interleave; ++q) interleave = tl[q].e_log2 == kWarpLong;
  if (interleave) {
    // kBlock / 32 warp-streamed rows summed together (interleaved_rows_sum); warp w then
    // finishes row w as if it had streamed it
    load_in(tl[warp], E0);
    if (!commit_only) interleaved_rows_sum(a.A.col, a.A.val, a.dx, tl, ipart, rs_all);
    finish(tl[warp], E0);
  } else if (nt > 0 && tl[0].e_log2 <= group_code(1)) {
    const int W = 1 << group_log2(tl[0].e_log2);
    const int q = warp / W, sub = warp % W;
    const bool has = q < nt;
    Tile t{};
    if (has) t = tl[q];
    if (has && sub == 0) load_in(t, E0);
    if (!commit_only) group_row_sum(a.A.col, a.A.val, a.dx, t, has, W, sub, wlane, rs);
    if (has && sub == 0) finish(t, E0);
  } else if (kDenseEpilogue<T>) {
    // warp tiles (never split): every row sum into the CTA's slot buffer, then the epilogue
    // with one row per thread, slot by slot (slot = the row's position among the tiles' rows)
    __shared__ T csum[kDenseSlots<T>];
    __shared__ int32_t slot_begin[kTilesPerCtaMax + 1];
    if (threadIdx.x == 0) {
      int o = 0;
      for (int q = 0; q < nt; ++q) {
        slot_begin[q] = o;
        o += tl[q].rows;
      }
      slot_begin[nt] = o;
    }
    __syncthreads();
    if (!commit_only) {
      for (int q = warp; q < nt; q += kBlock / 32) {
        const Tile t = tl[q];
        tile_load(a.A.row_ptr, a.plan.icol, a.plan.ival, t, L0);
        tile_sums<T, kSpanScan<T>>(a.A.col, a.A.val, a.dx, t, L0, rs);
        if (lane < t.rows) csum[slot_begin[q] + lane] = rs[lane];
        __syncwarp();
      }
    }
    __syncthreads();
    const int nslots = slot_begin[nt];
    for (int sl = threadIdx.x; sl < nslots; sl += kBlock) {
      int lo = 0, hi = nt - 1;   // the last tile starting at or before the slot (the non-empty one)
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (slot_begin[mid] <= sl) lo = mid;
        else hi = mid - 1;
      }
      const int i = tl[lo].row_begin + (sl - slot_begin[lo]);
      const T y = lds(ycur + i), kx = lds(kxcur + i);
      if (commit_only) {
        sts(a.sy + i, lds(a.sy + i) + y * w);
        sts(a.skx + i, lds(a.skx + i) + kx * w);
        continue;
      }
      const T bi = lds(a.b + i);
      if (pending) {
        sts(a.sy + i, lds(a.sy + i) + y * w);
        sts(a.skx + i, lds(a.skx + i) + kx * w);
      }
      const T rsum = csum[sl];
      const T kdx = direct ? rsum - kx : rsum;
      T v = y + od * ((bi - T(2) * kdx) - kx);   // (:247), extrapolation coefficient 1
      if (i >= tl[lo].aux) v = imax(v, T(0));      // (:254)
      const T d = v - y;
      ynew[i] = y + d;                             // y += dy (:306)
      sts(kxnew + i, direct ? rsum : kx + kdx);    // Kx += K dx (:304)
      acc_i = fma(kdx, d, acc_i);
      acc_d = fma(d, d, acc_d);
    }
  } else {
    for (int q = warp; q < nt; q += kBlock / 32) {
      const Tile t = tl[q];
      load_in(t, E0);
      if (!commit_only) {
        tile_load(a.A.row_ptr, a.plan.icol, a.plan.ival, t, L0);
        tile_sums<T, kSpanScan<T>>(a.A.col, a.A.val, a.dx, t, L0, rs);
      }
      finish(t, E0);
    }
  }
  const int inst = a.plan.cta_inst[b];
  const int c0 = a.plan.inst_cta_begin[inst], c1 = a.plan.inst_cta_begin[inst + 1];
  StepState* stw = a.st_mut + inst;
  if (!commit_only) {
    const T v[2] = {acc_i, acc_d};
    double o[2];
    cta_sums<2>(v, o, red);
    if (threadIdx.x == 0) {
      a.part_d[b] = o[0];
      a.part_d[a.plan.num_ctas + b] = o[1];
    }
    if (b == c0) {
      // the instance's primal ||dx||^2 in plan order (CTAs, then split rows), summed here
      // once so that the deciding CTA reads one value instead of every primal partial
      const int p0 = a.p_cta_begin[inst], p1 = a.p_cta_begin[inst + 1];
      const int q0 = a.p_split_begin[inst], q1 = a.p_split_begin[inst + 1];
      double sx[1] = {0.0};
      for (int k0 = p0 + (int)threadIdx.x; k0 < p1; k0 += 4 * kBlock) {
        double u[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) u[j] = k0 + j * kBlock < p1 ? __ldcg(a.part_p + k0 + j * kBlock) : 0.0;
#pragma unroll
        for (int j = 0; j < 4; ++j) sx[0] += u[j];
      }
      for (int k = q0 + (int)threadIdx.x; k < q1; k += kBlock) sx[0] += __ldcg(a.part_p_split + k);
      double ox[1];
      cta_sums<1>(sx, ox, red);
      if (threadIdx.x == 0) {
        // and the decision's other inputs that need no dual partial
        double f1, f2;
        step_factors(*st, st->total_iters + (st->constant_step ? 0 : 1), f1, f2);
        stw->half_w_dx2 = half_w_dx2(st->omega, ox[0]);
        stw->half_over_omega = 0.5 / st->omega;
        stw->f1 = f1;
        stw->f2 = f2;
      }
    }
  }
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned prev = atomicAdd(&stw->arrive, 1u);
    is_last = (prev == (unsigned)(c1 - c0 - 1)) ? 1 : 0;
  }
  __syncthreads();
  if (!is_last) return;
  if (commit_only) {
    if (threadIdx.x == 0) {
      stw->pending_commit = 0;
      stw->arrive = 0;
    }
    return;
  }
  // the instance's last CTA: the first threads copy the state from L2 (the first CTA's
  // fields are not in this SM's L1), one 8-byte word each, with the partials' loads; the
  // barriers of cta_sums order the copy before thread 0 uses it. Partials in a fixed order.
  __shared__ StepState s;
  static_assert(sizeof(StepState) % 8 == 0 && sizeof(StepState) / 8 <= kBlock, "StepState copy");
  if (threadIdx.x < sizeof(StepState) / 8)
    reinterpret_cast<unsigned long long*>(&s)[threadIdx.x] =
        __ldcg(reinterpret_cast<const unsigned long long*>(stw) + threadIdx.x);
  // one round of loads for both CTA ranges (interaction, ||dy||^2) up to 4 x kBlock CTAs,
  // all issued before any is added; split-row slots (rare) follow
  const int s0 = a.plan.inst_split_begin[inst], s1 = a.plan.inst_split_begin[inst + 1];
  double sd[2] = {0.0, 0.0};
  for (int k0 = c0 + (int)threadIdx.x; k0 < c1; k0 += 4 * kBlock) {
    double ui[4], ud[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const bool in = k0 + j * kBlock < c1;
      ui[j] = in ? __ldcg(a.part_d + k0 + j * kBlock) : 0.0;
      ud[j] = in ? __ldcg(a.part_d + a.plan.num_ctas + k0 + j * kBlock) : 0.0;
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      sd[0] += ui[j];
      sd[1] += ud[j];
    }
  }
  for (int k = s0 + (int)threadIdx.x; k < s1; k += kBlock) {
    sd[0] += __ldcg(a.part_d_split + 2 * k);
    sd[1] += __ldcg(a.part_d_split + 2 * k + 1);
  }
  double tot[2];
  cta_sums<2>(sd, tot, red);
  if (threadIdx.x == 0) {
    s.arrive = 0;
    if (pending) s.primal_spmv += 1;
    s.pending_commit = 0;
    step_decision(s, s.f1, s.f2, tot[0], s.half_w_dx2, s.half_over_omega, tot[1]);
  }
  __syncthreads();
  // the new state back to global memory, one 8-byte word per thread
  if (threadIdx.x < sizeof(StepState) / 8)
    reinterpret_cast<unsigned long long*>(stw)[threadIdx.x] = reinterpret_cast<const unsigned long long*>(&s)[threadIdx.x];
}

// Launches a step kernel with programmatic dependent launch enabled (see pdl_wait).
template <class Args>
inline void launch_step(void (*kernel)(Args), int grid, cudaStream_t s, const Args& args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(kBlock);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  CK(cudaLaunchKernelEx(&cfg, kernel, args));
}

}  // namespace gpdhg
