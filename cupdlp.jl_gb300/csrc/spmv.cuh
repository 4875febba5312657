// spmv.cuh — the CSR row-block SpMV shared by every step kernel.
//
// An item (one CTA) covers rows [row_begin, row_end); its `mode` picks the schedule:
//   kItemStaged  short rows whose nonzeros fit the CTA's stage (kStage = 256 x 8), at most
//                one row per group of `group` lanes (1..32) — steps 1-3 below;
//   kItemWarps   up to 8 rows of >= 64 nonzeros, one warp per row: register accumulation
//                (one FMA per nonzero, four independent loads per lane in flight);
//   kItemLong    one row longer than the stage, streamed by the whole CTA.
// Staged items:
//   1. the row's own epilogue loads (`pre`) are issued first;
//   2. every thread loads U (col, val) pairs of the item — fully unrolled, independent,
//      coalesced — then issues its U gathers, and stages the products in shared memory
//      (FP64 stages value and gathered entry apart, so the row sum is one FMA per nonzero on
//      GB300's scarce FP64 pipe): U loads in flight per thread instead of one dependent load
//      chain per nonzero;
//   3. after one barrier each group sums its row from shared memory in a fixed order and
//      its lane 0 runs the epilogue (`post`).
// Matrix streams use evict-first loads so the gathered vector stays in L2. The reduction
// order is fixed by the schedule, so results are deterministic.
#pragma once

#include "common.cuh"

namespace gpdhg {


template <class T>
__device__ __forceinline__ T group_sum(T v, int g) {
  for (int o = g >> 1; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o, g);
  return v;
}

// Row r of M times xg by the 32 lanes of a warp, four independent loads per lane in flight.
template <class T>
__device__ __forceinline__ T warp_row_dot(const CsrView<T>& M, const T* __restrict__ xg, int r, int lane) {
  const int s = M.row_ptr[r], e = M.row_ptr[r + 1];
  T a0 = T(0), a1 = T(0), a2 = T(0), a3 = T(0);
  int k = s + lane;
  for (; k + 96 < e; k += 128) {
    const int c0 = lds(M.col + k), c1 = lds(M.col + k + 32), c2 = lds(M.col + k + 64), c3 = lds(M.col + k + 96);
    const T v0 = lds(M.val + k), v1 = lds(M.val + k + 32), v2 = lds(M.val + k + 64), v3 = lds(M.val + k + 96);
    a0 += v0 * xg[c0];
    a1 += v1 * xg[c1];
    a2 += v2 * xg[c2];
    a3 += v3 * xg[c3];
  }
  for (; k < e; k += 32) a0 += lds(M.val + k) * xg[lds(M.col + k)];
  return warp_sum((a0 + a1) + (a2 + a3));
}

// Runs the item's rows. Every thread of the CTA must call it. `stage` holds kStage T, and
// so does `stage2` when T is double (unused otherwise).
template <class T, class Pre, class Post>
__device__ __forceinline__ void spmv_item(const CsrView<T>& M, const T* __restrict__ xg, int item, T* stage,
                                          T* stage2, T* wsum, Pre&& pre, Post&& post) {
  constexpr int U = kStageDepth;
  const RowItem it = M.items[item];
  const int tid = threadIdx.x;
  if (it.mode == kItemWarps) {
    const int lane = tid & 31;
    for (int base = it.row_begin; base < it.row_end; base += kBlock / 32) {
      const int r = base + (tid >> 5);
      if (r < it.row_end) {   // whole warps take this branch together
        decltype(pre(r)) p{};
        if (lane == 0) p = pre(r);
        const T sum = warp_row_dot(M, xg, r, lane);
        if (lane == 0) post(r, sum, p);
      }
    }
    return;
  }
  if (it.mode == kItemLong) {
    // one long row streamed by the whole CTA, U independent loads per thread per round
    const int r = it.row_begin;
    decltype(pre(r)) p{};
    if (tid == 0) p = pre(r);
    const int s = M.row_ptr[r], e = M.row_ptr[r + 1];
    T acc[U];
#pragma unroll
    for (int q = 0; q < U; ++q) acc[q] = T(0);
    for (int base = s; base < e; base += kBlock * U) {
      int c[U];
      T v[U];
#pragma unroll
      for (int q = 0; q < U; ++q) {
        const int k = base + q * kBlock + tid;
        c[q] = k < e ? lds(M.col + k) : 0;
        v[q] = k < e ? lds(M.val + k) : T(0);
      }
#pragma unroll
      for (int q = 0; q < U; ++q) acc[q] += v[q] * xg[c[q]];
    }
#pragma unroll
    for (int q = 1; q < U; ++q) acc[0] += acc[q];
    const T a = warp_sum(acc[0]);
    __syncthreads();
    if ((tid & 31) == 0) wsum[tid >> 5] = a;
    __syncthreads();
    if (tid == 0) {
      T sum = T(0);
      for (int w = 0; w < kBlock / 32; ++w) sum += wsum[w];
      post(r, sum, p);
    }
    return;
  }
  const int g = it.group;
  const int lane = tid & (g - 1);
  const int r = it.row_begin + tid / g;
  const bool owner = r < it.row_end && lane == 0;
  decltype(pre(r)) p{};
  if (owner) p = pre(r);
  const int s0 = M.row_ptr[it.row_begin];
  const int cnt = M.row_ptr[it.row_end] - s0;
  {
    int c[U];
    T v[U];
#pragma unroll
    for (int q = 0; q < U; ++q) {
      const int k = q * kBlock + tid;
      c[q] = k < cnt ? lds(M.col + s0 + k) : 0;
      v[q] = k < cnt ? lds(M.val + s0 + k) : T(0);
    }
#pragma unroll
    for (int q = 0; q < U; ++q) {
      const int k = q * kBlock + tid;
      if (k < cnt) {
        if constexpr (sizeof(T) == 8) {
          stage[k] = v[q];
          stage2[k] = xg[c[q]];
        } else {
          stage[k] = v[q] * xg[c[q]];
        }
      }
    }
  }
  __syncthreads();
  T sum = T(0);
  if (r < it.row_end) {
    const int a = M.row_ptr[r] - s0, b = M.row_ptr[r + 1] - s0;
    if constexpr (sizeof(T) == 8) {
      for (int k = a + lane; k < b; k += g) sum += stage[k] * stage2[k];
    } else {
      for (int k = a + lane; k < b; k += g) sum += stage[k];
    }
  }
  sum = group_sum(sum, g);
  if (owner) post(r, sum, p);
}

// y = M x over the row-block items of M. With row_inst non-NULL only the items whose first
// row belongs to an instance with active[instance] set run (the packed matrix of a batch;
// an item never spans two instances).
struct NoPre {};
template <class T>
__global__ void __launch_bounds__(kBlock) spmv_kernel(CsrView<T> M, const T* __restrict__ x, T* y,
                                                      const int32_t* __restrict__ row_inst,
                                                      const uint8_t* __restrict__ active) {
  __shared__ T stage[kStage];
  __shared__ T stage2[sizeof(T) == 8 ? kStage : 1];
  __shared__ T wsum[kBlock / 32];
  if ((int)blockIdx.x >= M.num_items) return;
  if (row_inst && !active[row_inst[M.items[blockIdx.x].row_begin]]) return;
  auto pre = [](int) { return NoPre{}; };
  auto post = [&](int i, T s, const NoPre&) { y[i] = s; };
  spmv_item(M, x, blockIdx.x, stage, stage2, wsum, pre, post);
}

}  // namespace gpdhg
