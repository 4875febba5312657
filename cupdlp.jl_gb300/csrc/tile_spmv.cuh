// tile_spmv.cuh — one warp's row sums of one tile, in registers.
#pragma once

#include "common.cuh"
#include "tiles.h"

namespace gpdhg {

// Row sums of tile t: rs[r] = sum of val * xg[col] over row t.row_begin + r, r < t.rows.
// Lane l takes the tile's nonzeros [l E, (l + 1) E), E = 2^e_log2, and issues all their
// column, value and gathered-entry loads before using any (up to 3 E independent loads in
// flight per lane), then sums them per row with one FMA per nonzero. The row offsets live
// in the lanes' registers (lane i holds rp[i]) and are read with shuffles; a row that
// crosses lanes is completed by a segmented shuffle scan of the lanes' trailing partial
// sums. Every sum's order depends only on the tile, so the result does not depend on the
// tile's position in memory. rs (32 entries per warp) is complete after the final __syncwarp.
template <class T>
__device__ __forceinline__ void tile_row_sums(const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ col,
                                              const T* __restrict__ val, const T* __restrict__ xg, const Tile& t,
                                              T* rs) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int E = 1 << t.e_log2;
  const int kb = lane << t.e_log2;
  const int ke = min(t.nnz, kb + E);
  int rpl = t.nnz;  // lane i: local offset of row i (i <= rows), clamped to the tile
  if (lane <= t.rows) {
    const int v = row_ptr[t.row_begin + lane] - t.nnz_begin;
    rpl = v < 0 ? 0 : (v > t.nnz ? t.nnz : v);
  }
  T vv[kTileEMax], xv[kTileEMax];
  {
    int c[kTileEMax];
#pragma unroll
    for (int j = 0; j < kTileEMax; ++j) {
      const bool in = j < E && kb + j < ke;
      c[j] = in ? lds(col + t.nnz_begin + kb + j) : 0;
      vv[j] = in ? lds(val + t.nnz_begin + kb + j) : T(0);
    }
#pragma unroll
    for (int j = 0; j < kTileEMax; ++j) xv[j] = (j < E && kb + j < ke) ? xg[c[j]] : T(0);
  }
  // first row whose end lies beyond kb (lane 0 starts at row 0: leading empty rows are its)
  int r;
  {
    int lo = 0, hi = t.rows > 0 ? t.rows - 1 : 0;
#pragma unroll
    for (int s = 0; s < 5; ++s) {
      const int mid = (lo + hi) >> 1;
      const int v = __shfl_sync(full, rpl, mid + 1);
      if (lo < hi) {
        if (v > kb) hi = mid;
        else lo = mid + 1;
      }
    }
    r = lane == 0 ? 0 : lo;
  }
  const bool active = kb < ke || (lane == 0 && t.rows > 0);
  const int rp_r = __shfl_sync(full, rpl, r);
  bool head = active && lane > 0 && rp_r < kb;  // row r began in an earlier lane
  int next = __shfl_sync(full, rpl, r + 1);
  int head_row = -1, tail_row = -1;
  T head_sum = T(0), tail_sum = T(0), s = T(0);
  bool tail_start = true;
#pragma unroll
  for (int j = 0; j < kTileEMax; ++j) {
    const int k = kb + j;
    const bool in = active && j < E && k < ke;
    while (true) {
      const bool need = in && k >= next;
      if (!__any_sync(full, need)) break;
      if (need) {
        if (head) { head_row = r; head_sum = s; }
        else rs[r] = s;
        head = false;
        s = T(0);
        ++r;
      }
      next = __shfl_sync(full, rpl, min(r + 1, 31));
    }
    if (in) s = fma(vv[j], xv[j], s);
  }
  while (true) {
    const bool need = active && r < t.rows && next <= ke;
    if (!__any_sync(full, need)) break;
    if (need) {
      if (head) { head_row = r; head_sum = s; }
      else rs[r] = s;
      head = false;
      s = T(0);
      ++r;
    }
    next = __shfl_sync(full, rpl, min(r + 1, 31));
  }
  if (active && kb < ke && r < t.rows) {
    tail_row = r;
    tail_sum = s;
    tail_start = !head;
  }
  if (__any_sync(full, head_row >= 0)) {
    // segmented inclusive scan of the trailing sums; a segment starts at a lane whose
    // trailing row began inside it (or that has none)
    T v = tail_row >= 0 ? tail_sum : T(0);
    int f = (tail_row < 0 || tail_start) ? 1 : 0;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const T vu = __shfl_up_sync(full, v, d);
      const int fu = __shfl_up_sync(full, f, d);
      if (lane >= d) {
        if (!f) v = vu + v;
        f |= fu;
      }
    }
    const T prev = __shfl_up_sync(full, v, 1);
    if (head_row >= 0) rs[head_row] = head_sum + prev;
  }
  __syncwarp();
}

// A piece of a split row: its partial goes to the row's carry slot, and the warp whose
// piece finishes last sums all slots in piece order into rs[0]. Returns (to the whole warp)
// whether this warp holds the finished row.
template <class T>
__device__ __forceinline__ bool split_finish(const Tile& t, const TileView<T>& plan, T* rs) {
  int last = 0;
  if ((threadIdx.x & 31) == 0) {
    plan.carry[t.carry + t.piece] = rs[0];
    __threadfence();
    const unsigned prev = atomicAdd(plan.counter + t.split, 1u);
    last = prev == (unsigned)(t.pieces - 1);
    if (last) {
      __threadfence();
      T s = T(0);
      for (int q = 0; q < t.pieces; ++q) s += __ldcg(plan.carry + t.carry + q);
      rs[0] = s;
      plan.counter[t.split] = 0u;
    }
  }
  last = __shfl_sync(0xffffffffu, last, 0);
  __syncwarp();
  return last != 0;
}

}  // namespace gpdhg
