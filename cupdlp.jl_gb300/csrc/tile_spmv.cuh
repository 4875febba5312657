// tile_spmv.cuh — one warp's row sums of one tile, in registers.
#pragma once

#include "common.cuh"
#include "tiles.h"

namespace gpdhg {

// The loads of one tile that do not depend on the gathered vector: this lane's local row
// offset (lane i holds rp[i], i <= rows), and its run of column indices and values.
template <class T>
struct TileLoad {
  int rpl;
  int c[TileTraits<T>::kEMax];
  T v[TileTraits<T>::kEMax];
};

// One 128-bit load of a lane: a group of 4 columns, 4 FP32 values or 2 FP64 values.
__device__ __forceinline__ void load_group(const int32_t* p, int32_t* d) {
  const int4 w = lds(reinterpret_cast<const int4*>(p));
  d[0] = w.x;
  d[1] = w.y;
  d[2] = w.z;
  d[3] = w.w;
}
__device__ __forceinline__ void load_group(const float* p, float* d) {
  const float4 w = lds(reinterpret_cast<const float4*>(p));
  d[0] = w.x;
  d[1] = w.y;
  d[2] = w.z;
  d[3] = w.w;
}
__device__ __forceinline__ void load_group(const double* p, double* d) {
  const double2 w = lds(reinterpret_cast<const double2*>(p));
  d[0] = w.x;
  d[1] = w.y;
}

// The lane's E elements (E = 2^e_log2) of one interleaved array (interleaved_slot): 128-bit
// group loads when E fills a group of G = 16 / sizeof(U), else one element per load; all are
// issued before any is used. Padding slots are loaded with the run (they exist).
template <class U, int kEMax>
__device__ __forceinline__ void load_run(const U* __restrict__ base, int data_begin, int e_log2, U* d) {
  constexpr int G = 16 / (int)sizeof(U);
  const int lane = threadIdx.x & 31;
  const int E = 1 << e_log2;
  if (E >= G) {
    const U* p = base + data_begin + G * lane;
#pragma unroll
    for (int g = 0; g < kEMax / G; ++g) {
      if (g * G >= E) break;  // uniform over the warp
      load_group(p + 32 * G * g, d + G * g);
    }
  } else {
#pragma unroll
    for (int j = 0; j < (G - 1 < kEMax ? G - 1 : kEMax); ++j) {
      if (j >= E) break;  // E is the same for the whole warp: a uniform exit
      d[j] = lds(base + data_begin + 32 * j + lane);
    }
  }
}

// Issues the loads of tile t (none is used here, so all are in flight together). The lane's
// columns and values come from the plan's lane-interleaved copy (interleaved_slot), so each
// load instruction of the warp is one coalesced access; padding slots are loaded with the
// lane's run but never gathered.
template <class T>
__device__ __forceinline__ void tile_load(const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ icol,
                                          const T* __restrict__ ival, const Tile& t, TileLoad<T>& L) {
  if (t.e_log2 < 0) return;  // a long row: streamed by long_row_sum / group_row_sum
  const int lane = threadIdx.x & 31;
  L.rpl = lane <= t.rows ? row_ptr[t.row_begin + lane] : 0;
  load_run<int32_t, TileTraits<T>::kEMax>(icol, t.data_begin, t.e_log2, L.c);
  load_run<T, TileTraits<T>::kEMax>(ival, t.data_begin, t.e_log2, L.v);
}

// A warp's rounds r0, r0 + step, ... (< nnz) of a long row: 32 x kLongRound coalesced
// (column, value) loads per round, all issued before the round's gathers, then one FMA per
// nonzero. FP32 keeps four independent accumulators (added pairwise at the end); FP64 keeps
// one: its FMAs issue at 2 lanes per SM and cycle, so a dependent chain costs no throughput
// and the three combining adds would. Returns the lane's sum (fixed order). (Keeping two
// rounds in flight needed more registers than the kernels' occupancy leaves and measured
// slower.)
template <class T>
__device__ __forceinline__ T stream_rounds(const int32_t* __restrict__ cp, const T* __restrict__ vp,
                                           const T* __restrict__ xg, int nnz, int r0, int step) {
  constexpr int kAcc = sizeof(T) == 8 ? 1 : 4;
  const int lane = threadIdx.x & 31;
  T acc[kAcc];
#pragma unroll
  for (int j = 0; j < kAcc; ++j) acc[j] = T(0);
  for (; r0 < nnz; r0 += step) {
    int c[kLongRound];
    T v[kLongRound];
#pragma unroll
    for (int j = 0; j < kLongRound; ++j) {
      const int k = r0 + j * 32 + lane;
      c[j] = k < nnz ? lds(cp + k) : 0;
      v[j] = k < nnz ? lds(vp + k) : T(0);
    }
#pragma unroll
    for (int j = 0; j < kLongRound; ++j)
      if (r0 + j * 32 + lane < nnz) acc[j % kAcc] = fma(v[j], xg[c[j]], acc[j % kAcc]);
  }
  if constexpr (kAcc == 1) return acc[0];
  else return (acc[0] + acc[1]) + (acc[2] + acc[3]);
}

// A CTA whose kBlock / 32 tiles are all warp-streamed rows (kWarpLong) sums them together:
// thread t takes row t % R (R = kBlock / 32 rows) and that row's nonzeros k = t / R + 32 i,
// so one warp-wide load covers R neighbouring rows at 32 / R consecutive positions each. When
// neighbouring rows have neighbouring columns at the same position (block-structured LPs:
// transportation, assignment, multicommodity flows) a warp's gathers touch R x 32 / R
// consecutive entries instead of 32 scattered ones. Row r's sum lands in rs_all[r][0]; the
// order is fixed (positions per thread, then the thread's four-lane group, then warps).
template <class T>
__device__ __forceinline__ void interleaved_rows_sum(const int32_t* __restrict__ col, const T* __restrict__ val,
                                                     const T* __restrict__ xg, const Tile* tl, T (*part)[kBlock / 32],
                                                     T (*rs_all)[32]) {
  constexpr int R = kBlock / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int r = threadIdx.x % R, u = threadIdx.x / R;
  const int len = tl[r].nnz;
  const int32_t* cp = col + tl[r].nnz_begin;
  const T* vp = val + tl[r].nnz_begin;
  int maxlen = 0;
#pragma unroll
  for (int q = 0; q < R; ++q) maxlen = max(maxlen, tl[q].nnz);
  T acc = T(0);
  for (int k0 = u; k0 < maxlen; k0 += 32 * kLongRound) {
    int c[kLongRound];
    T v[kLongRound];
#pragma unroll
    for (int j = 0; j < kLongRound; ++j) {
      const int k = k0 + j * 32;
      c[j] = k < len ? lds(cp + k) : 0;
      v[j] = k < len ? lds(vp + k) : T(0);
    }
#pragma unroll
    for (int j = 0; j < kLongRound; ++j)
      if (k0 + j * 32 < len) acc = fma(v[j], xg[c[j]], acc);
  }
  // lanes l, l + R, l + 2R, l + 3R of a warp hold row l
#pragma unroll
  for (int o = 16; o >= R; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if (lane < R) part[warp][lane] = acc;
  __syncthreads();
  if (threadIdx.x < R) {
    T sum = part[0][threadIdx.x];
#pragma unroll
    for (int w = 1; w < kBlock / 32; ++w) sum += part[w][threadIdx.x];
    rs_all[threadIdx.x][0] = sum;
  }
  __syncthreads();
}

// One row of up to kWarpShare nonzeros summed by the whole warp (valid in lane 0).
template <class T>
__device__ __forceinline__ T long_row_sum(const int32_t* __restrict__ col, const T* __restrict__ val,
                                          const T* __restrict__ xg, const Tile& t) {
  return warp_sum(stream_rounds(col + t.nnz_begin, val + t.nnz_begin, xg, t.nnz, 0, 32 * kLongRound));
}

// Group tiles: the CTA's warps form groups of W = 2^g; group q sums tile q's row (or piece),
// warp `sub` of the group streaming rounds sub, sub + W, ... The lanes' sums meet in shared
// memory (wlane, 32 per warp): lane l of the group's first warp adds lane l of each warp in
// warp order, and one shuffle tree finishes the row (W - 1 + 5 warp-wide adds instead of a
// shuffle tree per warp). Every thread must call it (warps without a tile pass has = false);
// the row's sum is in rs[0] of the group's first warp after the final __syncwarp.
template <class T>
__device__ __forceinline__ void group_row_sum(const int32_t* __restrict__ col, const T* __restrict__ val,
                                              const T* __restrict__ xg, const Tile& t, bool has, int W, int sub,
                                              T* wlane, T* rs) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T part = T(0);
  if (has)
    part = stream_rounds(col + t.nnz_begin, val + t.nnz_begin, xg, t.nnz, sub * 32 * kLongRound,
                         W * 32 * kLongRound);
  wlane[threadIdx.x] = part;
  __syncthreads();
  if (has && sub == 0) {
    T s = part;
    for (int w = 1; w < W; ++w) s += wlane[(warp + w) * 32 + lane];
    s = warp_sum(s);
    if (lane == 0) rs[0] = s;
  }
  __syncwarp();
}

// Row sums of tile t from its loads: rs[r] = sum of val * xg[col] over row t.row_begin + r,
// r < t.rows (a long-row tile, e_log2 < 0, goes to long_row_sum). Lane l owns the tile's
// nonzeros [l E, (l + 1) E), E = 2^e_log2: it gathers
// their entries of xg (all in flight together) and sums them per row with one FMA per
// nonzero. The row offsets are read from the lanes' registers with shuffles; a row that
// crosses lanes is completed by a segmented shuffle scan of the lanes' trailing partial
// sums. Every sum's order depends only on the tile, never on its position in memory. rs
// (32 entries per warp) is complete after the final __syncwarp.
template <class T, bool kSpanScan = false>
__device__ __forceinline__ void tile_sums(const int32_t* __restrict__ col, const T* __restrict__ val,
                                          const T* __restrict__ xg, const Tile& t, const TileLoad<T>& L, T* rs) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  if (t.e_log2 < 0) {
    const T sum = long_row_sum(col, val, xg, t);
    if (lane == 0) rs[0] = sum;
    __syncwarp();
    return;
  }
  const int E = 1 << t.e_log2;
  const int kb = lane << t.e_log2;
  const int ke = min(t.nnz, kb + E);
  int rpl = t.nnz;  // local offset of row `lane`, clamped to the tile
  if (lane <= t.rows) {
    const int v = L.rpl - t.nnz_begin;
    rpl = v < 0 ? 0 : (v > t.nnz ? t.nnz : v);
  }
  T xv[TileTraits<T>::kEMax];
#pragma unroll
  for (int j = 0; j < TileTraits<T>::kEMax; ++j) {
    if (j >= E) break;
    xv[j] = kb + j < ke ? xg[L.c[j]] : T(0);
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
  for (int j = 0; j < TileTraits<T>::kEMax; ++j) {
    if (j >= E) break;
    const int k = kb + j;
    const bool in = active && k < ke;
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
    if (in) s = fma(L.v[j], xv[j], s);
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
  // kSpanScan: a head lane needs the trailing sums of the lanes from its row's first lane on,
  // `span` lanes at most (0: no row crosses a lane boundary), so the scan stops after the
  // steps that reach that far: later steps change no value that a head lane reads (the FP64
  // pipe issues 2 lanes per SM and cycle, so each step costs the whole warp's time). Without
  // it every step runs (the primal kernel, whose compiled schedule measured up to 60% slower
  // with the span computed, and FP32 tiles; the FP64 dual kernel measured 6-9% faster).
  int span = 32;
  if constexpr (kSpanScan) {
    const int hstart = __shfl_sync(full, rpl, head_row >= 0 ? head_row : 0);
    span = __reduce_max_sync(full, head_row >= 0 ? lane - (hstart >> t.e_log2) : 0);
  } else {
    span = __any_sync(full, head_row >= 0) ? 32 : 0;
  }
  if (span > 0) {
    // segmented inclusive scan of the trailing sums; a segment starts at a lane whose
    // trailing row began inside it (or that has none)
    T v = tail_row >= 0 ? tail_sum : T(0);
    int f = (tail_row < 0 || tail_start) ? 1 : 0;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      if (kSpanScan && d >= span) break;  // uniform over the warp
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

// A CTA's tile descriptors, staged in shared memory once (one coalesced copy) so that no
// warp waits on a descriptor load before issuing a tile's loads.
__device__ __forceinline__ int stage_tiles(const Tile* __restrict__ tiles, int tb, int te, Tile* tl) {
  const int nt = te - tb;
  const int* src = reinterpret_cast<const int*>(tiles + tb);
  int* dst = reinterpret_cast<int*>(tl);
  constexpr int kWords = (int)(sizeof(Tile) / sizeof(int));
  for (int i = threadIdx.x; i < nt * kWords; i += kBlock) dst[i] = src[i];
  __syncthreads();
  return nt;
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
