// ingest.cu — A' of an uploaded CSR matrix, built on the GPU.
//
// The reference builds the transpose with CuSparseMatrixCSR(A') (src/cpu_to_gpu.jl:46).
// Here a stable LSD radix sort of the nonzeros by column (8-bit digits) yields, for every
// column, its nonzeros in increasing row order: the CSR of A' with sorted column indices,
// the order a counting-sort transpose gives. A block-diagonal A (a packed batch) gives the
// block diagonal of its blocks' transposes, each exactly what the block alone gives.
//
// One pass = a digit histogram per 4,096-key tile, one exclusive scan over (digit, tile), and
// a scatter in which every tile places its keys in order: per round of 256 keys each warp
// ranks its lanes among equal digits (__match_any_sync), a per-digit prefix over the warps
// orders the warps, and a per-digit running base orders the rounds. Stable by construction
// and deterministic (no atomics decide a position).
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "problem.h"

namespace gpdhg {
namespace {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 16;
constexpr int kSortTile = kSortThreads * kSortItems;
constexpr int kDigits = 256;

// rows[k] = the row of nonzero k (the last row i with rp[i] <= k; empty rows share offsets)
__global__ void row_of_kernel(int32_t m, long long nnz, const int32_t* __restrict__ rp, int32_t* __restrict__ rows) {
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += (long long)gridDim.x * blockDim.x) {
    int lo = 0, hi = m - 1;  // rp[lo] <= k < rp[m]
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (rp[mid] <= k) lo = mid;
      else hi = mid - 1;
    }
    rows[k] = lo;
  }
}

__global__ void iota_kernel(long long len, uint32_t* __restrict__ v) {
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < len; k += (long long)gridDim.x * blockDim.x)
    v[k] = (uint32_t)k;
}

// hist[d * tiles + t] = keys of tile t whose digit is d
__global__ void __launch_bounds__(kSortThreads) digit_hist_kernel(const uint32_t* __restrict__ keys, long long len,
                                                                  int shift, uint32_t* __restrict__ hist, int tiles) {
  __shared__ uint32_t h[kDigits];
  h[threadIdx.x] = 0;
  __syncthreads();
  const long long base = (long long)blockIdx.x * kSortTile;
  for (int i = threadIdx.x; i < kSortTile; i += kSortThreads) {
    const long long k = base + i;
    if (k < len) atomicAdd(&h[(keys[k] >> shift) & (kDigits - 1)], 1u);
  }
  __syncthreads();
  hist[(size_t)threadIdx.x * tiles + blockIdx.x] = h[threadIdx.x];
}

// In-place exclusive scan of len counts (one CTA: contiguous chunks per thread, then a scan
// of the chunk totals).
__global__ void __launch_bounds__(1024) exclusive_scan_kernel(uint32_t* __restrict__ v, long long len) {
  __shared__ uint32_t part[1024];
  const long long chunk = (len + 1023) / 1024;
  const long long b = threadIdx.x * chunk, e = min(len, b + chunk);
  uint32_t s = 0;
  for (long long i = b; i < e; ++i) s += v[i];
  part[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t run = 0;
    for (int t = 0; t < 1024; ++t) {
      const uint32_t c = part[t];
      part[t] = run;
      run += c;
    }
  }
  __syncthreads();
  uint32_t run = part[threadIdx.x];
  for (long long i = b; i < e; ++i) {
    const uint32_t c = v[i];
    v[i] = run;
    run += c;
  }
}

// Device-wide exclusive scan of len counts in three launches: per-block totals of
// kScanBlock consecutive counts (coalesced), one CTA scanning the totals in place
// (exclusive_scan_kernel), then each block scanning its counts from its total's offset.
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanBlock = kScanThreads * kScanItems;

__global__ void __launch_bounds__(kScanThreads) scan_block_totals_kernel(const uint32_t* __restrict__ v, long long len,
                                                                         uint32_t* __restrict__ totals) {
  __shared__ uint32_t warp_sum[kScanThreads / 32];
  const long long base = (long long)blockIdx.x * kScanBlock;
  uint32_t s = 0;
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    const long long i = base + j * kScanThreads + threadIdx.x;
    if (i < len) s += v[i];
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int w = 0; w < kScanThreads / 32; ++w) t += warp_sum[w];
    totals[blockIdx.x] = t;
  }
}

__global__ void __launch_bounds__(kScanThreads) scan_block_apply_kernel(uint32_t* __restrict__ v, long long len,
                                                                        const uint32_t* __restrict__ offsets) {
  __shared__ uint32_t sh[kScanBlock];
  __shared__ uint32_t warp_sum[kScanThreads / 32];
  const long long base = (long long)blockIdx.x * kScanBlock;
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    const int q = j * kScanThreads + threadIdx.x;
    sh[q] = base + q < len ? v[base + q] : 0u;
  }
  __syncthreads();
  // thread t scans its kScanItems consecutive counts
  uint32_t loc[kScanItems];
  uint32_t run = 0;
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    loc[j] = run;
    run += sh[threadIdx.x * kScanItems + j];
  }
  // exclusive scan of the thread totals: inclusive within the warp, then across warps
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t inc = run;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += u;
  }
  if (lane == 31) warp_sum[warp] = inc;
  __syncthreads();
  uint32_t before = offsets[blockIdx.x];
  for (int w = 0; w < warp; ++w) before += warp_sum[w];
  before += inc - run;
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) sh[threadIdx.x * kScanItems + j] = before + loc[j];
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    const int q = j * kScanThreads + threadIdx.x;
    if (base + q < len) v[base + q] = sh[q];
  }
}

void exclusive_scan(uint32_t* v, long long len, DBuf<uint32_t>& totals, cudaStream_t s) {
  const long long blocks = (len + kScanBlock - 1) / kScanBlock;
  if (blocks <= 1) {
    exclusive_scan_kernel<<<1, 1024, 0, s>>>(v, len);
    CK_LAUNCH();
    return;
  }
  if ((long long)totals.n < blocks) totals.alloc((size_t)blocks);
  scan_block_totals_kernel<<<(unsigned)blocks, kScanThreads, 0, s>>>(v, len, totals.get());
  CK_LAUNCH();
  exclusive_scan_kernel<<<1, 1024, 0, s>>>(totals.get(), blocks);
  CK_LAUNCH();
  scan_block_apply_kernel<<<(unsigned)blocks, kScanThreads, 0, s>>>(v, len, totals.get());
  CK_LAUNCH();
}

__global__ void __launch_bounds__(kSortThreads) digit_scatter_kernel(const uint32_t* __restrict__ keys,
                                                                     const uint32_t* __restrict__ vals, long long len,
                                                                     int shift, const uint32_t* __restrict__ offs,
                                                                     int tiles, uint32_t* __restrict__ keys_out,
                                                                     uint32_t* __restrict__ vals_out) {
  __shared__ uint32_t base[kDigits];                        // next output position per digit
  __shared__ uint32_t wcnt[kSortThreads / 32][kDigits];     // a round's per-warp digit counts
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  base[t] = offs[(size_t)t * tiles + blockIdx.x];
  const long long tile0 = (long long)blockIdx.x * kSortTile;
  for (int r = 0; r < kSortItems; ++r) {
    const long long k = tile0 + (long long)r * kSortThreads + t;
    const bool in = k < len;
    const uint32_t key = in ? keys[k] : 0u, val = in ? vals[k] : 0u;
    const int d = in ? (int)((key >> shift) & (kDigits - 1)) : kDigits;  // out-of-range lanes: a digit of their own
#pragma unroll
    for (int w = 0; w < kSortThreads / 32; ++w) wcnt[w][t] = 0;
    __syncthreads();
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int rank = __popc(peers & ((1u << lane) - 1u));
    if (in && rank == 0) wcnt[warp][d] = __popc(peers);
    __syncthreads();
    uint32_t run = 0;  // thread t: exclusive prefix of digit t over the warps
#pragma unroll
    for (int w = 0; w < kSortThreads / 32; ++w) {
      const uint32_t c = wcnt[w][t];
      wcnt[w][t] = run;
      run += c;
    }
    __syncthreads();
    if (in) {
      const uint32_t dst = base[d] + wcnt[warp][d] + (uint32_t)rank;
      keys_out[dst] = key;
      vals_out[dst] = val;
    }
    __syncthreads();
    base[t] += run;
  }
}

// A' = (row_ptr from the sorted columns, col = row of the nonzero, val)
__global__ void transpose_fill_kernel(long long nnz, const uint32_t* __restrict__ perm, const int32_t* __restrict__ rows,
                                      const double* __restrict__ val, int32_t* __restrict__ col_t,
                                      double* __restrict__ val_t) {
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < nnz; p += (long long)gridDim.x * blockDim.x) {
    const uint32_t k = perm[p];
    col_t[p] = rows[k];
    val_t[p] = val[k];
  }
}

__global__ void transpose_rowptr_kernel(long long nnz, int32_t n, const uint32_t* __restrict__ skeys,
                                        int32_t* __restrict__ rp_t) {
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p <= nnz; p += (long long)gridDim.x * blockDim.x) {
    const long long prev = p == 0 ? -1 : (long long)skeys[p - 1];
    const long long cur = p == nnz ? (long long)n : (long long)skeys[p];
    for (long long j = prev + 1; j <= cur; ++j) rp_t[j] = (int32_t)p;
  }
}

int grid_of(long long len) { return (int)std::max<long long>(1, std::min<long long>((len + 255) / 256, 8192)); }

}  // namespace

namespace {
// key[j] = max_key - (rp[j + 1] - rp[j]): ascending keys = decreasing row lengths
__global__ void length_key_kernel(int32_t n, const int32_t* __restrict__ rp, uint32_t max_key,
                                  uint32_t* __restrict__ key) {
  const int32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n) key[j] = max_key - (uint32_t)(rp[j + 1] - rp[j]);
}
}  // namespace

void order_rows_by_length(const DeviceMatrix& M, std::vector<int32_t>& order, cudaStream_t s) {
  const int32_t n = M.nrows;
  order.assign((size_t)n, 0);
  if (n == 0) return;
  uint32_t max_len = 0;
  for (int32_t j = 0; j < n; ++j) max_len = std::max<uint32_t>(max_len, (uint32_t)(M.host_rp[j + 1] - M.host_rp[j]));
  DBuf<uint32_t> k0((size_t)n), k1((size_t)n), v0((size_t)n), v1((size_t)n), hist, scan_totals;
  length_key_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, M.row_ptr.get(), max_len, k0.get());
  CK_LAUNCH();
  iota_kernel<<<grid_of(n), 256, 0, s>>>(n, v0.get());
  CK_LAUNCH();
  const int tiles = (int)((n + kSortTile - 1) / kSortTile);
  hist.alloc((size_t)kDigits * tiles);
  uint32_t *ka = k0.get(), *kb = k1.get(), *va = v0.get(), *vb = v1.get();
  for (int shift = 0; shift < 32 && (max_len >> shift) != 0u; shift += 8) {
    digit_hist_kernel<<<tiles, kSortThreads, 0, s>>>(ka, n, shift, hist.get(), tiles);
    CK_LAUNCH();
    exclusive_scan(hist.get(), (long long)kDigits * tiles, scan_totals, s);
    digit_scatter_kernel<<<tiles, kSortThreads, 0, s>>>(ka, va, n, shift, hist.get(), tiles, kb, vb);
    CK_LAUNCH();
    std::swap(ka, kb);
    std::swap(va, vb);
  }
  CK(cudaMemcpyAsync(order.data(), va, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
}

void transpose_on_device(const DeviceMatrix& A, DeviceMatrix& At, cudaStream_t s) {
  const int32_t m = A.nrows, n = A.ncols;
  const long long nnz = A.nnz;
  At.nrows = n;
  At.ncols = m;
  At.nnz = nnz;
  At.row_ptr.alloc((size_t)n + 1);
  At.col.alloc(std::max<long long>(nnz, 1));
  At.val64.alloc(std::max<long long>(nnz, 1));
  DBuf<uint32_t> k0(std::max<long long>(nnz, 1)), k1(std::max<long long>(nnz, 1));
  DBuf<uint32_t> v0(std::max<long long>(nnz, 1)), v1(std::max<long long>(nnz, 1));
  DBuf<int32_t> rows(std::max<long long>(nnz, 1));
  DBuf<uint32_t> hist;
  DBuf<uint32_t> scan_totals;
  if (nnz > 0) {
    row_of_kernel<<<grid_of(nnz), 256, 0, s>>>(m, nnz, A.row_ptr.get(), rows.get());
    CK_LAUNCH();
    CK(cudaMemcpyAsync(k0.get(), A.col.get(), sizeof(uint32_t) * nnz, cudaMemcpyDeviceToDevice, s));
    iota_kernel<<<grid_of(nnz), 256, 0, s>>>(nnz, v0.get());
    CK_LAUNCH();
    const int tiles = (int)((nnz + kSortTile - 1) / kSortTile);
    hist.alloc((size_t)kDigits * tiles);
    uint32_t *ka = k0.get(), *kb = k1.get(), *va = v0.get(), *vb = v1.get();
    for (int shift = 0; shift < 32 && n > 1 && ((uint32_t)(n - 1) >> shift) != 0u; shift += 8) {
      digit_hist_kernel<<<tiles, kSortThreads, 0, s>>>(ka, nnz, shift, hist.get(), tiles);
      CK_LAUNCH();
      exclusive_scan(hist.get(), (long long)kDigits * tiles, scan_totals, s);
      digit_scatter_kernel<<<tiles, kSortThreads, 0, s>>>(ka, va, nnz, shift, hist.get(), tiles, kb, vb);
      CK_LAUNCH();
      std::swap(ka, kb);
      std::swap(va, vb);
    }
    transpose_fill_kernel<<<grid_of(nnz), 256, 0, s>>>(nnz, va, rows.get(), A.val64.get(), At.col.get(),
                                                       At.val64.get());
    CK_LAUNCH();
    transpose_rowptr_kernel<<<grid_of(nnz + 1), 256, 0, s>>>(nnz, n, ka, At.row_ptr.get());
    CK_LAUNCH();
  } else {
    CK(cudaMemsetAsync(At.row_ptr.get(), 0, sizeof(int32_t) * ((size_t)n + 1), s));
  }
  At.host_rp.resize((size_t)n + 1);
  CK(cudaMemcpyAsync(At.host_rp.data(), At.row_ptr.get(), sizeof(int32_t) * ((size_t)n + 1), cudaMemcpyDeviceToHost, s));
  // the sort buffers are freed at return: wait for the kernels that use them (and the copy)
  CK(cudaStreamSynchronize(s));
}

}  // namespace gpdhg
