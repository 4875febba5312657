// pipe.cuh — the persistent, software-pipelined chunk engine under both step kernels.
//
// A matrix (A or A') is cut into chunks: runs of consecutive rows holding at most kS
// nonzeros and kR rows, and rows longer than kS split into pieces of kS. Each chunk's slice
// of the CSR is stored once, at plan build, as a 16-byte aligned blob in the layout the
// kernel computes from:
//     [ local row offsets: rows + 1 int32 | column indices: nnz int32 | values: padded ]
// values at index k + (k >> kPadShift), so that the row-sum pass, where every thread walks
// a contiguous run of nonzeros, reads shared memory without bank conflicts.
//
// A launch runs one CTA pair per SM (persistent); CTA b takes chunks b, b + G, b + 2G, ...
// through a three-stage ring of shared-memory buffers:
//   stage j+2: one elected thread issues cp.async.bulk copies of the blob and of the chunk's
//              slices of the epilogue vectors (x, c, l, u, ...), completing on an mbarrier;
//   stage j+1: once those land, every thread issues cp.async gathers of the multiplied
//              vector at the chunk's column indices into shared memory;
//   stage j:   row sums, split-row combination and the fused epilogue run from shared
//              memory and stream their results out.
// So HBM streams, L2 gathers and arithmetic of three chunks overlap in every CTA, without
// any dependent global load on the critical path. Every wait is bounded: a copy that does
// not land within kWaitCycles SM cycles records a fault in StepState::pipe_fault and the CTA
// stops, after waiting (again bounded) for its copies still in flight.
//
// Results do not depend on which CTA runs a chunk or where the chunk sits in the packed
// matrix: every sum's order is fixed by the chunk's own structure, so one LP gives the same
// bits alone and inside a batch.
#pragma once

#include "common.cuh"

namespace gpdhg {

// ------------------------------------------------------------------------------------
// Chunk schedule and blob layout (shared with the host builder).
// ------------------------------------------------------------------------------------
struct Chunk {
  long long blob;      // byte offset of the chunk's blob in its plan
  int32_t row_begin;   // first row (packed numbering)
  int32_t rows;        // rows of the chunk (1 for a piece of a split row)
  int32_t nnz_begin;   // first nonzero in the CSR
  int32_t nnz;         // nonzeros of the chunk
  int32_t inst;        // instance the rows belong to
  int32_t e_log2;      // log2 of the nonzeros per thread in the row-sum pass
  int32_t split;       // -1, or the counter of the split row this piece belongs to
  int32_t piece;       // piece index within the split row
  int32_t pieces;      // pieces of the split row
  int32_t carry;       // first carry slot of the split row
  int32_t aux;         // A chunks: first inequality row of the instance (packed numbering)
};

template <class T>
struct PipeTraits;
template <>
struct PipeTraits<float> {
  static constexpr int kS = 2048;      // nonzeros per chunk
  static constexpr int kR = 256;       // rows per chunk
  static constexpr int kPadShift = 5;  // one pad slot per 32 values (4-byte banks)
  static constexpr int kEMax = 8;      // longest per-thread run chosen from row lengths
};
template <>
struct PipeTraits<double> {
  static constexpr int kS = 1024;
  static constexpr int kR = 128;
  static constexpr int kPadShift = 4;  // one pad slot per 16 values (8-byte words)
  static constexpr int kEMax = 32;     // FP64 adds are scarce on GB300: few threads per row
};

constexpr int kPipeStages = 3;
constexpr long long kWaitCycles = 4000000000LL;  // ~2 s of SM clock before a copy counts as lost

__host__ __device__ constexpr long long pipe_align16(long long b) { return (b + 15) & ~15LL; }
__host__ __device__ constexpr int pad_index(int k, int shift) { return k + (k >> shift); }
__host__ __device__ constexpr int padded_len(int n, int shift) { return n + (n >> shift) + 1; }

template <class T>
__host__ __device__ constexpr int blob_rp_bytes(int rows) { return (int)pipe_align16(4LL * (rows + 1)); }
template <class T>
__host__ __device__ constexpr int blob_col_bytes(int nnz) { return (int)pipe_align16(4LL * nnz); }
template <class T>
__host__ __device__ constexpr int blob_val_bytes(int nnz) {
  return nnz == 0 ? 0 : (int)pipe_align16((long long)sizeof(T) * padded_len(nnz, PipeTraits<T>::kPadShift));
}
template <class T>
__host__ __device__ constexpr int blob_bytes(int rows, int nnz) {
  return blob_rp_bytes<T>(rows) + blob_col_bytes<T>(nnz) + blob_val_bytes<T>(nnz);
}

// Shared-memory layout of one pipeline stage with NV epilogue-vector slots.
template <class T, int NV>
struct StageLayout {
  static constexpr int S = PipeTraits<T>::kS, R = PipeTraits<T>::kR;
  static constexpr int V = 16 / (int)sizeof(T);  // elements per 16 bytes
  static constexpr int kBlob = blob_rp_bytes<T>(R) + blob_col_bytes<T>(S) + blob_val_bytes<T>(S);
  static constexpr int kXs = (int)pipe_align16((long long)sizeof(T) * padded_len(S, PipeTraits<T>::kPadShift));
  static constexpr int kVecLen = R + 2 * V;
  static constexpr int kVec = (int)pipe_align16((long long)sizeof(T) * kVecLen);
  static constexpr int kRs = (int)pipe_align16((long long)sizeof(T) * R);
  static constexpr int off_xs = kBlob;
  static constexpr int off_vec = off_xs + kXs;
  static constexpr int off_rs = off_vec + NV * kVec;
  static constexpr int kBytes = off_rs + kRs;
  static constexpr int kTotal = kPipeStages * kBytes + 128;  // + alignment slack of the ring
};

// Device view of a chunk plan.
template <class T>
struct ChunkView {
  const Chunk* chunks;
  int32_t num;
  const uint8_t* blob;
  T* carry;            // one partial row sum per piece of every split row
  unsigned* counter;   // pieces finished, per split row (returns to 0 after each launch)
};

// ------------------------------------------------------------------------------------
// PTX: mbarrier, bulk copies, cp.async gathers.
// ------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile(
      "{\n\t.reg .b64 state;\n\t"
      "mbarrier.arrive.expect_tx.shared::cta.b64 state, [%0], %1;\n\t}" ::"r"(smem_addr(bar)),
      "r"(bytes)
      : "memory");
}
// One poll of the phase with the given parity; may suspend the thread for up to ~1 us.
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity), "r"(1000u)
      : "memory");
  return ok != 0;
}
// Wait for the phase of the given parity to complete, bounded in time (kWaitCycles).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long t0 = clock64();
  while (clock64() - t0 < kWaitCycles)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ uint64_t policy_evict_first() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
// Global -> shared bulk copy completing on `bar` (both addresses and the size 16-byte multiples).
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}
__device__ __forceinline__ void bulk_load_stream(void* dst, const void* src, uint32_t bytes, uint64_t* bar,
                                                 uint64_t policy) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar)), "l"(policy)
      : "memory");
}
template <class T>
__device__ __forceinline__ void gather_async(T* dst, const T* src) {
  if constexpr (sizeof(T) == 4) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
  } else {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
  }
}
// Orders this thread's earlier generic-proxy shared-memory accesses (made visible to it by
// a barrier) before its following bulk copies into the same buffers.
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void async_wait_prev() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// ------------------------------------------------------------------------------------
// Per-stage header written by the issuing thread, read by the whole CTA.
// ------------------------------------------------------------------------------------
struct StageHdr {
  Chunk ch;
  int issued;    // copies were issued for this chunk (0: skipped, nothing to wait for)
  int pending;   // StepState::pending_commit of the chunk's instance
  int parity;    // StepState::parity
  int voff;      // index of the chunk's first row inside the vector slots
  double s0;     // kernel-specific scalars (weights, step ratios) of the instance
  double s1;
};

// Scratch of the row-sum pass.
template <class T>
struct ScanSmem {
  T v[kBlock / 32];
  int f[kBlock / 32];
};

// Row sums of one chunk from shared memory: rs[r] = sum_k val[k] * xs[k] over row r.
// Thread t takes the run of nonzeros [t E, (t + 1) E), E = 2^e_log2, sums it per row, and
// rows that cross runs are completed by a segmented scan of the runs' trailing partial sums
// (only when some row crosses a run boundary). Every thread must call it; rs is complete
// after the caller's next barrier.
template <class T>
__device__ __forceinline__ void chunk_row_sums(const int32_t* __restrict__ rp, const T* __restrict__ val,
                                               const T* __restrict__ xs, int rows, int nnz, int e_log2, T* rs,
                                               ScanSmem<T>& sc) {
  constexpr int SH = PipeTraits<T>::kPadShift;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int kb = tid << e_log2;
  const int ke = min(nnz, kb + (1 << e_log2));
  int head_row = -1, tail_row = -1;
  T head_sum = T(0), tail_sum = T(0);
  bool tail_start = true;
  if (kb < nnz || tid == 0) {
    int r = 0;
    if (tid > 0) {  // first row whose end lies beyond kb (exists: kb < nnz = rp[rows])
      int lo = 0, hi = rows - 1;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (rp[mid + 1] > kb) hi = mid;
        else lo = mid + 1;
      }
      r = lo;
    }
    bool head = tid > 0 && rp[r] < kb;  // row r began in an earlier run
    T s = T(0);
    int next = rows > 0 ? rp[r + 1] : 0;
    for (int k = kb; k < ke; ++k) {
      while (k >= next) {
        if (head) { head_row = r; head_sum = s; }
        else rs[r] = s;
        head = false;
        s = T(0);
        ++r;
        next = rp[r + 1];
      }
      const int q = pad_index(k, SH);
      s = fma(val[q], xs[q], s);
    }
    while (r < rows && rp[r + 1] <= ke) {
      if (head) { head_row = r; head_sum = s; }
      else rs[r] = s;
      head = false;
      s = T(0);
      ++r;
    }
    if (r < rows && kb < ke) {
      tail_row = r;
      tail_sum = s;
      tail_start = !head;
    }
  }
  if (!__syncthreads_or(head_row >= 0)) return;
  // segmented inclusive scan of the trailing sums; a segment starts at a run whose trailing
  // row began inside it (or that has no trailing row)
  T v = tail_row >= 0 ? tail_sum : T(0);
  int f = (tail_row < 0 || tail_start) ? 1 : 0;
  const unsigned full = 0xffffffffu;
  if (__any_sync(full, tail_row >= 0 || head_row >= 0)) {
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const T vu = __shfl_up_sync(full, v, d);
      const int fu = __shfl_up_sync(full, f, d);
      if (lane >= d) {
        if (!f) v = vu + v;
        f |= fu;
      }
    }
  }
  if (lane == 31) {
    sc.v[wid] = v;
    sc.f[wid] = f;
  }
  __syncthreads();
  T carry = T(0);  // inclusive scan at the last thread of the previous warp
  if (__any_sync(full, !f || (lane == 0 && head_row >= 0)))
    for (int w = 0; w < wid; ++w) carry = sc.f[w] ? sc.v[w] : carry + sc.v[w];
  const T S = f ? v : carry + v;
  T prev = __shfl_up_sync(full, S, 1);
  if (lane == 0) prev = carry;
  if (head_row >= 0) rs[head_row] = head_sum + prev;
}

// Combination of a split row's pieces: this piece's partial goes to its carry slot and the
// piece that finishes last sums all slots in piece order into rs[0]. Returns (to every
// thread) whether this CTA holds the finished row. Contains a barrier.
template <class T>
__device__ __forceinline__ bool split_combine(const Chunk& ch, const ChunkView<T>& plan, T* rs, int* flag) {
  if (threadIdx.x == 0) {
    plan.carry[ch.carry + ch.piece] = rs[0];
    __threadfence();
    const unsigned prev = atomicAdd(plan.counter + ch.split, 1u);
    const int last = prev == (unsigned)(ch.pieces - 1);
    if (last) {
      __threadfence();
      T s = T(0);
      for (int q = 0; q < ch.pieces; ++q) s += __ldcg(plan.carry + ch.carry + q);
      rs[0] = s;
      plan.counter[ch.split] = 0u;
    }
    *flag = last;
  }
  __syncthreads();
  return *flag != 0;
}

// Copies `count` elements of vector `src` starting at 16-byte aligned element `al` into a
// stage slot; returns the bytes issued.
template <class T>
__device__ __forceinline__ uint32_t issue_vec(T* slot, const T* src, int al, int count, uint64_t* bar) {
  const uint32_t bytes = (uint32_t)(count * (int)sizeof(T));
  if (bytes) bulk_load(slot, src + al, bytes, bar);
  return bytes;
}

// Sum of one value per thread; the result is valid in thread 0. One barrier; `sh` must not
// be written again before the caller's next barrier.
template <class T>
__device__ __forceinline__ double block_sum_1(T v, double* sh) {
  v = warp_sum(v);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = (double)v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < kBlock / 32; ++w) r += sh[w];
  return r;
}
template <class T>
__device__ __forceinline__ void block_sum_2(T a, T b, double* sh, double& ra, double& rb) {
  a = warp_sum(a);
  b = warp_sum(b);
  if ((threadIdx.x & 31) == 0) {
    sh[threadIdx.x >> 5] = (double)a;
    sh[kBlock / 32 + (threadIdx.x >> 5)] = (double)b;
  }
  __syncthreads();
  ra = rb = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < kBlock / 32; ++w) {
      ra += sh[w];
      rb += sh[kBlock / 32 + w];
    }
}

// Scalars of a chunk's instance that the issuing thread needs (read one chunk ahead).
struct StepScalars {
  int done, pending, parity;
  double w, tau, omega;
};
__device__ __forceinline__ StepScalars load_scalars(const StepState* st) {
  return StepScalars{st->done, st->pending_commit, st->parity, st->commit_weight, st->tau, st->omega};
}

// The persistent loop over chunks b0, b0 + G, ...: `issue(c, s, chunk, scalars)` (one
// thread) starts the copies of chunk c into stage s and fills hdr[s]; `gather(s)` (all
// threads) starts the cp.async gathers of stage s; `compute(c, s)` (all threads) consumes
// it. The issuing thread loads chunk descriptors two chunks ahead and instance scalars one
// chunk ahead, so no global load latency sits on the CTA's critical path. An instance's
// scalars cannot change while it still has chunks to run in this launch (its step decision
// waits for all of them), so reading them early is exact. Returns false after a lost copy.
template <class Issue, class Gather, class Compute>
__device__ __forceinline__ bool run_pipeline(const Chunk* __restrict__ chunks, int num_chunks,
                                             const StepState* st, uint64_t* bars, StageHdr* hdr, Issue&& issue,
                                             Gather&& gather, Compute&& compute) {
  const int G = gridDim.x, b0 = blockIdx.x, tid = threadIdx.x;
  const int J = b0 < num_chunks ? (num_chunks - b0 + G - 1) / G : 0;
  if (tid == 0) {
    for (int s = 0; s < kPipeStages; ++s) mbar_init(&bars[s], 1);
    mbar_fence_init();
  }
  __syncthreads();
  uint32_t phase = 0;        // bit s: parity of stage s's next phase
  uint32_t outstanding = 0;  // issuing thread: stages whose copies it has not seen land
  auto wait_stage = [&](int s) -> bool {
    if (!hdr[s].issued) return true;
    if (!mbar_wait(&bars[s], (phase >> s) & 1u)) return false;
    phase ^= 1u << s;
    outstanding &= ~(1u << s);
    return true;
  };
  // issuing thread's look-ahead: descriptor + scalars of the next chunk to issue, and the
  // descriptor of the one after it
  Chunk d1{}, d2{};
  StepScalars v1{};
  int next_j = 0;  // index j of the next chunk to issue
  auto advance = [&]() {
    // d1 <- d2, and start the loads that the next issue will use
    ++next_j;
    d1 = d2;
    if (next_j < J) v1 = load_scalars(st + d1.inst);
    if (next_j + 1 < J) d2 = chunks[b0 + (next_j + 1) * G];
  };
  auto issue_one = [&](int s) {
    fence_proxy_async();
    issue(b0 + next_j * G, s, d1, v1);
    if (hdr[s].issued) outstanding |= 1u << s;
    advance();
  };
  if (tid == 0) {
    if (J > 0) {
      d1 = chunks[b0];
      v1 = load_scalars(st + d1.inst);
    }
    if (J > 1) d2 = chunks[b0 + G];
    if (J > 0) issue_one(0);
    if (J > 1) issue_one(1);
  }
  __syncthreads();
  bool fail = false;
  if (J > 0) {
    if (wait_stage(0)) gather(0);
    else fail = true;
  }
  async_commit();
  for (int j = 0; j < J; ++j) {
    const int s = j % kPipeStages, s1 = (j + 1) % kPipeStages, s2 = (j + 2) % kPipeStages;
    if (j + 1 < J && !fail) {
      if (wait_stage(s1)) gather(s1);
      else fail = true;
    }
    async_commit();
    if (tid == 0 && j + 2 < J && !fail) issue_one(s2);
    async_wait_prev();
    if (__syncthreads_or(fail)) {
      // a copy did not land: wait (bounded) for whatever this CTA still has in flight
      async_wait_all();
      if (tid == 0)
        for (int q = 0; q < kPipeStages; ++q)
          if ((outstanding >> q) & 1u) mbar_wait(&bars[q], (phase >> q) & 1u);
      __syncthreads();
      return false;
    }
    compute(b0 + j * G, s);
    __syncthreads();
  }
  return true;
}

}  // namespace gpdhg
