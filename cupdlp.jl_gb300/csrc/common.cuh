// common.cuh — shared device/host helpers of libgpdhg (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <string>

#include "gpdhg.h"

namespace gpdhg {

// Phase timing of problem creation and solve set-up, printed to stderr when the environment
// variable GPDHG_TRACE is set (a diagnostic; nothing else reads it).
struct PhaseTrace {
  bool on;
  std::chrono::steady_clock::time_point t;
  PhaseTrace() : on(std::getenv("GPDHG_TRACE") != nullptr), t(std::chrono::steady_clock::now()) {}
  void mark(const char* what) {
    if (!on) return;
    const auto now = std::chrono::steady_clock::now();
    std::fprintf(stderr, "gpdhg trace: %-28s %8.2f ms\n", what,
                 std::chrono::duration<double, std::milli>(now - t).count());
    t = now;
  }
};

// A failure that maps onto one gpdhg_status at the ABI boundary.
struct Error : std::runtime_error {
  gpdhg_status status;
  Error(gpdhg_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

inline void cuda_check(cudaError_t e, const char* what, const char* file, int line) {
  if (e != cudaSuccess) {
    gpdhg_status s = (e == cudaErrorMemoryAllocation) ? GPDHG_ERR_OUT_OF_MEMORY : GPDHG_ERR_CUDA;
    throw Error(s, std::string(what) + ": " + cudaGetErrorString(e) + " (" + file + ":" + std::to_string(line) + ")");
  }
}
#define CK(call) ::gpdhg::cuda_check((call), #call, __FILE__, __LINE__)
#define CK_LAUNCH() ::gpdhg::cuda_check(cudaGetLastError(), "kernel launch", __FILE__, __LINE__)

constexpr int kBlock = 256;          // threads per CTA of every row-block kernel
constexpr int kStageDepth = 8;                // independent (col, val) loads per thread and item
constexpr int kStage = kBlock * kStageDepth;  // nonzeros staged per item (2048)
constexpr int kReduceBlocks = 304;   // 2 x 152 SMs for grid-stride reductions

// One CTA's share of a CSR matrix: rows [row_begin, row_end) and the schedule used for
// them (see spmv.cuh): staged short rows reduced by groups of `group` lanes, warp-per-row
// register accumulation, or one long row streamed by the whole CTA.
enum ItemMode : int32_t { kItemStaged = 0, kItemWarps = 1, kItemLong = 2 };
struct RowItem {
  int32_t row_begin;
  int32_t row_end;
  int32_t group;
  int32_t mode;
  int32_t nnz_begin;   // row_ptr[row_begin]
  int32_t nnz_count;   // row_ptr[row_end] - row_ptr[row_begin]
};

// A contiguous element range [begin, end) of one instance, reduced by one CTA of the
// segmented FP64 reductions (evaluation statistics, restart scores).
struct SegItem {
  int32_t begin;
  int32_t end;
  int32_t inst;
};

// Device view of a CSR matrix with its row-block schedule.
template <class T>
struct CsrView {
  int32_t nrows;
  int32_t ncols;
  const int32_t* row_ptr;
  const int32_t* col;
  const T* val;
  const RowItem* items;
  int32_t num_items;
};

// Scalar state of the step loop, resident on the device and updated by the last CTA
// of the dual kernel after every step attempt (the host mirrors it between chunks).
struct StepState {
  double tau;              // step size of the next attempt (take_step!'s local step_size)
  double omega;            // primal weight
  double iter_start_tau;   // solver_state.step_size at entry of take_step!: the averaging weight
  double commit_weight;    // averaging weight of the accepted step awaiting its commit
  double kkt_passes;       // cumulative_kkt_passes
  double sum_w_primal;     // sum_primal_solution_weights
  double sum_w_dual;       // sum_dual_solution_weights
  double reduction_exponent;
  double growth_exponent;
  double last_limit;       // diagnostics: last step-size limit
  long long total_iters;   // total_number_iterations (attempts)
  long long count_primal;  // sum_primal_solutions_count
  long long count_dual;    // sum_dual_solutions_count
  long long accepted;
  long long rejected;
  int parity;              // which y / K x buffer is current
  int pending_commit;      // an accepted step whose vector updates are not applied yet
  int done;                // the current chunk is finished
  int numerical_error;
  int accepted_in_chunk;
  int target_in_chunk;
  int attempts_in_chunk;
  int max_attempts_in_chunk;
  unsigned int arrive;     // CTAs of the dual kernel finished in this attempt
  int constant_step;       // ConstantStepsizeParams: every attempt is accepted
  long long primal_spmv;   // attempts whose primal kernel also ran A'y (a commit)
  const double* pow_table; // [1-(k+1)^-r, 1+(k+1)^-g] for k < pow_table_len (device)
  long long pow_table_len;
  // written in every attempt by the instance's first dual CTA, for the deciding CTA:
  double half_w_dx2;       // 0.5 * omega * ||dx|| * ||dx||: the primal part of the movement
  double half_over_omega;  // 0.5 / omega
  double f1, f2;           // step-size factors for this attempt's counter
  // 1 / sum_w_primal and 1 / sum_w_dual, set by the host before an evaluation averages
  double rcp_w_primal, rcp_w_dual;
};

// ----------------------------------------------------------------------------------
// Deterministic block reductions (fixed shuffle tree, fixed warp order).
// ----------------------------------------------------------------------------------
template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
template <class T>
__device__ __forceinline__ T warp_max(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  return v;
}

// Sum over the CTA; the result is valid in thread 0. `sh` holds >= 32 entries.
template <class T>
__device__ __forceinline__ T block_sum(T v, T* sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  T r = T(0);
  if (wid == 0) {
    r = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : T(0);
    r = warp_sum(r);
  }
  return r;
}
template <class T>
__device__ __forceinline__ T block_max(T v, T* sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v = warp_max(v);
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  T r = T(0);
  if (wid == 0) {
    r = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : T(0);
    r = warp_max(r);
  }
  return r;
}

// Julia's max/min (used by the reference's kernels) propagate NaN.
__device__ __forceinline__ double jmax(double a, double b) { return (a != a || b != b) ? a + b : (a > b ? a : b); }
__device__ __forceinline__ double jmin(double a, double b) { return (a != a || b != b) ? a + b : (a < b ? a : b); }
__device__ __forceinline__ float jmax(float a, float b) { return (a != a || b != b) ? a + b : (a > b ? a : b); }
__device__ __forceinline__ float jmin(float a, float b) { return (a != a || b != b) ? a + b : (a < b ? a : b); }

inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

// Streaming accesses (read or written once per pass): evict-first in L1 and L2, so the
// vectors gathered by the next kernel stay resident in L2.
template <class T>
__device__ __forceinline__ T lds(const T* p) { return __ldcs(p); }
template <class T>
__device__ __forceinline__ void sts(T* p, T v) { __stcs(p, v); }

// max / min of doubles on the integer pipe (GB300's FP64 pipe is the scarce resource):
// for non-NaN values the sign-magnitude bit pattern maps to an order-preserving int64 key.
__device__ __forceinline__ long long order_key(double v) {
  const long long b = __double_as_longlong(v);
  return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}
__device__ __forceinline__ double imax(double a, double b) { return order_key(a) < order_key(b) ? b : a; }
__device__ __forceinline__ double imin(double a, double b) { return order_key(b) < order_key(a) ? b : a; }
__device__ __forceinline__ float imax(float a, float b) { return fmaxf(a, b); }
__device__ __forceinline__ float imin(float a, float b) { return fminf(a, b); }

}  // namespace gpdhg
