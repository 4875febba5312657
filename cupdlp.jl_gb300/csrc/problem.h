// problem.h — device layout of one LP and the solver workspaces.
//
// Replaces CuLinearProgrammingProblem / CuScaledQpProblem (src/cpu_to_gpu.jl:1-21):
//   * scaled A as CSR (int32 row_ptr / col, FP64 values, FP32 values on demand),
//   * explicit CSR of A' (the reference builds it with CuSparseMatrixCSR(A'), :46),
//   * a row-block schedule for each (RowItem per CTA),
//   * scaled l, u, c, b and the ORIGINAL l, u, c, b plus the two rescaling vectors,
//     which is all the unscaled evaluation needs (the original matrix never is).
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <memory>
#include <vector>

#include "common.cuh"

namespace gpdhg {

// Start offset of the next large device buffer within its allocation: a multiple of 4 KB
// from 0 to 252 KB, stepping through the 64 values in a fixed order. Arrays that the step
// kernels stream at the same index (a tile's interleaved columns and values, the row vectors
// of an epilogue) otherwise begin at the same offset within the allocator's 2 MB pages and
// meet in the same memory channels; measured on the power-law LP, the FP32 dual kernel of a
// process's first problem took 130 µs with aligned starts and 123 µs with staggered ones
// (later problems 123-125 → 121.5-123).
inline size_t next_buffer_offset() {
  static std::atomic<unsigned> k{0};
  return (size_t)((k.fetch_add(1u) * 37u) % 64u) * 4096u;
}

template <class T>
struct DBuf {
  T* p = nullptr;
  void* raw = nullptr;   // the allocation (p lies at a staggered offset inside it)
  size_t n = 0;
  DBuf() = default;
  explicit DBuf(size_t count) { alloc(count); }
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  DBuf(DBuf&& o) noexcept : p(o.p), raw(o.raw), n(o.n) {
    o.p = nullptr;
    o.raw = nullptr;
    o.n = 0;
  }
  DBuf& operator=(DBuf&& o) noexcept {
    if (this != &o) {
      reset();
      p = o.p;
      raw = o.raw;
      n = o.n;
      o.p = nullptr;
      o.raw = nullptr;
      o.n = 0;
    }
    return *this;
  }
  ~DBuf() { reset(); }
  void alloc(size_t count) {
    reset();
    n = count;
    if (!count) return;
    // 64 spare bytes: bulk copies round their end up to 16 bytes; buffers of 1 MB and more
    // start at a staggered offset (next_buffer_offset)
    const size_t bytes = count * sizeof(T) + 64;
    const size_t offset = bytes >= ((size_t)1 << 20) ? next_buffer_offset() : 0;
    CK(cudaMalloc(&raw, bytes + offset));
    p = reinterpret_cast<T*>(static_cast<char*>(raw) + offset);
  }
  void reset() {
    if (raw) cudaFree(raw);
    raw = nullptr;
    p = nullptr;
    n = 0;
  }
  T* get() const { return p; }
};

template <class T>
struct PinnedBuf {
  T* p = nullptr;
  PinnedBuf() = default;
  explicit PinnedBuf(size_t count) { CK(cudaMallocHost(&p, count * sizeof(T) + 1)); }
  PinnedBuf(const PinnedBuf&) = delete;
  PinnedBuf& operator=(const PinnedBuf&) = delete;
  ~PinnedBuf() {
    if (p) cudaFreeHost(p);
  }
};

// Row-block schedule: consecutive rows packed while their nonzeros fit the SpMV stage
// (kStage) and there are at most kBlock of them; a longer row gets an item of its own.
std::vector<RowItem> build_row_items(const int32_t* row_ptr, int32_t nrows);

// CSR of A' built on the GPU from an uploaded A (ingest.cu: a stable radix sort of the
// nonzeros by column, so each row of A' lists its entries in increasing column of A' = row
// of A); fills At's device arrays and its host row pointer. Its row-block schedule is the
// caller's.
struct DeviceMatrix;
void transpose_on_device(const DeviceMatrix& A, DeviceMatrix& At, cudaStream_t s);

struct DeviceMatrix {
  int32_t nrows = 0, ncols = 0;
  long long nnz = 0;
  DBuf<int32_t> row_ptr, col;
  DBuf<double> val64;
  DBuf<float> val32;
  DBuf<RowItem> items;
  int32_t num_items = 0;
  std::vector<int32_t> host_rp;   // row pointer on the host (chunk plans are built from it)
  template <class T>
  CsrView<T> view() const;
};

template <>
inline CsrView<double> DeviceMatrix::view<double>() const {
  return CsrView<double>{nrows, ncols, row_ptr.get(), col.get(), val64.get(), items.get(), num_items};
}
template <>
inline CsrView<float> DeviceMatrix::view<float>() const {
  return CsrView<float>{nrows, ncols, row_ptr.get(), col.get(), val32.get(), items.get(), num_items};
}

template <class T>
struct Workspace;
// Out-of-line deleter so gpdhg_problem can be created where Workspace is incomplete.
struct WorkspaceDeleter {
  void operator()(Workspace<double>* w) const;
  void operator()(Workspace<float>* w) const;
};

}  // namespace gpdhg

struct gpdhg_problem {
  int32_t n = 0, m = 0, neq = 0;
  long long nnz = 0;
  double obj_const = 0.0;
  // host scalars derived once at creation
  double amax = 0.0;              // max |a_ij| of the scaled matrix: tau_0 = 1 / amax (:571)
  double norm2_c_scaled = 0.0;    // select_initial_primal_weight (src/saddle_point_gpu.jl:767-785)
  double norm2_b_scaled = 0.0;
  double linf_c = 0.0, linf_b = 0.0, l2_c = 0.0, l2_b = 0.0;  // CachedQuadraticProgramInfo (original)
  gpdhg::DeviceMatrix A, At;
  // scaled vectors (FP64; FP32 copies live in the FP32 workspace)
  gpdhg::DBuf<double> l, u, c, b;
  // original vectors and scaling
  gpdhg::DBuf<double> ol, ou, oc, ob, con, var;
  cudaStream_t stream = nullptr;
  std::unique_ptr<gpdhg::Workspace<double>, gpdhg::WorkspaceDeleter> ws64;
  std::unique_ptr<gpdhg::Workspace<float>, gpdhg::WorkspaceDeleter> ws32;
  std::vector<gpdhg_iteration_stats> history;
  std::vector<double> warm_x, warm_y;   // scaled warm start (empty: zero start)
  int last_precision = -1;              // workspace holding the last current iterate
  long long launches = 0;               // kernels launched on this handle so far
  // standard-form conversion of a two-sided problem: the caller's row behind each row, and
  // how many slack variables follow the caller's variables (empty / 0 otherwise)
  std::vector<int32_t> new_row_to_old;
  int32_t num_slacks = 0;
  // column order inside the handle (column_order): handle column k is the caller's column
  // col_perm[k]; empty when the handle keeps the caller's order
  std::vector<int32_t> col_perm;
  ~gpdhg_problem();
};

namespace gpdhg {
// validate (src/preprocess.jl:8-74) plus CSR structure checks; throws gpdhg::Error. The
// scans of large arrays run on host threads unless threads is false (the first bad entry,
// and so the error reported, is the serial scan's either way).
void validate_lp_desc(const gpdhg_lp_desc* d, bool threads);
// Builds the device problem from a descriptor (throws gpdhg::Error).
void problem_init(gpdhg_problem* p, const gpdhg_lp_desc* d);
// The solve loop (solver.cu); primal_out in the handle's column order.
void solve(gpdhg_problem* P, const gpdhg_params& prm, gpdhg_result* res, double* primal_out, double* dual_out);
// The same from the matrix in compressed sparse columns (index base 0 or 1, int64 indices, as
// Julia's SparseMatrixCSC): CSC(A) is uploaded as CSR(A') and A is built on the device.
void problem_init_csc(gpdhg_problem* p, const gpdhg_lp_desc* d, const int64_t* col_ptr, const int64_t* row_val,
                      const double* nz_val, int32_t base);
// transform_to_standard_form (src/quadratic_programming_io.jl:33-121) while the problem is
// built from a two-sided LP in compressed sparse columns; the matrix work runs on the device.
void problem_init_two_sided(gpdhg_problem* p, const gpdhg_two_sided_desc* t, const int64_t* col_ptr,
                            const int64_t* row_val, const double* nz_val, int32_t base);
// dst[k] = (float)src[k] on stream s.
void launch_convert_d2f(const double* src, float* dst, long long n, cudaStream_t s);
// dst[k] = 1 / src[k] on stream s.
void launch_reciprocal(const double* src, double* dst, long long n, cudaStream_t s);
// Ensures FP32 copies of the matrix values exist.
void ensure_fp32_values(gpdhg_problem* p);
// rescale_problem on the device (rescale.cu): rescales a problem built from an unscaled
// descriptor in place and recomputes its scaled host scalars.
void rescale_on_device(gpdhg_problem* p, const gpdhg_params& prm);
// Copies the constraint (m) and variable (n) rescaling vectors to the host.
void get_rescaling(const gpdhg_problem* p, double* con, double* var);

// Column order for the gathers of the dual step kernel (A dx gathers the primal candidate by
// column index, one 32-byte sector per nonzero). When the column degrees are skewed (at least
// kColumnOrderMinColumns columns, and the 1% most used columns hold at least
// kColumnOrderTopShare of the nonzeros) the columns are renumbered by decreasing degree
// (ties in the caller's order), so that the hot entries of the gathered vector share few
// cache lines; otherwise the caller's order is kept. The choice depends only on the degrees,
// so an LP gets the same order alone and inside a batch. Returns whether to renumber and
// fills perm (new column k = old column perm[k]).
constexpr int32_t kColumnOrderMinColumns = 1 << 16;
constexpr double kColumnOrderTopShare = 0.2;
bool choose_column_order(const std::vector<int32_t>& degree, std::vector<int32_t>& perm);
// Renumbers the columns of a built problem by choose_column_order's rule (the order sorted on
// the device; A's column indices, each row of A re-sorted by its new column, A' rebuilt,
// every n-vector permuted on the device) and records the order in col_perm.
void apply_column_order(gpdhg_problem* p);
// The rows of M in decreasing length, ties in row order (a stable radix sort on the device).
void order_rows_by_length(const DeviceMatrix& M, std::vector<int32_t>& order, cudaStream_t s);
// v (n entries, handle order) rewritten in the caller's column order, in place.
void to_caller_columns(const std::vector<int32_t>& perm, double* v);
// out[k] = in[perm[k]]: a caller-order vector in handle order.
void to_handle_columns(const std::vector<int32_t>& perm, const double* in, double* out);
}  // namespace gpdhg
