// problem.cu — validation and upload of one LP (replaces src/cpu_to_gpu.jl:26-81).
#include <algorithm>
#include <array>
#include <climits>
#include <cmath>
#include <cstring>
#include <exception>
#include <thread>

#include "problem.h"

namespace gpdhg {

std::vector<RowItem> build_row_items(const int32_t* rp, int32_t nrows) {
  // Rows with more than kCtaRow nonzeros get a CTA each (streamed, 8 loads per thread in
  // flight). The other rows are packed in order while their nonzeros fit the stage and there
  // are at most kBlock of them, whatever their lengths (splitting by length would fragment a
  // power-law matrix into thousands of tiny items); such an item of at most 8 rows averaging
  // >= 64 nonzeros runs warp-per-row, any other is staged, with the largest power-of-two lane
  // group (<= 32) that still gives every row its own group.
  constexpr int64_t kCtaRow = 256, kWarpRow = 64;
  std::vector<RowItem> items;
  auto len = [&](int32_t r) { return (int64_t)rp[r + 1] - rp[r]; };
  int32_t r = 0;
  while (r < nrows) {
    if (len(r) > kCtaRow) {
      items.push_back({r, r + 1, 0, kItemLong, rp[r], (int32_t)len(r)});
      ++r;
      continue;
    }
    const int32_t start = r;
    const int64_t base = rp[r];
    while (r < nrows && r - start < kBlock && len(r) <= kCtaRow && (int64_t)rp[r + 1] - base <= kStage) ++r;
    const int rows = r - start;
    const int64_t nnz = (int64_t)rp[r] - base;
    if (rows <= kBlock / 32 && nnz >= kWarpRow * rows) {
      items.push_back({start, r, 32, kItemWarps, rp[start], (int32_t)nnz});
      continue;
    }
    int g = 1;
    while (g < 32 && 2 * g * rows <= kBlock) g <<= 1;
    items.push_back({start, r, g, kItemStaged, rp[start], (int32_t)nnz});
  }
  return items;
}

namespace {

void upload_csr(DeviceMatrix& dm, int32_t nrows, int32_t ncols, const int32_t* rp, const int32_t* col,
                const double* val, cudaStream_t s) {
  dm.nrows = nrows;
  dm.ncols = ncols;
  dm.nnz = rp[nrows];
  dm.host_rp.assign(rp, rp + (size_t)nrows + 1);
  dm.row_ptr.alloc((size_t)nrows + 1);
  dm.col.alloc(std::max<long long>(dm.nnz, 1));
  dm.val64.alloc(std::max<long long>(dm.nnz, 1));
  CK(cudaMemcpyAsync(dm.row_ptr.get(), rp, sizeof(int32_t) * ((size_t)nrows + 1), cudaMemcpyHostToDevice, s));
  if (dm.nnz) {
    CK(cudaMemcpyAsync(dm.col.get(), col, sizeof(int32_t) * dm.nnz, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(dm.val64.get(), val, sizeof(double) * dm.nnz, cudaMemcpyHostToDevice, s));
  }
}

// The row-block schedule of the plain SpMV, from the matrix's host row pointer.
void set_row_items(DeviceMatrix& dm, cudaStream_t s) {
  std::vector<RowItem> items = build_row_items(dm.host_rp.data(), dm.nrows);
  if (items.empty()) items.push_back({0, 0, 1, kItemStaged, 0, 0});  // no rows: one idle CTA still runs the step decision
  dm.num_items = (int32_t)items.size();
  dm.items.alloc(std::max<size_t>(items.size(), 1));
  if (!items.empty())
    CK(cudaMemcpyAsync(dm.items.get(), items.data(), sizeof(RowItem) * items.size(), cudaMemcpyHostToDevice, s));
  // the schedule vector dies at return: wait for the copies before it does
  CK(cudaStreamSynchronize(s));
}

void upload_vec(DBuf<double>& d, const double* h, size_t n, cudaStream_t s) {
  d.alloc(std::max<size_t>(n, 1));
  if (n) CK(cudaMemcpyAsync(d.get(), h, sizeof(double) * n, cudaMemcpyHostToDevice, s));
}

void upload_vec_or_fill(DBuf<double>& d, const double* h, const double* fallback, size_t n, cudaStream_t s) {
  upload_vec(d, h ? h : fallback, n, s);
}

__global__ void fill_ones_kernel(double* __restrict__ v, long long n) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) v[k] = 1.0;
}

// d = h (n entries), or all ones when h is NULL (filled on the device)
void upload_vec_or_ones(DBuf<double>& d, const double* h, size_t n, cudaStream_t s) {
  if (h) return upload_vec(d, h, n, s);
  d.alloc(std::max<size_t>(n, 1));
  if (n) {
    fill_ones_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(d.get(), (long long)n);
    CK_LAUNCH();
  }
}

double norm2(const double* v, size_t n) {
  double s = 0.0;
  for (size_t i = 0; i < n; ++i) s += v[i] * v[i];
  return std::sqrt(s);
}
double norm_inf(const double* v, size_t n) {
  double s = 0.0;
  for (size_t i = 0; i < n; ++i) s = std::max(s, std::fabs(v[i]));
  return s;
}

}  // namespace

namespace {

// Host threads for a scan of len entries with `checks` tests each: one per 256k tests, at most
// 16 (a thread's start-up costs tens of microseconds, 256k tests a few hundred).
int scan_threads(int64_t len, int checks, bool threads) {
  if (!threads) return 1;
  const int64_t hw = std::max(1u, std::thread::hardware_concurrency());
  return (int)std::min<int64_t>(std::min<int64_t>(hw, 16), std::max<int64_t>(1, len * checks / 262144));
}

// For each of the K predicates, the smallest q in [0, len) with bad(q, k), or -1: one pass of
// contiguous chunks on host threads, so each answer is the serial scan's.
template <int K, class Bad>
std::array<int64_t, K> first_bad_each(int64_t len, Bad bad, bool threads) {
  const int T = scan_threads(len, K, threads);
  std::vector<std::array<int64_t, K>> first(T);
  auto scan = [&](int t) {
    std::array<int64_t, K>& f = first[t];
    f.fill(-1);
    int open = K;
    for (int64_t q = len * t / T, e = len * (t + 1) / T; q < e && open; ++q)
      for (int k = 0; k < K; ++k)
        if (f[k] < 0 && bad(q, k)) {
          f[k] = q;
          --open;
        }
  };
  if (T <= 1) {
    scan(0);
  } else {
    std::vector<std::thread> th;
    th.reserve(T);
    for (int t = 0; t < T; ++t) th.emplace_back(scan, t);
    for (auto& x : th) x.join();
  }
  std::array<int64_t, K> out;
  out.fill(-1);
  for (int k = 0; k < K; ++k)
    for (int t = 0; t < T && out[k] < 0; ++t) out[k] = first[t][k];
  return out;
}

// The smallest k in [0, len) with bad(k), or -1.
template <class Bad>
int64_t first_bad(int64_t len, Bad bad, bool threads) {
  return first_bad_each<1>(len, [&](int64_t q, int) { return bad(q); }, threads)[0];
}

}  // namespace

namespace {

// The descriptor's dimensions and vectors (validate, src/preprocess.jl:8-74, without the matrix).
void validate_dims(const gpdhg_lp_desc* d) {
  if (!d) throw Error(GPDHG_ERR_INVALID_ARGUMENT, "descriptor is NULL");
  if (d->num_variables <= 0) throw Error(GPDHG_ERR_INVALID_PROBLEM, "num_variables must be positive");
  if (d->num_constraints < 0) throw Error(GPDHG_ERR_INVALID_PROBLEM, "num_constraints must be >= 0");
  if (d->num_equalities < 0 || d->num_equalities > d->num_constraints)
    throw Error(GPDHG_ERR_INVALID_PROBLEM, "num_equalities out of [0, num_constraints]");
  if (!d->variable_lower_bound || !d->variable_upper_bound || !d->objective_vector ||
      (d->num_constraints > 0 && !d->right_hand_side))
    throw Error(GPDHG_ERR_INVALID_ARGUMENT, "required array pointer is NULL");
}

void validate_vectors(const gpdhg_lp_desc* d, bool threads) {
  const int32_t m = d->num_constraints, n = d->num_variables;
  const double *l = d->variable_lower_bound, *u = d->variable_upper_bound, *c = d->objective_vector;
  const double *ol = d->original_variable_lower_bound, *ou = d->original_variable_upper_bound;
  const double *oc = d->original_objective_vector, *var = d->variable_rescaling;
  const double *b = d->right_hand_side, *ob = d->original_right_hand_side, *con = d->constraint_rescaling;
  const bool obounds = ol && ou;
  auto bad_bounds = [](const double* lo, const double* hi, int64_t q) {
    return lo[q] == INFINITY || hi[q] == -INFINITY || std::isnan(lo[q]) || std::isnan(hi[q]);
  };
  auto not_pos = [](const double* v, int64_t q) { return !(v[q] > 0.0) || !std::isfinite(v[q]); };
  // every check of each side in one pass; failures are reported in the serial order below
  const std::array<int64_t, 5> fn = first_bad_each<5>(n, [&](int64_t q, int k) {
    switch (k) {
      case 0: return bad_bounds(l, u, q);
      case 1: return !std::isfinite(c[q]);
      case 2: return obounds && bad_bounds(ol, ou, q);
      case 3: return oc && !std::isfinite(oc[q]);
      default: return var && not_pos(var, q);
    }
  }, threads);
  const std::array<int64_t, 3> fm = first_bad_each<3>(m, [&](int64_t q, int k) {
    switch (k) {
      case 0: return !std::isfinite(b[q]);
      case 1: return ob && !std::isfinite(ob[q]);
      default: return con && not_pos(con, q);
    }
  }, threads);
  auto bounds_error = [](const double* lo, const double* hi, int64_t j) {
    if (lo[j] == INFINITY) throw Error(GPDHG_ERR_INVALID_PROBLEM, "variable_lower_bound contains +Inf");
    if (hi[j] == -INFINITY) throw Error(GPDHG_ERR_INVALID_PROBLEM, "variable_upper_bound contains -Inf");
    throw Error(GPDHG_ERR_INVALID_PROBLEM, "NaN found in variable bounds");
  };
  if (fn[0] >= 0) bounds_error(l, u, fn[0]);
  if (fn[1] >= 0) throw Error(GPDHG_ERR_INVALID_PROBLEM, "NaN or Inf found in objective vector");
  if (fm[0] >= 0) throw Error(GPDHG_ERR_INVALID_PROBLEM, "NaN or Inf found in right hand side");
  if (!std::isfinite(d->objective_constant)) throw Error(GPDHG_ERR_INVALID_PROBLEM, "objective constant not finite");
  if (fn[2] >= 0) bounds_error(ol, ou, fn[2]);
  if (fn[3] >= 0) throw Error(GPDHG_ERR_INVALID_PROBLEM, "NaN or Inf found in original objective vector");
  if (fm[1] >= 0) throw Error(GPDHG_ERR_INVALID_PROBLEM, "NaN or Inf found in original right hand side");
  if (fm[2] >= 0) throw Error(GPDHG_ERR_INVALID_PROBLEM, "constraint_rescaling must be positive and finite");
  if (fn[4] >= 0) throw Error(GPDHG_ERR_INVALID_PROBLEM, "variable_rescaling must be positive and finite");
}

}  // namespace

// validate (src/preprocess.jl:8-74) for the LP descriptor, plus structural CSR checks
// the reference gets from SparseMatrixCSC's invariants.
void validate_lp_desc(const gpdhg_lp_desc* d, bool threads) {
  validate_dims(d);
  if (!d->row_ptr) throw Error(GPDHG_ERR_INVALID_ARGUMENT, "required array pointer is NULL");
  const int32_t m = d->num_constraints, n = d->num_variables;
  if (d->row_ptr[0] != 0) throw Error(GPDHG_ERR_INVALID_PROBLEM, "row_ptr[0] must be 0");
  if (first_bad(m, [&](int64_t i) { return d->row_ptr[i + 1] < d->row_ptr[i]; }, threads) >= 0)
    throw Error(GPDHG_ERR_INVALID_PROBLEM, "row_ptr is not monotone");
  const int64_t nnz = d->row_ptr[m];
  if (nnz != d->nnz) throw Error(GPDHG_ERR_INVALID_PROBLEM, "nnz does not match row_ptr[m]");
  if (nnz > 0 && (!d->col_idx || !d->values)) throw Error(GPDHG_ERR_INVALID_ARGUMENT, "col_idx/values NULL");
  {
    auto bad_col = [&](int64_t k) { return d->col_idx[k] < 0 || d->col_idx[k] >= n; };
    const int64_t k = first_bad(nnz, [&](int64_t q) { return bad_col(q) || !std::isfinite(d->values[q]); }, threads);
    if (k >= 0) {
      if (bad_col(k)) throw Error(GPDHG_ERR_INVALID_PROBLEM, "column index out of range");
      throw Error(GPDHG_ERR_INVALID_PROBLEM, "NaN or Inf found in constraint matrix");
    }
  }
  validate_vectors(d, threads);
}

namespace {

// The part of problem creation after validation: build(s) uploads one of the two CSR copies
// and builds the other on the device; meanwhile a helper thread forms the host scalars
// (serial sums) from the matrix values (the first num_values of them; any others have
// magnitude at most amax_floor) and the vectors.
template <class Build>
void init_with(gpdhg_problem* p, const gpdhg_lp_desc* d, const double* values, int64_t num_values,
               double amax_floor, Build build) {
  const int32_t m = d->num_constraints, n = d->num_variables;
  p->n = n;
  p->m = m;
  p->neq = d->num_equalities;
  p->nnz = d->nnz;
  p->obj_const = d->objective_constant;
  CK(cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking));
  cudaStream_t s = p->stream;
  // the scalars: each serial sum on a thread of its own (same order, same bits as one loop);
  // the maximum |a_ij|, exact in any order, in chunks
  const double* c = d->objective_vector;
  const double* oc = d->original_objective_vector ? d->original_objective_vector : c;
  const double* bv = d->right_hand_side;
  const double* ob = d->original_right_hand_side ? d->original_right_hand_side : bv;
  const int ta = (int)std::max<int64_t>(1, std::min<int64_t>(8, num_values >> 20));
  std::vector<double> amax_part(ta, amax_floor);
  std::vector<std::thread> scalars;
  for (int t = 0; t < ta; ++t)
    scalars.emplace_back([&amax_part, values, num_values, ta, t] {
      double a = amax_part[t];
      for (int64_t k = num_values * t / ta; k < num_values * (t + 1) / ta; ++k) a = std::max(a, std::fabs(values[k]));
      amax_part[t] = a;
    });
  scalars.emplace_back([p, c, n] { p->norm2_c_scaled = norm2(c, n); });
  scalars.emplace_back([p, c, oc, n] {
    p->linf_c = norm_inf(oc, n);
    if (oc != c) p->l2_c = norm2(oc, n);
  });
  scalars.emplace_back([p, bv, ob, m] {
    p->norm2_b_scaled = m ? norm2(bv, m) : 0.0;
    p->linf_b = m ? norm_inf(ob, m) : 0.0;
    p->l2_b = m ? norm2(ob, m) : 0.0;
  });
  auto join_scalars = [&] {
    for (auto& x : scalars) x.join();
    p->amax = *std::max_element(amax_part.begin(), amax_part.end());
    if (oc == c) p->l2_c = p->norm2_c_scaled;
  };
  try {
    build(s);
    // the row-block schedules (a host pass over the rows of A and A') on a helper thread
    // while this one uploads the vectors
    std::exception_ptr items_err;
    int device = 0;
    CK(cudaGetDevice(&device));
    std::thread items([&] {
      try {
        CK(cudaSetDevice(device));   // a new host thread starts on device 0
        set_row_items(p->A, s);
        set_row_items(p->At, s);
      } catch (...) {
        items_err = std::current_exception();
      }
    });
    try {
      upload_vec(p->l, d->variable_lower_bound, n, s);
      upload_vec(p->u, d->variable_upper_bound, n, s);
      upload_vec(p->c, d->objective_vector, n, s);
      upload_vec(p->b, d->right_hand_side, m, s);
      upload_vec_or_fill(p->ol, d->original_variable_lower_bound, d->variable_lower_bound, n, s);
      upload_vec_or_fill(p->ou, d->original_variable_upper_bound, d->variable_upper_bound, n, s);
      upload_vec_or_fill(p->oc, d->original_objective_vector, d->objective_vector, n, s);
      upload_vec_or_fill(p->ob, d->original_right_hand_side, d->right_hand_side, m, s);
      upload_vec_or_ones(p->con, d->constraint_rescaling, m, s);
      upload_vec_or_ones(p->var, d->variable_rescaling, n, s);
    } catch (...) {
      items.join();
      throw;
    }
    items.join();
    if (items_err) std::rethrow_exception(items_err);
  } catch (...) {
    join_scalars();
    throw;
  }
  join_scalars();
  CK(cudaStreamSynchronize(s));
}

// dst[k] = (int32_t)(src[k] - base) on host threads
void narrow_indices(const int64_t* src, int64_t len, int64_t base, std::vector<int32_t>& dst) {
  dst.resize((size_t)len);
  const int T = (int)std::max<int64_t>(1, std::min<int64_t>(std::min(16u, std::max(1u, std::thread::hardware_concurrency())), len / 65536));
  std::vector<std::thread> th;
  for (int t = 0; t < T; ++t)
    th.emplace_back([&, t] {
      for (int64_t k = len * t / T; k < len * (t + 1) / T; ++k) dst[(size_t)k] = (int32_t)(src[k] - base);
    });
  for (auto& x : th) x.join();
}

}  // namespace

void problem_init(gpdhg_problem* p, const gpdhg_lp_desc* d) {
  PhaseTrace tr;
  validate_lp_desc(d, true);
  tr.mark("validate");
  init_with(p, d, d->values, d->nnz, 0.0, [&](cudaStream_t s) {
    upload_csr(p->A, d->num_constraints, d->num_variables, d->row_ptr, d->col_idx, d->values, s);
    tr.mark("upload A");
    transpose_on_device(p->A, p->At, s);
    tr.mark("transpose");
  });
  tr.mark("vectors, schedules, scalars");
  apply_column_order(p);
  tr.mark("column order");
}

namespace {

// Structure of a CSC matrix with int64 indices from index_base (Julia's SparseMatrixCSC
// invariants): col_ptr monotone from base, nnz = col_ptr[n] - base, row indices in range,
// finite values.
void validate_csc(int32_t n, int32_t m, int64_t nnz_declared, const int64_t* col_ptr, const int64_t* row_val,
                  const double* nz_val, int32_t base) {
  if (base != 0 && base != 1) throw Error(GPDHG_ERR_INVALID_ARGUMENT, "index_base must be 0 or 1");
  if (!col_ptr) throw Error(GPDHG_ERR_INVALID_ARGUMENT, "col_ptr is NULL");
  if (col_ptr[0] != base) throw Error(GPDHG_ERR_INVALID_PROBLEM, "col_ptr[0] must be index_base");
  if (first_bad(n, [&](int64_t j) { return col_ptr[j + 1] < col_ptr[j]; }, true) >= 0)
    throw Error(GPDHG_ERR_INVALID_PROBLEM, "col_ptr is not monotone");
  const int64_t nnz = col_ptr[n] - base;
  if (nnz != nnz_declared) throw Error(GPDHG_ERR_INVALID_PROBLEM, "nnz does not match col_ptr[n] - index_base");
  if (nnz >= (1LL << 31)) throw Error(GPDHG_ERR_INVALID_PROBLEM, "more than 2^31 - 1 nonzeros");
  if (nnz > 0 && (!row_val || !nz_val)) throw Error(GPDHG_ERR_INVALID_ARGUMENT, "row_val/nz_val NULL");
  auto bad_row = [&](int64_t k) { return row_val[k] < base || row_val[k] >= (int64_t)m + base; };
  const int64_t k = first_bad(nnz, [&](int64_t q) { return bad_row(q) || !std::isfinite(nz_val[q]); }, true);
  if (k >= 0) {
    if (bad_row(k)) throw Error(GPDHG_ERR_INVALID_PROBLEM, "row index out of range");
    throw Error(GPDHG_ERR_INVALID_PROBLEM, "NaN or Inf found in constraint matrix");
  }
}

// val[k] = -val[k] where the entry's row is flagged (the reference's `nzval[idx] *= -1` for
// "<=" rows, src/quadratic_programming_io.jl:52-56; an exact sign flip either way).
__global__ void negate_rows_kernel(long long nnz, const int32_t* __restrict__ row, const uint8_t* __restrict__ flip,
                                   double* __restrict__ val) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < nnz && flip[row[k]]) val[k] = -val[k];
}

}  // namespace

void problem_init_csc(gpdhg_problem* p, const gpdhg_lp_desc* d, const int64_t* col_ptr, const int64_t* row_val,
                      const double* nz_val, int32_t base) {
  validate_dims(d);
  if (d->row_ptr || d->col_idx || d->values)
    throw Error(GPDHG_ERR_INVALID_ARGUMENT, "a CSC descriptor carries no row_ptr, col_idx or values");
  const int32_t m = d->num_constraints, n = d->num_variables;
  validate_csc(n, m, d->nnz, col_ptr, row_val, nz_val, base);
  const int64_t nnz = d->nnz;
  validate_vectors(d, true);
  init_with(p, d, nz_val, nnz, 0.0, [&](cudaStream_t s) {
    // CSC(A) read as CSR(A'): its pointers become A's row pointer after the device transpose
    std::vector<int32_t> rp, ri;
    narrow_indices(col_ptr, (int64_t)n + 1, base, rp);
    narrow_indices(row_val, nnz, base, ri);
    upload_csr(p->At, n, m, rp.data(), ri.data(), nz_val, s);
    transpose_on_device(p->At, p->A, s);
  });
  apply_column_order(p);
}

void problem_init_two_sided(gpdhg_problem* p, const gpdhg_two_sided_desc* t, const int64_t* col_ptr,
                            const int64_t* row_val, const double* nz_val, int32_t base) {
  if (!t) throw Error(GPDHG_ERR_INVALID_ARGUMENT, "descriptor is NULL");
  const int32_t n = t->num_variables, m = t->num_constraints;
  if (n <= 0) throw Error(GPDHG_ERR_INVALID_PROBLEM, "num_variables must be positive");
  if (m < 0) throw Error(GPDHG_ERR_INVALID_PROBLEM, "num_constraints must be >= 0");
  if (!t->variable_lower_bound || !t->variable_upper_bound || !t->objective_vector ||
      (m > 0 && (!t->constraint_lower_bound || !t->constraint_upper_bound)))
    throw Error(GPDHG_ERR_INVALID_ARGUMENT, "required array pointer is NULL");
  validate_csc(n, m, t->nnz, col_ptr, row_val, nz_val, base);
  const int64_t nnz = t->nnz;
  const double* lc = t->constraint_lower_bound;
  const double* uc = t->constraint_upper_bound;
  for (int32_t i = 0; i < m; ++i)
    if (std::isnan(lc[i]) || std::isnan(uc[i])) throw Error(GPDHG_ERR_INVALID_PROBLEM, "NaN found in constraint bounds");
  // two_sided_rows_to_slacks (:85-121): rows with finite, unequal bounds get a slack column
  // (-1 in that row) with the row's bounds, and become "= 0" rows
  std::vector<int32_t> slack_row;
  for (int32_t i = 0; i < m; ++i)
    if (std::isfinite(lc[i]) && std::isfinite(uc[i]) && lc[i] != uc[i]) slack_row.push_back(i);
  const int32_t k = (int32_t)slack_row.size();
  if ((int64_t)n + k > INT32_MAX) throw Error(GPDHG_ERR_INVALID_PROBLEM, "too many variables after adding slacks");
  if (nnz + k >= (1LL << 31)) throw Error(GPDHG_ERR_INVALID_PROBLEM, "more than 2^31 - 1 nonzeros");
  std::vector<double> lo(lc, lc + m), hi(uc, uc + m);
  for (int32_t r : slack_row) lo[r] = hi[r] = 0.0;
  // transform_to_standard_form (:33-76): equality rows first, ">=" rows keep their sign,
  // "<=" rows are negated; each block keeps the caller's row order
  std::vector<uint8_t> eq(m), leq(m);
  std::vector<int32_t> new_row_to_old;
  new_row_to_old.reserve(m);
  for (int32_t i = 0; i < m; ++i) {
    eq[i] = lo[i] == hi[i];
    const bool geq = !eq[i] && std::isfinite(lo[i]);
    leq[i] = !eq[i] && std::isfinite(hi[i]);
    if (!eq[i] && !geq && !leq[i])
      throw Error(GPDHG_ERR_INVALID_PROBLEM, "Not all constraints have finite bounds on at least one side.");
    if (eq[i]) new_row_to_old.push_back(i);
  }
  const int32_t neq = (int32_t)new_row_to_old.size();
  for (int32_t i = 0; i < m; ++i)
    if (!eq[i]) new_row_to_old.push_back(i);
  std::vector<int32_t> old_to_new(m);
  bool identity = true;
  for (int32_t r = 0; r < m; ++r) {
    old_to_new[new_row_to_old[r]] = r;
    identity = identity && new_row_to_old[r] == r;
  }
  std::vector<double> rhs(m);
  std::vector<uint8_t> flip_new(std::max(m, 1), 0);
  for (int32_t r = 0; r < m; ++r) {
    const int32_t i = new_row_to_old[r];
    rhs[r] = leq[i] ? -hi[i] : lo[i];
    flip_new[r] = leq[i];
  }
  const int32_t ns = n + k;
  std::vector<double> l(t->variable_lower_bound, t->variable_lower_bound + n);
  std::vector<double> u(t->variable_upper_bound, t->variable_upper_bound + n);
  std::vector<double> c(t->objective_vector, t->objective_vector + n);
  for (int32_t r : slack_row) {
    l.push_back(lc[r]);
    u.push_back(uc[r]);
    c.push_back(0.0);
  }
  gpdhg_lp_desc d{};
  d.num_variables = ns;
  d.num_constraints = m;
  d.num_equalities = neq;
  d.nnz = nnz + k;
  d.variable_lower_bound = l.data();
  d.variable_upper_bound = u.data();
  d.objective_vector = c.data();
  d.right_hand_side = rhs.data();
  d.objective_constant = t->objective_offset;
  validate_vectors(&d, true);
  p->new_row_to_old = new_row_to_old;
  p->num_slacks = k;
  init_with(p, &d, nz_val, nnz, k ? 1.0 : 0.0, [&](cudaStream_t s) {
    // CSC([A S]) is CSR([A S]'): the narrowed row indices, renumbered on host threads when
    // the rows move; the slack columns hold one -1 each
    std::vector<int32_t> rp, ri;
    narrow_indices(col_ptr, (int64_t)n + 1, base, rp);
    narrow_indices(row_val, nnz, base, ri);
    rp.resize((size_t)ns + 1);
    ri.resize((size_t)(nnz + k));
    for (int32_t j = 0; j < k; ++j) {
      rp[(size_t)n + 1 + j] = (int32_t)(nnz + j + 1);
      ri[(size_t)(nnz + j)] = slack_row[j];
    }
    if (!identity) {
      const int T = (int)std::max<int64_t>(1, std::min<int64_t>(16, (nnz + k) / 65536));
      std::vector<std::thread> th;
      for (int q = 0; q < T; ++q)
        th.emplace_back([&, q] {
          for (int64_t e = (nnz + k) * q / T; e < (nnz + k) * (q + 1) / T; ++e) ri[(size_t)e] = old_to_new[ri[(size_t)e]];
        });
      for (auto& x : th) x.join();
    }
    DeviceMatrix& At = p->At;
    At.nrows = ns;
    At.ncols = m;
    At.nnz = nnz + k;
    At.host_rp = rp;
    At.row_ptr.alloc((size_t)ns + 1);
    At.col.alloc(std::max<long long>(At.nnz, 1));
    At.val64.alloc(std::max<long long>(At.nnz, 1));
    DBuf<uint8_t> flip((size_t)flip_new.size());
    CK(cudaMemcpyAsync(At.row_ptr.get(), rp.data(), sizeof(int32_t) * ((size_t)ns + 1), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(flip.get(), flip_new.data(), flip_new.size(), cudaMemcpyHostToDevice, s));
    std::vector<double> minus_one((size_t)std::max(k, 1), -1.0);
    if (At.nnz) CK(cudaMemcpyAsync(At.col.get(), ri.data(), sizeof(int32_t) * At.nnz, cudaMemcpyHostToDevice, s));
    if (nnz) {
      CK(cudaMemcpyAsync(At.val64.get(), nz_val, sizeof(double) * nnz, cudaMemcpyHostToDevice, s));
      negate_rows_kernel<<<(unsigned)((nnz + 255) / 256), 256, 0, s>>>(nnz, At.col.get(), flip.get(), At.val64.get());
      CK_LAUNCH();
    }
    if (k) CK(cudaMemcpyAsync(At.val64.get() + nnz, minus_one.data(), sizeof(double) * k, cudaMemcpyHostToDevice, s));
    // A is sorted out of A' as for any CSC; after a row renumbering, A' is rebuilt from A so
    // that its rows list their entries in increasing row again, as row_permute_in_place
    // leaves the columns of the CSC. The transposes synchronise the stream before returning,
    // so the host vectors above outlive the copies that read them.
    transpose_on_device(At, p->A, s);
    if (!identity) transpose_on_device(p->A, At, s);
  });
  apply_column_order(p);
}

bool choose_column_order(const std::vector<int32_t>& degree, std::vector<int32_t>& perm) {
  const int32_t n = (int32_t)degree.size();
  perm.clear();
  if (n < kColumnOrderMinColumns) return false;
  int32_t dmax = 0;
  long long total = 0;
  for (int32_t d : degree) {
    dmax = std::max(dmax, d);
    total += d;
  }
  if (total == 0) return false;
  // counting sort by decreasing degree, stable: bucket starts from the largest degree down
  std::vector<int64_t> start((size_t)dmax + 2, 0);
  for (int32_t d : degree) ++start[(size_t)(dmax - d) + 1];
  for (size_t q = 1; q < start.size(); ++q) start[q] += start[q - 1];
  std::vector<int32_t> order((size_t)n);
  for (int32_t j = 0; j < n; ++j) order[(size_t)start[(size_t)(dmax - degree[j])]++] = j;
  const int32_t top = std::max<int32_t>(1, (n + 99) / 100);
  long long top_nnz = 0;
  for (int32_t k = 0; k < top; ++k) top_nnz += degree[order[k]];
  if ((double)top_nnz < kColumnOrderTopShare * (double)total) return false;
  perm.swap(order);
  return true;
}

void to_caller_columns(const std::vector<int32_t>& perm, double* v) {
  if (perm.empty() || !v) return;
  std::vector<double> t(v, v + perm.size());
  for (size_t k = 0; k < perm.size(); ++k) v[perm[k]] = t[k];
}

void to_handle_columns(const std::vector<int32_t>& perm, const double* in, double* out) {
  for (size_t k = 0; k < perm.size(); ++k) out[k] = in[perm[k]];
}

namespace {
__global__ void relabel_kernel(long long nnz, const int32_t* __restrict__ inv, int32_t* col) {
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < nnz) col[k] = inv[col[k]];
}
__global__ void gather_kernel(int32_t n, const int32_t* __restrict__ perm, const double* __restrict__ src,
                              double* __restrict__ dst) {
  const int32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) dst[k] = src[perm[k]];
}
}  // namespace

void apply_column_order(gpdhg_problem* p) {
  PhaseTrace tr;
  const int32_t n = p->n;
  const long long total = p->At.host_rp[(size_t)n];
  if (n < kColumnOrderMinColumns || total == 0) return;
  // the rule needs the top 1% of columns to hold kColumnOrderTopShare of the nonzeros, which
  // the longest column alone decides against when top x its length falls short
  int32_t dmax = 0;
  for (int32_t j = 0; j < n; ++j) dmax = std::max(dmax, p->At.host_rp[(size_t)j + 1] - p->At.host_rp[(size_t)j]);
  const int32_t top = std::max<int32_t>(1, (n + 99) / 100);
  if ((double)dmax * (double)top < kColumnOrderTopShare * (double)total) return;
  cudaStream_t s = p->stream;
  // the order of choose_column_order (decreasing degree, ties by index), sorted on the device
  std::vector<int32_t> perm;
  order_rows_by_length(p->At, perm, s);
  long long top_nnz = 0;
  for (int32_t k = 0; k < top; ++k)
    top_nnz += p->At.host_rp[(size_t)perm[(size_t)k] + 1] - p->At.host_rp[(size_t)perm[(size_t)k]];
  if ((double)top_nnz < kColumnOrderTopShare * (double)total) return;
  tr.mark("  order: choose");
  std::vector<int32_t> inv((size_t)n);
  for (int32_t k = 0; k < n; ++k) inv[(size_t)perm[(size_t)k]] = k;
  DBuf<int32_t> dperm((size_t)n), dinv((size_t)n);
  CK(cudaMemcpyAsync(dperm.get(), perm.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(dinv.get(), inv.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, s));
  if (p->A.nnz > 0) {
    relabel_kernel<<<(unsigned)((p->A.nnz + 255) / 256), 256, 0, s>>>(p->A.nnz, dinv.get(), p->A.col.get());
    CK_LAUNCH();
  }
  // the permuted n-vectors: all gathers in flight together; the old vectors are freed after
  // the synchronisation below
  std::vector<DBuf<double>> old_vectors;
  for (DBuf<double>* v : {&p->l, &p->u, &p->c, &p->ol, &p->ou, &p->oc, &p->var}) {
    DBuf<double> t((size_t)n);
    gather_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, dperm.get(), v->get(), t.get());
    CK_LAUNCH();
    std::swap(*v, t);
    old_vectors.push_back(std::move(t));
  }
  // A' of the renumbered A (its rows are the columns in the new order, each listing its
  // entries in increasing row as before), then A again from A', so that every row of A lists
  // its entries in increasing new column (the layout a caller's own sorted CSR of the
  // renumbered LP gives, ties in their previous order)
  tr.mark("  order: relabel, gathers");
  transpose_on_device(p->A, p->At, s);
  transpose_on_device(p->At, p->A, s);
  tr.mark("  order: two transposes");
  set_row_items(p->At, s);
  tr.mark("  order: row items");
  // the 2-norms over the columns are summed in the new order (an LP whose caller already
  // sorted its columns gets the same scalars, bit for bit), from the permuted device vectors
  // (a copy back is faster than gathering the caller's arrays on the host)
  std::vector<double> hc((size_t)n), hoc((size_t)n);
  CK(cudaMemcpyAsync(hc.data(), p->c.get(), sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(hoc.data(), p->oc.get(), sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  p->norm2_c_scaled = norm2(hc.data(), n);
  p->l2_c = norm2(hoc.data(), n);
  p->col_perm.swap(perm);
  tr.mark("  order: norms");
}

void ensure_fp32_values(gpdhg_problem* p) {
  auto conv = [&](DeviceMatrix& dm) {
    if (dm.val32.get()) return;
    dm.val32.alloc(std::max<long long>(dm.nnz, 1));
    if (dm.nnz) launch_convert_d2f(dm.val64.get(), dm.val32.get(), dm.nnz, p->stream);
  };
  conv(p->A);
  conv(p->At);
}

}  // namespace gpdhg
