// batch.cu — batched solve of many independent LPs (gpdhg_batch_*).
//
// All instances are packed into one block-diagonal CSR of A and of A' (each instance's
// rows and columns shifted by its offsets), with one row-block schedule per instance, so
// one launch of each step kernel advances every unfinished instance by one attempt.
// Each instance keeps its own StepState (step size, primal weight, averaging weights,
// accept/reject counters) on the device, its own restart memory and termination state on
// the host, and its own evaluation cadence. The step loop is a CUDA graph of K
// [primal, dual] launches; after each graph the host looks at which instances reached
// their next evaluation point, evaluates exactly those with segmented FP64 reductions,
// retires the ones that terminated and re-arms the rest.
#include <algorithm>
#include <atomic>
#include <exception>
#include <thread>
#include <chrono>
#include <cmath>
#include <cstring>
#include <limits>
#include <vector>

#include "batch.h"
#include "batch_kernels.cuh"
#include "spmv.cuh"
#include "tiles.h"
#include "host_logic.h"

namespace gpdhg {

namespace {

using Clock = std::chrono::steady_clock;
constexpr int kBatchLevels = 6;   // graphs of 1, 2, ..., 32 [primal, dual] pairs

template <class T>
void alloc_all(std::initializer_list<DBuf<T>*> v, size_t n) {
  for (auto* b : v) b->alloc(std::max<size_t>(n, 1));
}

}  // namespace

void build_seg_items(const std::vector<int32_t>& off, std::vector<SegItem>& items, std::vector<int32_t>& begin) {
  const int count = (int)off.size() - 1;
  items.clear();
  begin.assign(count + 1, 0);
  for (int k = 0; k < count; ++k) {
    begin[k] = (int32_t)items.size();
    for (int32_t s = off[k]; s < off[k + 1]; s += kSegLen) items.push_back({s, std::min(off[k + 1], s + kSegLen), k});
  }
  begin[count] = (int32_t)items.size();
  if (items.empty()) items.push_back({0, 0, 0});
}

// Runs f(k) for k in [0, count) on host threads, instances handed out in order from a shared
// counter; each call writes only instance k's own outputs. An exception thrown by f(k) is
// rethrown after all threads joined: that of the lowest such k, as a serial loop would.
template <class F>
void for_each_instance(int count, F f) {
  const int T = std::max(1, std::min<int>(count, (int)std::min(16u, std::max(1u, std::thread::hardware_concurrency()))));
  if (T == 1) {
    for (int k = 0; k < count; ++k) f(k);
    return;
  }
  std::vector<std::exception_ptr> err(count);
  std::atomic<int> next{0};
  std::vector<std::thread> th;
  th.reserve(T);
  for (int t = 0; t < T; ++t)
    th.emplace_back([&] {
      for (int k = next++; k < count; k = next++) {
        try {
          f(k);
        } catch (...) {
          err[k] = std::current_exception();
        }
      }
    });
  for (auto& x : th) x.join();
  for (int k = 0; k < count; ++k)
    if (err[k]) std::rethrow_exception(err[k]);
}

// Allocator of host staging arrays that the instances' threads fill completely: a new element
// is left as it is (default-initialised) instead of zeroed, which for the packed matrix and
// vectors of a large batch spares one single-threaded pass over a few GB.
template <class T>
struct NoInitAlloc : std::allocator<T> {
  using value_type = T;
  NoInitAlloc() = default;
  template <class U>
  NoInitAlloc(const NoInitAlloc<U>&) noexcept {}
  template <class U>
  struct rebind {
    using other = NoInitAlloc<U>;
  };
  template <class U>
  void construct(U* p) noexcept {
    ::new ((void*)p) U;
  }
  template <class U, class... A>
  void construct(U* p, A&&... a) {
    ::new ((void*)p) U(std::forward<A>(a)...);
  }
};
template <class T>
using HostArray = std::vector<T, NoInitAlloc<T>>;

void batch_init(gpdhg_batch* B, int32_t count, const gpdhg_lp_desc* descs) {
  if (count <= 0 || !descs) throw Error(GPDHG_ERR_INVALID_ARGUMENT, "batch needs count > 0 and descriptors");
  PhaseTrace tr;
  B->count = count;
  B->row_off.assign(count + 1, 0);
  B->col_off.assign(count + 1, 0);
  B->info.resize(count);
  B->amax.assign(count, 0.0);
  B->norm_b.assign(count, 0.0);
  B->norm_c.assign(count, 0.0);
  B->neq.resize(count);
  B->col_perm.assign(count, {});
  // every descriptor validated (on host threads, one instance each); the error of the first
  // invalid instance is the one reported, as a serial loop would
  for_each_instance(count, [&](int k) { validate_lp_desc(&descs[k], false); });
  tr.mark("batch: validate");
  long long nnz_total = 0;
  std::vector<long long> nnz_off(count + 1, 0);
  for (int k = 0; k < count; ++k) {
    B->row_off[k + 1] = B->row_off[k] + descs[k].num_constraints;
    B->col_off[k + 1] = B->col_off[k] + descs[k].num_variables;
    nnz_total += descs[k].nnz;
    nnz_off[k + 1] = nnz_total;
    B->neq[k] = descs[k].num_equalities;
  }
  if (nnz_total >= (1LL << 31) || (long long)B->row_off[count] >= (1LL << 31) ||
      (long long)B->col_off[count] >= (1LL << 31))
    throw Error(GPDHG_ERR_INVALID_ARGUMENT, "packed batch exceeds int32 indexing");
  const int32_t M = B->row_off[count], N = B->col_off[count];
  B->M = M;
  B->N = N;
  CK(cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking));
  cudaStream_t s = B->stream;

  // pack A (block diagonal), the vectors, the per-instance schedules and host scalars: each
  // instance fills its own slices (on host threads); A' is built from A on the GPU
  std::vector<int32_t> arp(M + 1, 0);
  HostArray<int32_t> acol(nnz_total);
  HostArray<double> aval(nnz_total);
  HostArray<double> l(N), u(N), c(N), b(M), ol(N), ou(N), oc(N), ob(M), con(M), var(N);
  std::vector<uint8_t> ineq(std::max(M, 1), 0);
  std::vector<std::vector<RowItem>> a_items_of(count);
  for_each_instance(count, [&](int k) {
    const gpdhg_lp_desc& d = descs[k];
    const int32_t m = d.num_constraints, n = d.num_variables, ro = B->row_off[k], co = B->col_off[k];
    const long long z0 = nnz_off[k];
    for (int32_t i = 0; i < m; ++i) {
      arp[ro + i + 1] = (int32_t)(z0 + d.row_ptr[i + 1]);
      ineq[ro + i] = i >= d.num_equalities;
    }
    // the instance's column order, chosen from its column degrees as for a lone problem
    std::vector<int32_t> degree((size_t)n, 0);
    for (long long e = 0; e < d.nnz; ++e) ++degree[(size_t)d.col_idx[e]];
    std::vector<int32_t>& perm = B->col_perm[k];
    std::vector<int32_t> inv;
    if (choose_column_order(degree, perm)) {
      inv.resize((size_t)n);
      for (int32_t q = 0; q < n; ++q) inv[(size_t)perm[(size_t)q]] = q;
    }
    if (inv.empty()) {
      for (long long e = 0; e < d.nnz; ++e) {
        acol[z0 + e] = d.col_idx[e] + co;
        aval[z0 + e] = d.values[e];
      }
    } else {
      // renumbered columns, each row re-sorted by its new column (ties in their previous
      // order), as apply_column_order leaves a lone problem
      std::vector<std::pair<int32_t, double>> row;
      for (int32_t i = 0; i < m; ++i) {
        row.clear();
        for (int32_t e = d.row_ptr[i]; e < d.row_ptr[i + 1]; ++e) row.emplace_back(inv[(size_t)d.col_idx[e]], d.values[e]);
        std::stable_sort(row.begin(), row.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
        for (size_t q = 0; q < row.size(); ++q) {
          acol[z0 + d.row_ptr[i] + (long long)q] = row[q].first + co;
          aval[z0 + d.row_ptr[i] + (long long)q] = row[q].second;
        }
      }
    }
    for (RowItem it : build_row_items(d.row_ptr, m))
      a_items_of[k].push_back({it.row_begin + ro, it.row_end + ro, it.group, it.mode, it.nnz_begin + (int32_t)z0, it.nnz_count});
    if (m == 0) a_items_of[k].push_back({ro, ro, 1, kItemStaged, (int32_t)z0, 0});  // every instance owns a dual CTA: its decision runs there
    auto put = [](HostArray<double>& dst, int32_t off, const double* src, const double* fb, int len) {
      const double* p = src ? src : fb;
      if (p) std::copy(p, p + len, dst.begin() + off);
      else std::fill(dst.begin() + off, dst.begin() + off + len, 1.0);
    };
    // n-vectors in the instance's column order
    auto put_n = [&](HostArray<double>& dst, const double* src, const double* fb) {
      const double* p = src ? src : fb;
      if (!p) std::fill(dst.begin() + co, dst.begin() + co + n, 1.0);
      else if (perm.empty()) std::copy(p, p + n, dst.begin() + co);
      else to_handle_columns(perm, p, dst.data() + co);
    };
    put_n(l, d.variable_lower_bound, nullptr);
    put_n(u, d.variable_upper_bound, nullptr);
    put_n(c, d.objective_vector, nullptr);
    put(b, ro, d.right_hand_side, nullptr, m);
    put_n(ol, d.original_variable_lower_bound, d.variable_lower_bound);
    put_n(ou, d.original_variable_upper_bound, d.variable_upper_bound);
    put_n(oc, d.original_objective_vector, d.objective_vector);
    put(ob, ro, d.original_right_hand_side, d.right_hand_side, m);
    put(con, ro, d.constraint_rescaling, nullptr, m);
    put_n(var, d.variable_rescaling, nullptr);
    // host scalars (as problem_init)
    double amax = 0.0, nb = 0.0, nc = 0.0;
    for (int64_t e = 0; e < d.nnz; ++e) amax = std::max(amax, std::fabs(d.values[e]));
    for (int32_t i = 0; i < m; ++i) nb += d.right_hand_side[i] * d.right_hand_side[i];
    // column sums in the instance's column order, as apply_column_order has them
    auto col = [&](int32_t j) { return perm.empty() ? j : perm[(size_t)j]; };
    for (int32_t j = 0; j < n; ++j) nc += d.objective_vector[col(j)] * d.objective_vector[col(j)];
    B->amax[k] = amax;
    B->norm_b[k] = std::sqrt(nb);
    B->norm_c[k] = std::sqrt(nc);
    const double* occ = d.original_objective_vector ? d.original_objective_vector : d.objective_vector;
    const double* obb = d.original_right_hand_side ? d.original_right_hand_side : d.right_hand_side;
    InstanceInfo& qi = B->info[k];
    qi.obj_const = d.objective_constant;
    double s2 = 0.0, si = 0.0;
    for (int32_t j = 0; j < n; ++j) { s2 += occ[col(j)] * occ[col(j)]; si = std::max(si, std::fabs(occ[col(j)])); }
    qi.l2_c = std::sqrt(s2); qi.linf_c = si;
    s2 = 0.0; si = 0.0;
    for (int32_t i = 0; i < m; ++i) { s2 += obb[i] * obb[i]; si = std::max(si, std::fabs(obb[i])); }
    qi.l2_b = std::sqrt(s2); qi.linf_b = si;
  });
  tr.mark("batch: pack");
  std::vector<RowItem> a_items, t_items;
  for (auto& v : a_items_of) a_items.insert(a_items.end(), v.begin(), v.end());

  auto up_i = [&](DBuf<int32_t>& dst, const auto& v) {
    dst.alloc(std::max<size_t>(v.size(), 1));
    if (!v.empty()) CK(cudaMemcpyAsync(dst.get(), v.data(), 4 * v.size(), cudaMemcpyHostToDevice, s));
  };
  auto up_d = [&](DBuf<double>& dst, const auto& v) {
    dst.alloc(std::max<size_t>(v.size(), 1));
    if (!v.empty()) CK(cudaMemcpyAsync(dst.get(), v.data(), 8 * v.size(), cudaMemcpyHostToDevice, s));
  };
  auto up_items = [&](DeviceMatrix& dm, int32_t nrows, int32_t ncols, const std::vector<int32_t>& rp,
                      const HostArray<int32_t>& col, const HostArray<double>& val, const std::vector<RowItem>& it) {
    dm.nrows = nrows;
    dm.ncols = ncols;
    dm.nnz = (long long)col.size();
    dm.host_rp = rp;
    up_i(dm.row_ptr, rp);
    up_i(dm.col, col);
    up_d(dm.val64, val);
    dm.num_items = (int32_t)it.size();
    dm.items.alloc(std::max<size_t>(it.size(), 1));
    if (!it.empty()) CK(cudaMemcpyAsync(dm.items.get(), it.data(), sizeof(RowItem) * it.size(), cudaMemcpyHostToDevice, s));
  };
  up_items(B->A, M, N, arp, acol, aval, a_items);
  tr.mark("batch: upload A");
  // A' of the packed A on the GPU: the transpose of a block-diagonal matrix is block diagonal
  // with the blocks' transposes in the same order, each the counting sort's (ingest.cu)
  transpose_on_device(B->A, B->At, s);
  tr.mark("batch: transpose");
  for (int k = 0; k < count; ++k) {
    const int32_t co = B->col_off[k], n = B->col_off[k + 1] - co;
    // the instance's rows of A' from the packed row pointer (absolute nonzero offsets)
    for (RowItem it : build_row_items(B->At.host_rp.data() + co, n))
      t_items.push_back({it.row_begin + co, it.row_end + co, it.group, it.mode, it.nnz_begin, it.nnz_count});
  }
  B->At.num_items = (int32_t)t_items.size();
  B->At.items.alloc(std::max<size_t>(t_items.size(), 1));
  if (!t_items.empty())
    CK(cudaMemcpyAsync(B->At.items.get(), t_items.data(), sizeof(RowItem) * t_items.size(), cudaMemcpyHostToDevice, s));
  up_i(B->row_off_d, B->row_off);
  up_i(B->neq_d, B->neq);
  up_d(B->l, l); up_d(B->u, u); up_d(B->c, c); up_d(B->b, b);
  up_d(B->ol, ol); up_d(B->ou, ou); up_d(B->oc, oc); up_d(B->ob, ob);
  up_d(B->con, con); up_d(B->var, var);
  B->ineq_flag.alloc(ineq.size());
  CK(cudaMemcpyAsync(B->ineq_flag.get(), ineq.data(), ineq.size(), cudaMemcpyHostToDevice, s));
  std::vector<int32_t> col_inst(std::max(N, 1), 0), row_inst(std::max(M, 1), 0);
  for (int k = 0; k < count; ++k) {
    for (int32_t j = B->col_off[k]; j < B->col_off[k + 1]; ++j) col_inst[j] = k;
    for (int32_t i = B->row_off[k]; i < B->row_off[k + 1]; ++i) row_inst[i] = k;
  }
  up_i(B->col_inst, col_inst);
  up_i(B->row_inst, row_inst);
  std::vector<SegItem> sn, sm;
  std::vector<int32_t> bn, bm;
  build_seg_items(B->col_off, sn, bn);
  build_seg_items(B->row_off, sm, bm);
  B->nseg_n = (int)sn.size();
  B->nseg_m = (int)sm.size();
  B->seg_n.alloc(sn.size());
  B->seg_m.alloc(sm.size());
  CK(cudaMemcpyAsync(B->seg_n.get(), sn.data(), sizeof(SegItem) * sn.size(), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(B->seg_m.get(), sm.data(), sizeof(SegItem) * sm.size(), cudaMemcpyHostToDevice, s));
  up_i(B->seg_n_begin, bn);
  up_i(B->seg_m_begin, bm);
  CK(cudaStreamSynchronize(s));
  tr.mark("batch: vectors, schedules");
}

template <class T>
struct BatchWorkspace {
  gpdhg_batch* B;
  int count, N, M;
  DBuf<T> l_own, u_own, c_own, b_own, Aval32, Atval32;
  const T *l, *u, *c, *b;
  DBuf<T> x, dx, kty, sx, ax, agrad, grad, rx, rgrad, aty;
  DBuf<T> y0, y1, kx0, kx1, sy, skx, ay, akx, ry, rkx;
  DBuf<StepState> st_dev;
  PinnedBuf<StepState> st_host;
  DBuf<double> part_p, part_d, red_part, red_out;
  DBuf<double> rvar, rcon;   // 1 / variable and 1 / constraint rescaling (evaluation divisions)
  PinnedBuf<double> red_host;
  TilePlan<T> plan_p, plan_d;   // tiles of the packed A' and A, instance by instance
  DBuf<double> part_p_split, part_d_split;
  // launched CTAs: those of instances not yet retired (rebuilt when their count halves)
  DBuf<int32_t> map_p, map_d;
  int grid_p = 0, grid_d = 0;
  DBuf<uint8_t> flags;             // 4 x count: active, use_current, to_avg, restart
  PinnedBuf<uint8_t> flags_host;
  cudaGraphExec_t graphs[kBatchLevels] = {};
  long long launches = 0;
  DBuf<double> pow_table;
  double pow_r = -1.0, pow_g = -1.0;
  const int direct = sizeof(T) == sizeof(float) ? 1 : 0;
  const double* ensure_pow_table(double r, double g) {
    if (pow_table.get() && r == pow_r && g == pow_g) return pow_table.get();
    std::vector<double> t;
    fill_pow_table(t, r, g);
    pow_table.alloc(t.size());
    CK(cudaMemcpyAsync(pow_table.get(), t.data(), sizeof(double) * t.size(), cudaMemcpyHostToDevice, B->stream));
    CK(cudaStreamSynchronize(B->stream));
    pow_r = r;
    pow_g = g;
    return pow_table.get();
  }

  explicit BatchWorkspace(gpdhg_batch* b_) : B(b_), count(b_->count), N(b_->N), M(b_->M),
                                             st_host(b_->count), red_host((size_t)b_->count * 32),
                                             flags_host(4 * (size_t)b_->count) {
    PhaseTrace tr;
    cudaStream_t s = B->stream;
    if constexpr (sizeof(T) == sizeof(double)) {
      l = (const T*)B->l.get(); u = (const T*)B->u.get(); c = (const T*)B->c.get(); b = (const T*)B->b.get();
    } else {
      l_own.alloc(std::max(N, 1)); u_own.alloc(std::max(N, 1)); c_own.alloc(std::max(N, 1)); b_own.alloc(std::max(M, 1));
      launch_convert_d2f(B->l.get(), l_own.get(), N, s);
      launch_convert_d2f(B->u.get(), u_own.get(), N, s);
      launch_convert_d2f(B->c.get(), c_own.get(), N, s);
      if (M) launch_convert_d2f(B->b.get(), b_own.get(), M, s);
      l = l_own.get(); u = u_own.get(); c = c_own.get(); b = b_own.get();
      if (!B->A.val32.get()) {
        B->A.val32.alloc(std::max<long long>(B->A.nnz, 1));
        B->At.val32.alloc(std::max<long long>(B->At.nnz, 1));
        if (B->A.nnz) {
          launch_convert_d2f(B->A.val64.get(), B->A.val32.get(), B->A.nnz, s);
          launch_convert_d2f(B->At.val64.get(), B->At.val32.get(), B->At.nnz, s);
        }
      }
    }
    alloc_all<T>({&x, &dx, &kty, &sx, &ax, &agrad, &grad, &rx, &rgrad, &aty}, N);
    alloc_all<T>({&y0, &y1, &kx0, &kx1, &sy, &skx, &ay, &akx, &ry, &rkx}, M);
    rvar.alloc(std::max(N, 1));
    rcon.alloc(std::max(M, 1));
    launch_reciprocal(B->var.get(), rvar.get(), N, s);
    launch_reciprocal(B->con.get(), rcon.get(), M, s);
    st_dev.alloc(count);
    CK(cudaMemsetAsync(st_dev.get(), 0, sizeof(StepState) * count, s));
    tr.mark("batch ws: vectors");
    build_tile_plan(plan_p, B->At, B->col_off, {}, kPrimalCtasPerSm<T>, kTileSideAt, s);
    tr.mark("batch ws: primal plan");
    std::vector<int32_t> ineq_from(count);
    for (int k = 0; k < count; ++k) ineq_from[k] = B->row_off[k] + B->neq[k];
    build_tile_plan(plan_d, B->A, B->row_off, ineq_from, kDualCtasPerSm, kTileSideA, s);
    tr.mark("batch ws: dual plan");
    part_p.alloc(plan_p.num_ctas);
    part_d.alloc(2 * (size_t)plan_d.num_ctas);
    part_p_split.alloc(std::max(plan_p.num_splits, 1));
    part_d_split.alloc(2 * (size_t)std::max(plan_d.num_splits, 1));
    red_part.alloc((size_t)16 * std::max(B->nseg_n, B->nseg_m));
    red_out.alloc((size_t)count * 32);
    flags.alloc(4 * (size_t)count);
    compact(std::vector<char>(count, 0));
    tr.mark("batch ws: CTA maps, graphs");
  }
  ~BatchWorkspace() {
    for (cudaGraphExec_t g : graphs)
      if (g) cudaGraphExecDestroy(g);
  }
  TileView<T> view_p() const {
    TileView<T> v = plan_p.view();
    v.cta_map = map_p.get();
    return v;
  }
  TileView<T> view_d() const {
    TileView<T> v = plan_d.view();
    v.cta_map = map_d.get();
    return v;
  }
  // Launches only the CTAs of instances that are not retired; re-captures the step graphs.
  std::vector<int32_t> hbeg_p, hbeg_d;  // host copies of the plans' per-instance CTA ranges
  // CTAs the step kernels would launch with the given retirements (primal plan)
  int active_ctas(const std::vector<char>& retired) const {
    int a = 0;
    for (int k = 0; k < count; ++k)
      if (!retired[k]) a += hbeg_p[k + 1] - hbeg_p[k];
    return a;
  }
  void compact(const std::vector<char>& retired) {
    if (hbeg_p.empty()) {
      hbeg_p.resize(count + 1);
      hbeg_d.resize(count + 1);
      CK(cudaMemcpy(hbeg_p.data(), plan_p.inst_cta_begin.get(), sizeof(int32_t) * (count + 1), cudaMemcpyDeviceToHost));
      CK(cudaMemcpy(hbeg_d.data(), plan_d.inst_cta_begin.get(), sizeof(int32_t) * (count + 1), cudaMemcpyDeviceToHost));
    }
    std::vector<int32_t> mp, md;
    auto collect = [&](const std::vector<int32_t>& begin, std::vector<int32_t>& map) {
      for (int k = 0; k < count; ++k)
        if (!retired[k])
          for (int32_t c0 = begin[k]; c0 < begin[k + 1]; ++c0) map.push_back(c0);
    };
    collect(hbeg_p, mp);
    collect(hbeg_d, md);
    if (mp.empty() || md.empty()) return;  // nothing runs any more
    auto up = [&](DBuf<int32_t>& d, const std::vector<int32_t>& v) {
      d.alloc(v.size());
      CK(cudaMemcpy(d.get(), v.data(), sizeof(int32_t) * v.size(), cudaMemcpyHostToDevice));
    };
    up(map_p, mp);
    up(map_d, md);
    grid_p = (int)mp.size();
    grid_d = (int)md.size();
    for (cudaGraphExec_t& g : graphs) {
      if (g) cudaGraphExecDestroy(g);
      g = nullptr;
    }
    for (int lv = 0; lv < kBatchLevels; ++lv) graphs[lv] = capture(1 << lv);
  }
  PrimalArgs<T> pargs(int mode) {
    return PrimalArgs<T>{B->At.view<T>(), view_p(), c, l, u, x.get(), dx.get(), kty.get(), sx.get(),
                         y0.get(), y1.get(), st_dev.get(), part_p.get(), part_p_split.get(), mode, direct};
  }
  DualArgs<T> dargs(int mode) {
    return DualArgs<T>{B->A.view<T>(), view_d(), plan_p.inst_cta_begin.get(), plan_p.inst_split_begin.get(),
                       dx.get(), b, y0.get(), y1.get(), kx0.get(), kx1.get(), sy.get(), skx.get(), st_dev.get(),
                       part_p.get(), part_p_split.get(), part_d.get(), part_d_split.get(), mode, direct};
  }
  void launch_pair(int mode, cudaStream_t s) {
    launch_step(primal_step_kernel<T>, grid_p, s, pargs(mode));
    launch_step(dual_step_kernel<T>, grid_d, s, dargs(mode));
    launches += 2;
  }
  void launch_pair(int mode) { launch_pair(mode, B->stream); }
  cudaGraphExec_t capture(int pairs) {
    cudaStream_t s = B->stream;
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < pairs; ++k) {
      launch_step(primal_step_kernel<T>, grid_p, s, pargs(kStepNormal));
      launch_step(dual_step_kernel<T>, grid_d, s, dargs(kStepNormal));
    }
    cudaMemcpyAsync(st_host.p, st_dev.get(), sizeof(StepState) * count, cudaMemcpyDeviceToHost, s);
    CK(cudaStreamEndCapture(s, &g));
    cudaGraphExec_t ex = nullptr;
    CK(cudaGraphInstantiate(&ex, g, 0));
    cudaGraphDestroy(g);
    return ex;
  }
  void push_state() {
    CK(cudaMemcpyAsync(st_dev.get(), st_host.p, sizeof(StepState) * count, cudaMemcpyHostToDevice, B->stream));
    CK(cudaStreamSynchronize(B->stream));
  }
  void push_flags() {
    CK(cudaMemcpyAsync(flags.get(), flags_host.p, 4 * (size_t)count, cudaMemcpyHostToDevice, B->stream));
    CK(cudaStreamSynchronize(B->stream));
  }
  uint8_t* active() { return flags.get(); }
  uint8_t* use_current() { return flags.get() + count; }
  uint8_t* to_avg() { return flags.get() + 2 * count; }
  uint8_t* restart() { return flags.get() + 3 * count; }
  BatchVecArgs<T> vn(const uint8_t* flag) const { return BatchVecArgs<T>{B->col_inst.get(), flag, st_dev.get(), N}; }
  BatchVecArgs<T> vm(const uint8_t* flag) const { return BatchVecArgs<T>{B->row_inst.get(), flag, st_dev.get(), M}; }
  int grid(int len) const { return std::max(1, std::min(ceil_div(len, kBlock), 4096)); }

  template <int Q, unsigned MAXMASK, class F>
  void seg_reduce(bool n_side, F f, int out_offset) {
    const int nit = n_side ? B->nseg_n : B->nseg_m;
    const SegItem* items = n_side ? B->seg_n.get() : B->seg_m.get();
    const int32_t* beg = n_side ? B->seg_n_begin.get() : B->seg_m_begin.get();
    seg_reduce_kernel<Q, MAXMASK, F><<<nit, kBlock, 0, B->stream>>>(items, active(), f, red_part.get(), nit);
    CK_LAUNCH();
    seg_finalize_kernel<Q, MAXMASK><<<count, kBlock, 0, B->stream>>>(beg, active(), red_part.get(), nit,
                                                                      red_out.get() + out_offset, 32);
    CK_LAUNCH();
    launches += 2;
  }
  void fetch() {
    CK(cudaMemcpyAsync(red_host.p, red_out.get(), sizeof(double) * 32 * count, cudaMemcpyDeviceToHost, B->stream));
    CK(cudaStreamSynchronize(B->stream));
  }
};

template <class T>
static void run_batch(gpdhg_batch* B, BatchWorkspace<T>& W, const gpdhg_params& prm, gpdhg_result* results,
                      double* const* primal_out, double* const* dual_out,
                      const std::function<void(int)>* on_retire) {
  cudaStream_t s = B->stream;
  const int K = B->count;
  const int N = B->N, M = B->M;
  const long long freq = std::max(1, prm.termination_evaluation_frequency);
  const long long it_limit = prm.iteration_limit;
  const long long launches0 = W.launches;
  if (W.grid_p != W.plan_p.num_ctas) W.compact(std::vector<char>(K, 0));  // a new solve: every instance runs
  // initial state (:494-611) for every instance
  for (DBuf<T>* v : {&W.x, &W.kty, &W.sx, &W.dx, &W.ax, &W.agrad, &W.rx})
    CK(cudaMemsetAsync(v->get(), 0, sizeof(T) * v->n, s));
  for (DBuf<T>* v : {&W.y0, &W.y1, &W.kx0, &W.kx1, &W.sy, &W.skx, &W.ay, &W.akx, &W.ry, &W.rkx})
    CK(cudaMemsetAsync(v->get(), 0, sizeof(T) * v->n, s));
  CK(cudaMemcpyAsync(W.grad.get(), W.c, sizeof(T) * N, cudaMemcpyDeviceToDevice, s));   // c - K'0
  CK(cudaMemcpyAsync(W.rgrad.get(), W.c, sizeof(T) * N, cudaMemcpyDeviceToDevice, s));
  std::vector<long long> iteration(K, 1);
  std::vector<RestartMemory> mem(K);
  std::vector<char> retired(K, 0), due(K, 1);
  std::vector<double> basic(K, 0.0);
  StepState* st = W.st_host.p;
  const double* table = W.ensure_pow_table(prm.reduction_exponent, prm.growth_exponent);
  for (int k = 0; k < K; ++k) {
    StepState& q = st[k];
    std::memset(&q, 0, sizeof(q));
    q.reduction_exponent = prm.reduction_exponent;
    q.growth_exponent = prm.growth_exponent;
    q.pow_table = table;
    q.pow_table_len = kPowTableLen;
    q.kkt_passes = 0.5;
    q.tau = B->amax[k] > 0.0 ? 1.0 / B->amax[k] : 1.0;
    if (prm.scale_invariant_initial_primal_weight && B->norm_c[k] > 0.0 && B->norm_b[k] > 0.0)
      q.omega = prm.primal_importance * (B->norm_c[k] / B->norm_b[k]);
    else
      q.omega = prm.primal_importance;
    q.iter_start_tau = q.tau;
    q.done = 1;
  }
  W.push_state();
  const auto t0 = Clock::now();
  auto elapsed = [&]() { return std::chrono::duration<double>(Clock::now() - t0).count(); };
  uint8_t* fh = W.flags_host.p;
  int alive = K;
  long long rounds = 0;
  while (alive > 0) {
    // ---- evaluate every instance that reached its evaluation point ----
    std::memset(fh, 0, 4 * (size_t)K);
    bool any = false;
    for (int k = 0; k < K; ++k)
      if (!retired[k] && due[k]) {
        fh[k] = 1;
        fh[K + k] = (st[k].numerical_error || st[k].count_primal == 0 || st[k].count_dual == 0) ? 1 : 0;
        if (!fh[K + k]) {
          st[k].rcp_w_primal = 1.0 / st[k].sum_w_primal;
          st[k].rcp_w_dual = 1.0 / st[k].sum_w_dual;
        }
        st[k].kkt_passes += 2.0;
        st[k].done = 0;
        any = true;
      } else {
        st[k].done = 1;  // not being evaluated: keep its kernels idle
      }
    if (any) {
      W.push_state();
      W.push_flags();
      W.launch_pair(kStepCommitOnly);
      CK_LAUNCH();
      for (int k = 0; k < K; ++k)
        if (fh[k]) st[k].pending_commit = 0;
      // y-bar first, then the averages' K'y = A' y-bar of the instances evaluated now (as the
      // lone solve forms it), then x-bar and the average gradient
      if (M) {
        batch_average_m_kernel<T><<<W.grid(M), kBlock, 0, s>>>(W.vm(W.active()), W.use_current(), W.sy.get(),
                                                               W.skx.get(), W.y0.get(), W.y1.get(), W.kx0.get(),
                                                               W.kx1.get(), W.ay.get(), W.akx.get());
        CK_LAUNCH();
      }
      if (B->At.num_items > 0) {
        spmv_kernel<T><<<B->At.num_items, kBlock, 0, s>>>(B->At.view<T>(), W.ay.get(), W.aty.get(), B->col_inst.get(),
                                                          W.active());
        CK_LAUNCH();
      }
      batch_average_n_kernel<T><<<W.grid(N), kBlock, 0, s>>>(W.vn(W.active()), W.use_current(), W.sx.get(),
                                                             W.aty.get(), W.c, W.x.get(), W.grad.get(), W.ax.get(),
                                                             W.agrad.get());
      CK_LAUNCH();
      W.launches += 3;
      W.template seg_reduce<kEvalNQ, kEvalNMax>(
          true, EvalN<T>{W.ax.get(), W.agrad.get(), B->var.get(), W.rvar.get(), B->ol.get(), B->ou.get(), B->oc.get()},
          0);
      W.template seg_reduce<kEvalMQ, kEvalMMax>(
          false, EvalM<T>{W.ay.get(), W.akx.get(), B->con.get(), W.rcon.get(), B->ob.get(), 0, B->ineq_flag.get()},
          16);
      W.fetch();
      bool any_restart_check = false;
      std::vector<char> check(K, 0);
      for (int k = 0; k < K; ++k) {
        if (!fh[k]) continue;
        const double* en = W.red_host.p + (size_t)32 * k;
        gpdhg_iteration_stats stats;
        std::memset(&stats, 0, sizeof(stats));
        assemble_stats(B->info[k], prm, en, en + 16, stats);
        const long long it = iteration[k];
        stats.iteration_number = (int32_t)(it - 1);
        stats.cumulative_kkt_matrix_passes = st[k].kkt_passes;
        stats.cumulative_time_sec = elapsed();
        stats.step_size = st[k].tau;
        stats.primal_weight = st[k].omega;
        stats.precision = sizeof(T) == sizeof(double) ? GPDHG_PRECISION_FP64 : GPDHG_PRECISION_FP32;
        stats.time_spent_doing_basic_algorithm = basic[k];
        int reason = check_termination(prm, B->info[k], stats);
        if (st[k].numerical_error && reason == 0) reason = GPDHG_TERMINATION_REASON_NUMERICAL_ERROR;
        if (it < 10 && (reason == GPDHG_TERMINATION_REASON_PRIMAL_INFEASIBLE ||
                        reason == GPDHG_TERMINATION_REASON_DUAL_INFEASIBLE))
          reason = 0;
        if (reason != 0) {
          gpdhg_result& r = results[k];
          std::memset(&r, 0, sizeof(r));
          r.termination_reason = reason;
          r.iteration_count = (int32_t)(it - 1);
          r.total_number_iterations = st[k].total_iters;
          r.cumulative_kkt_matrix_passes = st[k].kkt_passes;
          r.solve_time_sec = stats.cumulative_time_sec;
          r.num_iteration_stats = 1;
          r.fp64_handoff_iteration = -1;
          r.last_iteration_stats = stats;
          r.accepted_steps = st[k].accepted;
          r.rejected_steps = st[k].rejected;
          r.primal_spmv_launches = st[k].primal_spmv;
          auto fetch_slice = [&](const T* dsrc, double* hdst, int off, int len) {
            if (!hdst || len == 0) return;
            std::vector<T> tmp(len);
            CK(cudaMemcpyAsync(tmp.data(), dsrc + off, sizeof(T) * len, cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            for (int q = 0; q < len; ++q) hdst[q] = (double)tmp[q];
          };
          fetch_slice(W.ax.get(), primal_out ? primal_out[k] : nullptr, B->col_off[k], B->col_off[k + 1] - B->col_off[k]);
          if (primal_out) to_caller_columns(B->col_perm[k], primal_out[k]);
          fetch_slice(W.ay.get(), dual_out ? dual_out[k] : nullptr, B->row_off[k], B->row_off[k + 1] - B->row_off[k]);
          retired[k] = 1;
          fh[k] = 0;
          st[k].done = 1;
          --alive;
          r.kernels_launched = W.launches - launches0;
          if (on_retire) (*on_retire)(k);
          continue;
        }
        if (st[k].count_primal > 0 && st[k].count_dual > 0) {
          check[k] = 1;
          any_restart_check = true;
        }
      }
      // buffer_primal_gradient = c - K'y (:742) for every instance that goes on
      for (int k = 0; k < K; ++k) fh[k] = (!retired[k] && due[k]) ? 1 : 0;
      W.push_flags();
      batch_grad_kernel<T><<<W.grid(N), kBlock, 0, s>>>(W.vn(W.active()), W.c, W.kty.get(), W.grad.get());
      CK_LAUNCH();
      ++W.launches;
      // run_restart_scheme for the instances that have an average
      for (int k = 0; k < K; ++k) fh[k] = check[k];
      if (any_restart_check) {
        W.push_flags();
        KktN<T> kn{W.l, W.u, W.c, W.x.get(), W.ax.get(), W.rx.get(), W.grad.get(), W.agrad.get(), W.rgrad.get()};
        W.template seg_reduce<kKktNQ, 0u>(true, kn, 0);
        W.fetch();
        std::vector<double> knv((size_t)32 * K);
        std::memcpy(knv.data(), W.red_host.p, sizeof(double) * 32 * K);
        // m side: one launch per buffer parity, so each instance reads its current y and K x
        for (int par = 0; par < 2; ++par) {
          bool have = false;
          for (int k = 0; k < K; ++k) {
            fh[k] = check[k] && st[k].parity == par;
            have |= fh[k] != 0;
          }
          if (!have) continue;
          W.push_flags();
          KktM<T> km{W.b, par ? W.y1.get() : W.y0.get(), W.ay.get(), W.ry.get(),
                     par ? W.kx1.get() : W.kx0.get(), W.akx.get(), W.rkx.get(), 0, B->ineq_flag.get()};
          W.template seg_reduce<kKktMQ, 0u>(false, km, 16);
        }
        for (int k = 0; k < K; ++k) fh[k] = check[k];
        W.fetch();
        bool any_restart = false;
        std::vector<uint8_t> ta(K, 0), rs(K, 0);
        for (int k = 0; k < K; ++k) {
          if (!check[k]) continue;
          const double* kn = knv.data() + (size_t)32 * k;
          const double* kmv = W.red_host.p + (size_t)32 * k + 16;
          const RestartDecision dec =
              decide_restart(prm, B->info[k], st[k].count_primal, st[k].tau, st[k].omega, iteration[k] - 1, kn, kmv, mem[k]);
          if (dec.restart_used != GPDHG_RESTART_CHOICE_NO_RESTART) {
            rs[k] = 1;
            ta[k] = dec.reset_to_average ? 1 : 0;
            st[k].count_primal = st[k].count_dual = 0;
            st[k].sum_w_primal = st[k].sum_w_dual = 0.0;
            st[k].omega = dec.new_omega;
            any_restart = true;
          }
        }
        if (any_restart) {
          for (int k = 0; k < K; ++k) {
            fh[k] = rs[k];
            fh[2 * K + k] = ta[k];
          }
          W.push_flags();
          W.push_state();  // restart kernels read each instance's parity
          batch_restart_n_kernel<T><<<W.grid(N), kBlock, 0, s>>>(W.vn(W.active()), W.to_avg(), W.ax.get(),
                                                                 W.agrad.get(), W.c, W.x.get(), W.kty.get(),
                                                                 W.grad.get(), W.sx.get(), W.rx.get(), W.rgrad.get());
          CK_LAUNCH();
          if (M) {
            batch_restart_m_kernel<T><<<W.grid(M), kBlock, 0, s>>>(W.vm(W.active()), W.to_avg(), W.ay.get(),
                                                                   W.akx.get(), W.y0.get(), W.y1.get(), W.kx0.get(),
                                                                   W.kx1.get(), W.sy.get(), W.skx.get(), W.ry.get(),
                                                                   W.rkx.get());
            CK_LAUNCH();
          }
          W.launches += 2;
        }
      }
      // re-arm: take_step! calls until each instance's next evaluation
      for (int k = 0; k < K; ++k) {
        if (retired[k] || !due[k]) continue;
        const long long it = iteration[k];
        st[k].done = 0;
        st[k].target_in_chunk = (int)std::min<long long>(next_eval_after(it, freq, it_limit) - it, 1 << 30);
        st[k].accepted_in_chunk = 0;
        st[k].attempts_in_chunk = 0;
        st[k].max_attempts_in_chunk = 1 << 30;
        st[k].iter_start_tau = st[k].tau;
        st[k].arrive = 0;
        due[k] = 0;
      }
    }
    if (alive == 0) break;
    // launch only the CTAs of running instances once retirements have halved them
    if (2 * W.active_ctas(retired) < W.grid_p) W.compact(retired);
    // ---- step graphs until every running instance reached its evaluation point ----
    W.push_state();
    const auto tb = Clock::now();
    long long graph_launches = 0;
    while (true) {
      int max_remaining = 0;
      for (int k = 0; k < K; ++k)
        if (!retired[k] && !st[k].done) max_remaining = std::max(max_remaining, st[k].target_in_chunk - st[k].accepted_in_chunk);
      if (max_remaining == 0) break;
      int lv = 0;
      while (lv + 1 < kBatchLevels && (1 << lv) < max_remaining) ++lv;
      CK(cudaGraphLaunch(W.graphs[lv], s));
      W.launches += 2 * (1 << lv);
      CK(cudaStreamSynchronize(s));
      bool all_done = true;
      for (int k = 0; k < K; ++k)
        if (!retired[k] && !st[k].done) all_done = false;
      if (all_done) break;
      if (++graph_launches > 1000000) throw Error(GPDHG_ERR_INTERNAL, "batch step chunk did not finish");
    }
    const double dt = std::chrono::duration<double>(Clock::now() - tb).count();
    for (int k = 0; k < K; ++k) {
      if (retired[k]) continue;
      basic[k] += dt;
      iteration[k] += st[k].accepted_in_chunk + (st[k].numerical_error ? 1 : 0);
      st[k].accepted_in_chunk = 0;
      due[k] = 1;
    }
    if (prm.time_sec_limit < std::numeric_limits<double>::infinity() && elapsed() > 10.0 * prm.time_sec_limit + 60.0)
      throw Error(GPDHG_ERR_INTERNAL, "batch exceeded its time limit by far");
    ++rounds;
  }
  const long long launched = W.launches - launches0;
  for (int k = 0; k < K; ++k) results[k].kernels_launched = launched;
}

void batch_solve(gpdhg_batch* B, const gpdhg_params& prm, gpdhg_result* results, double* const* primal_out,
                 double* const* dual_out, const std::function<void(int)>* on_retire) {
  if (prm.precision == GPDHG_PRECISION_FP64) {
    if (!B->ws64) B->ws64.reset(new BatchWorkspace<double>(B));
    run_batch(B, *B->ws64, prm, results, primal_out, dual_out, on_retire);
  } else {
    if (!B->ws32) B->ws32.reset(new BatchWorkspace<float>(B));
    run_batch(B, *B->ws32, prm, results, primal_out, dual_out, on_retire);
  }
}

void BatchWorkspaceDeleter::operator()(BatchWorkspace<double>* w) const { delete w; }
void BatchWorkspaceDeleter::operator()(BatchWorkspace<float>* w) const { delete w; }

}  // namespace gpdhg

gpdhg_batch::~gpdhg_batch() {
  ws64.reset();
  ws32.reset();
  if (stream) cudaStreamDestroy(stream);
}
