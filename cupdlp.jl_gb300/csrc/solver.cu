// solver.cu — the restarted PDHG loop of optimize() on one GPU.
//
// Host/device split (src/primal_dual_hybrid_gradient_gpu.jl:457-798):
//   * step attempts run as CUDA graphs of [primal_step_kernel, dual_step_kernel] pairs;
//     accept/reject and the step size live on the device (StepState), so a whole
//     evaluation interval (64 accepted steps) needs one or two host synchronisations
//     instead of ~5 per attempt;
//   * evaluations (every termination_evaluation_frequency iterations, the first 10,
//     and on a numerical error) run FP64 reduction kernels and read back ~40 scalars;
//     the termination test, restart scheme and primal-weight update are the reference's
//     scalar logic on the host;
//   * with GPDHG_PRECISION_FP32_REFINE the loop runs on FP32 copies of the matrix and
//     iterates until the relative KKT error reaches fp64_handoff_relative_kkt (or stalls),
//     then converts the state to FP64, recomputes K x and K'y exactly, and continues.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <exception>
#include <thread>
#include <limits>
#include <random>
#include <type_traits>
#include <vector>

#include "batch.h"
#include "batch_kernels.cuh"
#include "tiles.h"
#include "eval_kernels.cuh"
#include "host_logic.h"
#include "problem.h"
#include "spmv.cuh"
#include "step_kernels.cuh"

namespace gpdhg {

void launch_convert_d2f(const double* src, float* dst, long long n, cudaStream_t s) {
  const int grid = std::max(1, std::min(ceil_div(n, kBlock), 4096));
  convert_kernel<double, float><<<grid, kBlock, 0, s>>>(n, src, dst);
  CK_LAUNCH();
}

__global__ void reciprocal_kernel(long long len, const double* src, double* dst) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x)
    dst[i] = 1.0 / src[i];
}

void launch_reciprocal(const double* src, double* dst, long long n, cudaStream_t s) {
  if (n <= 0) return;
  const int grid = std::max(1, std::min(ceil_div(n, kBlock), 4096));
  reciprocal_kernel<<<grid, kBlock, 0, s>>>(n, src, dst);
  CK_LAUNCH();
}

template <class T>
struct DotF {
  const T* a;
  const T* b;
  __device__ __forceinline__ void operator()(long long i, double* acc) const { acc[0] += (double)a[i] * (double)b[i]; }
};

// Step graphs hold 1, 2, 4, ..., 64 [primal, dual] pairs; a chunk launches the smallest one
// that covers the accepted steps still missing, so finished chunks waste almost no launches.
constexpr int kGraphLevels = 7;
inline int graph_level(int remaining) {
  int lv = 0;
  while (lv + 1 < kGraphLevels && (1 << lv) < remaining) ++lv;
  return lv;
}
// Host table of the step-size factors (1 - (k+1)^-r, 1 + (k+1)^-g) of take_step!
// (:405-407): the device reads it instead of evaluating two FP64 pow() per attempt in one
// thread, and the values are the host libm's, as in the reference's host-side loop.
// The table of an exponent pair is computed once per process (on host threads, each entry
// by the same libm call whatever the thread) and kept for later problems.
void fill_pow_table(std::vector<double>& t, double r, double g) {
  static std::mutex mu;
  static std::vector<std::pair<std::pair<double, double>, std::shared_ptr<const std::vector<double>>>> cache;
  std::shared_ptr<const std::vector<double>> hit;
  {
    std::lock_guard<std::mutex> lock(mu);
    for (auto& e : cache)
      if (e.first.first == r && e.first.second == g) hit = e.second;
  }
  if (!hit) {
    auto v = std::make_shared<std::vector<double>>(2 * kPowTableLen);
    const int T = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    for (int q = 0; q < T; ++q)
      th.emplace_back([&, q] {
        for (long long k = kPowTableLen * q / T; k < kPowTableLen * (q + 1) / T; ++k) {
          const double k1 = (double)(k + 1);
          (*v)[2 * k] = 1.0 - 1.0 / std::pow(k1, r);
          (*v)[2 * k + 1] = 1.0 + 1.0 / std::pow(k1, g);
        }
      });
    for (auto& x : th) x.join();
    std::lock_guard<std::mutex> lock(mu);
    if (cache.size() >= 8) cache.erase(cache.begin());
    cache.push_back({{r, g}, v});
    hit = v;
  }
  t = *hit;
}

template <class T>
struct Workspace {
  gpdhg_problem* P = nullptr;
  int n = 0, m = 0;
  DBuf<T> l_own, u_own, c_own, b_own;
  const T *l = nullptr, *u = nullptr, *c = nullptr, *b = nullptr;
  DBuf<T> x, dx, kty, sx, ax, agrad, grad, rx, rgrad, tmp_n;
  DBuf<T> y0, y1, kx0, kx1, sy, skx, ay, akx, ry, rkx, tmp_m;
  DBuf<StepState> st_dev;
  PinnedBuf<StepState> st_host;
  DBuf<double> part_p, part_d, red_part, red_out;
  DBuf<double> rvar, rcon;   // 1 / variable and 1 / constraint rescaling (evaluation divisions)
  PinnedBuf<double> red_host;
  // KKT ingredients of the last restart point (KktN quantities 8-11, KktM 6-8), valid until
  // the restart point moves
  bool restart_kkt_valid = false;
  double restart_kkt_n[4] = {}, restart_kkt_m[3] = {};
  // segmented reductions over [0, n) and [0, m): the same layout a batch uses per instance
  DBuf<SegItem> seg_n, seg_m;
  DBuf<int32_t> seg_n_begin, seg_m_begin;
  DBuf<uint8_t> one;
  int nseg_n = 1, nseg_m = 1;
  cudaGraphExec_t graphs[kGraphLevels] = {};
  // profiled variants: an event between every pair of kernels
  std::vector<cudaEvent_t> pev;   // per-kernel timing events (params.profile_kernels)
  DBuf<double> pow_table;
  double pow_r = -1.0, pow_g = -1.0;
  const int direct = sizeof(T) == sizeof(float) ? 1 : 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // tile plans of A' (primal kernel) and A (dual kernel); the lone LP is a batch of one
  TilePlan<T> plan_p, plan_d;
  DBuf<double> part_p_split, part_d_split;

  explicit Workspace(gpdhg_problem* p) : P(p), n(p->n), m(p->m), st_host(1), red_host(64) {
    PhaseTrace tr;
    const size_t N = std::max(n, 1), M = std::max(m, 1);
    cudaStream_t s = P->stream;
    if constexpr (sizeof(T) == sizeof(double)) {
      l = (const T*)P->l.get();
      u = (const T*)P->u.get();
      c = (const T*)P->c.get();
      b = (const T*)P->b.get();
    } else {
      ensure_fp32_values(P);
      l_own.alloc(N); u_own.alloc(N); c_own.alloc(N); b_own.alloc(M);
      launch_convert_d2f(P->l.get(), l_own.get(), n, s);
      launch_convert_d2f(P->u.get(), u_own.get(), n, s);
      launch_convert_d2f(P->c.get(), c_own.get(), n, s);
      if (m) launch_convert_d2f(P->b.get(), b_own.get(), m, s);
      l = l_own.get(); u = u_own.get(); c = c_own.get(); b = b_own.get();
    }
    tr.mark("  ws: FP32 copies");
    // the primal plan (a host pass over the n rows of A') is built on a helper thread while
    // this one allocates the iterate vectors and builds the dual plan
    std::exception_ptr plan_err;
    int device = 0;
    CK(cudaGetDevice(&device));
    std::thread plan_thread([&] {
      try {
        CK(cudaSetDevice(device));   // a new host thread starts on device 0
        build_tile_plan(plan_p, P->At, {0, n}, {}, kPrimalCtasPerSm<T>, kTileSideAt, s);
      } catch (...) {
        plan_err = std::current_exception();
      }
    });
    try {
      for (DBuf<T>* v : {&x, &dx, &kty, &sx, &ax, &agrad, &grad, &rx, &rgrad, &tmp_n}) v->alloc(N);
      for (DBuf<T>* v : {&y0, &y1, &kx0, &kx1, &sy, &skx, &ay, &akx, &ry, &rkx, &tmp_m}) v->alloc(M);
      rvar.alloc(N);
      rcon.alloc(M);
      launch_reciprocal(P->var.get(), rvar.get(), n, s);
      launch_reciprocal(P->con.get(), rcon.get(), m, s);
      st_dev.alloc(1);
      CK(cudaMemsetAsync(st_dev.get(), 0, sizeof(StepState), s));
      tr.mark("  ws: iterate buffers");
      build_tile_plan(plan_d, P->A, {0, m}, {P->neq}, kDualCtasPerSm, kTileSideA, s);
      tr.mark("  ws: dual plan");
    } catch (...) {
      plan_thread.join();
      throw;
    }
    plan_thread.join();
    if (plan_err) std::rethrow_exception(plan_err);
    tr.mark(sizeof(T) == 8 ? "FP64 vectors and plans" : "FP32 vectors and plans");
    part_p.alloc(plan_p.num_ctas);
    part_d.alloc(2 * (size_t)plan_d.num_ctas);
    part_p_split.alloc(std::max(plan_p.num_splits, 1));
    part_d_split.alloc(2 * (size_t)std::max(plan_d.num_splits, 1));
    red_out.alloc(64);
    {
      std::vector<SegItem> it;
      std::vector<int32_t> beg;
      auto upload = [&](DBuf<SegItem>& d, DBuf<int32_t>& db, int len, int& count) {
        build_seg_items({0, len}, it, beg);
        count = (int)it.size();
        d.alloc(it.size());
        db.alloc(beg.size());
        CK(cudaMemcpyAsync(d.get(), it.data(), sizeof(SegItem) * it.size(), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(db.get(), beg.data(), sizeof(int32_t) * beg.size(), cudaMemcpyHostToDevice, s));
        CK(cudaStreamSynchronize(s));
      };
      upload(seg_n, seg_n_begin, n, nseg_n);
      upload(seg_m, seg_m_begin, m, nseg_m);
      red_part.alloc((size_t)32 * std::max(nseg_n, nseg_m));
      one.alloc(1);
      CK(cudaMemsetAsync(one.get(), 1, 1, s));
    }
    CK(cudaEventCreate(&ev0));
    CK(cudaEventCreate(&ev1));
    tr.mark("segments, partials");
    build_graphs();
    tr.mark("step graphs");
  }
  ~Workspace() {
    for (cudaGraphExec_t g : graphs)
      if (g) cudaGraphExecDestroy(g);
    for (cudaEvent_t e : pev) cudaEventDestroy(e);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
  }

  const T* ycur(int parity) const { return parity ? y1.get() : y0.get(); }
  const T* kxcur(int parity) const { return parity ? kx1.get() : kx0.get(); }
  T* ycur_mut(int parity) { return parity ? y1.get() : y0.get(); }
  T* kxcur_mut(int parity) { return parity ? kx1.get() : kx0.get(); }

  PrimalArgs<T> primal_args(int mode) {
    return PrimalArgs<T>{P->At.view<T>(), plan_p.view(), c, l, u, x.get(), dx.get(), kty.get(), sx.get(),
                         y0.get(), y1.get(), st_dev.get(), part_p.get(), part_p_split.get(), mode, direct};
  }
  DualArgs<T> dual_args(int mode) {
    return DualArgs<T>{P->A.view<T>(), plan_d.view(), plan_p.inst_cta_begin.get(), plan_p.inst_split_begin.get(),
                       dx.get(), b, y0.get(), y1.get(), kx0.get(), kx1.get(), sy.get(), skx.get(), st_dev.get(),
                       part_p.get(), part_p_split.get(), part_d.get(), part_d_split.get(), mode, direct};
  }
  void launch_primal(int mode, cudaStream_t s) { launch_step(primal_step_kernel<T>, plan_p.num_ctas, s, primal_args(mode)); }
  void launch_dual(int mode, cudaStream_t s) { launch_step(dual_step_kernel<T>, plan_d.num_ctas, s, dual_args(mode)); }

  void launch_pair(int mode, cudaStream_t s) {
    launch_primal(mode, s);
    launch_dual(mode, s);
    P->launches += 2;
  }

  cudaGraphExec_t capture(int pairs) {
    cudaStream_t s = P->stream;
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < pairs; ++k) {
      launch_primal(kStepNormal, s);
      launch_dual(kStepNormal, s);
    }
    cudaMemcpyAsync(st_host.p, st_dev.get(), sizeof(StepState), cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamEndCapture(s, &g);
    CK(e);
    cudaGraphExec_t ex = nullptr;
    CK(cudaGraphInstantiate(&ex, g, 0));
    cudaGraphDestroy(g);
    return ex;
  }
  void build_graphs() {
    for (int lv = 0; lv < kGraphLevels; ++lv) graphs[lv] = capture(1 << lv);
  }
  // The same pairs launched directly with an event between every two kernels, for
  // per-kernel CUDA-event timing (events recorded as graph nodes cannot be timed).
  void launch_profiled(int pairs) {
    if ((int)pev.size() < 2 * pairs + 1) {
      const size_t old = pev.size();
      pev.resize(2 * pairs + 1);
      for (size_t k = old; k < pev.size(); ++k) CK(cudaEventCreate(&pev[k]));
    }
    cudaStream_t s = P->stream;
    CK(cudaEventRecord(pev[0], s));
    for (int k = 0; k < pairs; ++k) {
      launch_primal(kStepNormal, s);
      CK(cudaEventRecord(pev[2 * k + 1], s));
      launch_dual(kStepNormal, s);
      CK(cudaEventRecord(pev[2 * k + 2], s));
    }
    CK_LAUNCH();
    CK(cudaMemcpyAsync(st_host.p, st_dev.get(), sizeof(StepState), cudaMemcpyDeviceToHost, s));
  }
  const double* ensure_pow_table(double r, double g) {
    if (pow_table.get() && r == pow_r && g == pow_g) return pow_table.get();
    std::vector<double> t;
    fill_pow_table(t, r, g);
    pow_table.alloc(t.size());
    CK(cudaMemcpyAsync(pow_table.get(), t.data(), sizeof(double) * t.size(), cudaMemcpyHostToDevice, P->stream));
    CK(cudaStreamSynchronize(P->stream));
    pow_r = r;
    pow_g = g;
    return pow_table.get();
  }

  void spmv(const DeviceMatrix& M, const T* xin, T* yout) {
    if (M.num_items == 0) return;
    spmv_kernel<T><<<M.num_items, kBlock, 0, P->stream>>>(M.view<T>(), xin, yout, nullptr, nullptr);
    CK_LAUNCH();
    ++P->launches;
  }

  // FP64 reduction of Q quantities over [0, n) (n_side) or [0, m), into red_out[out_offset..)
  template <int Q, unsigned MAXMASK, class F>
  void reduce(bool n_side, F f, int out_offset) {
    const int nit = n_side ? nseg_n : nseg_m;
    seg_reduce_kernel<Q, MAXMASK, F><<<nit, kBlock, 0, P->stream>>>(n_side ? seg_n.get() : seg_m.get(), one.get(), f,
                                                                     red_part.get(), nit);
    CK_LAUNCH();
    seg_finalize_kernel<Q, MAXMASK><<<1, kBlock, 0, P->stream>>>(n_side ? seg_n_begin.get() : seg_m_begin.get(),
                                                                  one.get(), red_part.get(), nit,
                                                                  red_out.get() + out_offset, 32);
    CK_LAUNCH();
    P->launches += 2;
  }
  void fetch_reductions(int count) {
    CK(cudaMemcpyAsync(red_host.p, red_out.get(), sizeof(double) * count, cudaMemcpyDeviceToHost, P->stream));
    CK(cudaStreamSynchronize(P->stream));
  }

  double dot(const T* a, const T* b2, long long len) {
    reduce<1, 0u>(len == n, DotF<T>{a, b2}, 0);
    fetch_reductions(1);
    return red_host.p[0];
  }

  int grid_for(long long len) const { return std::max(1, std::min(ceil_div(len, kBlock), 4096)); }
};

}  // namespace gpdhg

void gpdhg::WorkspaceDeleter::operator()(Workspace<double>* w) const { delete w; }
void gpdhg::WorkspaceDeleter::operator()(Workspace<float>* w) const { delete w; }

gpdhg_problem::~gpdhg_problem() {
  ws64.reset();
  ws32.reset();
  if (stream) cudaStreamDestroy(stream);
}

namespace gpdhg {

namespace {

using Clock = std::chrono::steady_clock;

// Host scalar state of the loop that is not part of StepState.
struct LoopState {
  long long iteration = 0;   // the reference's `iteration` (accepted steps + 1)
  double basic_time = 0.0;   // time_spent_doing_basic_algorithm
  Clock::time_point t0;
  RestartMemory restart;      // CuRestartInfo scalars
  double step_loop_sec = 0.0;
  double primal_kernel_sec = 0.0, dual_kernel_sec = 0.0;
  long long kernel_launches = 0;
  long long launches_at_start = 0;
  int precision = GPDHG_PRECISION_FP64;
  int handoff_iteration = -1;
  double best_rel_kkt = std::numeric_limits<double>::infinity();
  int evals_without_progress = 0;
  double elapsed() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

// The loop in one precision. Returns true when it terminated, false on an FP64 hand-off
// request (state left in W for the caller to convert).
template <class T>
bool run_phase(gpdhg_problem* P, Workspace<T>& W, const gpdhg_params& prm, LoopState& L, gpdhg_result* res,
               double* primal_out, double* dual_out, bool allow_handoff) {
  cudaStream_t s = P->stream;
  StepState& st = *W.st_host.p;
  const long long freq = std::max(1, prm.termination_evaluation_frequency);
  const long long it_limit = prm.iteration_limit;
  const int n = P->n, m = P->m;
  const int gn = W.grid_for(n), gm = W.grid_for(std::max(m, 1));
  InstanceInfo qi;
  qi.obj_const = P->obj_const;
  qi.linf_c = P->linf_c; qi.linf_b = P->linf_b; qi.l2_c = P->l2_c; qi.l2_b = P->l2_b;

  // The pinned mirror is edited right after this call, so the copy must have landed.
  auto push_state = [&]() {
    CK(cudaMemcpyAsync(W.st_dev.get(), W.st_host.p, sizeof(StepState), cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));
  };
  // The same copy when the mirror stays untouched until the stream has passed it (the step
  // graphs that follow end by copying the state back into the mirror, and the host reads it
  // only after synchronising with them).
  auto push_state_async = [&]() {
    CK(cudaMemcpyAsync(W.st_dev.get(), W.st_host.p, sizeof(StepState), cudaMemcpyHostToDevice, s));
  };

  while (true) {
    const long long it = L.iteration;
    if (eval_due(it, freq, it_limit, st.numerical_error != 0)) {
      st.kkt_passes += 2.0;  // KKT_PASSES_PER_TERMINATION_EVALUATION
      st.done = 0;
      push_state();
      if (st.pending_commit) {
        W.launch_pair(kStepCommitOnly, s);
        CK_LAUNCH();
        st.pending_commit = 0;
      }
      const int p = st.parity;
      // One pass per side (EvalPassM, then EvalPassN): the average, or the current point
      // (src/primal_dual_hybrid_gradient_gpu.jl:635-642); its unscaled statistics
      // (src/iteration_stats_utils_gpu.jl:447-502); buffer_primal_gradient = c - K'y (:742);
      // and the restart scheme's KKT ingredients, those of the last restart point only when
      // it moved since they were computed. Between them the average's K'y = A' y-bar (the
      // reference sums the steps' K'y with the averaging weights instead,
      // src/saddle_point_gpu.jl:176-189; the two agree in exact arithmetic). One read-back
      // for all of them.
      const bool use_current = st.numerical_error || st.count_primal == 0 || st.count_dual == 0;
      const double wx = st.sum_w_primal, wy = st.sum_w_dual;
      const double rwx = use_current ? 0.0 : 1.0 / wx, rwy = use_current ? 0.0 : 1.0 / wy;
      const bool with_restart = !W.restart_kkt_valid;
      W.template reduce<kEvalMQ + kKktMQ, kEvalMMax>(
          false,
          EvalPassM<T>{EvalM<T>{W.ay.get(), W.akx.get(), P->con.get(), W.rcon.get(), P->ob.get(), P->neq, nullptr},
                       KktM<T>{W.b, W.ycur(p), W.ay.get(), W.ry.get(), W.kxcur(p), W.akx.get(), W.rkx.get(), P->neq,
                               nullptr},
                       W.sy.get(), W.skx.get(), W.ay.get(), W.akx.get(), wx, wy, rwx, rwy, use_current ? 1 : 0,
                       with_restart ? 1 : 0},
          32);
      if (!use_current) W.spmv(P->At, W.ay.get(), W.tmp_n.get());
      W.template reduce<kEvalNQ + kKktNQ, kEvalNMax>(
          true,
          EvalPassN<T>{EvalN<T>{W.ax.get(), W.agrad.get(), P->var.get(), W.rvar.get(), P->ol.get(), P->ou.get(),
                                P->oc.get()},
                       KktN<T>{W.l, W.u, W.c, W.x.get(), W.ax.get(), W.rx.get(), W.grad.get(), W.agrad.get(),
                               W.rgrad.get()},
                       W.sx.get(), W.tmp_n.get(), W.kty.get(), W.ax.get(), W.agrad.get(), W.grad.get(), wx, wy, rwx,
                       rwy, use_current ? 1 : 0, with_restart ? 1 : 0},
          0);
      W.fetch_reductions(32 + kEvalMQ + kKktMQ);
      const double* en = W.red_host.p;            // EvalN, then KktN at kEvalNQ
      const double* em = W.red_host.p + 32;       // EvalM, then KktM at kEvalMQ
      double kn[kKktNQ], km[kKktMQ];
      std::memcpy(kn, en + kEvalNQ, sizeof(kn));
      std::memcpy(km, em + kEvalMQ, sizeof(km));
      if (with_restart) {
        std::memcpy(W.restart_kkt_n, kn + 8, sizeof(W.restart_kkt_n));
        std::memcpy(W.restart_kkt_m, km + 6, sizeof(W.restart_kkt_m));
        W.restart_kkt_valid = true;
      } else {
        std::memcpy(kn + 8, W.restart_kkt_n, sizeof(W.restart_kkt_n));
        std::memcpy(km + 6, W.restart_kkt_m, sizeof(W.restart_kkt_m));
      }
      gpdhg_iteration_stats stats;
      std::memset(&stats, 0, sizeof(stats));
      assemble_stats(qi, prm, en, em, stats);
      stats.iteration_number = (int32_t)(it - 1);
      stats.cumulative_kkt_matrix_passes = st.kkt_passes;
      stats.cumulative_time_sec = L.elapsed();
      stats.step_size = st.tau;
      stats.primal_weight = st.omega;
      stats.precision = L.precision;
      stats.time_spent_doing_basic_algorithm = L.basic_time;
      int reason = check_termination(prm, qi, stats);
      if (st.numerical_error && reason == 0) reason = GPDHG_TERMINATION_REASON_NUMERICAL_ERROR;
      if (it < 10 && (reason == GPDHG_TERMINATION_REASON_PRIMAL_INFEASIBLE ||
                      reason == GPDHG_TERMINATION_REASON_DUAL_INFEASIBLE))
        reason = 0;
      bool pushed = false;
      if (prm.record_iteration_stats || reason != 0) {
        P->history.push_back(stats);
        pushed = true;
      }
      if (reason != 0) {
        // copy the scaled average to the host (:713-720)
        auto fetch = [&](const T* dsrc, double* hdst, int len) {
          if (!hdst || len == 0) return;
          if constexpr (sizeof(T) == sizeof(double)) {
            CK(cudaMemcpyAsync(hdst, dsrc, sizeof(double) * len, cudaMemcpyDeviceToHost, s));
          } else {
            std::vector<float> tmp(len);
            CK(cudaMemcpyAsync(tmp.data(), dsrc, sizeof(float) * len, cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            for (int k = 0; k < len; ++k) hdst[k] = tmp[k];
          }
        };
        fetch(W.ax.get(), primal_out, n);
        fetch(W.ay.get(), dual_out, m);
        CK(cudaStreamSynchronize(s));
        std::memset(res, 0, sizeof(*res));
        res->termination_reason = reason;
        res->iteration_count = (int32_t)(it - 1);
        res->total_number_iterations = st.total_iters;
        res->cumulative_kkt_matrix_passes = st.kkt_passes;
        res->solve_time_sec = L.elapsed();
        res->num_iteration_stats = (int32_t)P->history.size();
        res->fp64_handoff_iteration = L.handoff_iteration;
        res->last_iteration_stats = stats;
        res->step_loop_device_sec = L.step_loop_sec;
        res->accepted_steps = st.accepted;
        res->rejected_steps = st.rejected;
        res->primal_kernel_sec = L.primal_kernel_sec;
        res->dual_kernel_sec = L.dual_kernel_sec;
        res->primal_kernel_launches = L.kernel_launches;
        res->primal_spmv_launches = st.primal_spmv;
        res->kernels_launched = P->launches - L.launches_at_start;
        P->last_precision = (sizeof(T) == sizeof(double)) ? GPDHG_PRECISION_FP64 : GPDHG_PRECISION_FP32;
        return true;
      }
      // FP64 hand-off check (FP32_REFINE)
      if (allow_handoff) {
        const double rk = relative_kkt(stats, prm.optimality_norm);
        if (rk < 0.5 * L.best_rel_kkt) {
          L.best_rel_kkt = rk;
          L.evals_without_progress = 0;
        } else {
          L.evals_without_progress++;
        }
        if (rk <= prm.fp64_handoff_relative_kkt ||
            (prm.fp64_handoff_stall_evaluations > 0 && L.evals_without_progress >= prm.fp64_handoff_stall_evaluations)) {
          // leave the evaluation to be repeated by the FP64 phase at the same iteration
          st.kkt_passes -= 2.0;
          if (pushed) P->history.pop_back();
          return false;
        }
      }
      // run_restart_scheme, src/saddle_point_gpu.jl:479-622 (buffer_primal_gradient was
      // refreshed by the column pass)
      int restart_used = GPDHG_RESTART_CHOICE_NO_RESTART;
      if (st.count_primal > 0 && st.count_dual > 0) {
        const RestartDecision dec =
            decide_restart(prm, qi, st.count_primal, st.tau, st.omega, it - 1, kn, km, L.restart);
        if (dec.restart_used != GPDHG_RESTART_CHOICE_NO_RESTART) {
          if (dec.reset_to_average) {
            restart_n_kernel<T><<<gn, kBlock, 0, s>>>(n, W.ax.get(), W.agrad.get(), W.c, W.x.get(), W.kty.get(),
                                                      W.grad.get());
            CK_LAUNCH();
            ++P->launches;
            if (m) {
              CK(cudaMemcpyAsync(W.ycur_mut(p), W.ay.get(), sizeof(T) * m, cudaMemcpyDeviceToDevice, s));
              CK(cudaMemcpyAsync(W.kxcur_mut(p), W.akx.get(), sizeof(T) * m, cudaMemcpyDeviceToDevice, s));
            }
          }
          W.restart_kkt_valid = false;  // the restart point moves below
          // reset_solution_weighted_average!
          CK(cudaMemsetAsync(W.sx.get(), 0, sizeof(T) * n, s));
          if (m) {
            CK(cudaMemsetAsync(W.sy.get(), 0, sizeof(T) * m, s));
            CK(cudaMemsetAsync(W.skx.get(), 0, sizeof(T) * m, s));
          }
          st.count_primal = st.count_dual = 0;
          st.sum_w_primal = st.sum_w_dual = 0.0;
          // update_last_restart_info!: the restart point becomes the (new) current point
          CK(cudaMemcpyAsync(W.rx.get(), W.x.get(), sizeof(T) * n, cudaMemcpyDeviceToDevice, s));
          CK(cudaMemcpyAsync(W.rgrad.get(), W.grad.get(), sizeof(T) * n, cudaMemcpyDeviceToDevice, s));
          if (m) {
            CK(cudaMemcpyAsync(W.ry.get(), W.ycur(p), sizeof(T) * m, cudaMemcpyDeviceToDevice, s));
            CK(cudaMemcpyAsync(W.rkx.get(), W.kxcur(p), sizeof(T) * m, cudaMemcpyDeviceToDevice, s));
          }
          st.omega = dec.new_omega;
          restart_used = dec.restart_used;
        }
      }
      if (pushed) P->history.back().restart_used = restart_used;
    }

    // take_step! calls until the next evaluation
    const long long target = next_eval_after(it, freq, it_limit) - it;
    st.done = 0;
    st.target_in_chunk = (int)std::min<long long>(target, 1 << 30);
    st.accepted_in_chunk = 0;
    st.attempts_in_chunk = 0;
    st.max_attempts_in_chunk = 1 << 30;
    st.iter_start_tau = st.tau;
    st.arrive = 0;
    push_state_async();
    const auto tb = Clock::now();
    long long launches = 0;
    const bool prof = prm.profile_kernels != 0;
    while (true) {
      const int remaining = st.target_in_chunk - st.accepted_in_chunk;
      const int attempts_before = st.attempts_in_chunk;
      const int lv = graph_level(remaining);
      CK(cudaEventRecord(W.ev0, s));
      if (prof)
        W.launch_profiled(1 << lv);
      else
        CK(cudaGraphLaunch(W.graphs[lv], s));
      P->launches += 2 * (1 << lv);
      CK(cudaEventRecord(W.ev1, s));
      CK(cudaStreamSynchronize(s));
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, W.ev0, W.ev1));
      L.step_loop_sec += 1e-3 * ms;
      if (prof) {
        const std::vector<cudaEvent_t>& ev = W.pev;
        const int did = st.attempts_in_chunk - attempts_before;
        for (int k = 0; k < did; ++k) {
          float a = 0.f, b2 = 0.f;
          CK(cudaEventElapsedTime(&a, ev[2 * k], ev[2 * k + 1]));
          CK(cudaEventElapsedTime(&b2, ev[2 * k + 1], ev[2 * k + 2]));
          L.primal_kernel_sec += 1e-3 * a;
          L.dual_kernel_sec += 1e-3 * b2;
        }
        L.kernel_launches += did;
      }
      if (st.done) break;
      // every launch runs >= kGraphSmall attempts; 10^6 launches without the chunk's
      // accepted steps means the step size never settles
      if (++launches > 1000000) throw Error(GPDHG_ERR_INTERNAL, "step chunk did not finish");
    }
    L.basic_time += std::chrono::duration<double>(Clock::now() - tb).count();
    L.iteration += st.accepted_in_chunk + (st.numerical_error ? 1 : 0);
  }
}

// Initial state of optimize() (:494-611) in workspace W.
template <class T>
void init_state(gpdhg_problem* P, Workspace<T>& W, const gpdhg_params& prm, LoopState& L) {
  cudaStream_t s = P->stream;
  const int n = P->n, m = P->m;
  for (DBuf<T>* v : {&W.x, &W.kty, &W.sx, &W.dx, &W.ax, &W.agrad})
    CK(cudaMemsetAsync(v->get(), 0, sizeof(T) * v->n, s));
  for (DBuf<T>* v : {&W.y0, &W.y1, &W.kx0, &W.kx1, &W.sy, &W.skx, &W.ay, &W.akx})
    CK(cudaMemsetAsync(v->get(), 0, sizeof(T) * v->n, s));
  if (!P->warm_x.empty() || !P->warm_y.empty()) {
    auto upload = [&](const std::vector<double>& h, T* d, int len) {
      if (h.empty() || len == 0) return;
      std::vector<T> tmp(h.begin(), h.end());
      CK(cudaMemcpyAsync(d, tmp.data(), sizeof(T) * len, cudaMemcpyHostToDevice, s));
      CK(cudaStreamSynchronize(s));
    };
    upload(P->warm_x, W.x.get(), n);
    upload(P->warm_y, W.y0.get(), m);
    W.spmv(P->A, W.x.get(), W.kx0.get());
    W.spmv(P->At, W.y0.get(), W.kty.get());
  }
  const int gn = W.grid_for(n);
  grad_kernel<T><<<gn, kBlock, 0, s>>>(n, W.c, W.kty.get(), W.grad.get());
  CK_LAUNCH();
  ++P->launches;
  StepState& st = *W.st_host.p;
  std::memset(&st, 0, sizeof(st));
  st.reduction_exponent = prm.reduction_exponent;
  st.growth_exponent = prm.growth_exponent;
  st.pow_table = W.ensure_pow_table(prm.reduction_exponent, prm.growth_exponent);
  st.pow_table_len = kPowTableLen;
  if (prm.step_size_policy == GPDHG_STEPSIZE_ADAPTIVE) {
    st.kkt_passes += 0.5;
    // 1 / norm(A, Inf): entrywise max (:571). An empty matrix (the reference fails before
    // this point) gets tau_0 = 1, since 1/0 would make every averaging weight infinite.
    st.tau = P->amax > 0.0 ? 1.0 / P->amax : 1.0;
  } else {
    // estimate_maximum_singular_value (:139-172) with 0.001 failure probability, 0.2 error
    const double rel = 0.2, eps = 1.0 - (1.0 - rel) * (1.0 - rel);
    auto fail = [&](long long k) {
      if (k < 2 || eps <= 0.0) return 1.0;
      return std::min(0.824, 0.354 / std::sqrt(eps * (k - 1))) * std::sqrt((double)n) * std::pow(1.0 - eps, (double)k - 0.5);
    };
    std::mt19937_64 rng(1);
    std::normal_distribution<double> nd;
    std::vector<T> hx(n);
    for (auto& v : hx) v = (T)nd(rng);
    CK(cudaMemcpyAsync(W.tmp_n.get(), hx.data(), sizeof(T) * n, cudaMemcpyHostToDevice, s));
    CK(cudaStreamSynchronize(s));
    long long k = 0;
    std::vector<T> h(n);
    while (fail(k) > 0.001) {
      const double nx = std::sqrt(W.dot(W.tmp_n.get(), W.tmp_n.get(), n));
      CK(cudaMemcpy(h.data(), W.tmp_n.get(), sizeof(T) * n, cudaMemcpyDeviceToHost));
      for (auto& v : h) v = (T)((double)v / nx);
      CK(cudaMemcpy(W.tmp_n.get(), h.data(), sizeof(T) * n, cudaMemcpyHostToDevice));
      W.spmv(P->A, W.tmp_n.get(), W.tmp_m.get());
      W.spmv(P->At, W.tmp_m.get(), W.dx.get());
      CK(cudaMemcpyAsync(W.tmp_n.get(), W.dx.get(), sizeof(T) * n, cudaMemcpyDeviceToDevice, s));
      ++k;
    }
    W.spmv(P->A, W.tmp_n.get(), W.tmp_m.get());
    W.spmv(P->At, W.tmp_m.get(), W.dx.get());
    const double xz = W.dot(W.tmp_n.get(), W.dx.get(), n);
    const double xx = W.dot(W.tmp_n.get(), W.tmp_n.get(), n);
    const double smax = std::sqrt(xz / xx);
    st.tau = (1.0 - rel) / smax;
    st.kkt_passes += (double)k;
    st.constant_step = 1;
    CK(cudaMemsetAsync(W.dx.get(), 0, sizeof(T) * n, s));
  }
  if (prm.scale_invariant_initial_primal_weight) {
    const double rhs = std::sqrt(1.0) * P->norm2_b_scaled, obj = std::sqrt(1.0) * P->norm2_c_scaled;
    st.omega = (obj > 0.0 && rhs > 0.0) ? prm.primal_importance * (obj / rhs) : prm.primal_importance;
  } else {
    st.omega = prm.primal_importance;
  }
  st.iter_start_tau = st.tau;
  // create_last_restart_info
  W.restart_kkt_valid = false;
  CK(cudaMemcpyAsync(W.rx.get(), W.x.get(), sizeof(T) * n, cudaMemcpyDeviceToDevice, s));
  CK(cudaMemcpyAsync(W.rgrad.get(), W.grad.get(), sizeof(T) * n, cudaMemcpyDeviceToDevice, s));
  if (m) {
    CK(cudaMemcpyAsync(W.ry.get(), W.y0.get(), sizeof(T) * m, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(W.rkx.get(), W.kx0.get(), sizeof(T) * m, cudaMemcpyDeviceToDevice, s));
  }
  CK(cudaStreamSynchronize(s));
  L.iteration = 1;
  L.t0 = Clock::now();
}

// FP32 -> FP64 hand-off: every vector converted, K x and K'y recomputed in FP64.
void handoff_to_fp64(gpdhg_problem* P, Workspace<float>& F, Workspace<double>& D) {
  cudaStream_t s = P->stream;
  auto conv = [&](const DBuf<float>& a, DBuf<double>& b) {
    const long long len = (long long)a.n;
    convert_kernel<float, double><<<std::max(1, std::min(ceil_div(len, kBlock), 4096)), kBlock, 0, s>>>(len, a.get(), b.get());
    CK_LAUNCH();
    ++P->launches;
  };
  conv(F.x, D.x); conv(F.dx, D.dx); conv(F.sx, D.sx); conv(F.ax, D.ax);
  conv(F.agrad, D.agrad); conv(F.grad, D.grad); conv(F.rx, D.rx); conv(F.rgrad, D.rgrad);
  conv(F.y0, D.y0); conv(F.y1, D.y1); conv(F.sy, D.sy); conv(F.skx, D.skx); conv(F.ay, D.ay);
  conv(F.akx, D.akx); conv(F.ry, D.ry); conv(F.rkx, D.rkx);
  StepState st = *F.st_host.p;
  const int n = P->n, m = P->m;
  // exact FP64 products of the current point
  D.spmv(P->A, D.x.get(), st.parity ? D.kx1.get() : D.kx0.get());
  D.spmv(P->At, st.parity ? D.y1.get() : D.y0.get(), D.kty.get());
  // The FP64 phase restarts its averages at the handed-over point: FP32-accumulated
  // sums (and the K x-bar they imply) are only consistent to ~1e-7 and would feed a
  // phantom residual to the dual update after a restart to the average.
  CK(cudaMemsetAsync(D.sx.get(), 0, sizeof(double) * D.sx.n, s));
  CK(cudaMemsetAsync(D.sy.get(), 0, sizeof(double) * D.sy.n, s));
  CK(cudaMemsetAsync(D.skx.get(), 0, sizeof(double) * D.skx.n, s));
  st.count_primal = st.count_dual = 0;
  st.sum_w_primal = st.sum_w_dual = 0.0;
  st.pending_commit = 0;
  st.pow_table = D.ensure_pow_table(st.reduction_exponent, st.growth_exponent);
  grad_kernel<double><<<D.grid_for(n), kBlock, 0, s>>>(n, D.c, D.kty.get(), D.grad.get());
  CK_LAUNCH();
  ++P->launches;
  D.restart_kkt_valid = false;
  CK(cudaMemcpyAsync(D.rx.get(), D.x.get(), sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  CK(cudaMemcpyAsync(D.rgrad.get(), D.grad.get(), sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  if (m) {
    CK(cudaMemcpyAsync(D.ry.get(), st.parity ? D.y1.get() : D.y0.get(), sizeof(double) * m, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(D.rkx.get(), st.parity ? D.kx1.get() : D.kx0.get(), sizeof(double) * m,
                       cudaMemcpyDeviceToDevice, s));
  }
  *D.st_host.p = st;
  CK(cudaStreamSynchronize(s));
}

}  // namespace

void solve(gpdhg_problem* P, const gpdhg_params& prm, gpdhg_result* res, double* primal_out, double* dual_out) {
  P->history.clear();
  LoopState L;
  L.launches_at_start = P->launches;
  const int prec = prm.precision;
  if (prec == GPDHG_PRECISION_FP64) {
    if (!P->ws64) P->ws64.reset(new Workspace<double>(P));
    L.precision = GPDHG_PRECISION_FP64;
    init_state(P, *P->ws64, prm, L);
    run_phase(P, *P->ws64, prm, L, res, primal_out, dual_out, false);
    return;
  }
  if (!P->ws32) P->ws32.reset(new Workspace<float>(P));
  L.precision = GPDHG_PRECISION_FP32;
  init_state(P, *P->ws32, prm, L);
  const bool refine = prec == GPDHG_PRECISION_FP32_REFINE;
  if (run_phase(P, *P->ws32, prm, L, res, primal_out, dual_out, refine)) return;
  if (!P->ws64) P->ws64.reset(new Workspace<double>(P));
  handoff_to_fp64(P, *P->ws32, *P->ws64);
  L.precision = GPDHG_PRECISION_FP64;
  L.handoff_iteration = (int)(L.iteration - 1);
  run_phase(P, *P->ws64, prm, L, res, primal_out, dual_out, false);
}

void current_iterate(const gpdhg_problem* P, double* x, double* y) {
  cudaStream_t s = P->stream;
  auto get = [&](auto& W) {
    const int p = W.st_host.p->parity;
    if constexpr (std::is_same_v<std::decay_t<decltype(*W.x.get())>, double>) {
      if (x) CK(cudaMemcpyAsync(x, W.x.get(), sizeof(double) * P->n, cudaMemcpyDeviceToHost, s));
      if (y && P->m) CK(cudaMemcpyAsync(y, W.ycur(p), sizeof(double) * P->m, cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
    } else {
      std::vector<float> tx(P->n), ty(std::max(P->m, 1));
      CK(cudaMemcpyAsync(tx.data(), W.x.get(), sizeof(float) * P->n, cudaMemcpyDeviceToHost, s));
      if (P->m) CK(cudaMemcpyAsync(ty.data(), W.ycur(p), sizeof(float) * P->m, cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      if (x) for (int j = 0; j < P->n; ++j) x[j] = tx[j];
      if (y) for (int i = 0; i < P->m; ++i) y[i] = ty[i];
    }
  };
  if (P->last_precision == GPDHG_PRECISION_FP64 && P->ws64) get(*P->ws64);
  else if (P->last_precision == GPDHG_PRECISION_FP32 && P->ws32) get(*P->ws32);
  else throw Error(GPDHG_ERR_INVALID_ARGUMENT, "no solve has completed on this problem");
}

}  // namespace gpdhg
