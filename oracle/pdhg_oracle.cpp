// pdhg_oracle.cpp — CPU FP64 restatement of cuPDLP.jl's restarted-PDHG solve path.
//
// TEST INFRASTRUCTURE ONLY. This file is the oracle that the CUDA library is checked
// against, and the host-core baseline that bench.py times beside it. Nothing in the
// product (libgpdhg.so, the `cupdlp` Python package) links, loads or calls it; only
// tests/, __graft_entry__.smoke() and bench.py's CPU legs do.
//
// It follows the reference step for step, including its quirks:
//   * tau_0 = 1 / max|a_ij| of the scaled matrix (entrywise, not the operator norm),
//     src/primal_dual_hybrid_gradient_gpu.jl:569-571;
//   * the averaging weight is solver_state.step_size at entry of take_step!, i.e. the
//     step size before this iteration's update (:309 vs :412);
//   * the step-size exponents use the attempt counter total_number_iterations (:353,:405-409);
//   * K*x is kept incrementally, Kx += K*dx (:304);
//   * termination is evaluated on the UNSCALED average (src/iteration_stats_utils_gpu.jl:
//     447-502) while restarts are scored in scaled space (src/saddle_point_gpu.jl:250-278);
//   * primal/dual infeasibility is ignored while iteration < 10 (:688-690);
//   * evaluation every termination_evaluation_frequency iterations plus the first 10 (:627-630);
//   * the dual-ray objective includes the objective constant (src/iteration_stats_utils_gpu.jl:235,354).
// Reductions use a fixed chunking (4096 elements per partial, partials summed in order),
// so results do not depend on the OpenMP thread count.
//
// Build: oracle/build_oracle.py (g++ -O2 -fopenmp -ffp-contract=off), output in oracle/_build/.

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <random>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/gpdhg.h"

namespace {

using Vec = std::vector<double>;
constexpr double kInf = std::numeric_limits<double>::infinity();
#ifndef ORACLE_CHUNK
#define ORACLE_CHUNK 4096
#endif
constexpr int64_t kChunk = ORACLE_CHUNK;

// Julia's max/min propagate NaN; C's fmax does not.
inline double jmax(double a, double b) {
  if (a != a || b != b) return std::numeric_limits<double>::quiet_NaN();
  return a > b ? a : b;
}
inline double jmin(double a, double b) {
  if (a != a || b != b) return std::numeric_limits<double>::quiet_NaN();
  return a < b ? a : b;
}

template <class F>
void par_for(int64_t n, F f) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) f(i);
}

// Deterministic chunked sum of f(i), i in [0,n).
template <class F>
double chunk_sum(int64_t n, F f) {
  int64_t nc = (n + kChunk - 1) / kChunk;
  std::vector<double> part(std::max<int64_t>(nc, 1), 0.0);
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < nc; ++c) {
    double s = 0.0;
    int64_t e = std::min(n, (c + 1) * kChunk);
    for (int64_t i = c * kChunk; i < e; ++i) s += f(i);
    part[c] = s;
  }
  double s = 0.0;
  for (int64_t c = 0; c < nc; ++c) s += part[c];
  return s;
}

template <class F>
double chunk_max(int64_t n, F f) {
  int64_t nc = (n + kChunk - 1) / kChunk;
  std::vector<double> part(std::max<int64_t>(nc, 1), 0.0);
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < nc; ++c) {
    double s = 0.0;
    int64_t e = std::min(n, (c + 1) * kChunk);
    for (int64_t i = c * kChunk; i < e; ++i) s = jmax(s, f(i));
    part[c] = s;
  }
  double s = 0.0;
  for (int64_t c = 0; c < nc; ++c) s = jmax(s, part[c]);
  return s;
}

double dot(const Vec& a, const Vec& b) {
  return chunk_sum((int64_t)a.size(), [&](int64_t i) { return a[i] * b[i]; });
}
double norm2(const Vec& a) {
  return std::sqrt(chunk_sum((int64_t)a.size(), [&](int64_t i) { return a[i] * a[i]; }));
}
double norm_inf(const Vec& a) {
  return chunk_max((int64_t)a.size(), [&](int64_t i) { return std::fabs(a[i]); });
}

struct Csr {
  int64_t nrows = 0, ncols = 0;
  std::vector<int64_t> ptr;
  std::vector<int32_t> idx;
  Vec val;
};

Csr transpose(const Csr& a) {
  Csr t;
  t.nrows = a.ncols;
  t.ncols = a.nrows;
  t.ptr.assign(t.nrows + 1, 0);
  int64_t nnz = a.ptr[a.nrows];
  t.idx.resize(nnz);
  t.val.resize(nnz);
  for (int64_t k = 0; k < nnz; ++k) t.ptr[a.idx[k] + 1]++;
  for (int64_t j = 0; j < t.nrows; ++j) t.ptr[j + 1] += t.ptr[j];
  std::vector<int64_t> fill(t.ptr.begin(), t.ptr.end() - 1);
  for (int64_t i = 0; i < a.nrows; ++i)
    for (int64_t k = a.ptr[i]; k < a.ptr[i + 1]; ++k) {
      int64_t p = fill[a.idx[k]]++;
      t.idx[p] = (int32_t)i;
      t.val[p] = a.val[k];
    }
  return t;
}

// y = M * x, each row summed sequentially in storage order.
void spmv(const Csr& a, const Vec& x, Vec& y) {
  par_for(a.nrows, [&](int64_t i) {
    double s = 0.0;
#ifdef ORACLE_REVERSE_SPMV
    for (int64_t k = a.ptr[i + 1] - 1; k >= a.ptr[i]; --k) s += a.val[k] * x[a.idx[k]];
#else
    for (int64_t k = a.ptr[i]; k < a.ptr[i + 1]; ++k) s += a.val[k] * x[a.idx[k]];
#endif
    y[i] = s;
  });
}

// CuLinearProgrammingProblem, src/cpu_to_gpu.jl:1-14 (host arrays).
struct Lp {
  int64_t n = 0, m = 0, neq = 0;
  Csr A, At;
  Vec l, u, c, b;
  std::vector<uint8_t> finl, finu;
  double obj_const = 0.0;
};

void set_finite_masks(Lp& p) {
  p.finl.resize(p.n);
  p.finu.resize(p.n);
  for (int64_t j = 0; j < p.n; ++j) {
    p.finl[j] = std::isfinite(p.l[j]);
    p.finu[j] = std::isfinite(p.u[j]);
  }
}

// --------------------------------------------------------------------------------
// Preprocessing: src/preprocess.jl:329-675 (LP case, objective_matrix == 0).
// --------------------------------------------------------------------------------

// scale_problem, src/preprocess.jl:541-561: A <- E^-1 A D^-1 computed as
// ((1/E_i) * a_ij) * (1/D_j); c ./= D; bounds .*= D; b ./= E.
void scale_problem(Lp& p, const Vec& con, const Vec& var) {
  for (int64_t j = 0; j < p.n; ++j) {
    p.c[j] /= var[j];
    p.u[j] *= var[j];
    p.l[j] *= var[j];
  }
  for (int64_t i = 0; i < p.m; ++i) p.b[i] /= con[i];
  for (int64_t i = 0; i < p.m; ++i) {
    double ir = 1.0 / con[i];
    for (int64_t k = p.A.ptr[i]; k < p.A.ptr[i + 1]; ++k) {
      double ic = 1.0 / var[p.A.idx[k]];
      p.A.val[k] = (ir * p.A.val[k]) * ic;
    }
  }
}

void col_max_abs(const Lp& p, Vec& out) {
  out.assign(p.n, 0.0);
  for (int64_t i = 0; i < p.m; ++i)
    for (int64_t k = p.A.ptr[i]; k < p.A.ptr[i + 1]; ++k)
      out[p.A.idx[k]] = std::max(out[p.A.idx[k]], std::fabs(p.A.val[k]));
}
void row_max_abs(const Lp& p, Vec& out) {
  out.assign(p.m, 0.0);
  for (int64_t i = 0; i < p.m; ++i)
    for (int64_t k = p.A.ptr[i]; k < p.A.ptr[i + 1]; ++k) out[i] = std::max(out[i], std::fabs(p.A.val[k]));
}

// ruiz_rescaling with p = Inf, src/preprocess.jl:398-463.
void ruiz_rescaling(Lp& p, int iters, Vec& cum_con, Vec& cum_var) {
  cum_con.assign(p.m, 1.0);
  cum_var.assign(p.n, 1.0);
  Vec var, con;
  for (int it = 0; it < iters; ++it) {
    col_max_abs(p, var);
    for (auto& v : var) v = std::sqrt(v);
    for (auto& v : var)
      if (v == 0.0) v = 1.0;
    row_max_abs(p, con);
    for (auto& v : con) v = std::sqrt(v);
    for (auto& v : con)
      if (v == 0.0) v = 1.0;
    scale_problem(p, con, var);
    for (int64_t i = 0; i < p.m; ++i) cum_con[i] *= con[i];
    for (int64_t j = 0; j < p.n; ++j) cum_var[j] *= var[j];
  }
}

// l2_norm, src/preprocess.jl:89-103 (scaled by the max |a| to avoid overflow).
void l2_norm_cols(const Lp& p, Vec& out) {
  Vec mx;
  col_max_abs(p, mx);
  for (auto& v : mx)
    if (v == 0.0) v = 1.0;
  out.assign(p.n, 0.0);
  for (int64_t i = 0; i < p.m; ++i)
    for (int64_t k = p.A.ptr[i]; k < p.A.ptr[i + 1]; ++k) {
      double t = p.A.val[k] * (1.0 / mx[p.A.idx[k]]);
      out[p.A.idx[k]] += t * t;
    }
  for (int64_t j = 0; j < p.n; ++j) out[j] = mx[j] * std::sqrt(out[j]);
}
void l2_norm_rows(const Lp& p, Vec& out) {
  Vec mx;
  row_max_abs(p, mx);
  for (auto& v : mx)
    if (v == 0.0) v = 1.0;
  out.assign(p.m, 0.0);
  for (int64_t i = 0; i < p.m; ++i) {
    double s = 0.0;
    for (int64_t k = p.A.ptr[i]; k < p.A.ptr[i + 1]; ++k) {
      double t = (1.0 / mx[i]) * p.A.val[k];
      s += t * t;
    }
    out[i] = mx[i] * std::sqrt(s);
  }
}

// l2_norm_rescaling, src/preprocess.jl:344-358.
void l2_norm_rescaling(Lp& p, Vec& con, Vec& var) {
  l2_norm_rows(p, con);
  l2_norm_cols(p, var);
  for (auto& v : con)
    if (v == 0.0) v = 1.0;
  for (auto& v : var)
    if (v == 0.0) v = 1.0;
  for (auto& v : var) v = std::sqrt(v);
  for (auto& v : con) v = std::sqrt(v);
  scale_problem(p, con, var);
}

// pock_chambolle_rescaling, src/preprocess.jl:494-525.
void pock_chambolle_rescaling(Lp& p, double alpha, Vec& con, Vec& var) {
  var.assign(p.n, 0.0);
  con.assign(p.m, 0.0);
  for (int64_t i = 0; i < p.m; ++i)
    for (int64_t k = p.A.ptr[i]; k < p.A.ptr[i + 1]; ++k)
      var[p.A.idx[k]] += std::pow(std::fabs(p.A.val[k]), 2.0 - alpha);
  for (int64_t i = 0; i < p.m; ++i) {
    double s = 0.0;
    for (int64_t k = p.A.ptr[i]; k < p.A.ptr[i + 1]; ++k) s += std::pow(std::fabs(p.A.val[k]), alpha);
    con[i] = s;
  }
  for (auto& v : var) v = std::sqrt(v);
  for (auto& v : con) v = std::sqrt(v);
  for (auto& v : var)
    if (v == 0.0) v = 1.0;
  for (auto& v : con)
    if (v == 0.0) v = 1.0;
  scale_problem(p, con, var);
}

// rescale_problem, src/preprocess.jl:619-675.
void rescale_problem(int ruiz, bool l2, double pc_alpha, Lp& p, Vec& con, Vec& var) {
  con.assign(p.m, 1.0);
  var.assign(p.n, 1.0);
  Vec c1, v1;
  if (ruiz > 0) {
    ruiz_rescaling(p, ruiz, c1, v1);
    for (int64_t i = 0; i < p.m; ++i) con[i] *= c1[i];
    for (int64_t j = 0; j < p.n; ++j) var[j] *= v1[j];
  }
  if (l2) {
    l2_norm_rescaling(p, c1, v1);
    for (int64_t i = 0; i < p.m; ++i) con[i] *= c1[i];
    for (int64_t j = 0; j < p.n; ++j) var[j] *= v1[j];
  }
  if (!std::isnan(pc_alpha)) {
    pock_chambolle_rescaling(p, pc_alpha, c1, v1);
    for (int64_t i = 0; i < p.m; ++i) con[i] *= c1[i];
    for (int64_t j = 0; j < p.n; ++j) var[j] *= v1[j];
  }
}

// --------------------------------------------------------------------------------
// Residuals and statistics: src/iteration_stats_utils_gpu.jl:23-372.
// --------------------------------------------------------------------------------

struct PrimalRes {   // compute_primal_residual! (:71-94) reduced to norms
  double linf, sumsq;
};

PrimalRes primal_residual(const Lp& p, const Vec& x, const Vec& Kx, const Vec& l, const Vec& u, const Vec* b) {
  // constraint violation (:26-45): eq rows b - Kx, ineq rows max(b - Kx, 0)
  auto cv = [&](int64_t i) {
    double bi = b ? (*b)[i] : 0.0;
    double v = bi - Kx[i];
    return i < p.neq ? v : jmax(v, 0.0);
  };
  auto lv = [&](int64_t j) { return jmax(l[j] - x[j], 0.0); };
  auto uv = [&](int64_t j) { return jmax(x[j] - u[j], 0.0); };
  PrimalRes r;
  r.linf = jmax(chunk_max(p.m, [&](int64_t i) { return std::fabs(cv(i)); }),
                jmax(chunk_max(p.n, [&](int64_t j) { return std::fabs(lv(j)); }),
                     chunk_max(p.n, [&](int64_t j) { return std::fabs(uv(j)); })));
  r.sumsq = chunk_sum(p.m, [&](int64_t i) { double v = cv(i); return v * v; }) +
            chunk_sum(p.n, [&](int64_t j) { double v = lv(j); return v * v; }) +
            chunk_sum(p.n, [&](int64_t j) { double v = uv(j); return v * v; });
  return r;
}

struct DualStats {   // compute_dual_stats! (:216-238) reduced to scalars
  double dual_objective;
  double res_inf;    // norm([dual_residual; reduced_costs_violation], Inf)
  double res_sumsq;  // squared 2-norm of the same concatenation
  double rc_inf;     // norm(reduced_costs, Inf)
};

// reduced costs (:157-174), dual residual (:198-211), objective contribution (:110-152).
DualStats dual_stats(const Lp& p, const Vec& y, const Vec& grad, const Vec& l, const Vec& u, const Vec& b) {
  auto rc = [&](int64_t j) {
    double g = grad[j];
    return (p.finl[j] ? jmax(g, 0.0) : 0.0) + (p.finu[j] ? jmin(g, 0.0) : 0.0);
  };
  auto rcv = [&](int64_t j) { return grad[j] - rc(j); };
  int64_t nineq = p.m - p.neq;
  auto dr = [&](int64_t k) { return jmax(-y[p.neq + k], 0.0); };
  DualStats s;
  s.res_inf = jmax(chunk_max(nineq, [&](int64_t k) { return std::fabs(dr(k)); }),
                   chunk_max(p.n, [&](int64_t j) { return std::fabs(rcv(j)); }));
  s.res_sumsq = chunk_sum(nineq, [&](int64_t k) { double v = dr(k); return v * v; }) +
                chunk_sum(p.n, [&](int64_t j) { double v = rcv(j); return v * v; });
  double base = dot(b, y) + p.obj_const;
  double contrib = chunk_sum(p.n, [&](int64_t j) {
    double r = rc(j);
    if (r > 0.0) return l[j] * r;
    if (r < 0.0) return u[j] * r;
    return 0.0;
  });
  s.dual_objective = base + contrib;
  s.rc_inf = chunk_max(p.n, [&](int64_t j) { return std::fabs(rc(j)); });
  return s;
}

struct QpCache {   // CachedQuadraticProgramInfo, src/termination.jl:123-137
  double linf_c, linf_b, l2_c, l2_b;
};

// compute_convergence_information, :251-309.
gpdhg_convergence_information convergence_info(const Lp& p, const QpCache& qc, const Vec& x, const Vec& y,
                                               double eps_ratio, const Vec& Kx, const Vec& grad) {
  gpdhg_convergence_information ci;
  std::memset(&ci, 0, sizeof(ci));
  PrimalRes pr = primal_residual(p, x, Kx, p.l, p.u, &p.b);
  ci.primal_objective = p.obj_const + dot(p.c, x);
  ci.l_inf_primal_residual = pr.linf;
  ci.l2_primal_residual = std::sqrt(pr.sumsq);
  ci.relative_l_inf_primal_residual = ci.l_inf_primal_residual / (eps_ratio + qc.linf_b);
  ci.relative_l2_primal_residual = ci.l2_primal_residual / (eps_ratio + qc.l2_b);
  ci.l_inf_primal_variable = norm_inf(x);
  ci.l2_primal_variable = norm2(x);
  DualStats ds = dual_stats(p, y, grad, p.l, p.u, p.b);
  ci.dual_objective = ds.dual_objective;
  ci.l_inf_dual_residual = ds.res_inf;
  ci.l2_dual_residual = std::sqrt(ds.res_sumsq);
  ci.relative_l_inf_dual_residual = ci.l_inf_dual_residual / (eps_ratio + qc.linf_c);
  ci.relative_l2_dual_residual = ci.l2_dual_residual / (eps_ratio + qc.l2_c);
  ci.l_inf_dual_variable = norm_inf(y);
  ci.l2_dual_variable = norm2(y);
  ci.corrected_dual_objective = ds.res_inf == 0.0 ? ds.dual_objective : -kInf;
  double gap = std::fabs(ci.primal_objective - ci.dual_objective);
  double abs_obj = std::fabs(ci.primal_objective) + std::fabs(ci.dual_objective);
  ci.relative_optimality_gap = gap / (eps_ratio + abs_obj);
  ci.candidate_type = GPDHG_POINT_TYPE_AVERAGE_ITERATE;
  return ci;
}

// compute_infeasibility_information, :314-372.
gpdhg_infeasibility_information infeasibility_info(const Lp& p, const Vec& x, const Vec& y, const Vec& Kx,
                                                   const Vec& grad) {
  gpdhg_infeasibility_information ii;
  std::memset(&ii, 0, sizeof(ii));
  double s = norm_inf(x);
  Vec xr = x, Kxr = Kx;
  if (s != 0.0) {
    for (auto& v : xr) v /= s;
    for (auto& v : Kxr) v /= s;
  }
  // ray problem: bounds 0 where finite, +-Inf elsewhere; right-hand side 0 (:335-338)
  Vec lr(p.n), ur(p.n);
  for (int64_t j = 0; j < p.n; ++j) {
    lr[j] = p.finl[j] ? 0.0 : -kInf;
    ur[j] = p.finu[j] ? 0.0 : kInf;
  }
  PrimalRes pr = primal_residual(p, xr, Kxr, lr, ur, nullptr);
  ii.max_primal_ray_infeasibility = pr.linf;
  ii.primal_ray_linear_objective = dot(p.c, xr);
  // dual ray: objective zero, original bounds and rhs; gradient - c (:346-354)
  Vec gr(p.n);
  for (int64_t j = 0; j < p.n; ++j) gr[j] = grad[j] - p.c[j];
  DualStats ds = dual_stats(p, y, gr, p.l, p.u, p.b);
  double sf = jmax(norm_inf(y), ds.rc_inf);
  if (sf != 0.0) {
    ii.max_dual_ray_infeasibility = ds.res_inf / sf;
    ii.dual_ray_objective = ds.dual_objective / sf;
  } else {
    ii.max_dual_ray_infeasibility = 0.0;
    ii.dual_ray_objective = 0.0;
  }
  ii.candidate_type = GPDHG_POINT_TYPE_AVERAGE_ITERATE;
  return ii;
}

// --------------------------------------------------------------------------------
// Termination: src/termination.jl:142-246.
// --------------------------------------------------------------------------------
int check_termination(const gpdhg_params& cr, const QpCache& qc, const gpdhg_iteration_stats& st) {
  const auto& ci = st.convergence_information;
  double abs_obj = std::fabs(ci.primal_objective) + std::fabs(ci.dual_objective);
  double gap = std::fabs(ci.primal_objective - ci.dual_objective);
  double pe, pb, de, db;
  if (cr.optimality_norm == GPDHG_L_INF) {
    pe = ci.l_inf_primal_residual;
    pb = qc.linf_b;
    de = ci.l_inf_dual_residual;
    db = qc.linf_c;
  } else {
    pe = ci.l2_primal_residual;
    pb = qc.l2_b;
    de = ci.l2_dual_residual;
    db = qc.l2_c;
  }
  double a = cr.eps_optimal_absolute, r = cr.eps_optimal_relative;
  if (de < a + r * db && pe < a + r * pb && gap < a + r * abs_obj) return GPDHG_TERMINATION_REASON_OPTIMAL;
  const auto& ii = st.infeasibility_information;
  if (ii.dual_ray_objective > 0.0 &&
      ii.max_dual_ray_infeasibility / ii.dual_ray_objective <= cr.eps_primal_infeasible)
    return GPDHG_TERMINATION_REASON_PRIMAL_INFEASIBLE;
  if (ii.primal_ray_linear_objective < 0.0 &&
      ii.max_primal_ray_infeasibility / (-ii.primal_ray_linear_objective) <= cr.eps_dual_infeasible)
    return GPDHG_TERMINATION_REASON_DUAL_INFEASIBLE;
  if (st.iteration_number >= cr.iteration_limit) return GPDHG_TERMINATION_REASON_ITERATION_LIMIT;
  if (st.cumulative_kkt_matrix_passes >= cr.kkt_matrix_pass_limit)
    return GPDHG_TERMINATION_REASON_KKT_MATRIX_PASS_LIMIT;
  if (st.cumulative_time_sec >= cr.time_sec_limit) return GPDHG_TERMINATION_REASON_TIME_LIMIT;
  return 0;
}

// --------------------------------------------------------------------------------
// The solve loop: src/primal_dual_hybrid_gradient_gpu.jl:457-798 and
// src/saddle_point_gpu.jl:63-785.
// --------------------------------------------------------------------------------

struct WeightedAverage {   // CuSolutionWeightedAverage, src/saddle_point_gpu.jl:71-80
  Vec sx, sy;
  int64_t cx = 0, cy = 0;
  double wx = 0.0, wy = 0.0;
  Vec sKx, sKty;
};

struct RestartInfo {       // CuRestartInfo, src/saddle_point_gpu.jl:280-335
  Vec x, y;
  int64_t last_len = 1;
  double pdist = 0.0, ddist = 0.0, ratio_last = 1.0;
  Vec Kx, grad;
};

// compute_weight_kkt_residual, src/saddle_point_gpu.jl:250-278 (scaled problem).
double weighted_kkt(const Lp& p, const Vec& x, const Vec& y, const Vec& Kx, const Vec& grad, double pw) {
  PrimalRes pr = primal_residual(p, x, Kx, p.l, p.u, &p.b);
  double pobj = p.obj_const + dot(p.c, x);
  double l2p = std::sqrt(pr.sumsq);
  DualStats ds = dual_stats(p, y, grad, p.l, p.u, p.b);
  double l2d = std::sqrt(ds.res_sumsq);
  double g = std::fabs(pobj - ds.dual_objective);
  return std::sqrt(pw * l2p * l2p + 1.0 / pw * l2d * l2d + g * g);
}

// power_method_failure_probability / estimate_maximum_singular_value, :139-172.
// The start vector comes from std::mt19937_64 + normal_distribution (seed 1), not
// Julia's MersenneTwister; the iteration count only depends on the dimension.
double power_method_failure_probability(int64_t dim, double eps, int64_t k) {
  if (k < 2 || eps <= 0.0) return 1.0;
  return std::min(0.824, 0.354 / std::sqrt(eps * (k - 1))) * std::sqrt((double)dim) *
         std::pow(1.0 - eps, (double)k - 0.5);
}

double estimate_max_singular_value(const Lp& p, double pfail, double rel_err, int64_t* iters) {
  double eps = 1.0 - (1.0 - rel_err) * (1.0 - rel_err);
  std::mt19937_64 rng(1);
  std::normal_distribution<double> nd;
  Vec x(p.n), t(p.m), z(p.n);
  for (auto& v : x) v = nd(rng);
  int64_t k = 0;
  while (power_method_failure_probability(p.n, eps, k) > pfail) {
    double nx = norm2(x);
    for (auto& v : x) v /= nx;
    spmv(p.A, x, t);
    spmv(p.At, t, z);
    x = z;
    ++k;
  }
  spmv(p.A, x, t);
  spmv(p.At, t, z);
  double nx = norm2(x);
  *iters = k;
  return std::sqrt(dot(x, z) / (nx * nx));
}

struct Solver {
  const gpdhg_params& P;
  Lp& s;            // scaled problem
  const Lp& o;      // original problem (vectors only are used)
  const Vec& con;   // constraint_rescaling
  const Vec& var;   // variable_rescaling
  QpCache qc;

  // CuPdhgSolverState, :26-39
  Vec x, y, Kx, Kty;
  WeightedAverage avg;
  double step = 0.0, pw = 1.0;
  bool numerical_error = false;
  double kkt_passes = 0.0;
  int64_t total_iters = 0;
  // CuBufferState, :42-46
  Vec dx, dy, dKx;
  // CuBufferAvgState
  Vec ax, ay, aKx, agrad;
  Vec grad;   // buffer_primal_gradient
  RestartInfo ri;
  int64_t accepted = 0, rejected = 0;
  // Decision margins (test diagnostics): the smallest relative distance of any discrete
  // decision to its threshold since the last evaluation. A tiny margin means round-off
  // alone can flip the decision, so implementations with different summation orders may
  // legitimately diverge from there on.
  double pending_margin = kInf;
  bool greedy_equivalent = false;  // a KKT_GREEDY tie between two numerically equal points
  std::vector<double>* margins = nullptr;
  static double rel_gap(double a, double b) {
    double d = std::fabs(a - b), s = std::max(std::fabs(a), std::fabs(b));
    return s > 0.0 ? d / s : (d > 0.0 ? kInf : 0.0);
  }
  void note(double margin) { pending_margin = std::min(pending_margin, margin); }

  Solver(const gpdhg_params& p, Lp& sc, const Lp& orig, const Vec& c_, const Vec& v_)
      : P(p), s(sc), o(orig), con(c_), var(v_) {}

  // compute_next_primal_solution_kernel!, :177-197
  void next_primal(double tau) {
    par_for(s.n, [&](int64_t j) {
      double v = x[j] - (tau / pw) * (s.c[j] - Kty[j]);
      v = jmin(s.u[j], jmax(s.l[j], v));
      dx[j] = v - x[j];
    });
    spmv(s.A, dx, dKx);   // :225
  }

  // compute_next_dual_solution_kernel!, :232-260 (extrapolation coefficient 1)
  void next_dual(double tau) {
    par_for(s.m, [&](int64_t i) {
      double v = y[i] + (pw * tau) * (s.b[i] - 2.0 * dKx[i] - 1.0 * Kx[i]);
      if (i >= s.neq) v = jmax(v, 0.0);
      dy[i] = v - y[i];
    });
  }

  // update_solution_in_solver_state! + add_to_solution_weighted_average!,
  // :297-319 and src/saddle_point_gpu.jl:131-221
  void update_solution() {
    par_for(s.n, [&](int64_t j) { x[j] += dx[j]; });
    par_for(s.m, [&](int64_t i) { Kx[i] += dKx[i]; });
    par_for(s.m, [&](int64_t i) { y[i] += dy[i]; });
    spmv(s.At, y, Kty);
    double w = step;
    par_for(s.n, [&](int64_t j) { avg.sx[j] += x[j] * w; });
    avg.cx++;
    avg.wx += w;
    par_for(s.m, [&](int64_t i) { avg.sy[i] += y[i] * w; });
    avg.cy++;
    avg.wy += w;
    par_for(s.m, [&](int64_t i) { avg.sKx[i] += Kx[i] * w; });
    par_for(s.n, [&](int64_t j) { avg.sKty[j] += Kty[j] * w; });
  }

  // take_step!(::AdaptiveStepsizeParams), :343-413
  void take_step_adaptive() {
    double tau = step;
    bool done = false;
    while (!done) {
      total_iters++;
      next_primal(tau);
      next_dual(tau);
      double inter = std::fabs(dot(dKx, dy));
      double ndx = norm2(dx), ndy = norm2(dy);
      double movement = 0.5 * pw * ndx * ndx + (0.5 / pw) * ndy * ndy;
      kkt_passes += 1.0;
      double limit;
      if (inter > 0.0) {
        limit = movement / inter;
        if (movement == 0.0) {
          numerical_error = true;
          break;
        }
      } else {
        limit = kInf;
      }
      if (std::isfinite(limit)) note(rel_gap(tau, limit));
      if (tau <= limit) {
        update_solution();
        done = true;
        accepted++;
      } else {
        rejected++;
      }
      double k1 = (double)(total_iters + 1);
      double first = (1.0 - 1.0 / std::pow(k1, P.reduction_exponent)) * limit;
      double second = (1.0 + 1.0 / std::pow(k1, P.growth_exponent)) * tau;
      tau = jmin(first, second);
    }
    step = tau;
  }

  // take_step!(::ConstantStepsizeParams), :418-452
  void take_step_constant() {
    next_primal(step);
    next_dual(step);
    kkt_passes += 1.0;
    update_solution();
    accepted++;
  }

  // compute_average!, src/saddle_point_gpu.jl:226-240
  void compute_average() {
    par_for(s.n, [&](int64_t j) { ax[j] = avg.sx[j] / avg.wx; });
    par_for(s.m, [&](int64_t i) { ay[i] = avg.sy[i] / avg.wy; });
    par_for(s.m, [&](int64_t i) { aKx[i] = avg.sKx[i] / avg.wx; });
    par_for(s.n, [&](int64_t j) {
      double g = -avg.sKty[j] / avg.wy;
      agrad[j] = g + s.c[j];
    });
  }

  // evaluate_unscaled_iteration_stats, src/iteration_stats_utils_gpu.jl:447-502
  gpdhg_iteration_stats evaluate(int64_t iteration, double time_sec) {
    Vec xo(s.n), go(s.n), yo(s.m), Kxo(s.m);
    par_for(s.n, [&](int64_t j) {
      xo[j] = ax[j] / var[j];
      go[j] = agrad[j] * var[j];
    });
    par_for(s.m, [&](int64_t i) {
      yo[i] = ay[i] / con[i];
      Kxo[i] = aKx[i] * con[i];
    });
    gpdhg_iteration_stats st;
    std::memset(&st, 0, sizeof(st));
    st.iteration_number = (int32_t)(iteration - 1);
    st.cumulative_kkt_matrix_passes = kkt_passes;
    st.cumulative_time_sec = time_sec;
    st.convergence_information =
        convergence_info(o, qc, xo, yo, P.eps_optimal_absolute / P.eps_optimal_relative, Kxo, go);
    st.infeasibility_information = infeasibility_info(o, xo, yo, Kxo, go);
    st.step_size = step;
    st.primal_weight = pw;
    st.precision = GPDHG_PRECISION_FP64;
    return st;
  }

  // run_restart_scheme, src/saddle_point_gpu.jl:479-622, with should_reset_to_average
  // (:419-429), should_do_adaptive_restart_kkt (:434-473), update_last_restart_info!
  // (:659-692) and reset_solution_weighted_average! (:111-126).
  int run_restart_scheme(int64_t iterations_completed, double pnp, double dnp) {
    if (!(avg.cx > 0 && avg.cy > 0)) return GPDHG_RESTART_CHOICE_NO_RESTART;
    int64_t restart_length = avg.cx;
    bool do_restart = false, artificial = false;
    if ((double)restart_length >= P.artificial_restart_threshold * (double)iterations_completed) {
      do_restart = true;
      artificial = true;
    }
    (void)artificial;
    bool reset_to_average;
    double candidate = std::numeric_limits<double>::quiet_NaN();
    if (P.restart_scheme == GPDHG_NO_RESTARTS) {
      reset_to_average = false;
    } else {
      double cur = weighted_kkt(s, x, y, Kx, grad, pw);
      double av = weighted_kkt(s, ax, ay, aKx, agrad, pw);
      reset_to_average = P.restart_to_current_metric == GPDHG_KKT_GREEDY ? (cur >= av) : true;
      if (P.restart_to_current_metric == GPDHG_KKT_GREEDY && rel_gap(cur, av) < 1e-9) {
        double dxn = std::sqrt(chunk_sum(s.n, [&](int64_t j) { double d = ax[j] - x[j]; return d * d; }));
        double dyn = std::sqrt(chunk_sum(s.m, [&](int64_t i) { double d = ay[i] - y[i]; return d * d; }));
        if (dxn <= 1e-12 * (1.0 + norm2(x)) && dyn <= 1e-12 * (1.0 + norm2(y)))
          greedy_equivalent = true;   // either choice restarts from the same point
        else
          note(rel_gap(cur, av));
      }
      candidate = reset_to_average ? av : cur;
    }
    if (!do_restart) {
      if (P.restart_scheme == GPDHG_ADAPTIVE_KKT) {
        double last = weighted_kkt(s, ri.x, ri.y, ri.Kx, ri.grad, pw);
        double ratio = candidate / last;
        note(rel_gap(ratio, P.necessary_reduction_for_restart));
        note(rel_gap(ratio, P.sufficient_reduction_for_restart));
        if (ratio < P.necessary_reduction_for_restart && ratio >= P.sufficient_reduction_for_restart)
          note(rel_gap(ratio, ri.ratio_last));
        if (ratio < P.necessary_reduction_for_restart) {
          if (ratio < P.sufficient_reduction_for_restart)
            do_restart = true;
          else if (ratio > ri.ratio_last)
            do_restart = true;
        }
        ri.ratio_last = ratio;
      } else if (P.restart_scheme == GPDHG_FIXED_FREQUENCY && P.restart_frequency_if_fixed <= restart_length) {
        do_restart = true;
      }
    }
    if (!do_restart) return GPDHG_RESTART_CHOICE_NO_RESTART;
    if (reset_to_average) {
      x = ax;
      y = ay;
      Kx = aKx;
      par_for(s.n, [&](int64_t j) { Kty[j] = s.c[j] - agrad[j]; });
      grad = agrad;
    }
    std::fill(avg.sx.begin(), avg.sx.end(), 0.0);
    std::fill(avg.sy.begin(), avg.sy.end(), 0.0);
    avg.cx = avg.cy = 0;
    avg.wx = avg.wy = 0.0;
    std::fill(avg.sKx.begin(), avg.sKx.end(), 0.0);
    std::fill(avg.sKty.begin(), avg.sKty.end(), 0.0);
    // update_last_restart_info!
    double dxn = std::sqrt(chunk_sum(s.n, [&](int64_t j) { double d = ax[j] - ri.x[j]; return d * d; }));
    double dyn = std::sqrt(chunk_sum(s.m, [&](int64_t i) { double d = ay[i] - ri.y[i]; return d * d; }));
    ri.pdist = std::sqrt(pnp) * dxn / std::sqrt(pw);
    ri.ddist = std::sqrt(dnp) * dyn * std::sqrt(pw);
    ri.x = x;
    ri.y = y;
    ri.last_len = restart_length;
    ri.Kx = Kx;
    ri.grad = grad;
    return reset_to_average ? GPDHG_RESTART_CHOICE_RESTART_TO_AVERAGE : GPDHG_RESTART_CHOICE_WEIGHTED_AVERAGE_RESET;
  }

  // compute_new_primal_weight, src/saddle_point_gpu.jl:627-654
  double new_primal_weight() {
    const double eps = std::numeric_limits<double>::epsilon();
    if (ri.pdist > eps && ri.ddist > eps) {
      double est = ri.ddist / ri.pdist;
      double th = P.primal_weight_update_smoothing;
      double lpw = th * std::log(est) + (1.0 - th) * std::log(pw);
      return std::exp(lpw);
    }
    return pw;
  }

  int run(gpdhg_result* res, std::vector<gpdhg_iteration_stats>& history, int max_stats) {
    const int64_t n = s.n, m = s.m;
    qc.linf_c = norm_inf(o.c);
    qc.linf_b = norm_inf(o.b);
    qc.l2_c = norm2(o.c);
    qc.l2_b = norm2(o.b);
    x.assign(n, 0.0);
    y.assign(m, 0.0);
    Kx.assign(m, 0.0);
    Kty.assign(n, 0.0);
    avg.sx.assign(n, 0.0);
    avg.sy.assign(m, 0.0);
    avg.sKx.assign(m, 0.0);
    avg.sKty.assign(n, 0.0);
    dx.assign(n, 0.0);
    dy.assign(m, 0.0);
    dKx.assign(m, 0.0);
    ax.assign(n, 0.0);
    ay.assign(m, 0.0);
    aKx.assign(m, 0.0);
    agrad.assign(n, 0.0);
    grad.resize(n);
    for (int64_t j = 0; j < n; ++j) grad[j] = s.c[j] - Kty[j];

    if (P.step_size_policy == GPDHG_STEPSIZE_ADAPTIVE) {
      kkt_passes += 0.5;
      double amax = 0.0;
      for (double v : s.A.val) amax = jmax(amax, std::fabs(v));
      // The reference cannot reach this point with an empty matrix (its launch with an
      // empty grid fails first); 1/0 would make every averaging weight infinite.
      step = amax > 0.0 ? 1.0 / amax : 1.0;
    } else {
      const double rel = 0.2;
      int64_t k = 0;
      double smax = estimate_max_singular_value(s, 0.001, rel, &k);
      step = (1.0 - rel) / smax;
      kkt_passes += (double)k;
    }
    if (P.scale_invariant_initial_primal_weight) {
      // select_initial_primal_weight, src/saddle_point_gpu.jl:767-785
      double rhs = std::sqrt(1.0) * norm2(s.b);
      double obj = std::sqrt(1.0) * norm2(s.c);
      pw = (obj > 0.0 && rhs > 0.0) ? P.primal_importance * (obj / rhs) : P.primal_importance;
    } else {
      pw = P.primal_importance;
    }
    // create_last_restart_info, src/saddle_point_gpu.jl:317-335
    ri.x = x;
    ri.y = y;
    ri.Kx = Kx;
    ri.grad = grad;

    auto t0 = std::chrono::steady_clock::now();
    auto now = [&]() { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); };
    double basic_time = 0.0;
    numerical_error = false;
    int64_t iteration = 0;
    const int64_t freq = P.termination_evaluation_frequency;
    while (true) {
      ++iteration;
      if ((iteration - 1) % freq == 0 || iteration == (int64_t)P.iteration_limit + 1 || iteration <= 10 ||
          numerical_error) {
        kkt_passes += 2.0;
        if (numerical_error || avg.cx == 0 || avg.cy == 0) {
          ax = x;
          ay = y;
          aKx = Kx;
          agrad = grad;
        } else {
          compute_average();
        }
        gpdhg_iteration_stats st = evaluate(iteration, now());
        st.time_spent_doing_basic_algorithm = basic_time;
        int reason = check_termination(P, qc, st);
        if (numerical_error && reason == 0) reason = GPDHG_TERMINATION_REASON_NUMERICAL_ERROR;
        if (iteration < 10 && (reason == GPDHG_TERMINATION_REASON_PRIMAL_INFEASIBLE ||
                               reason == GPDHG_TERMINATION_REASON_DUAL_INFEASIBLE))
          reason = 0;
        bool pushed = false;
        if (P.record_iteration_stats || reason != 0) {
          if ((int)history.size() < max_stats) {
            history.push_back(st);
            pushed = true;
            if (margins) margins->push_back(pending_margin);
          }
        }
        pending_margin = kInf;
        {  // optimality tests of check_termination_criteria, relative distance to threshold
          const auto& ci = st.convergence_information;
          const double a = P.eps_optimal_absolute, r = P.eps_optimal_relative;
          const bool l2n = P.optimality_norm != GPDHG_L_INF;
          note(rel_gap(l2n ? ci.l2_dual_residual : ci.l_inf_dual_residual, a + r * (l2n ? qc.l2_c : qc.linf_c)));
          note(rel_gap(l2n ? ci.l2_primal_residual : ci.l_inf_primal_residual, a + r * (l2n ? qc.l2_b : qc.linf_b)));
          note(rel_gap(std::fabs(ci.primal_objective - ci.dual_objective),
                       a + r * (std::fabs(ci.primal_objective) + std::fabs(ci.dual_objective))));
        }
        greedy_equivalent = false;
        if (reason != 0) {
          std::memset(res, 0, sizeof(*res));
          res->termination_reason = reason;
          res->iteration_count = (int32_t)(iteration - 1);
          res->total_number_iterations = total_iters;
          res->cumulative_kkt_matrix_passes = kkt_passes;
          res->solve_time_sec = now();
          res->num_iteration_stats = (int32_t)history.size();
          res->fp64_handoff_iteration = -1;
          st.restart_used = GPDHG_RESTART_CHOICE_UNSPECIFIED;
          res->last_iteration_stats = st;
          res->accepted_steps = accepted;
          res->rejected_steps = rejected;
          return 0;
        }
        for (int64_t j = 0; j < n; ++j) grad[j] = s.c[j] - Kty[j];
        double pnp = 1.0 / step * pw, dnp = 1.0 / step / pw;   // define_norms, :49-56
        int rc = run_restart_scheme(iteration - 1, pnp, dnp);
        if (pushed) history.back().restart_used = rc;
        if (pushed && greedy_equivalent) history.back().cumulative_rejected_steps = -1;  // marker, see oracle.py
        if (rc != GPDHG_RESTART_CHOICE_NO_RESTART) pw = new_primal_weight();
      }
      double tb = now();
      if (P.step_size_policy == GPDHG_STEPSIZE_ADAPTIVE)
        take_step_adaptive();
      else
        take_step_constant();
      basic_time += now() - tb;
    }
  }
};

bool build_lp(const gpdhg_lp_desc* d, Lp& p, bool use_original) {
  p.n = d->num_variables;
  p.m = d->num_constraints;
  p.neq = d->num_equalities;
  p.obj_const = d->objective_constant;
  auto pick = [&](const double* scaled, const double* orig) { return (use_original && orig) ? orig : scaled; };
  const double* l = pick(d->variable_lower_bound, d->original_variable_lower_bound);
  const double* u = pick(d->variable_upper_bound, d->original_variable_upper_bound);
  const double* c = pick(d->objective_vector, d->original_objective_vector);
  const double* b = pick(d->right_hand_side, d->original_right_hand_side);
  p.l.assign(l, l + p.n);
  p.u.assign(u, u + p.n);
  p.c.assign(c, c + p.n);
  p.b.assign(b, b + p.m);
  set_finite_masks(p);
  if (!use_original) {
    p.A.nrows = p.m;
    p.A.ncols = p.n;
    p.A.ptr.resize(p.m + 1);
    for (int64_t i = 0; i <= p.m; ++i) p.A.ptr[i] = d->row_ptr[i];
    int64_t nnz = p.A.ptr[p.m];
    p.A.idx.assign(d->col_idx, d->col_idx + nnz);
    p.A.val.assign(d->values, d->values + nnz);
  }
  return true;
}

// validate, src/preprocess.jl:8-74 (LP subset: sizes, NaN/Inf).
int validate(const gpdhg_lp_desc* d) {
  if (!d || d->num_variables < 0 || d->num_constraints < 0 || d->num_equalities < 0 ||
      d->num_equalities > d->num_constraints)
    return GPDHG_ERR_INVALID_ARGUMENT;
  for (int64_t j = 0; j < d->num_variables; ++j) {
    if (d->variable_lower_bound[j] == kInf || d->variable_upper_bound[j] == -kInf) return GPDHG_ERR_INVALID_PROBLEM;
    if (std::isnan(d->variable_lower_bound[j]) || std::isnan(d->variable_upper_bound[j]))
      return GPDHG_ERR_INVALID_PROBLEM;
    if (!std::isfinite(d->objective_vector[j])) return GPDHG_ERR_INVALID_PROBLEM;
  }
  for (int64_t i = 0; i < d->num_constraints; ++i)
    if (!std::isfinite(d->right_hand_side[i])) return GPDHG_ERR_INVALID_PROBLEM;
  int64_t nnz = d->row_ptr[d->num_constraints];
  for (int64_t k = 0; k < nnz; ++k)
    if (!std::isfinite(d->values[k])) return GPDHG_ERR_INVALID_PROBLEM;
  return 0;
}

int solve_scaled_impl(const gpdhg_lp_desc* d, const gpdhg_params* params, gpdhg_result* res, double* x_avg,
                      double* y_avg, double* x_cur, double* y_cur, gpdhg_iteration_stats* stats, int max_stats,
                      double* margins_out = nullptr) {
  Lp s, o;
  build_lp(d, s, false);
  s.At = transpose(s.A);
  build_lp(d, o, true);
  Vec con(s.m, 1.0), var(s.n, 1.0);
  if (d->constraint_rescaling) con.assign(d->constraint_rescaling, d->constraint_rescaling + s.m);
  if (d->variable_rescaling) var.assign(d->variable_rescaling, d->variable_rescaling + s.n);
  Solver sv(*params, s, o, con, var);
  std::vector<gpdhg_iteration_stats> hist;
  std::vector<double> margins;
  sv.margins = &margins;
  int rc = sv.run(res, hist, max_stats);
  if (margins_out) std::copy(margins.begin(), margins.end(), margins_out);
  if (x_avg) std::copy(sv.ax.begin(), sv.ax.end(), x_avg);
  if (y_avg) std::copy(sv.ay.begin(), sv.ay.end(), y_avg);
  if (x_cur) std::copy(sv.x.begin(), sv.x.end(), x_cur);
  if (y_cur) std::copy(sv.y.begin(), sv.y.end(), y_cur);
  if (stats) std::copy(hist.begin(), hist.end(), stats);
  return rc;
}

}  // namespace

extern "C" {

int oracle_set_threads(int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
  return omp_get_max_threads();
#else
  (void)nthreads;
  return 1;
#endif
}

// rescale_problem on an unscaled problem given as CSR: writes the scaled CSR values
// (same pattern), scaled vectors, and the cumulative rescaling vectors.
int oracle_rescale_problem(const gpdhg_lp_desc* d, int ruiz_iterations, int l2_norm_rescaling,
                           double pock_chambolle_alpha, double* values_out, double* l_out, double* u_out,
                           double* c_out, double* b_out, double* con_out, double* var_out) {
  int v = validate(d);
  if (v) return v;
  Lp p;
  build_lp(d, p, false);
  Vec con, var;
  rescale_problem(ruiz_iterations, l2_norm_rescaling != 0, pock_chambolle_alpha, p, con, var);
  std::copy(p.A.val.begin(), p.A.val.end(), values_out);
  std::copy(p.l.begin(), p.l.end(), l_out);
  std::copy(p.u.begin(), p.u.end(), u_out);
  std::copy(p.c.begin(), p.c.end(), c_out);
  std::copy(p.b.begin(), p.b.end(), b_out);
  std::copy(con.begin(), con.end(), con_out);
  std::copy(var.begin(), var.end(), var_out);
  return 0;
}

// The loop on an already-scaled problem (same descriptor contract as gpdhg_solve).
// x_avg/y_avg: scaled averaged output (what the reference copies to the host);
// x_cur/y_cur: scaled current iterate. Any output may be NULL.
// margins (optional, max_stats entries): for each recorded evaluation, the smallest
// relative distance of a discrete decision (accept/reject, restart tests, termination
// tests) to its threshold between the previous evaluation and this one.
int oracle_solve_scaled(const gpdhg_lp_desc* d, const gpdhg_params* params, gpdhg_result* res, double* x_avg,
                        double* y_avg, double* x_cur, double* y_cur, gpdhg_iteration_stats* stats,
                        int max_stats, double* margins) {
  int v = validate(d);
  if (v) return v;
  if (d->num_variables == 0) return GPDHG_ERR_INVALID_PROBLEM;
  return solve_scaled_impl(d, params, res, x_avg, y_avg, x_cur, y_cur, stats, max_stats, margins);
}

// optimize(): validate, rescale, loop, unscale (x ./ var, y ./ con).
int oracle_optimize(const gpdhg_lp_desc* d, const gpdhg_params* params, gpdhg_result* res, double* x_out,
                    double* y_out, gpdhg_iteration_stats* stats, int max_stats) {
  int v = validate(d);
  if (v) return v;
  if (d->num_variables == 0) return GPDHG_ERR_INVALID_PROBLEM;
  Lp p;
  build_lp(d, p, false);
  Vec con, var;
  rescale_problem(params->l_inf_ruiz_iterations, params->l2_norm_rescaling != 0, params->pock_chambolle_alpha, p,
                  con, var);
  std::vector<int32_t> rp(p.m + 1);
  for (int64_t i = 0; i <= p.m; ++i) rp[i] = (int32_t)p.A.ptr[i];
  gpdhg_lp_desc sd = *d;
  sd.row_ptr = rp.data();
  sd.values = p.A.val.data();
  sd.variable_lower_bound = p.l.data();
  sd.variable_upper_bound = p.u.data();
  sd.objective_vector = p.c.data();
  sd.right_hand_side = p.b.data();
  sd.original_variable_lower_bound = d->variable_lower_bound;
  sd.original_variable_upper_bound = d->variable_upper_bound;
  sd.original_objective_vector = d->objective_vector;
  sd.original_right_hand_side = d->right_hand_side;
  sd.constraint_rescaling = con.data();
  sd.variable_rescaling = var.data();
  Vec xa(p.n), ya(p.m);
  int rc = solve_scaled_impl(&sd, params, res, xa.data(), ya.data(), nullptr, nullptr, stats, max_stats);
  if (x_out)
    for (int64_t j = 0; j < p.n; ++j) x_out[j] = xa[j] / var[j];
  if (y_out)
    for (int64_t i = 0; i < p.m; ++i) y_out[i] = ya[i] / con[i];
  return rc;
}

}  // extern "C"
