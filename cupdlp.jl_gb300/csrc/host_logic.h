// host_logic.h — the reference's scalar decision logic, shared by the single-LP and
// the batched solver so both take exactly the same decisions from the same numbers.
//
//   check_termination     check_termination_criteria, src/termination.jl:142-246
//   assemble_stats        compute_convergence_information / compute_infeasibility_information,
//                         src/iteration_stats_utils_gpu.jl:251-372 (from FP64 reductions)
//   decide_restart        run_restart_scheme + should_reset_to_average +
//                         should_do_adaptive_restart_kkt + update_last_restart_info! +
//                         compute_new_primal_weight, src/saddle_point_gpu.jl:419-692
//   eval_due / next_eval_after   the evaluation cadence of optimize(), :627-630
#pragma once

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <vector>

#include "eval_kernels.cuh"

namespace gpdhg {

constexpr long long kPowTableLen = 1 << 18;
// Fills t with [1 - (k+1)^-r, 1 + (k+1)^-g] for k < kPowTableLen (take_step!, :405-407).
void fill_pow_table(std::vector<double>& t, double r, double g);

// CachedQuadraticProgramInfo (src/termination.jl:123-137) plus the objective constant.
struct InstanceInfo {
  double obj_const = 0.0;
  double linf_c = 0.0, linf_b = 0.0, l2_c = 0.0, l2_b = 0.0;
};

// CuRestartInfo scalars (src/saddle_point_gpu.jl:280-312).
struct RestartMemory {
  long long last_len = 1;
  double pdist = 0.0, ddist = 0.0, ratio_last = 1.0;
};

inline double jmax_h(double a, double b) {
  if (a != a || b != b) return a + b;
  return a > b ? a : b;
}

inline int check_termination(const gpdhg_params& cr, const InstanceInfo& qi, const gpdhg_iteration_stats& st) {
  const auto& ci = st.convergence_information;
  const double abs_obj = std::fabs(ci.primal_objective) + std::fabs(ci.dual_objective);
  const double gap = std::fabs(ci.primal_objective - ci.dual_objective);
  double pe, pb, de, db;
  if (cr.optimality_norm == GPDHG_L_INF) {
    pe = ci.l_inf_primal_residual; pb = qi.linf_b; de = ci.l_inf_dual_residual; db = qi.linf_c;
  } else {
    pe = ci.l2_primal_residual; pb = qi.l2_b; de = ci.l2_dual_residual; db = qi.l2_c;
  }
  const double a = cr.eps_optimal_absolute, r = cr.eps_optimal_relative;
  if (de < a + r * db && pe < a + r * pb && gap < a + r * abs_obj) return GPDHG_TERMINATION_REASON_OPTIMAL;
  const auto& ii = st.infeasibility_information;
  if (ii.dual_ray_objective > 0.0 && ii.max_dual_ray_infeasibility / ii.dual_ray_objective <= cr.eps_primal_infeasible)
    return GPDHG_TERMINATION_REASON_PRIMAL_INFEASIBLE;
  if (ii.primal_ray_linear_objective < 0.0 &&
      ii.max_primal_ray_infeasibility / (-ii.primal_ray_linear_objective) <= cr.eps_dual_infeasible)
    return GPDHG_TERMINATION_REASON_DUAL_INFEASIBLE;
  if (st.iteration_number >= cr.iteration_limit) return GPDHG_TERMINATION_REASON_ITERATION_LIMIT;
  if (st.cumulative_kkt_matrix_passes >= cr.kkt_matrix_pass_limit) return GPDHG_TERMINATION_REASON_KKT_MATRIX_PASS_LIMIT;
  if (st.cumulative_time_sec >= cr.time_sec_limit) return GPDHG_TERMINATION_REASON_TIME_LIMIT;
  return 0;
}

inline void assemble_stats(const InstanceInfo& qi, const gpdhg_params& prm, const double* en, const double* em,
                           gpdhg_iteration_stats& st) {
  const double eps_ratio = prm.eps_optimal_absolute / prm.eps_optimal_relative;
  auto& ci = st.convergence_information;
  ci.candidate_type = GPDHG_POINT_TYPE_AVERAGE_ITERATE;
  ci.primal_objective = qi.obj_const + en[kN_Cx];
  ci.l_inf_primal_residual = jmax_h(em[kM_CvMax], en[kN_LuMax]);
  ci.l2_primal_residual = std::sqrt(em[kM_CvSq] + en[kN_LuSq]);
  ci.relative_l_inf_primal_residual = ci.l_inf_primal_residual / (eps_ratio + qi.linf_b);
  ci.relative_l2_primal_residual = ci.l2_primal_residual / (eps_ratio + qi.l2_b);
  ci.l_inf_primal_variable = en[kN_XMax];
  ci.l2_primal_variable = std::sqrt(en[kN_XSq]);
  const double dual_res_inf = jmax_h(em[kM_DrMax], en[kN_RcvMax]);
  ci.dual_objective = em[kM_By] + qi.obj_const + en[kN_Contrib];
  ci.l_inf_dual_residual = dual_res_inf;
  ci.l2_dual_residual = std::sqrt(em[kM_DrSq] + en[kN_RcvSq]);
  ci.relative_l_inf_dual_residual = ci.l_inf_dual_residual / (eps_ratio + qi.linf_c);
  ci.relative_l2_dual_residual = ci.l2_dual_residual / (eps_ratio + qi.l2_c);
  ci.l_inf_dual_variable = em[kM_YMax];
  ci.l2_dual_variable = std::sqrt(em[kM_YSq]);
  ci.corrected_dual_objective = dual_res_inf == 0.0 ? ci.dual_objective : -std::numeric_limits<double>::infinity();
  const double gap = std::fabs(ci.primal_objective - ci.dual_objective);
  const double abs_obj = std::fabs(ci.primal_objective) + std::fabs(ci.dual_objective);
  ci.relative_optimality_gap = gap / (eps_ratio + abs_obj);

  auto& ii = st.infeasibility_information;
  ii.candidate_type = GPDHG_POINT_TYPE_AVERAGE_ITERATE;
  const double s = en[kN_XMax];
  const double scale = (s != 0.0) ? s : 1.0;
  ii.max_primal_ray_infeasibility = jmax_h(em[kM_RayCvMax], en[kN_RayLuMax]) / scale;
  ii.primal_ray_linear_objective = en[kN_Cx] / scale;
  const double res_inf_r = jmax_h(em[kM_DrMax], en[kN_RayRcvMax]);
  const double dual_obj_r = em[kM_By] + qi.obj_const + en[kN_RayContrib];
  const double sf = jmax_h(em[kM_YMax], en[kN_RayRcMax]);
  if (sf != 0.0) {
    ii.max_dual_ray_infeasibility = res_inf_r / sf;
    ii.dual_ray_objective = dual_obj_r / sf;
  } else {
    ii.max_dual_ray_infeasibility = 0.0;
    ii.dual_ray_objective = 0.0;
  }
}

inline double relative_kkt(const gpdhg_iteration_stats& st, int norm) {
  const auto& ci = st.convergence_information;
  if (norm == GPDHG_L_INF)
    return std::max({ci.relative_l_inf_primal_residual, ci.relative_l_inf_dual_residual, ci.relative_optimality_gap});
  return std::max({ci.relative_l2_primal_residual, ci.relative_l2_dual_residual, ci.relative_optimality_gap});
}

inline bool eval_due(long long it, long long freq, long long iteration_limit, bool numerical_error) {
  return (it - 1) % freq == 0 || it == iteration_limit + 1 || it <= 10 || numerical_error;
}

inline long long next_eval_after(long long it, long long freq, long long iteration_limit) {
  long long best = ((it - 1) / freq + 1) * freq + 1;
  if (it + 1 <= 10) best = std::min(best, it + 1);
  if (iteration_limit + 1 > it) best = std::min(best, iteration_limit + 1);
  return best;
}

struct RestartDecision {
  int restart_used = GPDHG_RESTART_CHOICE_NO_RESTART;
  bool reset_to_average = false;
  double new_omega = 0.0;
};

// kn / km: the KktN / KktM reductions (points 0 = current, 1 = average, 2 = last restart;
// kn[12] = ||avg x - last x||^2, km[9] = ||avg y - last y||^2). `count_primal` is
// sum_primal_solutions_count, `tau`/`omega` the current step size and primal weight.
inline RestartDecision decide_restart(const gpdhg_params& prm, const InstanceInfo& qi, long long count_primal,
                                      double tau, double omega, long long iterations_completed, const double* kn,
                                      const double* km, RestartMemory& mem) {
  RestartDecision d;
  d.new_omega = omega;
  auto wkkt = [&](int q) {
    const double l2p = std::sqrt(km[3 * q + 0] + kn[4 * q + 0]);
    const double pobj = qi.obj_const + kn[4 * q + 1];
    const double l2d = std::sqrt(km[3 * q + 1] + kn[4 * q + 2]);
    const double dobj = km[3 * q + 2] + qi.obj_const + kn[4 * q + 3];
    const double g = std::fabs(pobj - dobj);
    return std::sqrt(omega * l2p * l2p + 1.0 / omega * l2d * l2d + g * g);
  };
  const long long restart_length = count_primal;
  bool do_restart = (double)restart_length >= prm.artificial_restart_threshold * (double)iterations_completed;
  bool reset_to_average;
  double candidate = std::numeric_limits<double>::quiet_NaN();
  if (prm.restart_scheme == GPDHG_NO_RESTARTS) {
    reset_to_average = false;
  } else {
    const double cur = wkkt(0), avg = wkkt(1);
    reset_to_average = prm.restart_to_current_metric == GPDHG_KKT_GREEDY ? (cur >= avg) : true;
    candidate = reset_to_average ? avg : cur;
  }
  if (!do_restart) {
    if (prm.restart_scheme == GPDHG_ADAPTIVE_KKT) {
      const double ratio = candidate / wkkt(2);
      if (ratio < prm.necessary_reduction_for_restart) {
        if (ratio < prm.sufficient_reduction_for_restart)
          do_restart = true;
        else if (ratio > mem.ratio_last)
          do_restart = true;
      }
      mem.ratio_last = ratio;
    } else if (prm.restart_scheme == GPDHG_FIXED_FREQUENCY && prm.restart_frequency_if_fixed <= restart_length) {
      do_restart = true;
    }
  }
  if (!do_restart) return d;
  d.reset_to_average = reset_to_average;
  d.restart_used =
      reset_to_average ? GPDHG_RESTART_CHOICE_RESTART_TO_AVERAGE : GPDHG_RESTART_CHOICE_WEIGHTED_AVERAGE_RESET;
  const double pnp = 1.0 / tau * omega, dnp = 1.0 / tau / omega;   // define_norms (:49-56)
  mem.pdist = std::sqrt(pnp) * std::sqrt(kn[12]) / std::sqrt(omega);
  mem.ddist = std::sqrt(dnp) * std::sqrt(km[9]) * std::sqrt(omega);
  mem.last_len = restart_length;
  const double eps = std::numeric_limits<double>::epsilon();
  if (mem.pdist > eps && mem.ddist > eps) {
    const double est = mem.ddist / mem.pdist;
    const double th = prm.primal_weight_update_smoothing;
    d.new_omega = std::exp(th * std::log(est) + (1.0 - th) * std::log(omega));
  }
  return d;
}

}  // namespace gpdhg
