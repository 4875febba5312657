// abi.cu — extern "C" entry points of libgpdhg.so (declared in include/gpdhg.h).
// Every entry point catches everything: failures become a gpdhg_status plus a
// thread-local message, never an exception across the ABI.
#include <cmath>
#include <cstring>
#include <new>
#include <string>

#include "batch.h"
#include "problem.h"
#include "tiles.h"

namespace gpdhg {
void solve(gpdhg_problem* P, const gpdhg_params& prm, gpdhg_result* res, double* primal_out, double* dual_out);
void current_iterate(const gpdhg_problem* P, double* x, double* y);
void convergence_noalloc(int32_t n, int32_t m, int32_t neq, double obj_const, const double* l, const double* u,
                         const double* c, const double* b, const double* x, const double* y, const double* ax,
                         const double* aty, double eps_abs, double eps_rel, void* stream,
                         gpdhg_convergence_information* out);
}  // namespace gpdhg

namespace {

thread_local std::string g_last_error;

template <class F>
gpdhg_status guarded(F f) {
  try {
    f();
    g_last_error.clear();
    return GPDHG_OK;
  } catch (const gpdhg::Error& e) {
    g_last_error = e.what();
    return e.status;
  } catch (const std::bad_alloc&) {
    g_last_error = "host allocation failed";
    return GPDHG_ERR_OUT_OF_MEMORY;
  } catch (const std::exception& e) {
    g_last_error = e.what();
    return GPDHG_ERR_INTERNAL;
  } catch (...) {
    g_last_error = "unknown error";
    return GPDHG_ERR_INTERNAL;
  }
}

// Parameter checks of the reference: construct_restart_parameters' assertions
// (src/saddle_point_gpu.jl:397-403), the primal_importance check
// (src/primal_dual_hybrid_gradient_gpu.jl:483-485) and validate_termination_criteria
// (src/termination.jl:101-117).
void check_params(const gpdhg_params* p) {
  using gpdhg::Error;
  if (!p) throw Error(GPDHG_ERR_INVALID_ARGUMENT, "params is NULL");
  if (!(p->primal_importance > 0.0) || !std::isfinite(p->primal_importance))
    throw Error(GPDHG_ERR_INVALID_ARGUMENT, "primal_importance must be positive and finite");
  if (p->termination_evaluation_frequency <= 0)
    throw Error(GPDHG_ERR_INVALID_ARGUMENT, "termination_evaluation_frequency must be positive");
  if (!(p->eps_optimal_relative > 0.0) && !(p->eps_optimal_absolute >= 0.0))
    throw Error(GPDHG_ERR_INVALID_ARGUMENT, "eps_optimal_* must be nonnegative");
  if (p->eps_primal_infeasible < 0 || p->eps_dual_infeasible < 0)
    throw Error(GPDHG_ERR_INVALID_ARGUMENT, "eps_*_infeasible must be nonnegative");
  if (p->restart_frequency_if_fixed <= 1) throw Error(GPDHG_ERR_INVALID_ARGUMENT, "restart_frequency_if_fixed must be > 1");
  if (!(p->artificial_restart_threshold > 0.0 && p->artificial_restart_threshold <= 1.0))
    throw Error(GPDHG_ERR_INVALID_ARGUMENT, "artificial_restart_threshold must be in (0, 1]");
  if (!(0.0 < p->sufficient_reduction_for_restart && p->sufficient_reduction_for_restart <= p->necessary_reduction_for_restart &&
        p->necessary_reduction_for_restart <= 1.0))
    throw Error(GPDHG_ERR_INVALID_ARGUMENT, "need 0 < sufficient <= necessary <= 1");
  if (!(p->primal_weight_update_smoothing >= 0.0 && p->primal_weight_update_smoothing <= 1.0))
    throw Error(GPDHG_ERR_INVALID_ARGUMENT, "primal_weight_update_smoothing must be in [0, 1]");
  if (p->step_size_policy != GPDHG_STEPSIZE_ADAPTIVE && p->step_size_policy != GPDHG_STEPSIZE_CONSTANT)
    throw Error(GPDHG_ERR_INVALID_ARGUMENT, "unknown step_size_policy");
  if (p->precision < GPDHG_PRECISION_FP64 || p->precision > GPDHG_PRECISION_FP32)
    throw Error(GPDHG_ERR_INVALID_ARGUMENT, "unknown precision");
  if (p->restart_scheme < GPDHG_NO_RESTARTS || p->restart_scheme > GPDHG_ADAPTIVE_KKT)
    throw Error(GPDHG_ERR_INVALID_ARGUMENT, "unknown restart_scheme");
  if (p->optimality_norm != GPDHG_L_INF && p->optimality_norm != GPDHG_L2)
    throw Error(GPDHG_ERR_INVALID_ARGUMENT, "unknown optimality_norm");
}

}  // namespace

extern "C" {

int32_t gpdhg_abi_version(void) { return GPDHG_ABI_VERSION; }

const char* gpdhg_last_error(void) { return g_last_error.c_str(); }

void gpdhg_default_params(gpdhg_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->l_inf_ruiz_iterations = 10;
  p->l2_norm_rescaling = 0;
  p->pock_chambolle_alpha = 1.0;
  p->primal_importance = 1.0;
  p->scale_invariant_initial_primal_weight = 1;
  p->verbosity = 2;
  p->record_iteration_stats = 1;
  p->termination_evaluation_frequency = 64;
  p->optimality_norm = GPDHG_L2;
  p->iteration_limit = 2147483647;
  p->eps_optimal_absolute = 1e-4;
  p->eps_optimal_relative = 1e-4;
  p->eps_primal_infeasible = 1e-8;
  p->eps_dual_infeasible = 1e-8;
  p->time_sec_limit = 3600.0;
  p->kkt_matrix_pass_limit = INFINITY;
  p->restart_scheme = GPDHG_ADAPTIVE_KKT;
  p->restart_to_current_metric = GPDHG_KKT_GREEDY;
  p->restart_frequency_if_fixed = 1000;
  p->artificial_restart_threshold = 0.36;
  p->sufficient_reduction_for_restart = 0.2;
  p->necessary_reduction_for_restart = 0.8;
  p->primal_weight_update_smoothing = 0.5;
  p->step_size_policy = GPDHG_STEPSIZE_ADAPTIVE;
  p->precision = GPDHG_PRECISION_FP64;
  p->reduction_exponent = 0.3;
  p->growth_exponent = 0.6;
  p->fp64_handoff_relative_kkt = 1e-6;
  p->fp64_handoff_stall_evaluations = 20;
}

gpdhg_status gpdhg_problem_create(const gpdhg_lp_desc* desc, gpdhg_problem** out) {
  return guarded([&] {
    if (!out) throw gpdhg::Error(GPDHG_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    gpdhg_problem* p = new gpdhg_problem();
    try {
      gpdhg::problem_init(p, desc);
    } catch (...) {
      delete p;
      throw;
    }
    *out = p;
  });
}

gpdhg_status gpdhg_solve(gpdhg_problem* p, const gpdhg_params* params, gpdhg_result* result, double* primal_out,
                         double* dual_out) {
  return guarded([&] {
    if (!p || !result) throw gpdhg::Error(GPDHG_ERR_INVALID_ARGUMENT, "problem or result is NULL");
    check_params(params);
    gpdhg::solve(p, *params, result, primal_out, dual_out);
    gpdhg::to_caller_columns(p->col_perm, primal_out);
  });
}

gpdhg_status gpdhg_problem_create_unscaled(const gpdhg_lp_desc* desc, const gpdhg_params* params,
                                           gpdhg_problem** out) {
  return guarded([&] {
    if (!out) throw gpdhg::Error(GPDHG_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    if (!desc || !params) throw gpdhg::Error(GPDHG_ERR_INVALID_ARGUMENT, "desc or params is NULL");
    if (desc->original_variable_lower_bound || desc->original_variable_upper_bound ||
        desc->original_objective_vector || desc->original_right_hand_side || desc->constraint_rescaling ||
        desc->variable_rescaling)
      throw gpdhg::Error(GPDHG_ERR_INVALID_ARGUMENT,
                         "an unscaled descriptor carries no original_* or rescaling vectors");
    if (params->l_inf_ruiz_iterations < 0)
      throw gpdhg::Error(GPDHG_ERR_INVALID_ARGUMENT, "l_inf_ruiz_iterations must be >= 0");
    gpdhg_problem* p = new gpdhg_problem();
    try {
      gpdhg::problem_init(p, desc);
      gpdhg::rescale_on_device(p, *params);
    } catch (...) {
      delete p;
      throw;
    }
    *out = p;
  });
}

gpdhg_status gpdhg_problem_create_csc(const gpdhg_lp_desc* desc, const int64_t* col_ptr, const int64_t* row_val,
                                      const double* nz_val, int32_t index_base, const gpdhg_params* unscaled_params,
                                      gpdhg_problem** out) {
  return guarded([&] {
    if (!out) throw gpdhg::Error(GPDHG_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    if (!desc) throw gpdhg::Error(GPDHG_ERR_INVALID_ARGUMENT, "desc is NULL");
    if (unscaled_params) {
      if (desc->original_variable_lower_bound || desc->original_variable_upper_bound ||
          desc->original_objective_vector || desc->original_right_hand_side || desc->constraint_rescaling ||
          desc->variable_rescaling)
        throw gpdhg::Error(GPDHG_ERR_INVALID_ARGUMENT,
                           "an unscaled descriptor carries no original_* or rescaling vectors");
      if (unscaled_params->l_inf_ruiz_iterations < 0)
        throw gpdhg::Error(GPDHG_ERR_INVALID_ARGUMENT, "l_inf_ruiz_iterations must be >= 0");
    }
    gpdhg_problem* p = new gpdhg_problem();
    try {
      gpdhg::problem_init_csc(p, desc, col_ptr, row_val, nz_val, index_base);
      if (unscaled_params) gpdhg::rescale_on_device(p, *unscaled_params);
    } catch (...) {
      delete p;
      throw;
    }
    *out = p;
  });
}

gpdhg_status gpdhg_problem_create_two_sided(const gpdhg_two_sided_desc* desc, const int64_t* col_ptr,
                                            const int64_t* row_val, const double* nz_val, int32_t index_base,
                                            const gpdhg_params* unscaled_params, gpdhg_problem** out) {
  return guarded([&] {
    if (!out) throw gpdhg::Error(GPDHG_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    if (!desc) throw gpdhg::Error(GPDHG_ERR_INVALID_ARGUMENT, "desc is NULL");
    if (unscaled_params && unscaled_params->l_inf_ruiz_iterations < 0)
      throw gpdhg::Error(GPDHG_ERR_INVALID_ARGUMENT, "l_inf_ruiz_iterations must be >= 0");
    gpdhg_problem* p = new gpdhg_problem();
    try {
      gpdhg::problem_init_two_sided(p, desc, col_ptr, row_val, nz_val, index_base);
      if (unscaled_params) gpdhg::rescale_on_device(p, *unscaled_params);
    } catch (...) {
      delete p;
      throw;
    }
    *out = p;
  });
}

gpdhg_status gpdhg_get_standard_form(const gpdhg_problem* p, int32_t* num_variables, int32_t* num_equalities,
                                     int32_t* num_slacks, int32_t* new_row_to_old) {
  return guarded([&] {
    if (!p) throw gpdhg::Error(GPDHG_ERR_INVALID_ARGUMENT, "problem is NULL");
    if (num_variables) *num_variables = p->n;
    if (num_equalities) *num_equalities = p->neq;
    if (num_slacks) *num_slacks = p->num_slacks;
    if (new_row_to_old)
      for (int32_t r = 0; r < p->m; ++r) new_row_to_old[r] = p->new_row_to_old.empty() ? r : p->new_row_to_old[r];
  });
}

gpdhg_status gpdhg_get_rescaling(const gpdhg_problem* p, double* constraint_rescaling, double* variable_rescaling) {
  return guarded([&] {
    if (!p) throw gpdhg::Error(GPDHG_ERR_INVALID_ARGUMENT, "problem is NULL");
    gpdhg::get_rescaling(p, constraint_rescaling, variable_rescaling);
    gpdhg::to_caller_columns(p->col_perm, variable_rescaling);
  });
}

gpdhg_status gpdhg_get_stats(const gpdhg_problem* p, int32_t index, gpdhg_iteration_stats* out) {
  return guarded([&] {
    if (!p || !out) throw gpdhg::Error(GPDHG_ERR_INVALID_ARGUMENT, "problem or out is NULL");
    if (index < 0 || (size_t)index >= p->history.size())
      throw gpdhg::Error(GPDHG_ERR_INVALID_ARGUMENT, "stats index out of range");
    *out = p->history[index];
  });
}

gpdhg_status gpdhg_set_warm_start(gpdhg_problem* p, const double* x0, const double* y0) {
  return guarded([&] {
    if (!p) throw gpdhg::Error(GPDHG_ERR_INVALID_ARGUMENT, "problem is NULL");
    p->warm_x.clear();
    p->warm_y.clear();
    if (x0) {
      p->warm_x.assign(x0, x0 + p->n);
      if (!p->col_perm.empty()) gpdhg::to_handle_columns(p->col_perm, x0, p->warm_x.data());
    }
    if (y0) p->warm_y.assign(y0, y0 + p->m);
  });
}

gpdhg_status gpdhg_get_current_iterate(const gpdhg_problem* p, double* x, double* y) {
  return guarded([&] {
    if (!p) throw gpdhg::Error(GPDHG_ERR_INVALID_ARGUMENT, "problem is NULL");
    gpdhg::current_iterate(p, x, y);
    gpdhg::to_caller_columns(p->col_perm, x);
  });
}

void* gpdhg_problem_stream(const gpdhg_problem* p) { return p ? (void*)p->stream : nullptr; }

gpdhg_status gpdhg_set_tile_override(int32_t precision, int32_t side, int32_t tile_nnz, int32_t e_floor,
                                     int32_t tpc_max) {
  return guarded([&] {
    if (precision != GPDHG_PRECISION_FP64 && precision != GPDHG_PRECISION_FP32)
      throw gpdhg::Error(GPDHG_ERR_INVALID_ARGUMENT, "precision must be FP64 or FP32");
    if (tile_nnz == 0) {
      gpdhg::set_tile_override(precision, side, nullptr);
      return;
    }
    const gpdhg::TileConfig c{tile_nnz, e_floor, tpc_max};
    gpdhg::set_tile_override(precision, side, &c);
  });
}

gpdhg_status gpdhg_batch_create(int32_t count, const gpdhg_lp_desc* descs, gpdhg_batch** out) {
  return guarded([&] {
    if (!out) throw gpdhg::Error(GPDHG_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    gpdhg_batch* b = new gpdhg_batch();
    try {
      gpdhg::batch_init(b, count, descs);
    } catch (...) {
      delete b;
      throw;
    }
    *out = b;
  });
}

gpdhg_status gpdhg_batch_solve(gpdhg_batch* b, const gpdhg_params* params, gpdhg_result* results,
                               double* const* primal_out, double* const* dual_out) {
  return guarded([&] {
    if (!b || !results) throw gpdhg::Error(GPDHG_ERR_INVALID_ARGUMENT, "batch or results is NULL");
    check_params(params);
    if (params->precision == GPDHG_PRECISION_FP32_REFINE)
      throw gpdhg::Error(GPDHG_ERR_NOT_SUPPORTED, "batched solves run in FP64 or FP32 (no FP64 hand-off)");
    if (params->step_size_policy != GPDHG_STEPSIZE_ADAPTIVE)
      throw gpdhg::Error(GPDHG_ERR_NOT_SUPPORTED, "batched solves use the adaptive step size");
    gpdhg::batch_solve(b, *params, results, primal_out, dual_out);
  });
}

gpdhg_status gpdhg_convergence_noalloc(int32_t num_variables, int32_t num_constraints, int32_t num_equalities,
                                       double objective_constant, const double* variable_lower_bound,
                                       const double* variable_upper_bound, const double* objective_vector,
                                       const double* right_hand_side, const double* primal, const double* dual,
                                       const double* primal_product, const double* dual_product,
                                       double eps_optimal_absolute, double eps_optimal_relative, void* stream,
                                       gpdhg_convergence_information* out) {
  return guarded([&] {
    gpdhg::convergence_noalloc(num_variables, num_constraints, num_equalities, objective_constant,
                               variable_lower_bound, variable_upper_bound, objective_vector, right_hand_side, primal,
                               dual, primal_product, dual_product, eps_optimal_absolute, eps_optimal_relative, stream,
                               out);
  });
}

double gpdhg_server_footprint(const gpdhg_lp_desc* desc, const gpdhg_params* params) {
  if (!desc || !params) return -1.0;
  return gpdhg::footprint_bytes(*desc, *params);
}

gpdhg_status gpdhg_server_create(const gpdhg_server_config* cfg, gpdhg_server** out) {
  return guarded([&] {
    if (!out) throw gpdhg::Error(GPDHG_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    gpdhg_server_config c{};
    if (cfg) c = *cfg;
    *out = gpdhg::server_create(c);
  });
}

gpdhg_status gpdhg_server_submit(gpdhg_server* s, const gpdhg_lp_desc* desc, const gpdhg_params* params,
                                 uint64_t* ticket) {
  return guarded([&] {
    if (!s || !desc || !ticket) throw gpdhg::Error(GPDHG_ERR_INVALID_ARGUMENT, "server, desc or ticket is NULL");
    check_params(params);
    *ticket = gpdhg::server_submit(s, *desc, *params);
  });
}

namespace {
gpdhg_status server_take(gpdhg_server* s, uint64_t ticket, double timeout_sec, gpdhg_result* result,
                         double* primal_out, double* dual_out) {
  gpdhg_status st = GPDHG_OK;
  const gpdhg_status g = guarded([&] {
    if (!s) throw gpdhg::Error(GPDHG_ERR_INVALID_ARGUMENT, "server is NULL");
    std::string err;
    st = gpdhg::server_take(s, ticket, timeout_sec, result, primal_out, dual_out, err);
    if (st == GPDHG_ERR_NOT_READY) err = "request has not terminated yet";
    if (st != GPDHG_OK) throw gpdhg::Error(st, err);
  });
  return g;
}
}  // namespace

gpdhg_status gpdhg_server_poll(gpdhg_server* s, uint64_t ticket, gpdhg_result* result, double* primal_out,
                               double* dual_out) {
  return server_take(s, ticket, 0.0, result, primal_out, dual_out);
}

gpdhg_status gpdhg_server_wait(gpdhg_server* s, uint64_t ticket, double timeout_sec, gpdhg_result* result,
                               double* primal_out, double* dual_out) {
  return server_take(s, ticket, timeout_sec > 0.0 ? timeout_sec : 0.0, result, primal_out, dual_out);
}

gpdhg_status gpdhg_server_destroy(gpdhg_server* s) {
  return guarded([&] { gpdhg::server_destroy(s); });
}

gpdhg_status gpdhg_batch_destroy(gpdhg_batch* b) {
  return guarded([&] { delete b; });
}

gpdhg_status gpdhg_problem_destroy(gpdhg_problem* p) {
  return guarded([&] { delete p; });
}

}  // extern "C"
