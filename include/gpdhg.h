/*
 * gpdhg.h — C ABI of libgpdhg.so, a GB300 (sm_103a) restarted-PDHG LP engine.
 *
 * The library replaces the GPU part of cuPDLP.jl's solve loop,
 *   optimize(params::PdhgParameters, problem::QuadraticProgrammingProblem)
 *   (src/primal_dual_hybrid_gradient_gpu.jl:457-798),
 * from the host->device transfer (src/primal_dual_hybrid_gradient_gpu.jl:488-490,
 * src/cpu_to_gpu.jl:26-81) up to the copy of the averaged iterate back to the host
 * (src/primal_dual_hybrid_gradient_gpu.jl:713-720, src/cpu_to_gpu.jl:86-94).
 * Validation, `rescale_problem` (src/preprocess.jl:619-675) and
 * `unscaled_saddle_point_output` (src/saddle_point_gpu.jl:40-61) stay with the
 * caller, exactly where the reference keeps them, so a caller hands the library the
 * already-scaled problem plus the original vectors and the two scaling vectors.
 *
 * Conventions
 *   - Every entry point returns a gpdhg_status; nothing throws across the ABI.
 *     gpdhg_last_error() returns a thread-local description of the last failure.
 *   - All arrays are plain host pointers owned by the caller; the library copies what
 *     it needs and owns every byte of device memory it allocates.
 *   - One handle per host thread; distinct handles may be used concurrently.
 *   - Indices are 0-based. Matrices are CSR with int32 indices.
 *   - Enum values equal the reference's Julia enums (0-based declaration order).
 */
#ifndef GPDHG_H
#define GPDHG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GPDHG_ABI_VERSION 1

typedef enum gpdhg_status {
  GPDHG_OK = 0,
  GPDHG_ERR_INVALID_ARGUMENT = 1, /* null pointer, negative size, bad parameter */
  GPDHG_ERR_INVALID_PROBLEM = 2,  /* validate() failure: sizes, NaN/Inf data */
  GPDHG_ERR_OUT_OF_MEMORY = 3,    /* device or host allocation failed */
  GPDHG_ERR_CUDA = 4,             /* any other CUDA runtime error */
  GPDHG_ERR_NOT_SUPPORTED = 5,    /* feature not available (e.g. quadratic objective) */
  GPDHG_ERR_ADMISSION = 6,        /* server: request can never fit the HBM budget */
  GPDHG_ERR_NOT_READY = 7,        /* server: result not available yet */
  GPDHG_ERR_DEVICE_TIMEOUT = 8,   /* a bounded device-side wait gave up */
  GPDHG_ERR_INTERNAL = 9
} gpdhg_status;

/* TerminationReason, src/solve_log.jl:323-334 (same values). */
enum {
  GPDHG_TERMINATION_REASON_UNSPECIFIED = 0,
  GPDHG_TERMINATION_REASON_OPTIMAL = 1,
  GPDHG_TERMINATION_REASON_PRIMAL_INFEASIBLE = 2,
  GPDHG_TERMINATION_REASON_DUAL_INFEASIBLE = 3,
  GPDHG_TERMINATION_REASON_TIME_LIMIT = 4,
  GPDHG_TERMINATION_REASON_ITERATION_LIMIT = 5,
  GPDHG_TERMINATION_REASON_KKT_MATRIX_PASS_LIMIT = 6,
  GPDHG_TERMINATION_REASON_NUMERICAL_ERROR = 7,
  GPDHG_TERMINATION_REASON_INVALID_PROBLEM = 8,
  GPDHG_TERMINATION_REASON_OTHER = 9
};

/* RestartChoice, src/solve_log.jl:19-24. */
enum {
  GPDHG_RESTART_CHOICE_UNSPECIFIED = 0,
  GPDHG_RESTART_CHOICE_NO_RESTART = 1,
  GPDHG_RESTART_CHOICE_WEIGHTED_AVERAGE_RESET = 2,
  GPDHG_RESTART_CHOICE_RESTART_TO_AVERAGE = 3
};

/* PointType, src/solve_log.jl:39-45. */
enum {
  GPDHG_POINT_TYPE_UNSPECIFIED = 0,
  GPDHG_POINT_TYPE_CURRENT_ITERATE = 1,
  GPDHG_POINT_TYPE_ITERATE_DIFFERENCE = 2,
  GPDHG_POINT_TYPE_AVERAGE_ITERATE = 3,
  GPDHG_POINT_TYPE_NONE = 4
};

/* OptimalityNorm, src/termination.jl:6. */
enum { GPDHG_L_INF = 0, GPDHG_L2 = 1 };

/* RestartScheme and RestartToCurrentMetric, src/saddle_point_gpu.jl:343,350. */
enum { GPDHG_NO_RESTARTS = 0, GPDHG_FIXED_FREQUENCY = 1, GPDHG_ADAPTIVE_KKT = 2 };
enum { GPDHG_NO_RESTART_TO_CURRENT = 0, GPDHG_KKT_GREEDY = 1 };

/* step_size_policy_params: AdaptiveStepsizeParams / ConstantStepsizeParams,
 * src/primal_dual_hybrid_gradient_gpu.jl:2-7. */
enum { GPDHG_STEPSIZE_ADAPTIVE = 0, GPDHG_STEPSIZE_CONSTANT = 1 };

/* Arithmetic of the bulk iteration (appended to PdhgParameters; no reference
 * counterpart: the reference runs everything in FP64). */
enum {
  GPDHG_PRECISION_FP64 = 0,        /* FP64 matrix, iterates and reductions */
  GPDHG_PRECISION_FP32_REFINE = 1, /* FP32 matrix/iterates, FP64 norms/scalars, then an FP64 phase */
  GPDHG_PRECISION_FP32 = 2         /* FP32 bulk only (FP64 norms/scalars), no FP64 phase */
};

/*
 * Solver parameters. The first block mirrors PdhgParameters
 * (src/primal_dual_hybrid_gradient_gpu.jl:9-24) with TerminationCriteria
 * (src/termination.jl:9-77), RestartParameters (src/saddle_point_gpu.jl:353-383) and
 * AdaptiveStepsizeParams flattened in, field for field and in the same order.
 * The rescaling fields (l_inf_ruiz_iterations, l2_norm_rescaling,
 * pock_chambolle_alpha) are read only by gpdhg_problem_create_unscaled().
 * Fields after `growth_exponent` are additions.
 */
typedef struct gpdhg_params {
  int32_t l_inf_ruiz_iterations;
  int32_t l2_norm_rescaling;       /* Bool */
  double pock_chambolle_alpha;     /* NaN means `nothing` */
  double primal_importance;
  int32_t scale_invariant_initial_primal_weight; /* Bool */
  int32_t verbosity;
  int32_t record_iteration_stats;  /* Bool */
  int32_t termination_evaluation_frequency;
  /* TerminationCriteria */
  int32_t optimality_norm;
  int32_t iteration_limit;
  double eps_optimal_absolute;
  double eps_optimal_relative;
  double eps_primal_infeasible;
  double eps_dual_infeasible;
  double time_sec_limit;
  double kkt_matrix_pass_limit;
  /* RestartParameters */
  int32_t restart_scheme;
  int32_t restart_to_current_metric;
  int64_t restart_frequency_if_fixed;
  double artificial_restart_threshold;
  double sufficient_reduction_for_restart;
  double necessary_reduction_for_restart;
  double primal_weight_update_smoothing;
  /* step_size_policy_params */
  int32_t step_size_policy;
  int32_t precision;               /* GPDHG_PRECISION_* (addition) */
  double reduction_exponent;
  double growth_exponent;
  /* additions */
  double fp64_handoff_relative_kkt; /* FP32_REFINE: switch to FP64 below this relative KKT error */
  int32_t fp64_handoff_stall_evaluations; /* FP32_REFINE: or after this many evaluations without progress */
  int32_t profile_kernels;         /* time every step kernel with CUDA events (result.*_kernel_sec) */
  double reserved[6];
} gpdhg_params;

/* ConvergenceInformation, src/solve_log.jl:51-155. */
typedef struct gpdhg_convergence_information {
  int32_t candidate_type;
  int32_t pad0;
  double primal_objective;
  double dual_objective;
  double corrected_dual_objective;
  double l_inf_primal_residual;
  double l2_primal_residual;
  double l_inf_dual_residual;
  double l2_dual_residual;
  double relative_l_inf_primal_residual;
  double relative_l2_primal_residual;
  double relative_l_inf_dual_residual;
  double relative_l2_dual_residual;
  double relative_optimality_gap;
  double l_inf_primal_variable;
  double l2_primal_variable;
  double l_inf_dual_variable;
  double l2_dual_variable;
} gpdhg_convergence_information;

/* InfeasibilityInformation, src/solve_log.jl:161-212. */
typedef struct gpdhg_infeasibility_information {
  int32_t candidate_type;
  int32_t pad0;
  double max_primal_ray_infeasibility;
  double primal_ray_linear_objective;
  double max_dual_ray_infeasibility;
  double dual_ray_objective;
} gpdhg_infeasibility_information;

/* IterationStats, src/solve_log.jl:219-302 (one convergence and one
 * infeasibility entry, as the reference always records). */
typedef struct gpdhg_iteration_stats {
  int32_t iteration_number;
  int32_t cumulative_rejected_steps;
  int32_t restart_used;            /* RestartChoice */
  int32_t precision;               /* GPDHG_PRECISION_FP64 or _FP32 phase that produced it */
  gpdhg_convergence_information convergence_information;
  gpdhg_infeasibility_information infeasibility_information;
  double cumulative_kkt_matrix_passes;
  double cumulative_time_sec;
  double step_size;
  double primal_weight;
  double time_spent_doing_basic_algorithm; /* method_specific_stats entry */
} gpdhg_iteration_stats;

typedef struct gpdhg_result {
  int32_t termination_reason;      /* TerminationReason */
  int32_t iteration_count;         /* SaddlePointOutput.iteration_count (= iteration - 1) */
  int64_t total_number_iterations; /* step attempts, accepted or rejected */
  double cumulative_kkt_matrix_passes;
  double solve_time_sec;           /* wall time from loop start to termination */
  int32_t num_iteration_stats;     /* entries readable with gpdhg_get_stats */
  int32_t fp64_handoff_iteration;  /* iteration at which the FP64 phase began, -1 if none */
  gpdhg_iteration_stats last_iteration_stats;
  /* measurement (additions): device time of the step loop, attempts per phase */
  double step_loop_device_sec;     /* CUDA-event time of all step launches */
  int64_t accepted_steps;
  int64_t rejected_steps;
  /* with params.profile_kernels: summed CUDA-event durations of the step kernels that did
   * work, and how many primal launches also ran the A'y product of a commit */
  double primal_kernel_sec;
  double dual_kernel_sec;
  int64_t primal_kernel_launches;
  int64_t primal_spmv_launches;
  int64_t kernels_launched;        /* every kernel this solve launched (graph nodes included) */
} gpdhg_result;

/*
 * Problem descriptor. The scaled problem is the output of rescale_problem
 * (src/preprocess.jl:619-675); the "original_*" vectors are the unscaled ones the
 * reference evaluates termination on (src/iteration_stats_utils_gpu.jl:447-502).
 * constraint_rescaling / variable_rescaling are ScaledQpProblem's vectors
 * (src/quadratic_programming.jl:284-289). Any original_* pointer or rescaling pointer
 * may be NULL, meaning "same as scaled" / "all ones".
 * Rows [0, num_equalities) are equalities, the rest are ">=" rows
 * (src/quadratic_programming.jl:6-24).
 */
typedef struct gpdhg_lp_desc {
  int32_t num_variables;           /* n */
  int32_t num_constraints;         /* m */
  int32_t num_equalities;
  int32_t pad0;
  int64_t nnz;
  const int32_t* row_ptr;          /* m+1, CSR of the scaled constraint matrix */
  const int32_t* col_idx;          /* nnz */
  const double* values;            /* nnz */
  const double* variable_lower_bound;  /* n, may hold -Inf */
  const double* variable_upper_bound;  /* n, may hold +Inf */
  const double* objective_vector;      /* n */
  const double* right_hand_side;       /* m */
  double objective_constant;
  const double* original_variable_lower_bound;
  const double* original_variable_upper_bound;
  const double* original_objective_vector;
  const double* original_right_hand_side;
  const double* constraint_rescaling;  /* m */
  const double* variable_rescaling;    /* n */
} gpdhg_lp_desc;

typedef struct gpdhg_problem gpdhg_problem;

/* Library identity and errors. */
int32_t gpdhg_abi_version(void);
const char* gpdhg_last_error(void);

/* Defaults of scripts/solve.jl:163-196 (the CLI) with tolerance 1e-4, i.e. the
 * reference's PdhgParameters(10, false, 1.0, 1.0, true, 2, true, 64, ...). */
void gpdhg_default_params(gpdhg_params* params);

/*
 * Replaces scaledqp_cpu_to_gpu + qp_cpu_to_gpu (src/cpu_to_gpu.jl:26-81): validates
 * the descriptor, uploads FP64 (and FP32) copies of the scaled matrix, builds CSR(A^T)
 * and the row schedules on the device, and returns a handle that owns it all.
 */
gpdhg_status gpdhg_problem_create(const gpdhg_lp_desc* desc, gpdhg_problem** out);

/*
 * Same, for an UNSCALED problem: the library runs rescale_problem
 * (src/preprocess.jl:619-675: Ruiz L-inf, optional L2, Pock-Chambolle) on the GPU with
 * the rescaling fields of `params`, then behaves as gpdhg_problem_create.
 * `desc` must have all original_* and rescaling pointers NULL. On success the scaling
 * vectors can be read back with gpdhg_get_rescaling.
 */
gpdhg_status gpdhg_problem_create_unscaled(const gpdhg_lp_desc* desc, const gpdhg_params* params,
                                           gpdhg_problem** out);
gpdhg_status gpdhg_get_rescaling(const gpdhg_problem* p, double* constraint_rescaling,
                                 double* variable_rescaling);

/*
 * The constraint matrix in compressed sparse COLUMNS, as Julia's SparseMatrixCSC holds it
 * (col_ptr: n+1, row_val: nnz, nz_val: nnz; index_base 1 for Julia's 1-based arrays, 0 for
 * 0-based ones). CSC(A) is CSR(A^T): the library uploads it as A^T and builds A on the
 * device (src/cpu_to_gpu.jl:45-46 builds the CSR copies from the CSC on the host). `desc`
 * gives the dimensions, nnz and the vectors; its row_ptr, col_idx and values must be NULL.
 * With `unscaled_params` NULL the data are the scaled problem, as for gpdhg_problem_create;
 * otherwise they are unscaled and rescaled on the device as by gpdhg_problem_create_unscaled
 * (then `desc` carries no original_* or rescaling vectors). For a CSC whose row indices
 * increase within each column the handle is the one the CSR of the same matrix gives.
 */
gpdhg_status gpdhg_problem_create_csc(const gpdhg_lp_desc* desc, const int64_t* col_ptr, const int64_t* row_val,
                                      const double* nz_val, int32_t index_base, const gpdhg_params* unscaled_params,
                                      gpdhg_problem** out);

/*
 * TwoSidedQpProblem (src/quadratic_programming_io.jl:5-22) with a zero objective matrix:
 * l <= x <= u and constraint_lower_bound <= A x <= constraint_upper_bound, as an MPS
 * reader returns it. The matrix is passed separately in compressed sparse columns.
 */
typedef struct gpdhg_two_sided_desc {
  int32_t num_variables;               /* n */
  int32_t num_constraints;             /* m */
  int64_t nnz;
  const double* variable_lower_bound;  /* n */
  const double* variable_upper_bound;  /* n */
  const double* constraint_lower_bound; /* m, may hold -Inf */
  const double* constraint_upper_bound; /* m, may hold +Inf */
  const double* objective_vector;      /* n */
  double objective_offset;
} gpdhg_two_sided_desc;

/*
 * transform_to_standard_form (src/quadratic_programming_io.jl:33-76, with
 * two_sided_rows_to_slacks :85-121 and row_permute_in_place, src/preprocess.jl:586-611)
 * done while the problem is built: each row with two finite, unequal bounds becomes
 * A x - s = 0 with a new variable s in [lower, upper] (appended after the n variables, in
 * row order); rows with only a finite upper bound are negated into ">=" rows; equality rows
 * move to the front, each block keeping its row order. The matrix (CSC, index base 0 or 1,
 * as for gpdhg_problem_create_csc) is uploaded once: the sign flips, the row renumbering,
 * the slack entries and both CSR copies are made on the device. With `unscaled_params` the
 * standard-form problem is then rescaled on the device as by gpdhg_problem_create_unscaled;
 * with NULL it is solved unscaled. A row with neither bound finite fails with
 * GPDHG_ERR_INVALID_PROBLEM, as the reference's error() does.
 */
gpdhg_status gpdhg_problem_create_two_sided(const gpdhg_two_sided_desc* desc, const int64_t* col_ptr,
                                            const int64_t* row_val, const double* nz_val, int32_t index_base,
                                            const gpdhg_params* unscaled_params, gpdhg_problem** out);
/*
 * The standard form a handle solves: its variable count (n plus one slack per two-sided
 * row), equality count, slack count and, in new_row_to_old (m entries, 0-based), the row
 * of the caller's problem behind each standard-form row (the reference's new_row_to_old).
 * For a handle not made by gpdhg_problem_create_two_sided: n, num_equalities, 0 and the
 * identity. Any output pointer may be NULL.
 */
gpdhg_status gpdhg_get_standard_form(const gpdhg_problem* p, int32_t* num_variables, int32_t* num_equalities,
                                     int32_t* num_slacks, int32_t* new_row_to_old);

/*
 * Runs the restarted PDHG loop of optimize() (src/primal_dual_hybrid_gradient_gpu.jl:
 * 494-797) on the handle's problem from a zero starting point (or the warm start set
 * with gpdhg_set_warm_start). On return `primal_out` (n) and `dual_out` (m) hold the
 * SCALED averaged iterate that the reference copies to the host at :713-720; the
 * caller unscales it (unscaled_saddle_point_output). Either output pointer may be NULL.
 */
gpdhg_status gpdhg_solve(gpdhg_problem* p, const gpdhg_params* params, gpdhg_result* result,
                         double* primal_out, double* dual_out);

/* The per-evaluation IterationStats history of the last solve (the reference pushes
 * one per evaluation when record_iteration_stats, else only the final one: :694-696). */
gpdhg_status gpdhg_get_stats(const gpdhg_problem* p, int32_t index, gpdhg_iteration_stats* out);

/* Optional scaled starting point (x0: n, y0: m) for the next solve; NULL clears it.
 * No reference counterpart (the reference always starts from zero, :494-507). */
gpdhg_status gpdhg_set_warm_start(gpdhg_problem* p, const double* x0, const double* y0);

/* The scaled CURRENT iterate (not the average) at the end of the last solve, for
 * diagnostics and step-level parity checks (solver_state.current_primal_solution /
 * current_dual_solution, src/primal_dual_hybrid_gradient_gpu.jl:26-39). */
gpdhg_status gpdhg_get_current_iterate(const gpdhg_problem* p, double* x, double* y);

gpdhg_status gpdhg_problem_destroy(gpdhg_problem* p);

/* The cudaStream_t (as void*) every kernel of this handle runs on, so a caller can
 * order its own work or record CUDA events around gpdhg_solve. */
void* gpdhg_problem_stream(const gpdhg_problem* p);

/* ---------------------------------------------------------------------------------
 * Batched solve: many independent LPs packed into one segmented CSR and advanced
 * together by persistent kernels, each instance with its own step size, primal
 * weight, restart and termination state. No reference counterpart beyond calling
 * optimize() once per instance.
 * ------------------------------------------------------------------------------- */
typedef struct gpdhg_batch gpdhg_batch;

gpdhg_status gpdhg_batch_create(int32_t count, const gpdhg_lp_desc* descs, gpdhg_batch** out);
/* results: `count` entries; primal_out[i] / dual_out[i] may be NULL (or the arrays
 * themselves NULL). Each instance terminates under its own criteria. */
gpdhg_status gpdhg_batch_solve(gpdhg_batch* b, const gpdhg_params* params, gpdhg_result* results,
                               double* const* primal_out, double* const* dual_out);
gpdhg_status gpdhg_batch_destroy(gpdhg_batch* b);

/* ---------------------------------------------------------------------------------
 * Allocation-free evaluation. No counterpart in the reference.
 *
 * The reference's termination statistics (ConvergenceInformation of
 * compute_convergence_information) of a candidate (x, y) of an unscaled LP, for callers that
 * may not allocate GPU memory when they want a solution checked: a host whose own memory pool
 * owns the device (a caching allocator that must not be bypassed), or a serving path with a
 * fixed memory budget. Every pointer except `out` is a DEVICE pointer the caller owns: bounds
 * and objective (n), right-hand side (m), x (n), y (m), primal_product = A x (m),
 * dual_product = A'y (n). `stream` is a cudaStream_t or NULL. The call is synchronous (it
 * copies the statistics back and waits for `stream`), so a stream that is being captured into
 * a CUDA graph is refused with GPDHG_ERR_NOT_SUPPORTED before any other CUDA call, leaving the
 * capture valid. The library allocates nothing: its scratch is one fixed device array of
 * 608.3 KiB that every GPU loading the library holds until the process exits, so n and m are
 * limited to 16,777,216 each (GPDHG_ERR_INVALID_ARGUMENT beyond). The first call in each CUDA
 * context looks the array's address up; calls that overlap on the GPU share the array and race.
 * ------------------------------------------------------------------------------- */
gpdhg_status gpdhg_convergence_noalloc(int32_t num_variables, int32_t num_constraints, int32_t num_equalities,
                                       double objective_constant, const double* variable_lower_bound,
                                       const double* variable_upper_bound, const double* objective_vector,
                                       const double* right_hand_side, const double* primal, const double* dual,
                                       const double* primal_product, const double* dual_product,
                                       double eps_optimal_absolute, double eps_optimal_relative, void* stream,
                                       gpdhg_convergence_information* out);

/* ---------------------------------------------------------------------------------
 * Tile-plan tuning hook. No counterpart in the reference.
 *
 * The step kernels' work plan (warp tiles, lane runs, tiles per CTA) takes its parameters
 * from a table measured on GB300 and keyed by the row-length histogram of each instance's
 * matrix. The sweep that measures the table (cupdlp.jl_gb300/tune_tiles.py) pins the
 * parameters with this process-wide override for plans built afterwards: precision
 * GPDHG_PRECISION_FP64 or GPDHG_PRECISION_FP32, side 0 for the primal kernel's plan (rows of
 * A') and 1 for the dual kernel's (rows of A); tile_nnz = 0 removes the override. Values are
 * clamped to what the kernels take (tile_nnz 32..32 x the lane run limit, e_floor 1..the
 * lane run limit, tpc_max 8..96). Results depend on the plan only through summation order.
 * ------------------------------------------------------------------------------- */
gpdhg_status gpdhg_set_tile_override(int32_t precision, int32_t side, int32_t tile_nnz, int32_t e_floor,
                                     int32_t tpc_max);

/* ---------------------------------------------------------------------------------
 * Serving loop: continuous batching of arriving LPs (no reference counterpart: a request
 * loop around optimize(), src/primal_dual_hybrid_gradient_gpu.jl:457).
 *
 * Requests wait in a FIFO queue. Each of `workers` host threads owns a CUDA stream and
 * repeatedly packs the waiting requests that share the head request's parameters (at most
 * max_cohort of them, after lingering up to linger_sec for more) into one device batch
 * (gpdhg_batch_*, a segmented CSR with per-instance step size, restarts and termination)
 * and solves it. A cohort is admitted only while the estimated device footprint of all
 * resident requests stays within hbm_budget_bytes and at most max_resident requests are
 * resident, so requests arriving while others run start as soon as memory and a worker
 * are free, and their kernels overlap with the running cohorts' on the device. An instance
 * that terminates stops launching work at once and its result can be collected at that
 * moment; its cohort's memory is released when the cohort's last instance terminates.
 * Once at most a quarter of a cohort's instances still run, the cohort no longer counts
 * against `workers`: a new cohort of waiting requests starts beside its stragglers (the
 * server keeps 2 x workers threads for this). Requests whose parameters a batch does not take (FP32_REFINE with its FP64 hand-off, the
 * constant step size) are solved one after another as lone problems by the worker that picks
 * them. Each result is bit-identical to solving the same LP alone with the same parameters
 * (a batch gives every instance the same arithmetic as a lone solve). Zero config fields
 * take the defaults in brackets.
 * ------------------------------------------------------------------------------- */
typedef struct gpdhg_server gpdhg_server;

typedef struct gpdhg_server_config {
  double hbm_budget_bytes;   /* admission budget for resident requests [half the free device memory] */
  int32_t max_resident;      /* requests resident on the device at once, all cohorts [4096] */
  int32_t max_cohort;        /* requests packed into one device batch [256] */
  int32_t workers;           /* cohorts advanced concurrently, stragglers not counted [2] */
  int32_t reserved_int;
  double linger_sec;         /* a free worker waits this long for more requests [0.002] */
  double reserved[2];
} gpdhg_server_config;

/* Estimated device bytes one request occupies while resident (the admission measure). */
double gpdhg_server_footprint(const gpdhg_lp_desc* desc, const gpdhg_params* params);
gpdhg_status gpdhg_server_create(const gpdhg_server_config* cfg, gpdhg_server** out);
/* Copies the request; `ticket` identifies it. GPDHG_ERR_ADMISSION if it can never fit. */
gpdhg_status gpdhg_server_submit(gpdhg_server* s, const gpdhg_lp_desc* desc, const gpdhg_params* params,
                                 uint64_t* ticket);
/* Non-blocking: GPDHG_ERR_NOT_READY until the request has terminated. A request's result
 * is handed out once: after a successful poll or wait its ticket is released. primal_out
 * and dual_out (n and m doubles, or NULL) receive the scaled average iterate. */
gpdhg_status gpdhg_server_poll(gpdhg_server* s, uint64_t ticket, gpdhg_result* result,
                               double* primal_out, double* dual_out);
/* Blocks until the request has terminated or `timeout_sec` passes (GPDHG_ERR_NOT_READY). */
gpdhg_status gpdhg_server_wait(gpdhg_server* s, uint64_t ticket, double timeout_sec, gpdhg_result* result,
                               double* primal_out, double* dual_out);
gpdhg_status gpdhg_server_destroy(gpdhg_server* s);

#ifdef __cplusplus
}
#endif

#endif /* GPDHG_H */
