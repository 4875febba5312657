# GpdhgShim.jl — the ccall layer that lets cuPDLP.jl's `optimize` run its solve loop in
# libgpdhg.so (GB300, sm_103a).
#
# cuPDLP.jl's optimize (src/primal_dual_hybrid_gradient_gpu.jl:457-798) keeps `validate`
# (:461), `cached_quadratic_program_info` (:462), `rescale_problem` (:465) and
# `unscaled_saddle_point_output` (:732); only lines :488-797 (host->device transfer, the
# PDHG loop, the copy of the average back to the host) are replaced by `GpdhgShim.solve`.
# Struct layouts mirror include/gpdhg.h field for field (all isbits, C alignment).
#
# Usage inside cuPDLP:
#     include("GpdhgShim.jl")
#     function optimize(params::PdhgParameters, original_problem::QuadraticProgrammingProblem)
#         validate(original_problem)
#         scaled_problem = rescale_problem(params.l_inf_ruiz_iterations, params.l2_norm_rescaling,
#                                          params.pock_chambolle_alpha, params.verbosity, original_problem)
#         avg_primal, avg_dual, reason, iterations, stats = GpdhgShim.solve(params, scaled_problem)
#         return unscaled_saddle_point_output(scaled_problem, avg_primal, avg_dual, reason, iterations, stats)
#     end
module GpdhgShim

import SparseArrays

const libgpdhg = get(ENV, "GPDHG_LIB", joinpath(@__DIR__, "..", "lib", "libgpdhg.so"))

struct GpdhgParams
    l_inf_ruiz_iterations::Int32
    l2_norm_rescaling::Int32
    pock_chambolle_alpha::Float64
    primal_importance::Float64
    scale_invariant_initial_primal_weight::Int32
    verbosity::Int32
    record_iteration_stats::Int32
    termination_evaluation_frequency::Int32
    optimality_norm::Int32
    iteration_limit::Int32
    eps_optimal_absolute::Float64
    eps_optimal_relative::Float64
    eps_primal_infeasible::Float64
    eps_dual_infeasible::Float64
    time_sec_limit::Float64
    kkt_matrix_pass_limit::Float64
    restart_scheme::Int32
    restart_to_current_metric::Int32
    restart_frequency_if_fixed::Int64
    artificial_restart_threshold::Float64
    sufficient_reduction_for_restart::Float64
    necessary_reduction_for_restart::Float64
    primal_weight_update_smoothing::Float64
    step_size_policy::Int32
    precision::Int32
    reduction_exponent::Float64
    growth_exponent::Float64
    fp64_handoff_relative_kkt::Float64
    fp64_handoff_stall_evaluations::Int32
    profile_kernels::Int32
    reserved::NTuple{6,Float64}
end

struct GpdhgConvergenceInformation
    candidate_type::Int32
    pad0::Int32
    primal_objective::Float64
    dual_objective::Float64
    corrected_dual_objective::Float64
    l_inf_primal_residual::Float64
    l2_primal_residual::Float64
    l_inf_dual_residual::Float64
    l2_dual_residual::Float64
    relative_l_inf_primal_residual::Float64
    relative_l2_primal_residual::Float64
    relative_l_inf_dual_residual::Float64
    relative_l2_dual_residual::Float64
    relative_optimality_gap::Float64
    l_inf_primal_variable::Float64
    l2_primal_variable::Float64
    l_inf_dual_variable::Float64
    l2_dual_variable::Float64
end

struct GpdhgInfeasibilityInformation
    candidate_type::Int32
    pad0::Int32
    max_primal_ray_infeasibility::Float64
    primal_ray_linear_objective::Float64
    max_dual_ray_infeasibility::Float64
    dual_ray_objective::Float64
end

struct GpdhgIterationStats
    iteration_number::Int32
    cumulative_rejected_steps::Int32
    restart_used::Int32
    precision::Int32
    convergence_information::GpdhgConvergenceInformation
    infeasibility_information::GpdhgInfeasibilityInformation
    cumulative_kkt_matrix_passes::Float64
    cumulative_time_sec::Float64
    step_size::Float64
    primal_weight::Float64
    time_spent_doing_basic_algorithm::Float64
end

struct GpdhgResult
    termination_reason::Int32
    iteration_count::Int32
    total_number_iterations::Int64
    cumulative_kkt_matrix_passes::Float64
    solve_time_sec::Float64
    num_iteration_stats::Int32
    fp64_handoff_iteration::Int32
    last_iteration_stats::GpdhgIterationStats
    step_loop_device_sec::Float64
    accepted_steps::Int64
    rejected_steps::Int64
    primal_kernel_sec::Float64
    dual_kernel_sec::Float64
    primal_kernel_launches::Int64
    primal_spmv_launches::Int64
    kernels_launched::Int64
end

struct GpdhgLpDesc
    num_variables::Int32
    num_constraints::Int32
    num_equalities::Int32
    pad0::Int32
    nnz::Int64
    row_ptr::Ptr{Int32}
    col_idx::Ptr{Int32}
    values::Ptr{Float64}
    variable_lower_bound::Ptr{Float64}
    variable_upper_bound::Ptr{Float64}
    objective_vector::Ptr{Float64}
    right_hand_side::Ptr{Float64}
    objective_constant::Float64
    original_variable_lower_bound::Ptr{Float64}
    original_variable_upper_bound::Ptr{Float64}
    original_objective_vector::Ptr{Float64}
    original_right_hand_side::Ptr{Float64}
    constraint_rescaling::Ptr{Float64}
    variable_rescaling::Ptr{Float64}
end

function check(status::Cint)
    if status != 0
        msg = unsafe_string(ccall((:gpdhg_last_error, libgpdhg), Cstring, ()))
        error("libgpdhg status $status: $msg")
    end
end

"""
Flattens cuPDLP's PdhgParameters (with its TerminationCriteria, RestartParameters and
step-size policy) into the C struct. `pock_chambolle_alpha == nothing` becomes NaN.
"""
function c_params(p, precision::Integer = 0)
    tc = p.termination_criteria
    rp = p.restart_params
    adaptive = hasfield(typeof(p.step_size_policy_params), :reduction_exponent)
    return GpdhgParams(
        Int32(p.l_inf_ruiz_iterations), Int32(p.l2_norm_rescaling),
        p.pock_chambolle_alpha === nothing ? NaN : Float64(p.pock_chambolle_alpha),
        p.primal_importance, Int32(p.scale_invariant_initial_primal_weight), Int32(p.verbosity),
        Int32(p.record_iteration_stats), Int32(p.termination_evaluation_frequency),
        Int32(Int(tc.optimality_norm)), Int32(min(tc.iteration_limit, typemax(Int32))),
        tc.eps_optimal_absolute, tc.eps_optimal_relative, tc.eps_primal_infeasible, tc.eps_dual_infeasible,
        tc.time_sec_limit, tc.kkt_matrix_pass_limit,
        Int32(Int(rp.restart_scheme)), Int32(Int(rp.restart_to_current_metric)), Int64(rp.restart_frequency_if_fixed),
        rp.artificial_restart_threshold, rp.sufficient_reduction_for_restart, rp.necessary_reduction_for_restart,
        rp.primal_weight_update_smoothing,
        Int32(adaptive ? 0 : 1), Int32(precision),
        adaptive ? p.step_size_policy_params.reduction_exponent : 0.3,
        adaptive ? p.step_size_policy_params.growth_exponent : 0.6,
        1e-6, Int32(20), Int32(0), ntuple(_ -> 0.0, 6))
end

"""
    solve(params, scaled_problem; precision = 0)

Runs optimize()'s loop in libgpdhg on a ScaledQpProblem and returns
(avg_primal, avg_dual, termination_reason, iteration_count, iteration_stats), the
SCALED average that :713-720 copies to the host, ready for unscaled_saddle_point_output.
`iteration_stats` holds the library's per-evaluation records as NamedTuples.
"""
function solve(params, scaled_problem; precision::Integer = 0)
    s = scaled_problem.scaled_qp
    o = scaled_problem.original_qp
    m, n = size(s.constraint_matrix)
    # The SparseMatrixCSC goes in as it is (1-based, Int64 indices): gpdhg_problem_create_csc
    # uploads it as CSR(A') and builds CSR(A) on the GPU. `convert` copies only when the index
    # type is not Int64 already.
    A = s.constraint_matrix
    colptr = convert(Vector{Int64}, A.colptr)
    rowval = convert(Vector{Int64}, A.rowval)
    nzval = convert(Vector{Float64}, A.nzval)
    arrays = (colptr, rowval, nzval, s.variable_lower_bound, s.variable_upper_bound, s.objective_vector,
              s.right_hand_side, o.variable_lower_bound, o.variable_upper_bound, o.objective_vector,
              o.right_hand_side, scaled_problem.constraint_rescaling, scaled_problem.variable_rescaling)
    avg_primal = zeros(n)
    avg_dual = zeros(m)
    result = Ref{GpdhgResult}()
    GC.@preserve arrays avg_primal avg_dual begin
        desc = Ref(GpdhgLpDesc(Int32(n), Int32(m), Int32(s.num_equalities), Int32(0), Int64(length(nzval)),
                               Ptr{Int32}(C_NULL), Ptr{Int32}(C_NULL), Ptr{Float64}(C_NULL),
                               pointer(s.variable_lower_bound), pointer(s.variable_upper_bound),
                               pointer(s.objective_vector), pointer(s.right_hand_side), s.objective_constant,
                               pointer(o.variable_lower_bound), pointer(o.variable_upper_bound),
                               pointer(o.objective_vector), pointer(o.right_hand_side),
                               pointer(scaled_problem.constraint_rescaling),
                               pointer(scaled_problem.variable_rescaling)))
        handle = Ref{Ptr{Cvoid}}(C_NULL)
        check(ccall((:gpdhg_problem_create_csc, libgpdhg), Cint,
                    (Ref{GpdhgLpDesc}, Ptr{Int64}, Ptr{Int64}, Ptr{Float64}, Int32, Ptr{Cvoid}, Ref{Ptr{Cvoid}}),
                    desc, colptr, rowval, nzval, Int32(1), C_NULL, handle))
        try
            cp = Ref(c_params(params, precision))
            check(ccall((:gpdhg_solve, libgpdhg), Cint,
                        (Ptr{Cvoid}, Ref{GpdhgParams}, Ref{GpdhgResult}, Ptr{Float64}, Ptr{Float64}),
                        handle[], cp, result, avg_primal, avg_dual))
            stats = Vector{GpdhgIterationStats}(undef, result[].num_iteration_stats)
            for k in 1:length(stats)
                r = Ref{GpdhgIterationStats}()
                check(ccall((:gpdhg_get_stats, libgpdhg), Cint, (Ptr{Cvoid}, Int32, Ref{GpdhgIterationStats}),
                            handle[], Int32(k - 1), r))
                stats[k] = r[]
            end
            return avg_primal, avg_dual, result[].termination_reason, result[].iteration_count, stats
        finally
            ccall((:gpdhg_problem_destroy, libgpdhg), Cint, (Ptr{Cvoid},), handle[])
        end
    end
end

struct GpdhgTwoSidedDesc
    num_variables::Int32
    num_constraints::Int32
    nnz::Int64
    variable_lower_bound::Ptr{Float64}
    variable_upper_bound::Ptr{Float64}
    constraint_lower_bound::Ptr{Float64}
    constraint_upper_bound::Ptr{Float64}
    objective_vector::Ptr{Float64}
    objective_offset::Float64
end

"""
    solve_two_sided(params, qp::TwoSidedQpProblem; precision=0)

The MPS path (`qps_reader_to_standard_form`, src/quadratic_programming_io.jl:139-186)
without the host conversion: `transform_to_standard_form` (:33-121) and `rescale_problem`
run on the GPU inside gpdhg_problem_create_two_sided, then the loop runs as in `solve`.
Returns (primal, dual, termination_reason, iteration_count, new_row_to_old,
num_equalities): the UNSCALED average of the standard form (slack variables after the
original ones; rows in the standard form's order, i.e. row r is the caller's row
new_row_to_old[r], 1-based, negated when that row was a "<=" row), which is what the
reference's MPS path returns.
"""
function solve_two_sided(params, qp; precision::Integer = 0)
    A = qp.constraint_matrix
    m, n = size(A)
    colptr = convert(Vector{Int64}, A.colptr)
    rowval = convert(Vector{Int64}, A.rowval)
    nzval = convert(Vector{Float64}, A.nzval)
    arrays = (colptr, rowval, nzval, qp.variable_lower_bound, qp.variable_upper_bound,
              qp.constraint_lower_bound, qp.constraint_upper_bound, qp.objective_vector)
    result = Ref{GpdhgResult}()
    GC.@preserve arrays begin
        desc = Ref(GpdhgTwoSidedDesc(Int32(n), Int32(m), Int64(length(nzval)), pointer(qp.variable_lower_bound),
                                     pointer(qp.variable_upper_bound), pointer(qp.constraint_lower_bound),
                                     pointer(qp.constraint_upper_bound), pointer(qp.objective_vector),
                                     qp.objective_offset))
        cp = Ref(c_params(params, precision))
        handle = Ref{Ptr{Cvoid}}(C_NULL)
        check(ccall((:gpdhg_problem_create_two_sided, libgpdhg), Cint,
                    (Ref{GpdhgTwoSidedDesc}, Ptr{Int64}, Ptr{Int64}, Ptr{Float64}, Int32, Ref{GpdhgParams},
                     Ref{Ptr{Cvoid}}),
                    desc, colptr, rowval, nzval, Int32(1), cp, handle))
        try
            nv, neq, ns = Ref{Int32}(0), Ref{Int32}(0), Ref{Int32}(0)
            order = zeros(Int32, m)
            check(ccall((:gpdhg_get_standard_form, libgpdhg), Cint,
                        (Ptr{Cvoid}, Ref{Int32}, Ref{Int32}, Ref{Int32}, Ptr{Int32}), handle[], nv, neq, ns, order))
            primal = zeros(nv[])
            dual = zeros(m)
            check(ccall((:gpdhg_solve, libgpdhg), Cint,
                        (Ptr{Cvoid}, Ref{GpdhgParams}, Ref{GpdhgResult}, Ptr{Float64}, Ptr{Float64}),
                        handle[], cp, result, primal, dual))
            con = zeros(m)
            var = zeros(nv[])
            check(ccall((:gpdhg_get_rescaling, libgpdhg), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}),
                        handle[], con, var))
            # unscaled_saddle_point_output (src/saddle_point_gpu.jl:40-61)
            return primal ./ var, dual ./ con, result[].termination_reason, result[].iteration_count,
                   order .+ 1, Int(neq[])
        finally
            ccall((:gpdhg_problem_destroy, libgpdhg), Cint, (Ptr{Cvoid},), handle[])
        end
    end
end

end # module
