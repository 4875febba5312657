"""Independent numpy check of the reference's optimality measures on an unscaled
solution (compute_convergence_information, src/iteration_stats_utils_gpu.jl:251-309,
and optimality_criteria_met, src/termination.jl:142-170, L2 norm)."""
import numpy as np
import scipy.sparse as sp


def kkt_measures(p, x, y):
    a = sp.csr_matrix(p.constraint_matrix)
    neq = p.num_equalities
    l, u, c, b = p.variable_lower_bound, p.variable_upper_bound, p.objective_vector, p.right_hand_side
    kx = a @ x
    cv = b - kx
    cv[neq:] = np.maximum(cv[neq:], 0.0)
    lv = np.maximum(l - x, 0.0)
    uv = np.maximum(x - u, 0.0)
    pres = np.sqrt(np.sum(cv * cv) + np.sum(lv * lv) + np.sum(uv * uv))
    g = c - a.T @ y
    rc = np.where(np.isfinite(l), np.maximum(g, 0.0), 0.0) + np.where(np.isfinite(u), np.minimum(g, 0.0), 0.0)
    rcv = g - rc
    dr = np.maximum(-y[neq:], 0.0)
    dres = np.sqrt(np.sum(dr * dr) + np.sum(rcv * rcv))
    pobj = p.objective_constant + c @ x
    contrib = np.where(rc > 0, np.where(np.isfinite(l), l, 0.0) * rc, np.where(rc < 0, np.where(np.isfinite(u), u, 0.0) * rc, 0.0))
    dobj = b @ y + p.objective_constant + contrib.sum()
    return dict(primal_residual=pres, dual_residual=dres, primal_objective=pobj, dual_objective=dobj,
                rel_primal=pres / (1.0 + np.linalg.norm(b)), rel_dual=dres / (1.0 + np.linalg.norm(c)),
                rel_gap=abs(pobj - dobj) / (1.0 + abs(pobj) + abs(dobj)))


def meets_tolerance(p, x, y, tol, slack=1.0):
    k = kkt_measures(p, x, y)
    return (k["primal_residual"] < slack * (tol + tol * np.linalg.norm(p.right_hand_side))
            and k["dual_residual"] < slack * (tol + tol * np.linalg.norm(p.objective_vector))
            and abs(k["primal_objective"] - k["dual_objective"]) < slack * (
                tol + tol * (abs(k["primal_objective"]) + abs(k["dual_objective"])))), k


def convergence_information(p, x, y, eps_abs, eps_rel, ax=None, aty=None):
    """Every field of the reference's ConvergenceInformation for a candidate (x, y) of an
    unscaled LP (compute_convergence_information, src/iteration_stats_utils_gpu.jl:251-309,
    with the problem norms of cached_quadratic_program_info, src/termination.jl:123-137),
    restated in numpy. `ax` / `aty` default to A x and A'y."""
    a = sp.csr_matrix(p.constraint_matrix)
    neq = p.num_equalities
    l, u, c, b = p.variable_lower_bound, p.variable_upper_bound, p.objective_vector, p.right_hand_side
    ax = a @ x if ax is None else ax
    aty = a.T @ y if aty is None else aty
    cv = b - ax
    cv[neq:] = np.maximum(cv[neq:], 0.0)
    lv = np.maximum(l - x, 0.0)
    uv = np.maximum(x - u, 0.0)
    g = c - aty
    rc = np.where(np.isfinite(l), np.maximum(g, 0.0), 0.0) + np.where(np.isfinite(u), np.minimum(g, 0.0), 0.0)
    rcv = g - rc
    dr = np.maximum(-y[neq:], 0.0)
    contrib = np.where(rc > 0, np.where(np.isfinite(l), l, 0.0) * rc,
                       np.where(rc < 0, np.where(np.isfinite(u), u, 0.0) * rc, 0.0))
    ratio = eps_abs / eps_rel
    linf = lambda *vs: max([float(np.max(np.abs(v))) if v.size else 0.0 for v in vs])
    l2 = lambda *vs: float(np.sqrt(sum(float(np.dot(v, v)) for v in vs)))
    out = dict(primal_objective=p.objective_constant + float(c @ x),
               dual_objective=float(b @ y) + p.objective_constant + float(contrib.sum()),
               l_inf_primal_residual=linf(cv, lv, uv), l2_primal_residual=l2(cv, lv, uv),
               l_inf_dual_residual=linf(dr, rcv), l2_dual_residual=l2(dr, rcv),
               l_inf_primal_variable=linf(x), l2_primal_variable=l2(x),
               l_inf_dual_variable=linf(y), l2_dual_variable=l2(y))
    out["relative_l_inf_primal_residual"] = out["l_inf_primal_residual"] / (ratio + linf(b))
    out["relative_l2_primal_residual"] = out["l2_primal_residual"] / (ratio + l2(b))
    out["relative_l_inf_dual_residual"] = out["l_inf_dual_residual"] / (ratio + linf(c))
    out["relative_l2_dual_residual"] = out["l2_dual_residual"] / (ratio + l2(c))
    po, do = out["primal_objective"], out["dual_objective"]
    out["relative_optimality_gap"] = abs(po - do) / (ratio + abs(po) + abs(do))
    out["corrected_dual_objective"] = do if out["l_inf_dual_residual"] == 0.0 else -np.inf
    return out
