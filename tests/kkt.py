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
