"""Generates tests/golden/golden.json: independent pins for the oracle and the library.

cuPDLP.jl ships no golden vectors or known-answer tests for its solve loop (its only
test runs MathOptInterface's conformance suite at rtol 1e-1), and it cannot run here.
So the pins are:
  * the planted optimum of each known-optimum instance (exact by construction);
  * scipy.optimize.linprog(method="highs") optimal objectives, an independent FP64 solver;
  * the oracle's own statistics at a fixed iteration count, so oracle regressions show,
    with the same statistics from the oracle built with another summation order: their
    distance is the round-off envelope within which two correct implementations agree.
Each instance is re-generated from (generator, seed, sizes); a checksum of the
generated data guards against a different numpy random stream.

The power-law section pins reduced instances of the large power-law generator: its planted
optimum against HiGHS, and how many iterations the oracle needs (the family converges slowly
under PDHG: most instances with m >= 1,000 do not reach 1e-4 within 300,000 iterations).

The full-size section holds the FP64 oracle's optimum of the transportation benchmark
(1M columns) at 1e-8, the reference objective its benchmark result is measured against.

Run:  python tests/golden/make_golden.py [--power-law-only | --full-size-only |
                                           --power-law-iterations-only]
"""
import hashlib
import json
import os
import sys

import numpy as np
import scipy.optimize as so
import scipy.sparse as sp

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "cupdlp.jl_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))

import cupdlp  # noqa: E402
from cupdlp import synthetic  # noqa: E402
import oracle  # noqa: E402

INSTANCES = [
    {"gen": "known_optimum_lp", "seed": 0, "kw": {}},                                  # the plain FP64 workload
    {"gen": "known_optimum_lp", "seed": 11, "kw": {"m": 200, "n": 400, "density": 0.03}},
    {"gen": "known_optimum_lp", "seed": 12, "kw": {"m": 300, "n": 500, "neq": 300, "density": 0.02}},
    {"gen": "known_optimum_lp", "seed": 13, "kw": {"m": 300, "n": 500, "neq": 0, "density": 0.02}},
    {"gen": "transportation_lp", "seed": 14, "kw": {"supplies": 20, "demands": 80}},
    {"gen": "transportation_lp", "seed": 15, "kw": {"supplies": 50, "demands": 200}},
]


# Reduced power-law LPs (synthetic.power_law_lp with smaller m, n, nnz). "converge": the oracle
# reaches 1e-8 on them; "study": HiGHS-pinned only, with the oracle's state after a fixed budget.
POWER_LAW = [
    {"gen": "power_law_lp", "seed": 6, "kw": {"m": 300, "n": 600, "target_nnz": 3000}, "kind": "converge"},
    {"gen": "power_law_lp", "seed": 3, "kw": {"m": 300, "n": 600, "target_nnz": 3000}, "kind": "converge"},
    {"gen": "power_law_lp", "seed": 7, "kw": {"m": 2000, "n": 4000, "target_nnz": 40000}, "kind": "study",
     "budget": 20000},
]
# Iterations the oracle needs on the family as it grows (recorded, not re-run by the tests):
# to 1e-4 and to 1e-8 within a cap of `budget` iterations.
POWER_LAW_ITERATIONS = [
    {"gen": "power_law_lp", "seed": s, "kw": {"m": m, "n": 2 * m, "target_nnz": 10 * m}, "budget": cap}
    for (m, cap) in ((300, 300000), (1000, 300000), (3000, 300000), (20000, 100000))
    for s in (1, 3, 5, 7)
]


def make(spec):
    return getattr(synthetic, spec["gen"])(spec["seed"], **spec["kw"])


def checksum(p):
    a = sp.csc_matrix(p.constraint_matrix)
    h = hashlib.sha256()
    for arr in (a.indptr.astype(np.int64), a.indices.astype(np.int64), a.data, p.objective_vector,
                p.right_hand_side, p.variable_lower_bound, p.variable_upper_bound):
        h.update(np.ascontiguousarray(arr).tobytes())
    return h.hexdigest()[:16]


def highs_objective(p, presolve=True):
    a = sp.csr_matrix(p.constraint_matrix)
    neq = p.num_equalities
    bounds = list(zip(np.where(np.isfinite(p.variable_lower_bound), p.variable_lower_bound, None),
                      np.where(np.isfinite(p.variable_upper_bound), p.variable_upper_bound, None)))
    res = so.linprog(p.objective_vector, A_ub=-a[neq:] if a.shape[0] > neq else None,
                     b_ub=-p.right_hand_side[neq:] if a.shape[0] > neq else None,
                     A_eq=a[:neq] if neq else None, b_eq=p.right_hand_side[:neq] if neq else None,
                     bounds=bounds, method="highs", options={"presolve": presolve})
    assert res.status == 0, res.message
    return float(res.fun) + p.objective_constant


def power_law_entry(spec):
    lp = make(spec)
    p = lp.problem
    entry = dict(spec)
    entry["checksum"] = checksum(p)
    entry["m"], entry["n"], entry["nnz"] = p.num_constraints, p.num_variables, int(p.constraint_matrix.nnz)
    entry["planted_objective"] = lp.optimal_objective
    # HiGHS' presolve declares one of these (coefficients spread over four decades) infeasible;
    # its simplex without presolve reaches the planted optimum
    entry["highs_objective"] = highs_objective(p, presolve=False)
    if spec["kind"] == "converge":
        for tol, key in ((1e-4, "oracle_1e4"), (1e-8, "oracle_1e8")):
            res, x, y, st = oracle.optimize(p, cupdlp.default_parameters(tolerance=tol, iteration_limit=400000))
            ci = res.last_iteration_stats.convergence_information
            entry[key] = {"termination_reason": res.termination_reason, "iteration_count": res.iteration_count,
                          "primal_objective": ci.primal_objective, "dual_objective": ci.dual_objective}
    else:
        res, x, y, st = oracle.optimize(p, cupdlp.default_parameters(tolerance=1e-4,
                                                                     iteration_limit=spec["budget"]))
        ci = res.last_iteration_stats.convergence_information
        entry["oracle_budget"] = {"termination_reason": res.termination_reason,
                                  "iteration_count": res.iteration_count,
                                  "primal_objective": ci.primal_objective, "dual_objective": ci.dual_objective,
                                  "relative_optimality_gap": ci.relative_optimality_gap,
                                  "relative_l2_primal_residual": ci.relative_l2_primal_residual}
    print(entry["gen"], entry["seed"], entry["highs_objective"], entry.get("oracle_1e8", entry.get("oracle_budget")))
    return entry


FULL_SIZE = {"transportation": {"gen": "transportation_lp", "seed": 1, "kw": {}}}


def full_size_entry(spec):
    p = make(spec).problem
    entry = dict(spec)
    entry["checksum"] = checksum(p)
    for tol, key in ((1e-4, "oracle_1e4"), (1e-8, "oracle_1e8")):
        res, x, y, st = oracle.optimize(p, cupdlp.default_parameters(tolerance=tol), max_stats=1000)
        ci = res.last_iteration_stats.convergence_information
        entry[key] = {"termination_reason": res.termination_reason, "iteration_count": res.iteration_count,
                      "kkt_passes": res.cumulative_kkt_matrix_passes,
                      "primal_objective": ci.primal_objective, "dual_objective": ci.dual_objective}
    print(entry["gen"], entry["oracle_1e8"])
    return entry


def iterations_entry(spec):
    p = make(spec).problem
    entry = dict(spec)
    entry["nnz"] = int(p.constraint_matrix.nnz)
    for tol, key in ((1e-4, "tol_1e4"), (1e-8, "tol_1e8")):
        res, x, y, st = oracle.optimize(p, cupdlp.default_parameters(tolerance=tol, iteration_limit=spec["budget"]),
                                        max_stats=10)
        ci = res.last_iteration_stats.convergence_information
        entry[key] = {"termination_reason": res.termination_reason, "iteration_count": res.iteration_count,
                      "relative_optimality_gap": ci.relative_optimality_gap}
        if res.termination_reason != 1:
            break
    print(spec["kw"]["m"], spec["seed"], entry.get("tol_1e4"), entry.get("tol_1e8"), flush=True)
    return entry


def main():
    oracle.set_threads(8)
    path = os.path.join(HERE, "golden.json")
    if "--power-law-iterations-only" in sys.argv:
        out = json.load(open(path))
        out["power_law_iterations"] = [iterations_entry(spec) for spec in POWER_LAW_ITERATIONS]
        with open(path, "w") as f:
            json.dump(out, f, indent=1)
        return
    if "--full-size-only" in sys.argv:
        out = json.load(open(path))
        out["full_size"] = {k: full_size_entry(v) for k, v in FULL_SIZE.items()}
        with open(path, "w") as f:
            json.dump(out, f, indent=1)
        return
    if "--power-law-only" in sys.argv:
        out = json.load(open(path))
        out["power_law"] = [power_law_entry(spec) for spec in POWER_LAW]
        with open(path, "w") as f:
            json.dump(out, f, indent=1)
        return
    out = {"instances": []}
    for spec in INSTANCES:
        lp = make(spec)
        p = lp.problem
        entry = dict(spec)
        entry["checksum"] = checksum(p)
        entry["m"], entry["n"], entry["nnz"] = p.num_constraints, p.num_variables, int(p.constraint_matrix.nnz)
        entry["planted_objective"] = lp.optimal_objective
        entry["highs_objective"] = highs_objective(p)
        params = cupdlp.default_parameters(tolerance=1e-8)
        res, x, y, st = oracle.optimize(p, params)
        ci = res.last_iteration_stats.convergence_information
        entry["oracle_1e8"] = {"termination_reason": res.termination_reason, "iteration_count": res.iteration_count,
                               "primal_objective": ci.primal_objective, "dual_objective": ci.dual_objective}
        params = cupdlp.default_parameters(tolerance=1e-8, iteration_limit=100)
        sq = cupdlp.rescale_problem(10, False, 1.0, 0, p)
        pert = oracle.solve_scaled(sq, params, perturbed=True).result.last_iteration_stats.convergence_information
        res, x, y, st = oracle.optimize(p, params)
        ci = res.last_iteration_stats.convergence_information
        entry["oracle_it100_perturbed"] = {"primal_objective": pert.primal_objective,
                                           "l2_dual_residual": pert.l2_dual_residual}
        entry["oracle_it100"] = {"primal_objective": ci.primal_objective, "dual_objective": ci.dual_objective,
                                 "l2_primal_residual": ci.l2_primal_residual, "l2_dual_residual": ci.l2_dual_residual,
                                 "step_size": res.last_iteration_stats.step_size,
                                 "primal_weight": res.last_iteration_stats.primal_weight,
                                 "kkt_passes": res.cumulative_kkt_matrix_passes}
        out["instances"].append(entry)
        print(entry["gen"], entry["seed"], entry["highs_objective"], entry["oracle_1e8"])
    out["power_law"] = [power_law_entry(spec) for spec in POWER_LAW]
    out["full_size"] = {k: full_size_entry(v) for k, v in FULL_SIZE.items()}
    out["power_law_iterations"] = [iterations_entry(spec) for spec in POWER_LAW_ITERATIONS]
    with open(path, "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
