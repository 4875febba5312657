"""Seeded synthetic LP generators for the five measured workloads.

No public benchmark set is named for this path, so seeded synthetic problems with the
stated shapes and value distributions stand in for real instances. All use
numpy.random.default_rng(seed).

  known_optimum_lp      plain FP64 LP with a planted optimum (x*, y*, reduced costs):
                        m=1,000 (600 '=', 400 '>='), n=2,000, 0.5% uniform density,
                        values N(0,1), 0 <= x <= 10.
  transportation_lp     500 supply x 2,000 demand nodes: n=1,000,000, m=2,500, nnz=2,000,000
                        (exactly 2 per column), demand rows '=' first, supply rows '<='
                        negated into '>=' (as src/quadratic_programming_io.jl:52-65 does).
  power_law_lp          m=1,000,000, n=2,000,000, nnz~20M: column degrees Zipf(1.5) capped at
                        5,000 and rescaled to the target nnz (stochastic rounding, floor 1);
                        row indices drawn from a shuffled row popularity proportional to
                        rank^-ROW_POPULARITY_EXPONENT (0.5), so row lengths are skewed too;
                        values N(0,1)*10^U(-2,2); bounds [0, U(1,100)]; planted optimum.
  batch_lps             256 instances: m log-normal (median 2,000, clipped to [200, 50,000]),
                        n = 2m, nnz/row ~ U(5,40); 25% transportation-structured with
                        S + D = m, S = round(m/5), and m reduced until S*D <= 1,000,000.
  two_sided_lp          a planted-optimum LP rewritten as an MPS reader returns it: '>=' rows
                        split three ways into '>=', negated '<=' and two-sided rows (upper
                        bound 0.5-2 above the planted A x*), then all rows shuffled.
  serving_stream        Poisson arrivals; mixture 70% small (m 200-2k), 25% medium
                        (m 10k-100k), 5% large (m 500k, nnz 10M).
"""
from __future__ import annotations

import dataclasses
from typing import List, Optional

import numpy as np
import scipy.sparse as sp

from .types import QuadraticProgrammingProblem, TwoSidedQpProblem

ROW_POPULARITY_EXPONENT = 0.5


@dataclasses.dataclass
class SyntheticLp:
    problem: QuadraticProgrammingProblem
    name: str
    optimal_objective: Optional[float] = None   # exact, from the planted optimum
    x_star: Optional[np.ndarray] = None
    y_star: Optional[np.ndarray] = None


def _empty_q(n):
    return sp.csc_matrix((n, n), dtype=np.float64)


def _planted(rng, a: sp.csc_matrix, neq: int, ub: np.ndarray, name: str) -> SyntheticLp:
    """Planted optimum on a given matrix, bounds [0, ub]: x* 30% at 0, 10% at ub, the
    rest interior; b = A x* minus slack U(0,1) on half of the '>=' rows; y* N(0,1) on
    '=' rows, |N(0,1)| on tight '>=' rows, 0 on slack rows; c = A'y* + lambda with
    lambda >= 0 at lower bounds, <= 0 at upper bounds, 0 in the interior."""
    m, n = a.shape
    kind = rng.random(n)
    at_lo = kind < 0.3
    at_hi = (kind >= 0.3) & (kind < 0.4)
    x = ub * rng.uniform(0.01, 0.99, n)
    x[at_lo] = 0.0
    x[at_hi] = ub[at_hi]
    ax = a @ x
    nineq = m - neq
    slack_rows = np.zeros(m, dtype=bool)
    if nineq > 0:
        ineq_idx = np.arange(neq, m)
        pick = rng.permutation(nineq)[: nineq // 2]
        slack_rows[ineq_idx[pick]] = True
    b = ax.copy()
    b[slack_rows] -= rng.uniform(0.0, 1.0, int(slack_rows.sum()))
    y = rng.standard_normal(m)
    y[neq:] = np.abs(y[neq:])
    y[slack_rows] = 0.0
    lam = np.zeros(n)
    lam[at_lo] = np.abs(rng.standard_normal(int(at_lo.sum())))
    lam[at_hi] = -np.abs(rng.standard_normal(int(at_hi.sum())))
    c = a.T @ y + lam
    prob = QuadraticProgrammingProblem(np.zeros(n), ub.astype(np.float64), _empty_q(n), c, 0.0, a, b, neq)
    return SyntheticLp(prob, name, float(c @ x), x, y)


def known_optimum_lp(seed: int = 0, m: int = 1000, n: int = 2000, neq: Optional[int] = None,
                     density: float = 0.005) -> SyntheticLp:
    rng = np.random.default_rng(seed)
    neq = int(round(0.6 * m)) if neq is None else neq
    nnz = int(round(density * m * n))
    lin = rng.choice(m * n, size=nnz, replace=False)
    rows, cols = np.divmod(lin, n)
    vals = rng.standard_normal(nnz)
    a = sp.csc_matrix((vals, (rows, cols)), shape=(m, n))
    a.sort_indices()
    return _planted(rng, a, neq, np.full(n, 10.0), f"known_optimum_m{m}_n{n}_s{seed}")


@dataclasses.dataclass
class SyntheticTwoSidedLp:
    problem: TwoSidedQpProblem
    name: str
    optimal_objective: Optional[float] = None   # the planted optimum's, unchanged by the rewrite


def two_sided_lp(seed: int = 5, m: int = 400, n: int = 900, neq: Optional[int] = None,
                 density: float = 0.01) -> SyntheticTwoSidedLp:
    """known_optimum_lp's LP as constraint_lower_bound <= A x <= constraint_upper_bound: '='
    rows keep l = u = b; each '>=' row stays (b, +Inf), is negated into (-Inf, -b), or gets a
    finite upper bound 0.5-2 above A x* (x* stays feasible, hence optimal); rows shuffled."""
    base = known_optimum_lp(seed, m=m, n=n, neq=neq, density=density)
    rng = np.random.default_rng(seed + 1000)
    p = base.problem
    a = sp.csr_matrix(p.constraint_matrix)
    b = p.right_hand_side
    lo, hi = b.copy(), b.copy()
    ineq = np.arange(p.num_equalities, m)
    kind = rng.integers(0, 3, ineq.size)
    hi[ineq] = np.inf
    neg = ineq[kind == 1]
    lo[neg], hi[neg] = -np.inf, -b[neg]
    two = ineq[kind == 2]
    hi[two] = (a @ base.x_star)[two] + rng.uniform(0.5, 2.0, two.size)
    sign = np.ones(m)
    sign[neg] = -1.0
    a = sp.diags(sign) @ a
    perm = rng.permutation(m)
    qp = TwoSidedQpProblem(p.variable_lower_bound.copy(), p.variable_upper_bound.copy(), lo[perm], hi[perm],
                           sp.csc_matrix(a[perm]), 0.0, p.objective_vector.copy())
    qp.constraint_matrix.sort_indices()
    return SyntheticTwoSidedLp(qp, f"two_sided_m{m}_n{n}_s{seed}", base.optimal_objective)


def transportation_two_sided(seed: int = 1, supplies: int = 500, demands: int = 2000) -> SyntheticTwoSidedLp:
    """transportation_lp as its MPS file states it: demand rows '=' and supply rows '<='
    (sum_j x_ij <= s_i), before the reader's standard-form conversion."""
    t = transportation_lp(seed, supplies, demands).problem
    D = t.num_equalities
    a = sp.csr_matrix(t.constraint_matrix)
    sign = np.ones(t.num_constraints)
    sign[D:] = -1.0
    lo = t.right_hand_side.copy()
    hi = t.right_hand_side.copy()
    lo[D:] = -np.inf
    hi[D:] = -t.right_hand_side[D:]
    qp = TwoSidedQpProblem(t.variable_lower_bound.copy(), t.variable_upper_bound.copy(), lo, hi,
                           sp.csc_matrix(sp.diags(sign) @ a), 0.0, t.objective_vector.copy())
    qp.constraint_matrix.sort_indices()
    return SyntheticTwoSidedLp(qp, f"transportation_two_sided_{supplies}x{demands}_s{seed}")


def transportation_lp(seed: int = 1, supplies: int = 500, demands: int = 2000) -> SyntheticLp:
    rng = np.random.default_rng(seed)
    S, D = supplies, demands
    n = S * D
    m = S + D
    cost = rng.uniform(1.0, 100.0, n)
    demand = rng.uniform(10.0, 50.0, D)
    supply = rng.uniform(50.0, 150.0, S)
    supply *= 1.1 * demand.sum() / supply.sum()
    j = np.arange(n, dtype=np.int64)
    s_of, d_of = np.divmod(j, D)
    # column j = (s, d): +1 in demand row d (equalities first), -1 in supply row D + s
    indptr = np.arange(0, 2 * n + 1, 2, dtype=np.int64)
    indices = np.empty(2 * n, dtype=np.int32)
    indices[0::2] = d_of
    indices[1::2] = D + s_of
    data = np.empty(2 * n)
    data[0::2] = 1.0
    data[1::2] = -1.0
    a = sp.csc_matrix((data, indices, indptr), shape=(m, n))
    b = np.concatenate([demand, -supply])
    prob = QuadraticProgrammingProblem(np.zeros(n), np.full(n, np.inf), _empty_q(n), cost, 0.0, a, b, D)
    return SyntheticLp(prob, f"transportation_{S}x{D}_s{seed}")


def _zipf_degrees(rng, n, target_nnz, s=1.5, cap=5000):
    d = np.minimum(rng.zipf(s, n), cap).astype(np.float64)
    d *= target_nnz / d.sum()
    fl = np.floor(d)
    d = fl + (rng.random(n) < (d - fl))
    return np.maximum(d, 1).astype(np.int64)


def power_law_lp(seed: int = 2, m: int = 1_000_000, n: int = 2_000_000, target_nnz: int = 20_000_000,
                 row_exponent: float = ROW_POPULARITY_EXPONENT) -> SyntheticLp:
    rng = np.random.default_rng(seed)
    deg = _zipf_degrees(rng, n, target_nnz)
    deg = np.minimum(deg, m)
    pop = np.arange(1, m + 1, dtype=np.float64) ** (-row_exponent)
    pop = pop[rng.permutation(m)]
    cdf = np.cumsum(pop)
    cdf /= cdf[-1]
    total = int(deg.sum())
    rows = np.searchsorted(cdf, rng.random(total), side="right").astype(np.int64)
    np.minimum(rows, m - 1, out=rows)
    cols = np.repeat(np.arange(n, dtype=np.int64), deg)
    vals = rng.standard_normal(total) * 10.0 ** rng.uniform(-2.0, 2.0, total)
    a = sp.csc_matrix((vals, (rows, cols)), shape=(m, n))
    a.sum_duplicates()
    a.sort_indices()
    ub = rng.uniform(1.0, 100.0, n)
    neq = int(round(0.6 * m))
    return _planted(rng, a, neq, ub, f"power_law_m{m}_n{n}_s{seed}")


def batch_lps(seed: int = 3, count: int = 256, median_m: int = 2000, m_range=(200, 50_000),
              transport_fraction: float = 0.25, transport_cap: int = 1_000_000) -> List[SyntheticLp]:
    rng = np.random.default_rng(seed)
    out = []
    ms = np.clip(np.round(median_m * np.exp(rng.normal(0.0, 1.0, count))), *m_range).astype(int)
    is_tr = rng.random(count) < transport_fraction
    for k in range(count):
        sub = int(rng.integers(0, 2**31 - 1))
        m = int(ms[k])
        if is_tr[k]:
            S = max(2, int(round(m / 5)))
            D = max(2, m - S)
            while S * D > transport_cap:
                m = int(m * 0.9)
                S = max(2, int(round(m / 5)))
                D = max(2, m - S)
            out.append(transportation_lp(sub, S, D))
        else:
            n = 2 * m
            per_row = rng.uniform(5.0, 40.0)
            out.append(known_optimum_lp(sub, m=m, n=n, density=per_row / n))
    return out


@dataclasses.dataclass
class Request:
    arrival_sec: float
    lp: SyntheticLp
    kind: str


def serving_mixture_lp(rng, kind: str) -> SyntheticLp:
    sub = int(rng.integers(0, 2**31 - 1))
    if kind == "small":
        m = int(rng.integers(200, 2001))
        return known_optimum_lp(sub, m=m, n=2 * m, density=rng.uniform(5, 40) / (2 * m))
    if kind == "medium":
        m = int(rng.integers(10_000, 100_001))
        return known_optimum_lp(sub, m=m, n=2 * m, density=rng.uniform(5, 40) / (2 * m))
    return power_law_lp(sub, m=500_000, n=1_000_000, target_nnz=10_000_000)


def serving_stream(seed: int, rate_per_sec: float, duration_sec: float, mix=(0.70, 0.25, 0.05),
                   max_requests: Optional[int] = None) -> List[Request]:
    rng = np.random.default_rng(seed)
    t = 0.0
    reqs = []
    while True:
        t += rng.exponential(1.0 / rate_per_sec)
        if t > duration_sec or (max_requests is not None and len(reqs) >= max_requests):
            break
        u = rng.random()
        kind = "small" if u < mix[0] else ("medium" if u < mix[0] + mix[1] else "large")
        reqs.append(Request(t, serving_mixture_lp(rng, kind), kind))
    return reqs
