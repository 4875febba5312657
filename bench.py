"""Benchmark of the restarted-PDHG solve loop (KKT matrix passes per second).

Workload (default): the power-law LP — m = 1,000,000 rows (600k '=', 400k '>='),
n = 2,000,000 columns, 21.2M nonzeros (Zipf(1.5) column degrees, skewed row lengths, values
N(0,1) x 10^U(-2,2)), boxes [0, U(1,100)], planted optimum, seeded synthetic data; FP32 bulk
iterates with FP64 norms, restarts and termination, and the FP64 hand-off (FP32_REFINE). One
step = the first 1,000 iterations of the solve from the zero start (a fixed-iteration
protocol: neither the reference loop nor this one reaches 1e-4 on this family within a
benchmark's time; the oracle needs >300,000 iterations already at m = 1,000), with the scaled
problem resident in HBM. `--workload transportation` is the transportation LP (500 x 2,000,
1M columns, 2M nonzeros, FP64) solved to the relative KKT tolerance 1e-4, one solve per step.

  value       KKT matrix passes / s (the reference's cumulative_kkt_matrix_passes per
              second of solve time), timed with CUDA events on the solver's stream; the
              solves run as they do for a user (evaluation intervals as CUDA graphs).
  e2e         the same metric through the C ABI with host buffers (pinned host memory, filled
              once before timing): gpdhg_problem_create
              (host->device copy of the CSR matrix and vectors, transpose and schedule),
              gpdhg_solve, and the device->host copy of the solution, every step
              (create_sec_per_step: the gpdhg_problem_create part alone).
  objective_error  the result's primal and dual objectives against the FP64 reference
              optimum: the planted optimum (power-law, plain LP; exact by construction and
              equal to HiGHS' on reduced instances) or the FP64 oracle at 1e-8
              (transportation, tests/golden/golden.json).
  roofline    the dominant step kernel's algorithmic bytes / its CUDA-event time, measured
              live right after the timed steps on the same number of solves launched kernel
              by kernel with an event between every two (params.profile_kernels; events
              cannot split the kernels of a CUDA graph). traffic and
              fp64_pipe_active_pct_ncu come from the committed ncu capture (profiles/).
  cpu_baseline  the oracle (the CPU FP64 restatement of the reference loop) on the host
              cores: the same 1,000 iterations (power-law), the full solve (transportation).
  reference_gpu_equiv  the reference's loop in its own GPU form on the same GPU
              (baseline/ref_equiv.cu: cuSPARSE CSR_ALG2 FP64 SpMV, one kernel per reference
              kernel or broadcast with the reference's synchronisations, dot / nrm2 read back by
              the host every attempt), on the same problem, parameters and iteration budget.

--impl reference times that CPU implementation alone (the reference itself is Julia
and cannot be installed here). Multi-GPU: replicas only (a single LP does not shard).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "cupdlp.jl_gb300"))

import numpy as np  # noqa: E402

L2_BYTES = 129 * 2**20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="powerlaw",
                    choices=["transportation", "plain", "powerlaw", "batch", "serve"])
    ap.add_argument("--serve-rates", default="50,200,1000", help="Poisson arrival rates (LPs/s)")
    ap.add_argument("--serve-duration", type=float, default=5.0, help="seconds of arrivals per rate")
    ap.add_argument("--serve-drain-cap", type=float, default=90.0,
                    help="seconds after the last arrival before unfinished requests are counted as such")
    ap.add_argument("--batch-count", type=int, default=256)
    ap.add_argument("--tolerance", type=float, default=1e-4)
    ap.add_argument("--cpu-sample-iters", type=int, default=0, help="oracle iteration cap (0: automatic)")
    ap.add_argument("--iters", type=int, default=0,
                    help="iteration budget per step (default: run to the tolerance; the power-law "
                         "workload uses 1000, since neither the reference loop nor this one "
                         "reaches 1e-4 on it within a benchmark's time)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--precision", choices=["fp64", "fp32", "fp32_refine"], default=None,
                    help="override the workload's precision (profiling one precision's kernels)")
    ap.add_argument("--no-reference-gpu", action="store_true", help="skip the reference-form GPU baseline")
    return ap.parse_args()


DEFAULT_ITERS = {"powerlaw": 1000}          # fixed-iteration protocol of the power-law LP
CPU_SAMPLE_ITERS = {"powerlaw": 1000}       # the oracle on the same iterations (0: full solve)
REFERENCE_ARM_ITERS = {"powerlaw": 200}     # per step of --impl reference (25 steps in minutes)


def workload(name):
    import cupdlp
    from cupdlp import synthetic
    if name == "transportation":
        lp = synthetic.transportation_lp(1)
        prec = cupdlp.Precision.FP64
        desc = "transportation LP 500x2000: m=2,500, n=1,000,000, nnz=2,000,000, FP64"
    elif name == "plain":
        lp = synthetic.known_optimum_lp(0)
        prec = cupdlp.Precision.FP64
        desc = "plain LP with planted optimum: m=1,000, n=2,000, nnz=10,000, FP64"
    else:
        lp = synthetic.power_law_lp(2)
        prec = cupdlp.Precision.FP32_REFINE
        desc = ("power-law LP: m=1,000,000, n=2,000,000, nnz=21.2M (Zipf(1.5) column degrees), "
                "FP32 bulk + FP64 norms/restarts/termination + FP64 hand-off")
    return lp, prec, desc


def reference_objective(name, lp):
    """(objective, what it is) of the FP64 reference optimum of the workload."""
    if lp.optimal_objective is not None:
        return lp.optimal_objective, "planted optimum (exact by construction)"
    try:
        g = json.load(open(os.path.join(REPO, "tests", "golden", "golden.json")))["full_size"][name]
        return g["oracle_1e8"]["primal_objective"], "FP64 oracle at relative tolerance 1e-8"
    except (OSError, KeyError):
        return None, None


def objective_error(name, lp, ci):
    ref, what = reference_objective(name, lp)
    if ref is None:
        return None
    rel = lambda v: abs(v - ref) / max(1.0, abs(ref))
    return {"reference": what, "reference_objective": ref, "primal_rel": rel(ci.primal_objective),
            "dual_rel": rel(ci.dual_objective), "relative_optimality_gap": ci.relative_optimality_gap,
            "relative_l2_primal_residual": ci.relative_l2_primal_residual,
            "relative_l2_dual_residual": ci.relative_l2_dual_residual}


def precision_name(prec):
    return {0: "FP64", 1: "FP32_REFINE", 2: "FP32"}.get(int(prec), str(prec))


def bytes_model(m, n, nnz, prec):
    """Algorithmic bytes of the two step kernels (minimum traffic of the fused schedule,
    gathered vectors counted once)."""
    sv = 8 if prec == 0 else 4   # matrix values
    sx = sv                      # iterate vectors
    si = 4                       # int32 indices
    mat_t = (sv + si) * nnz + si * (n + 1)   # CSR of A' (n rows)
    mat_a = (sv + si) * nnz + si * (m + 1)   # CSR of A (m rows)
    return {
        # primal kernel with a commit: A' stream, gather y, read x dx c l u sx,
        # write x dx kty sx
        "primal_commit": mat_t + sx * m + 10 * sx * n,
        # primal kernel after a rejection: read x kty c l u, write dx
        "primal_plain": 6 * sx * n,
        # dual kernel: A stream, gather dx, read y kx b, write y' kx'
        "dual": mat_a + sx * n + 5 * sx * m,
        # extra dual traffic when it commits the sums: sy skx read+write
        "dual_commit_extra": 4 * sx * m,
    }


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return None
        rows = [r.split(", ") for r in open(self.path).read().strip().splitlines() if r.count(",") >= 8]
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = max(float(r[2]) for r in rows)
        load = [v for v in sm if v > 0.5 * mx] or sm
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].strip() == "Active"})
        return {"sm_mhz": statistics.median(load) if load else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(rows)}


def pinned_desc(d):
    """The same LP descriptor over copies of its arrays in page-locked host memory: the e2e
    steps copy their inputs from pinned buffers, as a caller that stages its LP for the GPU
    would. The copies are made once, outside any timed region."""
    import torch
    from cupdlp.solver import _Desc
    keep = []

    def pin(a):
        if a is None:
            return None
        t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
        keep.append(t)
        return t.numpy()

    a = {k: pin(v) for k, v in d.arrays.items()}
    q = d.desc
    out = _Desc(q.num_variables, q.num_constraints, q.num_equalities, a["rptr"], a["cols"], a["vals"], a["l"],
                a["u"], a["c"], a["b"], q.objective_constant, a["ol"], a["ou"], a["oc"], a["ob"], a["con"], a["var"])
    for k, v in a.items():
        assert v is None or out.arrays[k].ctypes.data == v.ctypes.data, k   # no pageable copy was made
    out._pinned = keep
    return out


def dist_setup(n_gpus):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        backend = "nccl"
        try:
            import torch
            torch.cuda.set_device(local)
        except Exception:
            backend = "gloo"
        dist.init_process_group(backend=backend)
        pg = dist
    return world, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def _reduce_over_ranks(pg, v, op):
    if pg is None:
        return v
    import torch
    # NCCL reduces device tensors, gloo (the CPU fallback) host tensors
    dev = "cuda" if pg.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    pg.all_reduce(t, op=op)
    return float(t.item())


def max_over_ranks(pg, v):
    return v if pg is None else _reduce_over_ranks(pg, v, pg.ReduceOp.MAX)


def sum_over_ranks(pg, v):
    return v if pg is None else _reduce_over_ranks(pg, v, pg.ReduceOp.SUM)


PROFILE_FILES = {"transportation": "step_kernels_transportation_fp64.md", "powerlaw": "step_kernels_powerlaw_fp32.md"}


def _profile_rows(workload_name, kernel):
    """The table rows of `kernel` in the committed ncu capture of this workload (profiles/)."""
    fn = PROFILE_FILES.get(workload_name)
    if not fn:
        return []
    try:
        text = open(os.path.join(REPO, "profiles", fn)).read()
    except OSError:
        return []
    rows = []
    for line in text.splitlines():
        cells = [c.strip() for c in line.strip().strip("|").split("|")]
        if len(cells) > 7 and cells[0].startswith(kernel + "<"):
            rows.append(cells)
    return rows


def _profile_mean(rows, f):
    vals = []
    for cells in rows:
        try:
            vals.append(f(cells))
        except ValueError:
            pass
    return sum(vals) / len(vals) if vals else None


def profile_traffic(workload_name, kernel):
    """DRAM bytes per launch (read + write) of `kernel` in the committed ncu capture of this
    workload, averaged over the captured launches; None if there is none."""
    return _profile_mean(_profile_rows(workload_name, kernel), lambda c: (float(c[2]) + float(c[3])) * 1e6)


def profile_fp64_pipe(workload_name, kernel):
    """FP64 pipe activity (% of peak) of `kernel` in the same capture: the unit that binds the
    FP64 kernels, which the HBM fraction alone does not show."""
    return _profile_mean(_profile_rows(workload_name, kernel), lambda c: float(c[7]))


def cpu_baseline(lp_problem, params, iters_cap, threads=None):
    """The oracle on a bounded sample: the first `iters_cap` iterations of the same solve, or
    the whole solve to the tolerance when iters_cap is 0."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    import cupdlp
    threads = threads or os.cpu_count() or 1
    oracle.set_threads(threads)
    sq = cupdlp.rescale_problem(10, False, 1.0, 0, lp_problem)
    p = cupdlp.default_parameters(tolerance=params.termination_criteria.eps_optimal_relative,
                                  iteration_limit=iters_cap or 2**31 - 1)
    t0 = time.perf_counter()
    run = oracle.solve_scaled(sq, p, max_stats=100000)
    wall = time.perf_counter() - t0
    r = run.result
    what = (f"first {r.iteration_count} iterations" if iters_cap else
            f"the full solve to {p.termination_criteria.eps_optimal_relative:g} ({r.iteration_count} iterations, "
            f"termination {r.termination_reason})")
    return {"value": r.cumulative_kkt_matrix_passes / r.solve_time_sec, "unit": "KKT passes/s", "cores": threads,
            "kind": "port",
            "sample": f"oracle FP64 restatement, {what} ({r.cumulative_kkt_matrix_passes:.1f} KKT passes, "
                      f"{r.solve_time_sec:.2f} s of loop, {wall:.1f} s wall)",
            "solve_sec": r.solve_time_sec, "iterations": r.iteration_count,
            "kkt_passes": r.cumulative_kkt_matrix_passes}


def reference_gpu_equiv(sq, params, repeats=2):
    """The reference-form GPU baseline on the same scaled problem: KKT passes / s of its solve
    (host wall clock around its loop, as the reference times itself), best of `repeats`."""
    sys.path.insert(0, os.path.join(REPO, "baseline"))
    import cupdlp
    import ref_equiv
    p64 = cupdlp.default_parameters(tolerance=params.termination_criteria.eps_optimal_relative,
                                    iteration_limit=params.termination_criteria.iteration_limit,
                                    record_iteration_stats=False)
    best = None
    for _ in range(repeats):
        r, _, _ = ref_equiv.solve_scaled(sq, p64, want_solution=False)
        if best is None or r.solve_time_sec < best.solve_time_sec:
            best = r
    ci = best.last_iteration_stats.convergence_information
    return best, {"value": best.cumulative_kkt_matrix_passes / best.solve_time_sec, "unit": "KKT passes/s",
                  "solve_sec": best.solve_time_sec, "iterations": best.iteration_count,
                  "kkt_passes": best.cumulative_kkt_matrix_passes, "termination": best.termination_reason,
                  "primal_objective": ci.primal_objective, "kernels_per_iteration":
                      best.kernels_launched / max(1, best.iteration_count),
                  "form": "reference call pattern on this GPU: cuSPARSE CSR_ALG2 FP64 SpMV, per-kernel "
                          "sync, host-side dot/nrm2 every attempt (baseline/ref_equiv.cu); best of "
                          f"{repeats} solves"}


def run_reference(args):
    world, rank, local, pg = dist_setup(args.gpus)
    if rank != 0:
        return 0
    import cupdlp
    lp, prec, desc = workload(args.workload)
    params = cupdlp.default_parameters(tolerance=args.tolerance, precision=prec)
    cap = args.cpu_sample_iters or REFERENCE_ARM_ITERS.get(args.workload, 0)
    vals = []
    for k in range(args.warmup + args.steps):
        cb = cpu_baseline(lp.problem, params, cap)
        if k >= args.warmup:
            vals.append(cb["value"])
    v = float(np.mean(vals))
    line = {"metric": "KKT mults/sec", "value": v, "unit": "KKT passes/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)", "impl": "reference",
            "config": {"workload": desc, "tolerance": args.tolerance, "l2": "n/a (CPU)"},
            "cpu_baseline": {"value": v, "unit": "KKT passes/s", "cores": cb["cores"], "kind": "port",
                             "sample": cb["sample"]},
            "e2e": {"value": v, "unit": "KKT passes/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_batch(args):
    """256 LPs of uneven size (m log-normal around 2,000, n = 2m, 25% transportation-shaped)
    packed into one segmented CSR and solved together, FP32 bulk with FP64 termination at the
    tolerance; value = solves/s. Also times the same instances solved one after another through
    the single-LP path (the plain per-instance form) on the same GPU."""
    world, rank, local, pg = dist_setup(args.gpus)
    import torch
    import cupdlp
    from cupdlp import synthetic
    from cupdlp.solver import DeviceBatch, DeviceProblem, scaled_desc
    torch.cuda.set_device(local)
    torch.zeros(1, device="cuda")
    lps = synthetic.batch_lps(3 + rank, count=args.batch_count)
    params = cupdlp.default_parameters(tolerance=args.tolerance, precision=cupdlp.Precision.FP32,
                                       record_iteration_stats=False, time_sec_limit=600.0)
    scaled = [cupdlp.rescale_problem(10, False, 1.0, 0, lp.problem) for lp in lps]
    descs = [scaled_desc(sq) for sq in scaled]
    nnz = sum(d.desc.nnz for d in descs)
    db = DeviceBatch(descs)
    for _ in range(args.warmup):
        db.solve(params, want_solution=False)
    barrier(pg)
    torch.cuda.synchronize()
    times, results = [], None
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            t0 = time.perf_counter()
            results, _, _ = db.solve(params, want_solution=False)
            times.append(time.perf_counter() - t0)
    clocks = clk.summary()
    t_max = max_over_ranks(pg, sum(times))
    solves = sum_over_ranks(pg, len(lps) * args.steps)
    value = solves / t_max
    opt = sum(1 for r in results if r.termination_reason == 1)
    err = []
    for lp, r in zip(lps, results):
        if lp.optimal_objective:
            po = r.last_iteration_stats.convergence_information.primal_objective
            err.append(abs(po - lp.optimal_objective) / max(1.0, abs(lp.optimal_objective)))
    launches = results[0].kernels_launched * args.steps
    # the plain per-instance form: each LP alone through gpdhg_problem_create + gpdhg_solve
    t0 = time.perf_counter()
    for d in descs:
        with DeviceProblem(d) as dp:
            dp.solve(params, want_solution=False)
    seq = time.perf_counter() - t0
    # the reference's loop in its own GPU form, one instance after another, on every 8th
    # instance (a sample of the same size mix), FP64 as the reference computes
    rge = None
    if rank == 0:
        try:
            sys.path.insert(0, os.path.join(REPO, "baseline"))
            import ref_equiv
            p64 = cupdlp.default_parameters(tolerance=args.tolerance, record_iteration_stats=False,
                                            time_sec_limit=600.0)
            sample = list(range(0, len(scaled), 8))
            t0 = time.perf_counter()
            ok = 0
            for k in sample:
                r, _, _ = ref_equiv.solve_scaled(scaled[k], p64, want_solution=False)
                ok += int(r.termination_reason == 1)
            tr = time.perf_counter() - t0
            rge = {"value": len(sample) / tr, "unit": "solves/s", "sample": f"{len(sample)} of {len(scaled)} "
                   f"instances (every 8th), solved one after another, {tr:.1f} s", "terminated_optimal": ok,
                   "ours_over_reference": value / world / (len(sample) / tr),
                   "form": "reference call pattern on this GPU: cuSPARSE CSR_ALG2 FP64 SpMV, per-kernel sync, "
                           "host-side dot/nrm2 every attempt (baseline/ref_equiv.cu)"}
        except Exception as e:
            rge = {"unavailable": f"{type(e).__name__}: {e}"}
    # e2e: the batched call with host buffers in pinned memory (pack + upload + solve + copy
    # back), averaged over up to two passes
    pinned = [pinned_desc(d) for d in descs]
    e2e_runs = max(1, min(args.steps, 2))
    t0 = time.perf_counter()
    for _ in range(e2e_runs):
        with DeviceBatch(pinned) as dq:
            dq.solve(params, want_solution=True)
    e2e_sec = (time.perf_counter() - t0) / e2e_runs
    h2d = sum(sum(a.nbytes for a in d.arrays.values() if a is not None) for d in pinned)
    d2h = sum(8 * (d.desc.num_variables + d.desc.num_constraints) for d in descs)
    line = {
        "metric": "batched solves/sec", "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max * 1e3 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (seeded)",
        "config": {"workload": f"{len(lps)} LPs, m log-normal (median 2,000, 200-50,000), n = 2m, "
                               f"nnz/row U(5,40), 25% transportation-shaped; {nnz} nonzeros in total",
                   "tolerance": args.tolerance, "terminated_optimal": opt,
                   "max_objective_error_vs_planted": max(err) if err else None,
                   "sequential_single_lp_solves_per_sec": len(lps) / seq,
                   "l2": "batch working set > L2"},
        "e2e": {"value": len(lps) / e2e_sec, "unit": "solves/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(launches), "clocks": clocks,
    }
    if rge:
        line["reference_gpu_equiv"] = rge
    db.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if pg is not None:
        pg.destroy_process_group()
    return 0


def run_serve(args):
    """Continuous batching (gpdhg_server_*) under Poisson arrivals: 70% small LPs (m 200-2,000),
    25% medium (m 10k-100k), 5% large (power-law m = 500k, nnz = 10M), drawn from a seeded pool
    of pre-generated, pre-scaled instances; small and medium in FP64, large in FP32, tolerance
    1e-4. Latency = result available on the host - arrival; value = completed requests / s at the
    middle rate. Beside it, the plain per-request form on the same GPU: one gpdhg_problem at a
    time in arrival order, its latencies from the queue driven by each pool LP's measured
    create + solve + copy-back time."""
    world, rank, local, pg = dist_setup(args.gpus)
    import threading
    import torch
    import cupdlp
    from cupdlp import synthetic
    from cupdlp.solver import DeviceProblem, Server, scaled_desc
    torch.cuda.set_device(local)
    torch.zeros(1, device="cuda")
    rng = np.random.default_rng(7 + rank)
    pool = {"small": [], "medium": [], "large": []}
    sizes = {"small": 16, "medium": 4, "large": 1}
    for kind, cnt in sizes.items():
        for _ in range(cnt):
            lp = synthetic.serving_mixture_lp(rng, kind)
            sq = cupdlp.rescale_problem(10, False, 1.0, 0, lp.problem)
            pool[kind].append(scaled_desc(sq))
    p64 = cupdlp.default_parameters(tolerance=1e-4, precision=cupdlp.Precision.FP64, record_iteration_stats=False,
                                    iteration_limit=20_000, time_sec_limit=120.0)
    p32 = cupdlp.default_parameters(tolerance=1e-4, precision=cupdlp.Precision.FP32, record_iteration_stats=False,
                                    iteration_limit=1_000, time_sec_limit=120.0)
    par = {"small": p64, "medium": p64, "large": p32}
    # measured service time of every pool LP alone (create + solve + copy back), after a warm-up
    service = {}
    for kind, descs in pool.items():
        for i, d in enumerate(descs):
            for rep in range(2):
                t0 = time.perf_counter()
                with DeviceProblem(d) as dp:
                    dp.solve(par[kind], want_solution=True)
                service[(kind, i)] = time.perf_counter() - t0
    rates = [float(r) for r in args.serve_rates.split(",")]
    mix = (0.70, 0.25, 0.05)
    per_rate = {}
    launches = 0
    with ClockSampler(local) as clk:
        for rate in rates:
            arr = []
            t = 0.0
            while True:
                t += rng.exponential(1.0 / rate)
                if t > args.serve_duration:
                    break
                u = rng.random()
                kind = "small" if u < mix[0] else ("medium" if u < mix[0] + mix[1] else "large")
                arr.append((t, kind, int(rng.integers(0, len(pool[kind])))))
            done = {}
            lock = threading.Lock()
            with Server(hbm_budget_bytes=150e9, workers=3, max_cohort=256, linger_sec=0.002) as srv:
                tickets = {}
                stop = threading.Event()

                def collect():
                    while not stop.is_set() or len(done) < len(tickets):
                        with lock:
                            pending = [(tk, q) for q, tk in tickets.items() if q not in done]
                        for tk, q in pending:
                            if srv.poll(tk) is not None:
                                done[q] = time.perf_counter()
                        if stop.is_set() and time.perf_counter() > deadline:
                            return
                        time.sleep(0.0005)

                deadline = float("inf")
                col = threading.Thread(target=collect, daemon=True)
                col.start()
                t_start = time.perf_counter()
                for q, (ta, kind, i) in enumerate(arr):
                    now = time.perf_counter() - t_start
                    if ta > now:
                        time.sleep(ta - now)
                    tk = srv.submit(pool[kind][i], par[kind])
                    with lock:
                        tickets[q] = tk
                deadline = time.perf_counter() + args.serve_drain_cap
                stop.set()
                col.join()
            lat = sorted(done[q] - (t_start + arr[q][0]) for q in done)
            span = (max(done.values()) - t_start) if done else float("nan")
            # the plain per-request form: one LP at a time in arrival order
            free_at, seq_lat = 0.0, []
            for (ta, kind, i) in arr:
                start = max(ta, free_at)
                free_at = start + service[(kind, i)]
                seq_lat.append(free_at - ta)
            seq_lat.sort()
            pct = lambda v, p: v[min(len(v) - 1, int(p * len(v)))] if v else None
            per_rate[str(int(rate))] = {
                "requests": len(arr), "completed": len(done), "unfinished": len(arr) - len(done),
                "solves_per_sec": len(done) / span if done else 0.0,
                "p50_latency_sec": pct(lat, 0.50), "p99_latency_sec": pct(lat, 0.99),
                "plain_per_request": {"solves_per_sec": len(arr) / free_at if free_at else None,
                                      "p50_latency_sec": pct(seq_lat, 0.50), "p99_latency_sec": pct(seq_lat, 0.99)},
                "mix": {k: sum(1 for a in arr if a[1] == k) for k in pool},
            }
    clocks = clk.summary()
    mid = per_rate[str(int(rates[len(rates) // 2]))]
    line = {
        "metric": "served solves/sec (p50/p99 latency in config)", "value": mid["solves_per_sec"], "unit": "solves/s",
        "n_gpus": world, "steps": len(rates), "warmup": 1, "ms_per_step": None, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64 (small, medium) / f32+f64 (large)",
        "data": "synthetic (seeded), Poisson arrivals",
        "config": {"workload": "serving stream: 70% small (m 200-2,000), 25% medium (m 10k-100k), 5% large "
                               "(power-law m 500k, nnz 10M); pool 16/4/1 pre-scaled instances; FP64 tol 1e-4 "
                               "(large: FP32, 1,000-iteration cap)",
                   "duration_sec_per_rate": args.serve_duration, "hbm_budget_bytes": 150e9, "workers": 3,
                   "rates": per_rate,
                   "service_sec_alone": {f"{k}[{i}]": v for (k, i), v in service.items()}},
        "e2e": {"value": mid["solves_per_sec"], "unit": "solves/s", "note": "host LP in, host solution out"},
        "gpu_launches": None, "clocks": clocks,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if pg is not None:
        pg.destroy_process_group()
    return 0


def run_ours(args):
    if args.workload == "serve":
        return run_serve(args)
    if args.workload == "batch":
        return run_batch(args)
    world, rank, local, pg = dist_setup(args.gpus)
    import torch
    import cupdlp
    from cupdlp.solver import DeviceProblem, scaled_desc
    torch.cuda.set_device(local)
    torch.zeros(1, device="cuda")
    lp, prec, desc = workload(args.workload)
    if args.precision:
        prec = {"fp64": cupdlp.Precision.FP64, "fp32": cupdlp.Precision.FP32,
                "fp32_refine": cupdlp.Precision.FP32_REFINE}[args.precision]
        desc += f" (precision set to {prec.name})"
    iters = args.iters or DEFAULT_ITERS.get(args.workload, 0)
    params = cupdlp.default_parameters(tolerance=args.tolerance, precision=prec, record_iteration_stats=False,
                                       iteration_limit=iters or 2**31 - 1)
    if iters:
        desc += f", first {iters} iterations per step"
    sq = cupdlp.rescale_problem(10, False, 1.0, 0, lp.problem)
    d = scaled_desc(sq)
    m, n, nnz = d.desc.num_constraints, d.desc.num_variables, d.desc.nnz
    dp = DeviceProblem(d)
    stream = torch.cuda.ExternalStream(dp.lib.gpdhg_problem_stream(dp.handle))
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")

    for _ in range(args.warmup):
        dp.solve(params, want_solution=False)

    cparams = cupdlp.params_to_c(params)
    import ctypes as C
    from cupdlp import _abi

    def timed_solves(profile):
        # solves with the inputs resident, each bracketed by CUDA events on the problem's
        # stream, L2 flushed before each. The profiled solves of an FP32_REFINE workload run
        # its FP32 bulk phase alone (plain FP32, same iterations), so that every profiled
        # launch is an FP32 launch, the precision the byte model counts.
        cparams.profile_kernels = 1 if profile else 0
        cparams.precision = int(cupdlp.Precision.FP32 if profile and prec == cupdlp.Precision.FP32_REFINE
                                else prec)
        out, ms = [], 0.0
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            res = _abi.Result()
            _abi.check(dp.lib.gpdhg_solve(dp.handle, C.byref(cparams), C.byref(res), None, None), dp.lib)
            e1.record(stream)
            e1.synchronize()
            ms += e0.elapsed_time(e1)
            out.append(res)
        return out, ms

    barrier(pg)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        results, ms_total = timed_solves(profile=False)
    torch.cuda.synchronize()
    barrier(pg)
    clocks = clk.summary()
    kkt = sum(r.cumulative_kkt_matrix_passes for r in results)
    t_max = max_over_ranks(pg, ms_total / 1e3)
    kkt_all = sum_over_ranks(pg, kkt)
    value = kkt_all / t_max
    launches = sum(r.kernels_launched for r in results)

    # roofline of the dominant step kernel: the same solves again with a CUDA event between
    # every two step kernels (launched one by one: events inside a CUDA graph cannot split
    # its kernels), per-kernel durations summed over all attempts
    prof, _ = timed_solves(profile=True)
    bm = bytes_model(m, n, nnz, 0 if prec == cupdlp.Precision.FP64 else 1)
    attempts = sum(r.primal_kernel_launches for r in prof)
    spmv = sum(r.primal_spmv_launches for r in prof)
    tp = sum(r.primal_kernel_sec for r in prof)
    td = sum(r.dual_kernel_sec for r in prof)
    bytes_p = spmv * bm["primal_commit"] + (attempts - spmv) * bm["primal_plain"]
    bytes_d = attempts * bm["dual"] + spmv * bm["dual_commit_extra"]
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    dom = "primal_step_kernel" if tp >= td else "dual_step_kernel"
    b_dom, t_dom = (bytes_p, tp) if tp >= td else (bytes_d, td)
    achieved = (b_dom / t_dom / 1e9) if t_dom > 0 else None
    traffic = profile_traffic(args.workload, dom)
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                "traffic_unit": "bytes per launch (ncu dram__bytes_read.sum + dram__bytes_write.sum, cold cache; "
                                "profiles/" + PROFILE_FILES.get(args.workload, "-") + ")",
                "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback 6.8 TB/s",
                "share_of_step_time": {"primal_step_kernel": tp / max(tp + td, 1e-30),
                                       "dual_step_kernel": td / max(tp + td, 1e-30)},
                "bytes_per_launch": {"primal_with_commit": bm["primal_commit"], "dual": bm["dual"]},
                "fp64_pipe_active_pct_ncu": profile_fp64_pipe(args.workload, dom),
                "profiled_precision": "FP32 (the bulk phase)" if prec == cupdlp.Precision.FP32_REFINE else
                                      precision_name(prec),
                "step_pair_GBps": ((bytes_p + bytes_d) / (tp + td) / 1e9) if tp + td > 0 else None}

    # e2e through the C ABI with host buffers (create -> solve -> copy back), every step; the
    # inputs sit in pinned host memory
    e2e_times, e2e_kkt = [], 0.0
    dpin = pinned_desc(d)
    h2d = sum(a.nbytes for a in dpin.arrays.values() if a is not None)
    d2h = 8 * (n + m)
    create_times = []
    for k in range(max(1, min(args.steps, 3))):
        t0 = time.perf_counter()
        with DeviceProblem(dpin) as dq:
            create_times.append(time.perf_counter() - t0)
            r, x, y = dq.solve(params, want_solution=True)
        e2e_times.append(time.perf_counter() - t0)
        e2e_kkt += r.cumulative_kkt_matrix_passes
    e2e_value = e2e_kkt / sum(e2e_times)

    cb = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cap = args.cpu_sample_iters or (iters if iters else CPU_SAMPLE_ITERS.get(args.workload, 0))
        cb = cpu_baseline(lp.problem, params, cap)
        # the same work on both sides: time to the same result (tolerance or iteration budget)
        cb["gpu_speedup_time_to_result"] = cb["solve_sec"] / (t_max / args.steps)

    # the reference's loop in its own GPU form, same problem and iteration budget (rank 0)
    rge = None
    if rank == 0 and not args.no_reference_gpu:
        try:
            _, rge = reference_gpu_equiv(sq, params)
            our_sec = t_max / args.steps
            rge["ours_over_reference_kkt_rate"] = value / world / rge["value"]
            rge["ours_over_reference_time_to_result"] = rge["solve_sec"] / our_sec
        except Exception as e:   # the baseline is reported, never required
            rge = {"unavailable": f"{type(e).__name__}: {e}"}

    r0 = results[-1]
    ci = r0.last_iteration_stats.convergence_information
    line = {
        "metric": "KKT mults/sec", "value": value, "unit": "KKT passes/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max * 1e3 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64" if prec == cupdlp.Precision.FP64 else "f32+f64",
        "data": "synthetic (seeded)",
        "config": {"workload": desc, "tolerance": args.tolerance, "parallelism": f"replicas x{world}",
                   "l2": "flushed between steps (256 MB write); working set > L2",
                   "iterations_per_solve": r0.iteration_count, "attempts_per_solve": r0.total_number_iterations,
                   "kkt_passes_per_solve": r0.cumulative_kkt_matrix_passes,
                   "termination": int(r0.termination_reason), "primal_objective": ci.primal_objective,
                   "dual_objective": ci.dual_objective,
                   "fp64_handoff_iteration": int(r0.fp64_handoff_iteration)},
        "objective_error": objective_error(args.workload, lp, ci),
        "e2e": {"value": e2e_value, "unit": "KKT passes/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "sec_per_step": statistics.mean(e2e_times),
                "create_sec_per_step": statistics.mean(create_times)},
        "roofline": roofline,
        "gpu_launches": int(launches),
        "clocks": clocks,
    }
    if cb:
        line["cpu_baseline"] = cb
    if rge:
        line["reference_gpu_equiv"] = rge
    dp.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if pg is not None:
        pg.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
