"""Tile-plan autotuner: measures the step kernels under every candidate plan parameter set on
a family of tuning matrices and writes csrc/tile_table.h, which the planner consults by
row-length histogram (choose_tile_config in csrc/tiles.cu).

Run on a GB300 from the repository root, then rebuild the library:

    python cupdlp.jl_gb300/tune_tiles.py [--iters 200] [--quick] [--min-gain 0.03]
    python cupdlp.jl_gb300/tune_tiles.py --reapply [--min-gain 0.03]   # the rule on the stored times

For each tuning matrix, precision (FP32, FP64) and candidate (tile_nnz, e_floor, tpc_max),
the parameters are pinned with gpdhg_set_tile_override, a problem handle is built and
solved for a fixed number of iterations with per-kernel CUDA-event timing
(params.profile_kernels), and the primal and dual kernels' time per launch is recorded. The
primal kernel's time depends only on the plan of A' and the dual's only on the plan of A, so
each side keeps its own best candidate. The table stores, per matrix, precision and side, the
row-length histogram of that side's matrix and the best parameters; the measured times of
the default and of the best candidate are kept as comments. A candidate replaces the default
parameters only where it is faster by at least --min-gain (3%): smaller differences are within
the run-to-run spread of one measurement and would change a plan for nothing.
"""
from __future__ import annotations

import argparse
import ctypes as C
import itertools
import math
import os
import re
import sys
import time

import numpy as np
import scipy.sparse as sp

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import cupdlp  # noqa: E402
from cupdlp import _abi, synthetic  # noqa: E402
from cupdlp.solver import DeviceProblem, scaled_desc  # noqa: E402

TABLE = os.path.join(HERE, "csrc", "tile_table.h")
HIST_BINS = 16

CANDIDATES = {
    "FP32": list(itertools.product((128, 256), (1, 8), (24, 96))),
    "FP64": list(itertools.product((64, 128), (1, 4), (24, 96))),
}
DEFAULT = {"FP32": (256, 8, 96), "FP64": (128, 4, 96)}


def matrices(quick: bool):
    """(name, LP) pairs spanning row-length shapes: power-law (skewed rows and columns),
    transportation (two per column, rows of 500 and 2,000), uniform random rows, small."""
    out = [("powerlaw_mid", synthetic.power_law_lp(4, m=200_000, n=400_000, target_nnz=4_000_000)),
           ("transportation", synthetic.transportation_lp(1)),
           ("uniform", synthetic.known_optimum_lp(3, m=100_000, n=200_000, density=20 / 200_000)),
           ("small", synthetic.known_optimum_lp(5, m=5_000, n=10_000, density=20 / 10_000))]
    if not quick:
        out.insert(0, ("powerlaw_full", synthetic.power_law_lp(2)))
    return out


def row_histogram(rp: np.ndarray) -> list:
    """The planner's histogram (row_histogram in csrc/tiles.cu): nonzero share per log2 bin of
    row length, then log2(nonzeros) / 32."""
    lens = np.diff(rp.astype(np.int64))
    lens = lens[lens > 0]
    total = int(lens.sum())
    h = [0.0] * (HIST_BINS + 1)
    if total == 0:
        return h
    bins = np.minimum(np.floor(np.log2(lens)).astype(np.int64), HIST_BINS - 1)
    w = np.bincount(bins, weights=lens, minlength=HIST_BINS)
    h[:HIST_BINS] = (w / total).tolist()
    h[HIST_BINS] = math.log2(total) / 32.0
    return h


def measure(lib, desc, precision, cfg, iters):
    """(primal seconds per launch, dual seconds per launch) under cfg on both sides."""
    p = _abi.PRECISION_FP64 if precision == "FP64" else _abi.PRECISION_FP32
    for side in (0, 1):
        _abi.check(lib.gpdhg_set_tile_override(p, side, *cfg), lib)
    try:
        params = cupdlp.default_parameters(tolerance=1e-12, iteration_limit=iters,
                                           precision=cupdlp.Precision(p), record_iteration_stats=False)
        cp = cupdlp.params_to_c(params)
        cp.profile_kernels = 1
        with DeviceProblem(desc) as dp:
            for _ in range(2):   # the first solve builds the plans and graphs
                res = _abi.Result()
                _abi.check(lib.gpdhg_solve(dp.handle, C.byref(cp), C.byref(res), None, None), lib)
        return (res.primal_kernel_sec / max(1, res.primal_kernel_launches),
                res.dual_kernel_sec / max(1, res.primal_kernel_launches))
    finally:
        for side in (0, 1):
            lib.gpdhg_set_tile_override(p, side, 0, 0, 0)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--iters", type=int, default=200)
    ap.add_argument("--quick", action="store_true", help="leave out the 21M-nonzero power-law LP")
    ap.add_argument("--out", default=TABLE)
    ap.add_argument("--min-gain", type=float, default=0.03)
    ap.add_argument("--reapply", action="store_true", help="re-apply --min-gain to the stored table")
    args = ap.parse_args()
    if args.reapply:
        entries, iters = read_table(TABLE)
        write_table(args.out, entries, iters, args.min_gain)
        return
    lib = _abi.load()
    entries = []
    for name, lp in matrices(args.quick):
        t0 = time.time()
        sq = cupdlp.rescale_problem(10, False, 1.0, 0, lp.problem)
        desc = scaled_desc(sq)
        a = sp.csr_matrix(sq.scaled_qp.constraint_matrix)
        hist = {1: row_histogram(a.indptr), 0: row_histogram(sp.csc_matrix(a).indptr)}
        for precision, cands in CANDIDATES.items():
            times = {cfg: measure(lib, desc, precision, cfg, args.iters) for cfg in cands}
            for side in (0, 1):
                best = min(cands, key=lambda c: times[c][side])
                entries.append(dict(name=name, fp64=precision == "FP64", side=side, hist=hist[side], cfg=best,
                                    best=best, t_best=times[best][side], t_default=times[DEFAULT[precision]][side]))
                print(f"{name:15s} {precision} side {side}: best {best} {times[best][side] * 1e6:8.1f} us, "
                      f"default {times[DEFAULT[precision]][side] * 1e6:8.1f} us", flush=True)
        print(f"  ({time.time() - t0:.0f} s)", flush=True)
    write_table(args.out, entries, args.iters, args.min_gain)


def read_table(path):
    """The entries of a written table, with their measured times (from the comments)."""
    text = open(path).read()
    iters = int(re.search(r"over (\d+) iterations", text).group(1))
    pat = re.compile(r'// (\w+) (FP32|FP64) side (\d): ([\d.]+) us \(default ([\d.]+) us; measured best '
                     r'\((\d+), (\d+), (\d+)\)\)\n\s*\{"\w+", \w+, \d, \{([^}]*)\}')
    entries = []
    for m in pat.finditer(text):
        best = (int(m.group(6)), int(m.group(7)), int(m.group(8)))
        entries.append(dict(name=m.group(1), fp64=m.group(2) == "FP64", side=int(m.group(3)),
                            t_best=float(m.group(4)) * 1e-6, t_default=float(m.group(5)) * 1e-6, best=best,
                            hist=[float(v.rstrip("f")) for v in m.group(9).split(",")]))
    return entries, iters


def write_table(path, entries, iters, min_gain):
    for e in entries:
        prec = "FP64" if e["fp64"] else "FP32"
        gain = 1.0 - e["t_best"] / e["t_default"] if e["t_default"] > 0 else 0.0
        e["cfg"] = e["best"] if gain >= min_gain else DEFAULT[prec]
    lines = ['// tile_table.h — measured tile plan parameters by row-length histogram.', '//',
             '// Written by cupdlp.jl_gb300/tune_tiles.py from a sweep of the plan parameters on one',
             '// GB300: for each tuning matrix, precision and kernel side, the histogram of its rows',
             '// (row_histogram) and the parameters with the lowest measured kernel time. The planner',
             '// takes the entry nearest to an instance\'s histogram (choose_tile_config).',
             f'// Kernel times: microseconds per launch over {iters} iterations, best vs default parameters;',
             f'// the best replaces the default where it is at least {100 * min_gain:.0f}% faster.',
             '#pragma once', '', '#include <cstdint>', '', 'namespace gpdhg {', '',
             'struct TileTableEntry {', '  const char* name;', '  bool fp64;', '  int side;', '  float hist[17];',
             '  int32_t tile_nnz, e_floor, tpc_max;', '};', '', 'inline constexpr TileTableEntry kTileTable[] = {']
    for e in entries:
        h = ", ".join(f"{v:.4f}f" for v in e["hist"])
        lines.append(f'    // {e["name"]} {"FP64" if e["fp64"] else "FP32"} side {e["side"]}: '
                     f'{e["t_best"] * 1e6:.1f} us (default {e["t_default"] * 1e6:.1f} us; measured best '
                     f'({e["best"][0]}, {e["best"][1]}, {e["best"][2]}))')
        lines.append(f'    {{"{e["name"]}", {"true" if e["fp64"] else "false"}, {e["side"]}, {{{h}}}, '
                     f'{e["cfg"][0]}, {e["cfg"][1]}, {e["cfg"][2]}}},')
    lines += ['};', '', '}  // namespace gpdhg', '']
    with open(path, "w") as f:
        f.write("\n".join(lines))
    print("wrote", path)


if __name__ == "__main__":
    main()
