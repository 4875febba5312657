"""The measured tile-plan table (csrc/tile_table.h, written by cupdlp.jl_gb300/tune_tiles.py)
and the histogram the planner keys it by (no GPU needed)."""
import os
import re
import sys

import numpy as np
import scipy.sparse as sp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(REPO, "cupdlp.jl_gb300"))

import tune_tiles  # noqa: E402

TABLE = os.path.join(REPO, "cupdlp.jl_gb300", "csrc", "tile_table.h")


def _entries():
    text = open(TABLE).read()
    pat = re.compile(r'\{"(\w+)", (true|false), (-?\d), \{([^}]*)\}, (\d+), (\d+), (\d+)\}')
    return [(m.group(1), m.group(2) == "true", int(m.group(3)),
             [float(v.rstrip("f")) for v in m.group(4).split(",") if v.strip()],
             int(m.group(5)), int(m.group(6)), int(m.group(7))) for m in pat.finditer(text)]


def test_table_entries_are_within_the_kernels_limits():
    for name, fp64, side, hist, tile_nnz, e_floor, tpc in _entries():
        if side < 0:
            continue   # placeholder
        assert side in (0, 1)
        assert len(hist) == 17
        assert abs(sum(hist[:16]) - 1.0) < 1e-3 and 0.0 < hist[16] <= 1.0
        e_max = 4 if fp64 else 8
        assert 32 <= tile_nnz <= 32 * e_max and 1 <= e_floor <= e_max and 8 <= tpc <= 96


def test_histogram_matches_the_planners_bins():
    # rows of lengths 1, 2, 3, 4, 7, 8 and 40000: bins floor(log2(len)), the last bin open
    lens = np.array([1, 2, 3, 4, 7, 8, 40000])
    rp = np.concatenate([[0], np.cumsum(lens)])
    h = tune_tiles.row_histogram(rp)
    total = lens.sum()
    want = np.zeros(16)
    for n in lens:
        want[min(int(np.floor(np.log2(n))), 15)] += n / total
    np.testing.assert_allclose(h[:16], want, rtol=1e-12)
    assert h[16] == np.log2(total) / 32


def test_tuning_candidates_include_the_defaults():
    for prec, cands in tune_tiles.CANDIDATES.items():
        assert tune_tiles.DEFAULT[prec] in cands
