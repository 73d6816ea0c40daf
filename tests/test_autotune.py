"""The schedule autotuner: selection logic on the CPU with a stand-in timer,
and on the GPU a real tuning run whose chosen setting still factorizes to
the oracle's accuracy."""
import numpy as np
import pytest

from conftest import make_case
from suitesparse_gb300 import autotune as AT
from suitesparse_gb300 import cholmod as CH
from suitesparse_gb300 import matrices as M


class _Opts:
    """Records the options the tuner sets (stands in for cholmod_common)."""

    def __init__(self):
        self.opts = {}

    def set_option(self, k, v):
        self.opts[k] = v


def test_picks_fastest_and_leaves_it_set():
    times = {(64, 4_000_000): 5.0, (64, 0): 3.0, (32, 4_000_000): 4.0}
    c = _Opts()
    calls = []

    def timer(A, L, common, mixed):
        key = (common.opts[CH.GB300_OPT_SMALL_COLS], common.opts[CH.GB300_OPT_SUBTREE_WORK])
        calls.append(key)
        return times[key]

    best, table = AT.autotune(None, None, c, candidates=list(times), reps=2, timer=timer)
    assert best == (64, 0) and table == times
    assert c.opts[CH.GB300_OPT_SMALL_COLS] == 64 and c.opts[CH.GB300_OPT_SUBTREE_WORK] == 0
    assert len(calls) == 3 * len(times)          # warm-up + 2 repetitions each


@pytest.mark.gpu
def test_tuned_setting_factorizes_correctly(golden, lib, oracle_mod):
    meta, arrays = golden
    c = CH.Common()
    n, Ap, Ai, Ax = make_case(meta, "c1")
    A = CH.sparse(n, Ap, Ai, Ax, c)
    L = CH.analyze_perm(A, arrays["c1_Perm"].astype(np.int64), c)
    best, table = AT.autotune(A, L, c, candidates=((64, 4_000_000), (64, 0), (16, 1_000_000)),
                              reps=1, mixed=True)
    assert best in table and all(v > 0 for v in table.values())
    assert CH.factorize_mixed(A, L, c) == 1
    B = M.rhs(n, 2, 8)
    X, info = CH.solve_refined(A, L, B, c, tol=1e-12)
    assert oracle_mod.backward_error(n, Ap, Ai, Ax, X, B).max() <= 1e-12
    # the FP64 form with the tuned plan matches the reference factor
    assert CH.factorize(A, L, c) == 1
    X64 = CH.solve(L, B, c)
    assert oracle_mod.backward_error(n, Ap, Ai, Ax, X64, B).max() <= 1e-14
    CH.free_factor(L, c)
    CH.free_sparse(A, c)
