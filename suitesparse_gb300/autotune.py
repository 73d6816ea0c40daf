"""Autotuner for the factorization's schedule parameters.

Two parameters shape the task graph of a pattern: the small/large
supernode cutoff (GB300_OPT_SMALL_COLS: supernodes at most this wide are
factorized whole by one thread block, wider ones by 64 x 64 tile tasks) and
the subtree work limit (GB300_OPT_SUBTREE_WORK: subtrees of small supernodes
up to this estimated work run as one task).  The best values depend on the
pattern (a batch of small grids wants large subtrees, a 3D separator tree
wants more parallel tasks).  `autotune` times the factorization of one
matrix under each candidate setting (device time from the library's CUDA
events, median of a few repetitions after a warm-up that builds the plan)
and leaves the fastest setting on the cholmod_common.
"""
import statistics

from . import cholmod as CH

DEFAULT_CANDIDATES = (
    (64, 4_000_000), (64, 16_000_000), (64, 1_000_000), (64, 0),
    (32, 4_000_000), (16, 4_000_000),
)


def _factor_ms(A, L, common, mixed):
    ok = CH.factorize_mixed(A, L, common) if mixed else CH.factorize(A, L, common)
    if not ok:
        raise RuntimeError(f"factorization failed, status {common.status}")
    return common.stats()[0]


def autotune(A, L, common, candidates=DEFAULT_CANDIDATES, reps=3, mixed=True, timer=None):
    """Returns (best (small_cols, subtree_work), {setting: median ms}).

    timer(A, L, common, mixed) -> milliseconds of one factorization; by
    default the library's device time of gb300_factorize_mixed (or of the
    FP64 factorization when mixed is False)."""
    timer = timer or _factor_ms
    table = {}
    for small, work in candidates:
        common.set_option(CH.GB300_OPT_SMALL_COLS, small)
        common.set_option(CH.GB300_OPT_SUBTREE_WORK, work)
        timer(A, L, common, mixed)                    # plan rebuilt for the setting
        table[(small, work)] = statistics.median(timer(A, L, common, mixed) for _ in range(reps))
    best = min(table, key=table.get)
    common.set_option(CH.GB300_OPT_SMALL_COLS, best[0])
    common.set_option(CH.GB300_OPT_SUBTREE_WORK, best[1])
    return best, table
