"""Python face of the library's autotuner (gb300_autotune, csrc/gb_autotune.c).

Three plan options shape the task graph of a pattern: the small/large
supernode cutoff (GB300_OPT_SMALL_COLS), the subtree work limit
(GB300_OPT_SUBTREE_WORK) and the depth of the wide supernodes' trailing
tile products (GB300_OPT_UPD_GROUP: g panels per 64 x 64 x 64 g product).
The tuner in the C library times the factorization under each candidate
(device time of the library's CUDA events, median of a few repetitions
after a warm-up that builds the candidate's plan) and leaves the fastest
candidate set on the cholmod_common; C callers reach the same tuner through
gb300_autotune or GB300_OPT_AUTOTUNE.
"""
import ctypes as C

from . import cholmod as CH


def default_candidates():
    """The library's default list of (small_cols, subtree_work, upd_group)."""
    n = CH.lib().gb300_autotune_candidates(None, 0)
    buf = (C.c_int64 * (3 * n))()
    CH.lib().gb300_autotune_candidates(buf, n)
    return [tuple(buf[3 * i:3 * i + 3]) for i in range(n)]


def _cand_array(candidates):
    rows = []
    for c in candidates:
        c = tuple(int(v) for v in c)
        rows.append(c if len(c) == 3 else c + (4,))
    buf = (C.c_int64 * (3 * len(rows)))(*[v for r in rows for v in r])
    return rows, buf


def autotune(A, L, common, candidates=None, reps=3, mixed=True, timer=None):
    """Returns (best (small_cols, subtree_work, upd_group), {candidate: median ms}).

    candidates: (small_cols, subtree_work[, upd_group]) tuples (group 4 when
    left out), or None for the library's default list.  timer(common) ->
    milliseconds of one run under the options set on common replaces the
    library's own timing of the factorization of A (A and L are then not
    used)."""
    rows, buf = _cand_array(candidates if candidates is not None else default_candidates())
    ms = (C.c_double * len(rows))()
    if timer is None:
        best = CH.lib().gb300_autotune(A, L, int(bool(mixed)), reps, buf, len(rows), ms,
                                       common.ptr)
    else:
        cb = CH.TUNE_TIMER(lambda _c, _ud: float(timer(common)))
        best = CH.lib().gb300_autotune_with(buf, len(rows), reps, ms, cb, None, common.ptr)
    if best < 0:
        raise RuntimeError(f"factorization failed during tuning, status {common.status}")
    return rows[best], {r: ms[i] for i, r in enumerate(rows)}
