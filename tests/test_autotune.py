"""The plan-option autotuner of the C library (gb300_autotune,
csrc/gb_autotune.c): its selection logic on the CPU with a stand-in timer
(through gb300_autotune_with), and on the GPU real tuning runs whose chosen
setting still factorizes to the oracle's accuracy, every update group
giving the oracle's factor, and the automatic tuning of an unchanged
cholmod_l_super_numeric caller (GB300_OPT_AUTOTUNE)."""
import numpy as np
import pytest

from conftest import make_case
from suitesparse_gb300 import autotune as AT
from suitesparse_gb300 import cholmod as CH
from suitesparse_gb300 import matrices as M

OPTS = (CH.GB300_OPT_SMALL_COLS, CH.GB300_OPT_SUBTREE_WORK, CH.GB300_OPT_UPD_GROUP)


def _current(c):
    return tuple(c.get_option(o) for o in OPTS)


def test_picks_fastest_and_leaves_it_set(lib):
    times = {(64, 4_000_000, 4): 5.0, (64, 0, 2): 3.0, (32, 4_000_000, 1): 4.0}
    c = CH.Common()
    calls = []

    def timer(common):
        key = _current(common)
        calls.append(key)
        return times[key]

    best, table = AT.autotune(None, None, c, candidates=list(times), reps=2, timer=timer)
    assert best == (64, 0, 2) and table == times
    assert _current(c) == (64, 0, 2)
    assert len(calls) == 3 * len(times)          # warm-up + 2 repetitions each
    c.finish()


def test_median_and_failure_restores(lib):
    c = CH.Common()
    seq = iter([9.0, 7.0, 1.0, 8.0,          # candidate 0: warm-up, then 7, 1, 8 -> median 7
                9.0, 6.0, 6.5, 5.0])         # candidate 1: median 6
    best, table = AT.autotune(None, None, c, candidates=[(64, 0, 4), (16, 0, 1)], reps=3,
                              timer=lambda common: next(seq))
    assert best == (16, 0, 1) and table[(64, 0, 4)] == 7.0 and table[(16, 0, 1)] == 6.0
    # a failing run ends the tuning and restores the options set before it
    c.set_option(CH.GB300_OPT_SMALL_COLS, 48)
    c.set_option(CH.GB300_OPT_UPD_GROUP, 3)
    before = _current(c)
    with pytest.raises(RuntimeError):
        AT.autotune(None, None, c, candidates=[(64, 0, 4), (16, 0, 1)], reps=1,
                    timer=lambda common: -1.0)
    assert _current(c) == before
    c.finish()


def test_default_candidates_and_option_limits(lib):
    cand = AT.default_candidates()
    assert len(cand) >= 6 and len(set(cand)) == len(cand)
    assert all(1 <= s <= 64 and w >= 0 and 1 <= g <= 4 for s, w, g in cand)
    c = CH.Common()
    assert _current(c) == (64, 4_000_000, 4)                 # defaults
    c.set_option(CH.GB300_OPT_UPD_GROUP, 9)
    assert c.get_option(CH.GB300_OPT_UPD_GROUP) == 4         # clamped to 1..4
    c.set_option(CH.GB300_OPT_UPD_GROUP, 0)
    assert c.get_option(CH.GB300_OPT_UPD_GROUP) == 1
    assert c.get_option(CH.GB300_OPT_AUTOTUNE) == 0
    c.finish()


@pytest.mark.gpu
def test_tuned_setting_factorizes_correctly(golden, lib, oracle_mod):
    meta, arrays = golden
    c = CH.Common()
    n, Ap, Ai, Ax = make_case(meta, "c1")
    A = CH.sparse(n, Ap, Ai, Ax, c)
    L = CH.analyze_perm(A, arrays["c1_Perm"].astype(np.int64), c)
    best, table = AT.autotune(A, L, c, candidates=((64, 4_000_000), (64, 0, 2), (16, 1_000_000, 1)),
                              reps=1, mixed=True)
    assert best in table and all(v > 0 for v in table.values())
    assert _current(c) == best
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


def _p40():
    # 40^3 variable-coefficient Laplacian, nested dissection: supernodes up
    # to ~1,600 wide, so every update group shapes many tile products
    return M.laplace3d(40, seed=1), M.grid_nd_perm((40, 40, 40))


@pytest.mark.gpu
@pytest.mark.parametrize("group", [1, 2, 3])
def test_update_groups_give_the_oracle_factor(lib, oracle_mod, group):
    (n, Ap, Ai, Ax), perm = _p40()
    facs = {}
    for g in (group, 4):
        c = CH.Common()
        assert c.set_option(CH.GB300_OPT_UPD_GROUP, g)
        A = CH.sparse(n, Ap, Ai, Ax, c)
        L = CH.analyze_perm(A, perm, c)
        assert CH.factorize(A, L, c) == 1 and c.status == CH.CHOLMOD_OK
        facs[g] = CH.factor_arrays(L)
        if g == group:
            B = M.rhs(n, 2, 5)
            assert CH.factorize_mixed(A, L, c) == 1
            X, info = CH.solve_refined(A, L, B, c, tol=1e-12)
            assert oracle_mod.backward_error(n, Ap, Ai, Ax, X, B).max() <= 1e-12
            assert not info["fp64_fallback"] and info["iterations"] <= 3, info
        CH.free_factor(L, c)
        CH.free_sparse(A, c)
        c.finish()
    f = facs[group]
    sym = {k: f[k] for k in ("Super", "Pi", "Px", "Ls")}
    sym["n"] = n
    Sp, Si, Sx = oracle_mod.permute_lower(n, Ap, Ai, Ax, perm)
    st, minor, Lref = oracle_mod.factor(sym, Sp, Si, Sx)
    assert st == 0
    for g in (group, 4):
        err = np.linalg.norm(facs[g]["Lx"] - Lref) / np.linalg.norm(Lref)
        assert err <= 1e-10, (g, err)


@pytest.mark.gpu
def test_automatic_tuning_on_first_super_numeric(golden, lib, oracle_mod):
    """GB300_OPT_AUTOTUNE: an unchanged caller of cholmod_l_super_numeric
    gets the tuned options on its first call, and that call's factor is the
    oracle's; the second call does not tune again."""
    meta, arrays = golden
    n, Ap, Ai, Ax = make_case(meta, "c1")
    perm = arrays["c1_Perm"].astype(np.int64)
    c = CH.Common()
    assert c.set_option(CH.GB300_OPT_AUTOTUNE, 1)
    A = CH.sparse(n, Ap, Ai, Ax, c)
    L = CH.analyze_perm(A, perm, c)
    launches0 = c.stats()[5]
    assert CH.factorize(A, L, c) == 1 and c.status == CH.CHOLMOD_OK
    launches1 = c.stats()[5]
    ncand = len(AT.default_candidates())
    # every candidate: a warm-up and one timed factorization, then the call's own
    assert launches1 - launches0 >= 2 * ncand + 1
    assert _current(c) in AT.default_candidates()
    f = CH.factor_arrays(L)
    sym = {k: f[k] for k in ("Super", "Pi", "Px", "Ls")}
    sym["n"] = n
    Sp, Si, Sx = oracle_mod.permute_lower(n, Ap, Ai, Ax, perm)
    st, minor, Lref = oracle_mod.factor(sym, Sp, Si, Sx)
    assert np.linalg.norm(f["Lx"] - Lref) / np.linalg.norm(Lref) <= 1e-10
    assert CH.factorize(A, L, c) == 1
    assert c.stats()[5] - launches1 <= launches1 - launches0   # no second tuning
    CH.free_factor(L, c)
    CH.free_sparse(A, c)
