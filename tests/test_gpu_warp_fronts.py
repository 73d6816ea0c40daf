"""One-warp fronts (GB300_OPT_WARP_ROWS): a front of at most that many rows
assembled and factorized by one warp gives the same factor, bit for bit, as
the same front on a whole thread block, whatever the subtree grouping
(GB300_OPT_SUBTREE_WORK) -- in FP64, in FP32, and for a matrix that is not
positive definite; the sweeps' one-warp leaf subtrees keep both solve forms
at their accuracy bars."""
import numpy as np
import pytest

from conftest import make_case
from suitesparse_gb300 import cholmod as CH
from suitesparse_gb300 import matrices as M

pytestmark = pytest.mark.gpu

SETTINGS = [(0, 0), (32, 0), (64, 0), (0, 4_000_000), (16, 4_000_000), (32, 4_000_000),
            (48, 4_000_000), (64, 4_000_000), (64, 10**9)]


def _factor(meta, arrays, name, warp_rows, sub_work, dtype="d"):
    c = CH.Common()
    c.set_option(CH.GB300_OPT_WARP_ROWS, warp_rows)
    c.set_option(CH.GB300_OPT_SUBTREE_WORK, sub_work)
    n, Ap, Ai, Ax = make_case(meta, name)
    A = CH.sparse(n, Ap, Ai, Ax if dtype == "d" else Ax.astype(np.float32), c, dtype=dtype)
    L = CH.analyze_perm(A, arrays[name + "_Perm"].astype(np.int64), c)
    assert CH.factorize(A, L, c) == 1
    f = CH.factor_arrays(L)
    out = (c.status, f["minor"], np.array(f["Lx"], copy=True))
    CH.free_factor(L, c)
    CH.free_sparse(A, c)
    return out


def _tiny_share(meta, arrays, name):
    c = CH.Common()
    n, Ap, Ai, Ax = make_case(meta, name)
    A = CH.sparse(n, Ap, Ai, Ax, c)
    L = CH.analyze_perm(A, arrays[name + "_Perm"].astype(np.int64), c)
    f = CH.factor_arrays(L)
    share = float(np.mean(np.diff(f["Pi"]) <= 32))
    CH.free_factor(L, c)
    CH.free_sparse(A, c)
    return share


@pytest.mark.parametrize("dtype", ["d", "s"])
@pytest.mark.parametrize("name", ["g2v", "g3", "e27", "c1"])
def test_same_factor_bit_for_bit(golden, lib, name, dtype):
    meta, arrays = golden
    assert _tiny_share(meta, arrays, name) > 0.05     # the case exercises the warp path
    ref = _factor(meta, arrays, name, 0, 0, dtype)
    assert ref[0] == CH.CHOLMOD_OK
    for wr, sw in SETTINGS[1:]:
        st, minor, Lx = _factor(meta, arrays, name, wr, sw, dtype)
        assert st == ref[0] and minor == ref[1]
        assert np.array_equal(Lx, ref[2]), (wr, sw)


def test_not_positive_definite_same_state(golden, lib):
    meta, arrays = golden
    ref = _factor(meta, arrays, "npd", 0, 0)
    assert ref[0] == CH.CHOLMOD_NOT_POSDEF and ref[1] == meta["npd"]["minor"]
    for wr, sw in SETTINGS[1:]:
        st, minor, Lx = _factor(meta, arrays, "npd", wr, sw)
        assert st == ref[0] and minor == ref[1]
        assert np.array_equal(Lx, ref[2]), (wr, sw)


@pytest.mark.parametrize("name", ["g2v", "c1"])
@pytest.mark.parametrize("nrhs", [1, 3, 20])
def test_solves_with_and_without_warp_paths(golden, lib, oracle_mod, name, nrhs):
    """The sweeps run leaf subtrees of one-warp fronts (GB300_OPT_WARP_ROWS >
    0) in launches of their own; with and without them both the FP64 solve
    and the mixed form's refined solve reach their accuracy bars."""
    meta, arrays = golden
    n, Ap, Ai, Ax = make_case(meta, name)
    B = M.rhs(n, nrhs, 4)
    sols = []
    for wr in (0, 32):
        c = CH.Common()
        c.set_option(CH.GB300_OPT_WARP_ROWS, wr)
        A = CH.sparse(n, Ap, Ai, Ax, c)
        L = CH.analyze_perm(A, arrays[name + "_Perm"].astype(np.int64), c)
        assert CH.factorize(A, L, c) == 1
        X = CH.solve(L, B, c)
        assert oracle_mod.backward_error(n, Ap, Ai, Ax, X, B).max() <= 1e-14
        sols.append(np.array(X, copy=True))
        assert CH.factorize_mixed(A, L, c) == 1
        Xm, info = CH.solve_refined(A, L, B, c, tol=1e-12)
        assert oracle_mod.backward_error(n, Ap, Ai, Ax, Xm, B).max() <= 1e-12
        assert info["iterations"] <= 3
        CH.free_factor(L, c)
        CH.free_sparse(A, c)
    np.testing.assert_allclose(sols[1], sols[0], rtol=1e-10, atol=1e-12 * np.abs(sols[0]).max())


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_random_orderings_match_oracle(lib, oracle_mod, seed):
    """Random permutations give irregular elimination trees (subtrees that
    are not index ranges, fronts of every height): the one-warp fronts, the
    subtree waves and the sweeps' leaf subtrees still give the oracle's
    factor and accurate solves."""
    rng = np.random.default_rng(seed)
    n, Ap, Ai, Ax = M.laplace2d(24 + 6 * seed, seed=seed)
    perm = rng.permutation(n).astype(np.int64)
    c = CH.Common()
    A = CH.sparse(n, Ap, Ai, Ax, c)
    L = CH.analyze_perm(A, perm, c)
    assert CH.factorize(A, L, c) == 1 and c.status == CH.CHOLMOD_OK
    f = CH.factor_arrays(L)
    sym = {k: f[k] for k in ("Super", "Pi", "Px", "Ls")}
    sym["n"] = n
    Sp, Si, Sx = oracle_mod.permute_lower(n, Ap, Ai, Ax, perm)
    st, minor, Lref = oracle_mod.factor(sym, Sp, Si, Sx)
    rel = np.linalg.norm(f["Lx"] - Lref) / np.linalg.norm(Lref)
    assert rel < 1e-10, rel
    B = M.rhs(n, 3, seed)
    X = CH.solve(L, B, c)
    assert oracle_mod.backward_error(n, Ap, Ai, Ax, X, B).max() <= 1e-14
    assert CH.factorize_mixed(A, L, c) == 1
    Xm, info = CH.solve_refined(A, L, B, c, tol=1e-12)
    assert oracle_mod.backward_error(n, Ap, Ai, Ax, Xm, B).max() <= 1e-12
    CH.free_factor(L, c)
    CH.free_sparse(A, c)
