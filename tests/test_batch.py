"""Batches of independent systems: the symbolic factor of the block-diagonal
batch built by concatenation (gb300_batch_analyze) equals the analysis of the
block-diagonal matrix itself, and the batch factorizes and solves as one
system whose refinement measures every system's backward error."""
import numpy as np
import pytest

from conftest import make_case
from suitesparse_gb300 import cholmod as CH
from suitesparse_gb300 import matrices as M


def _perm_rcm(n, Ap, Ai):
    """A deterministic fill-reducing-ish permutation (reverse level order of a
    breadth-first search from vertex 0) so the cases have bushy etrees."""
    import scipy.sparse as sp
    from scipy.sparse.csgraph import reverse_cuthill_mckee
    A = sp.csc_matrix((np.ones(len(Ai)), Ai, Ap), shape=(n, n))
    return np.asarray(reverse_cuthill_mckee((A + A.T).tocsr(), symmetric_mode=True), dtype=np.int64)


_GENS = [lambda sd: M.laplace2d(6, 5, seed=sd), lambda sd: M.laplace2d(9, seed=sd),
         lambda sd: M.laplace3d(4, seed=sd)]


def _systems():
    """Three patterns; seven systems, each with its own coefficients (same
    structure as its pattern, different values)."""
    pats = [g(11 + q) for q, g in enumerate(_GENS)]
    perms = [_perm_rcm(p[0], p[1], p[2]) for p in pats]
    sys_pat = np.array([1, 0, 2, 1, 1, 0, 2], dtype=np.int32)
    mats = [_GENS[q](100 + i) for i, q in enumerate(sys_pat)]
    for i, q in enumerate(sys_pat):
        assert np.array_equal(mats[i][1], pats[q][1]) and np.array_equal(mats[i][2], pats[q][2])
    return pats, perms, sys_pat, mats


def _fields(L):
    f = L.contents
    ns, n = f.nsuper, f.n
    g = lambda ptr, k: np.ctypeslib.as_array(C.cast(ptr, C.POINTER(C.c_int64)), (k,)).copy()
    return dict(n=n, nsuper=ns, ssize=f.ssize, xsize=f.xsize, maxcsize=f.maxcsize,
                maxesize=f.maxesize, super=g(f.super, ns + 1), pi=g(f.pi, ns + 1),
                px=g(f.px, ns + 1), s=g(f.s, f.ssize), Perm=g(f.Perm, n),
                ColCount=g(f.ColCount, n))


import ctypes as C  # noqa: E402


def test_batch_analyze_equals_block_diagonal_analysis(lib):
    pats, perms, sys_pat, mats = _systems()
    c = CH.Common()
    Lpats = []
    for (n, Ap, Ai, Ax), perm in zip(pats, perms):
        A = CH.sparse(n, Ap, Ai, Ax, c)
        Lpats.append(CH.analyze_perm(A, perm, c))
        CH.free_sparse(A, c)
    Lb = CH.batch_analyze(Lpats, sys_pat, c)
    nb, Ap, Ai, Ax = M.block_diag_lower(mats)
    offs = np.cumsum([0] + [m[0] for m in mats])
    perm = np.concatenate([offs[i] + perms[q] for i, q in enumerate(sys_pat)])
    Ab = CH.sparse(nb, Ap, Ai, Ax, c)
    Ld = CH.analyze_perm(Ab, perm, c)
    fb, fd = _fields(Lb), _fields(Ld)
    for k in fb:
        assert np.array_equal(np.asarray(fb[k]), np.asarray(fd[k])), k
    for L in Lpats + [Lb, Ld]:
        CH.free_factor(L, c)
    CH.free_sparse(Ab, c)


def test_batch_analyze_rejects_bad_input(lib):
    c = CH.Common()
    n, Ap, Ai, Ax = M.laplace2d(4, seed=1)
    A = CH.sparse(n, Ap, Ai, Ax, c)
    L = CH.analyze_perm(A, np.arange(n, dtype=np.int64), c)
    with pytest.raises(RuntimeError):
        CH.batch_analyze([L], np.array([0, 1], dtype=np.int32), c)
    assert c.status == CH.CHOLMOD_INVALID
    CH.free_factor(L, c)
    CH.free_sparse(A, c)


@pytest.mark.gpu
@pytest.mark.parametrize("mixed", [False, True])
def test_batch_factor_solve_per_system(lib, oracle_mod, mixed):
    """Each system of the batch reaches the accuracy target on its own, and
    its block of the batch factor equals its standalone factor bit for bit."""
    pats, perms, sys_pat, mats = _systems()
    c = CH.Common()
    Lpats = []
    for (n, Ap, Ai, Ax), perm in zip(pats, perms):
        A = CH.sparse(n, Ap, Ai, Ax, c)
        Lpats.append(CH.analyze_perm(A, perm, c))
        CH.free_sparse(A, c)
    Lb = CH.batch_analyze(Lpats, sys_pat, c)
    nb, Ap, Ai, Ax = M.block_diag_lower(mats)
    Ab = CH.sparse(nb, Ap, Ai, Ax, c)
    B = M.rhs(nb, 4, 9)
    offs = np.cumsum([0] + [m[0] for m in mats])
    if mixed:
        assert CH.factorize_mixed(Ab, Lb, c) == 1
        X, info = CH.solve_refined(Ab, Lb, B, c, tol=1e-12)
        assert info["berr"] <= 1e-12
    else:
        assert CH.factorize(Ab, Lb, c) == 1 and c.status == CH.CHOLMOD_OK
        X = CH.solve(Lb, B, c)
    for i, (n, p, ii, x) in enumerate(mats):
        lo, hi = offs[i], offs[i + 1]
        be = oracle_mod.backward_error(n, p, ii, x, X[lo:hi], B[lo:hi])
        assert be.max() <= (1e-12 if mixed else 1e-14), (i, be)
    if not mixed:
        # the batch factor's supernodes of system i are its standalone factor's
        fb = CH.factor_arrays(Lb)
        for i, q in enumerate(sys_pat):
            n, p, ii, x = mats[i]
            A = CH.sparse(n, p, ii, x, c)
            Ls = CH.analyze_perm(A, perms[q], c)
            assert CH.factorize(A, Ls, c) == 1
            fs = CH.factor_arrays(Ls)
            s0 = int(np.searchsorted(fb["Super"], offs[i]))
            assert fb["Super"][s0] == offs[i]
            x0 = int(fb["Px"][s0])
            xs = fs["Lx"]
            # the same arithmetic in the same order: equal bit for bit
            assert np.array_equal(fb["Lx"][x0:x0 + len(xs)], xs), i
            CH.free_factor(Ls, c)
            CH.free_sparse(A, c)
    for L in Lpats + [Lb]:
        CH.free_factor(L, c)
    CH.free_sparse(Ab, c)


@pytest.mark.gpu
def test_batch_refinement_freezes_converged_systems(lib, oracle_mod):
    """The refined solve of a batch refines only the systems still above the
    tolerance: a system whose backward error is reached stops (its sweep
    tasks are skipped, its correction is zero), so every system's solution
    is the one its own refined solve gives, even beside a system that needs
    more steps."""
    nx = 24
    mats = [M.laplace2d(nx, seed=31, lo=0.5, hi=2.0), M.laplace2d(nx, seed=32, lo=1e-5, hi=1e5, shift=0.0),
            M.laplace2d(nx, seed=33, lo=0.5, hi=2.0), M.laplace2d(nx, seed=34, lo=1e-3, hi=1e3)]
    n, Ap, Ai, _ = mats[0]
    perm = _perm_rcm(n, Ap, Ai)
    c = CH.Common()
    alone, iters = [], []
    for i, (n, p, ii, x) in enumerate(mats):
        A = CH.sparse(n, p, ii, x, c)
        L = CH.analyze_perm(A, perm, c)
        assert CH.factorize_mixed(A, L, c) == 1
        X, info = CH.solve_refined(A, L, M.rhs(n, 2, 40 + i), c, tol=1e-12)
        assert info["berr"] <= 1e-12 and not info["fp64_fallback"]
        alone.append(np.array(X, copy=True))
        iters.append(info["iterations"])
        CH.free_factor(L, c)
        CH.free_sparse(A, c)
    assert len(set(iters)) > 1, iters            # the systems need different step counts
    A0 = CH.sparse(n, Ap, Ai, mats[0][3], c)
    Lpat = CH.analyze_perm(A0, perm, c)
    CH.free_sparse(A0, c)
    Lb = CH.batch_analyze([Lpat], np.zeros(len(mats), dtype=np.int32), c)
    nb, bp, bi, bx = M.block_diag_lower(mats)
    Ab = CH.sparse(nb, bp, bi, bx, c)
    B = np.vstack([M.rhs(n, 2, 40 + i) for i in range(len(mats))])
    assert CH.factorize_mixed(Ab, Lb, c) == 1
    X, info = CH.solve_refined(Ab, Lb, B, c, tol=1e-12)
    assert info["iterations"] == max(iters) and info["berr"] <= 1e-12
    for i, (n, p, ii, x) in enumerate(mats):
        Xi = X[i * n:(i + 1) * n]
        assert oracle_mod.backward_error(n, p, ii, x, Xi, B[i * n:(i + 1) * n]).max() <= 1e-12
        # the batch's arithmetic for system i is its own: the same solution
        assert np.array_equal(Xi, alone[i]), (i, iters, np.abs(Xi - alone[i]).max())
    for L in (Lpat, Lb):
        CH.free_factor(L, c)
    CH.free_sparse(Ab, c)
