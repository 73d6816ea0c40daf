"""Sparse right-hand sides (cholmod_l_spsolve) and the sys values of the
solve.  On the CPU: the oracle's restatement against the reference's own
cholmod_l_spsolve output for every sys (tests/golden/spsolve.npz, made by
tests/golden/make_spsolve.py), and the argument checks of the C ABI.  On the
GPU: cholmod_l_spsolve and gb300_solve(sys) through the C ABI against the
same fixture and the oracle."""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import make_case
from suitesparse_gb300 import cholmod as CH
from suitesparse_gb300 import matrices as M

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = ("g3a", "e27", "g2c")
SYS = range(9)
VAL_TOL = 1e-12        # |x - x_ref| <= VAL_TOL * max|x_ref| per column, FP64


@pytest.fixture(scope="module")
def spfix():
    return dict(np.load(os.path.join(HERE, "golden", "spsolve.npz")))


def symbolic(meta, arrays, name, c):
    n, Ap, Ai, Ax = make_case(meta, name)
    A = CH.sparse(n, Ap, Ai, Ax, c)
    perm = arrays[name + "_Perm"].astype(np.int64)
    L = CH.analyze_perm(A, perm, c)
    f = CH.factor_arrays(L, with_x=False)
    sym = {k: f[k] for k in ("Super", "Pi", "Px", "Ls")}
    sym["n"] = n
    return (n, Ap, Ai, Ax), A, L, perm, sym


def check_sparse(got, fix, name, sys_):
    Xp, Xi, Xx = got[:3]
    want_p = fix[f"{name}_{sys_}_Xp"]
    want_i = fix[f"{name}_{sys_}_Xi"].astype(np.int64)
    want_x = fix[f"{name}_{sys_}_Xx"]
    np.testing.assert_array_equal(Xp, want_p)
    np.testing.assert_array_equal(Xi, want_i)
    for j in range(len(want_p) - 1):
        a, b = int(want_p[j]), int(want_p[j + 1])
        if a < b:
            scale = np.abs(want_x[a:b]).max()
            assert np.abs(Xx[a:b] - want_x[a:b]).max() <= VAL_TOL * scale


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference(golden, spfix, oracle_mod, lib, name):
    """The oracle's spsolve on the reference's own factor gives the
    reference's sparse X: the same pattern, values to rounding."""
    meta, arrays = golden
    c = CH.Common()
    mat, A, L, perm, sym = symbolic(meta, arrays, name, c)
    Lx = arrays[name + "_Lx"]
    Bp, Bi, Bx = spfix[name + "_Bp"], spfix[name + "_Bi"], spfix[name + "_Bx"]
    for sys_ in SYS:
        got = oracle_mod.spsolve(sym, Lx, perm, mat[0], Bp, Bi, Bx, sys_)
        check_sparse(got, spfix, name, sys_)
        assert int(spfix[f"{name}_{sys_}_nzmax"][0]) == max(int(got[0][-1]), 1)
    CH.free_factor(L, c)
    CH.free_sparse(A, c)


def test_argument_checks(lib):
    """The reference's checks, before any GPU work."""
    n, Ap, Ai, Ax = M.laplace2d(6, seed=1)
    c = CH.Common()
    A = CH.sparse(n, Ap, Ai, Ax, c)
    L = CH.analyze_perm(A, np.arange(n, dtype=np.int64), c)
    f = L.contents
    f.xtype = CH.CHOLMOD_REAL          # looks numeric; the checks come first
    sp = lib.cholmod_l_spsolve
    Bp = np.array([0, 1], np.int64)
    B = CH.sparse(n, Bp, np.array([0], np.int64), np.array([1.0]), c, stype=0, ncol=1)
    assert not sp(0, L, None, c.ptr) and c.status == CH.CHOLMOD_INVALID
    assert not sp(0, None, B, c.ptr) and c.status == CH.CHOLMOD_INVALID
    Bs = CH.sparse(n, Bp, np.array([0], np.int64), np.array([1.0]), c, stype=-1, ncol=1)
    assert not sp(0, L, Bs, c.ptr) and c.status == CH.CHOLMOD_INVALID     # symmetric B
    Bw = CH.sparse(n + 1, Bp, np.array([0], np.int64), np.array([1.0]), c, stype=0, ncol=1)
    assert not sp(0, L, Bw, c.ptr) and c.status == CH.CHOLMOD_INVALID     # n mismatch
    Bf = CH.sparse(n, Bp, np.array([0], np.int64), np.array([1.0]), c, stype=0, ncol=1,
                   dtype="s")
    assert not sp(0, L, Bf, c.ptr) and c.status == CH.CHOLMOD_INVALID     # dtype mismatch
    assert not sp(9, L, B, c.ptr) and c.status == CH.CHOLMOD_INVALID      # no such sys
    Bo = CH.sparse(n, Bp, np.array([n], np.int64), np.array([1.0]), c, stype=0, ncol=1)
    assert not sp(0, L, Bo, c.ptr) and c.status == CH.CHOLMOD_INVALID     # row out of range
    for M_ in (B, Bs, Bw, Bf, Bo):
        CH.free_sparse(M_, c)
    f.xtype = CH.CHOLMOD_PATTERN
    CH.free_factor(L, c)
    CH.free_sparse(A, c)


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------

def gpu_factor(meta, arrays, name, c, dtype="d"):
    n, Ap, Ai, Ax = make_case(meta, name)
    A = CH.sparse(n, Ap, Ai, Ax if dtype == "d" else Ax.astype(np.float32), c, dtype=dtype)
    perm = arrays[name + "_Perm"].astype(np.int64)
    L = CH.analyze_perm(A, perm, c)
    assert CH.factorize(A, L, c) == 1 and c.status == CH.CHOLMOD_OK
    f = CH.factor_arrays(L)
    sym = {k: f[k] for k in ("Super", "Pi", "Px", "Ls")}
    sym["n"] = n
    return (n, Ap, Ai, Ax), A, L, perm, sym, f["Lx"]


@pytest.mark.gpu
@pytest.mark.parametrize("keep", [0, 1])
@pytest.mark.parametrize("name", CASES)
def test_spsolve_matches_reference(golden, spfix, lib, name, keep):
    """cholmod_l_spsolve on the GPU factor: the reference's pattern exactly,
    its values to VAL_TOL, nzmax = nnz(X); with the factor on the host
    (copied up) and kept on the device."""
    meta, arrays = golden
    c = CH.Common()
    c.set_option(CH.GB300_OPT_KEEP_ON_DEVICE, keep)
    mat, A, L, perm, sym, Lx = gpu_factor(meta, arrays, name, c)
    Bp, Bi, Bx = spfix[name + "_Bp"], spfix[name + "_Bi"], spfix[name + "_Bx"]
    for sys_ in SYS:
        got = CH.spsolve(L, mat[0], Bp, Bi, Bx, c, sys=sys_)
        assert c.status == CH.CHOLMOD_OK
        check_sparse(got, spfix, name, sys_)
        assert got[3] == int(spfix[f"{name}_{sys_}_nzmax"][0])
    CH.free_factor(L, c)
    CH.free_sparse(A, c)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["g3", "e27"])
def test_solve_sys_matches_oracle(golden, lib, oracle_mod, name):
    """gb300_solve for every sys against the oracle on the same factor."""
    meta, arrays = golden
    c = CH.Common()
    mat, A, L, perm, sym, Lx = gpu_factor(meta, arrays, name, c)
    B = M.rhs(mat[0], 3, 11)
    for sys_ in SYS:
        X = CH.solve(L, B, c, sys=sys_)
        Xo = oracle_mod.solve_sys(sym, Lx, perm, B, sys_)
        if sys_ in (6, 7, 8):
            np.testing.assert_array_equal(X, Xo)     # pure data movement
        else:
            assert np.abs(X - Xo).max() <= VAL_TOL * np.abs(Xo).max()
    CH.free_factor(L, c)
    CH.free_sparse(A, c)


def random_sparse_rhs(n, ncol, per_col, seed):
    rng = np.random.default_rng(seed)
    Bp = np.zeros(ncol + 1, np.int64)
    Bi, Bx = [], []
    for j in range(ncol):
        k = int(rng.integers(0, per_col + 1))
        Bi.append(np.sort(rng.choice(n, k, replace=False)))
        Bx.append(rng.standard_normal(k))
        Bp[j + 1] = Bp[j] + k
    return Bp, np.concatenate(Bi).astype(np.int64), np.concatenate(Bx)


@pytest.mark.gpu
@pytest.mark.parametrize("sys_", [CH.CHOLMOD_A, CH.CHOLMOD_L, CH.CHOLMOD_Lt])
def test_spsolve_many_columns(golden, lib, oracle_mod, sys_):
    """150 columns (three device passes of up to 64): the sparse result is
    the dense GPU solve's nonzero entries, bit for bit, pass by pass; and the
    oracle's spsolve to VAL_TOL with the same pattern."""
    meta, arrays = golden
    c = CH.Common()
    mat, A, L, perm, sym, Lx = gpu_factor(meta, arrays, "g3", c)
    n = mat[0]
    Bp, Bi, Bx = random_sparse_rhs(n, 150, 4, 5)
    Xp, Xi, Xx, nzmax = CH.spsolve(L, n, Bp, Bi, Bx, c, sys=sys_)
    assert nzmax == max(int(Xp[-1]), 1)
    Bd = np.zeros((n, 150))
    for j in range(150):
        Bd[Bi[Bp[j]:Bp[j + 1]], j] = Bx[Bp[j]:Bp[j + 1]]
    for j0 in range(0, 150, 64):
        j1 = min(150, j0 + 64)
        Xd = CH.solve(L, Bd[:, j0:j1], c, sys=sys_)
        for j in range(j0, j1):
            rows = np.nonzero(Xd[:, j - j0] != 0)[0]
            np.testing.assert_array_equal(Xi[Xp[j]:Xp[j + 1]], rows)
            np.testing.assert_array_equal(Xx[Xp[j]:Xp[j + 1]], Xd[rows, j - j0])
    op, oi, ox = oracle_mod.spsolve(sym, Lx, perm, n, Bp, Bi, Bx, sys_)
    np.testing.assert_array_equal(Xp, op)
    np.testing.assert_array_equal(Xi, oi)
    assert np.abs(Xx - ox).max() <= VAL_TOL * np.abs(ox).max()
    CH.free_factor(L, c)
    CH.free_sparse(A, c)


@pytest.mark.gpu
def test_spsolve_unpacked_and_single(golden, spfix, lib, oracle_mod):
    """An unpacked B (per-column counts, gaps between columns) gives the
    packed B's result; a single-precision factor and B give the oracle's
    FP32 pattern and values to FP32 rounding."""
    meta, arrays = golden
    name = "e27"
    c = CH.Common()
    mat, A, L, perm, sym, Lx = gpu_factor(meta, arrays, name, c)
    n = mat[0]
    Bp, Bi, Bx = spfix[name + "_Bp"], spfix[name + "_Bi"], spfix[name + "_Bx"]
    ncol = len(Bp) - 1
    ref = CH.spsolve(L, n, Bp, Bi, Bx, c)
    # unpacked: column j at 2*Bp[j] with Bnz[j] entries, garbage in the gaps
    nz = int(Bp[-1])
    B = CH.lib().gb300_allocate_sparse(n, ncol, 2 * nz + 1, 1, 0, 0, CH.CHOLMOD_REAL, c.ptr)
    b = B.contents
    P = CH._arr(b.p, np.int64, ncol + 1)
    I = CH._arr(b.i, np.int64, 2 * nz + 1)
    X = CH._arr(b.x, np.float64, 2 * nz + 1)
    Z = CH._arr(b.nz, np.int64, ncol)
    I[:] = 0
    X[:] = 7.0
    for j in range(ncol):
        P[j] = 2 * Bp[j]
        Z[j] = Bp[j + 1] - Bp[j]
        I[P[j]:P[j] + Z[j]] = Bi[Bp[j]:Bp[j + 1]]
        X[P[j]:P[j] + Z[j]] = Bx[Bp[j]:Bp[j + 1]]
    P[ncol] = 2 * nz
    Xs = CH.lib().cholmod_l_spsolve(CH.CHOLMOD_A, L, B, c.ptr)
    assert Xs and c.status == CH.CHOLMOD_OK
    got = CH.sparse_arrays(Xs)
    for a, w in zip(got, ref[:3]):
        np.testing.assert_array_equal(a, w)
    CH.free_sparse(Xs, c)
    CH.lib().gb300_free_sparse(C.byref(B), c.ptr)
    CH.free_factor(L, c)
    CH.free_sparse(A, c)

    c2 = CH.Common()
    mat, A, L, perm, sym, Lx = gpu_factor(meta, arrays, name, c2, dtype="s")
    Xp, Xi, Xx, nzmax = CH.spsolve(L, n, Bp, Bi, Bx.astype(np.float32), c2, dtype="s")
    assert Xx.dtype == np.float32
    op, oi, ox = oracle_mod.spsolve(sym, Lx, perm, n, Bp, Bi, Bx.astype(np.float32), 0,
                                    dtype="s")
    np.testing.assert_array_equal(Xp, op)
    np.testing.assert_array_equal(Xi, oi)
    assert np.abs(Xx - ox).max() <= 1e-4 * np.abs(ox).max()
    CH.free_factor(L, c2)
    CH.free_sparse(A, c2)
