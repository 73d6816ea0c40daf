"""The FP64 fallback of the mixed form and non-finite inputs.

gb300_factorize_mixed / gb300_solve_refined switch to an FP64 factor when
(1) the FP32 factorization fails, (2) an FP32 pivot is small
(min L(k,k)^2 <= 2^-GB300_OPT_PIVOT_LOG2 max L(k,k)^2), or (3) refinement
stalls (the backward error does not halve in 2 steps).  Each trigger is
forced here on a matrix whose FP32 arithmetic is known exactly, and the
solution must still reach the FP64 target against the oracle.  A NaN in b
must never be reported as converged."""
import numpy as np
import pytest

from conftest import make_case
from suitesparse_gb300 import cholmod as CH
from suitesparse_gb300 import matrices as M

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _with_pair(c):
    """A 12 x 12 unit-coefficient 2D Laplacian (diagonal 4, off-diagonal -1:
    its scaled form D A D is exact in FP32, every pivot^2 >= 1/2) followed by
    an independent 2 x 2 block [[1, c], [c, 1]], whose second scaled pivot^2
    is 1 - c^2.  Identity ordering (each component's etree is a chain)."""
    n0, Ap0, Ai0, Ax0 = M.laplace2d(12)
    n = n0 + 2
    Ap = np.concatenate([Ap0, [Ap0[-1] + 2, Ap0[-1] + 3]]).astype(np.int64)
    Ai = np.concatenate([Ai0, [n0, n0 + 1, n0 + 1]]).astype(np.int64)
    Ax = np.concatenate([Ax0, [1.0, c, 1.0]])
    return n, Ap, Ai, Ax


def _run(mat, nrhs=2, tol=TOL, pivot_log2=None):
    n, Ap, Ai, Ax = mat
    c = CH.Common()
    if pivot_log2 is not None:
        assert c.set_option(CH.GB300_OPT_PIVOT_LOG2, pivot_log2)
    A = CH.sparse(n, Ap, Ai, Ax, c)
    L = CH.analyze_perm(A, np.arange(n, dtype=np.int64), c)
    assert CH.factorize_mixed(A, L, c) == 1 and c.status == CH.CHOLMOD_OK
    reason_after_factor = CH.mixed_reason(L, c)
    B = M.rhs(n, nrhs, 11)
    X, info = CH.solve_refined(A, L, B, c, tol=tol)
    reason = CH.mixed_reason(L, c)
    CH.free_factor(L, c)
    CH.free_sparse(A, c)
    c.finish()
    return B, X, info, reason_after_factor, reason


def test_fp32_failure_takes_fp64(lib, oracle_mod):
    """c = -(1 - 1e-10) rounds to -1 in FP32: the scaled pivot is exactly 0
    there (the FP32 factorization fails), 2e-10 in FP64 (condition ~2e10)."""
    mat = _with_pair(-(1.0 - 1e-10))
    B, X, info, r0, r1 = _run(mat)
    assert r0 == CH.GB300_REASON_FP32_FAILED and r1 == r0
    assert info["fp64_fallback"] and info["status"] == CH.CHOLMOD_OK
    be = oracle_mod.backward_error(*mat, X, B)
    assert be.max() <= TOL and info["berr"] <= TOL, (be, info)


@pytest.mark.parametrize("pivot_log2,expect", [(9, CH.GB300_REASON_SMALL_PIVOT),
                                               (10, CH.GB300_REASON_NONE)])
def test_small_pivot_threshold(lib, oracle_mod, pivot_log2, expect):
    """c = -(1 - 2^-10): the FP32 pivot^2 1 - c^2 = 2^-9 - 2^-20 is exact
    (with or without a fused multiply-add), just below 2^-9 and twice
    2^-10, so the fallback fires at threshold 2^-9 and not at 2^-10."""
    mat = _with_pair(-(1.0 - 2.0 ** -10))
    B, X, info, r0, r1 = _run(mat, pivot_log2=pivot_log2)
    assert r0 == expect and r1 == expect
    assert info["fp64_fallback"] == (expect != CH.GB300_REASON_NONE)
    be = oracle_mod.backward_error(*mat, X, B)
    assert be.max() <= TOL and info["status"] == CH.CHOLMOD_OK, (be, info)


def test_threshold_zero_always_takes_fp64(golden, lib, oracle_mod):
    """2^-0 = 1: min <= max holds for every factor."""
    meta, arrays = golden
    n, Ap, Ai, Ax = make_case(meta, "g3")
    c = CH.Common()
    assert c.set_option(CH.GB300_OPT_PIVOT_LOG2, 0)
    A = CH.sparse(n, Ap, Ai, Ax, c)
    L = CH.analyze_perm(A, arrays["g3_Perm"].astype(np.int64), c)
    assert CH.factorize_mixed(A, L, c) == 1
    assert CH.mixed_reason(L, c) == CH.GB300_REASON_SMALL_PIVOT
    B = M.rhs(n, 3, 4)
    X, info = CH.solve_refined(A, L, B, c, tol=TOL)
    assert info["fp64_fallback"] and info["iterations"] <= 3
    assert oracle_mod.backward_error(n, Ap, Ai, Ax, X, B).max() <= TOL
    CH.free_factor(L, c)
    CH.free_sparse(A, c)


def test_stall_takes_fp64_then_stops(golden, lib, oracle_mod):
    """A tolerance no factor reaches (1e-300: only an exactly zero residual
    would; FP64 residuals of this system end near 1e-17): the FP32 factor's
    refinement stalls and the FP64 factor takes over; that stalls too, the
    call stops with CHOLMOD_DSMALL and the FP64-accurate solution."""
    meta, arrays = golden
    n, Ap, Ai, Ax = make_case(meta, "g3")
    c = CH.Common()
    A = CH.sparse(n, Ap, Ai, Ax, c)
    L = CH.analyze_perm(A, arrays["g3_Perm"].astype(np.int64), c)
    assert CH.factorize_mixed(A, L, c) == 1
    assert CH.mixed_reason(L, c) == CH.GB300_REASON_NONE
    B = M.rhs(n, 2, 6)
    X, info = CH.solve_refined(A, L, B, c, tol=1e-300)
    assert CH.mixed_reason(L, c) == CH.GB300_REASON_STALLED
    assert info["fp64_fallback"] and info["status"] == CH.CHOLMOD_DSMALL
    assert 0 < info["berr"] <= 1e-14
    assert oracle_mod.backward_error(n, Ap, Ai, Ax, X, B).max() <= 1e-14
    CH.free_factor(L, c)
    CH.free_sparse(A, c)


def test_nan_in_b_is_not_converged(golden, lib):
    """One NaN entry of b: the backward error is NaN, never <= tol, and the
    call ends with CHOLMOD_DSMALL (a plain fmax reduction would drop the
    NaN rows and report convergence)."""
    meta, arrays = golden
    n, Ap, Ai, Ax = make_case(meta, "g3")
    c = CH.Common()
    A = CH.sparse(n, Ap, Ai, Ax, c)
    L = CH.analyze_perm(A, arrays["g3_Perm"].astype(np.int64), c)
    assert CH.factorize_mixed(A, L, c) == 1
    B = M.rhs(n, 2, 8)
    B[n // 3, 1] = np.nan
    X, info = CH.solve_refined(A, L, B, c, tol=TOL)
    assert np.isnan(info["berr"]), info
    assert info["status"] == CH.CHOLMOD_DSMALL
    # the clean column is still solved; the next solve with a finite b converges
    B2 = M.rhs(n, 2, 9)
    X2, info2 = CH.solve_refined(A, L, B2, c, tol=TOL)
    assert info2["berr"] <= TOL and info2["status"] == CH.CHOLMOD_OK
    CH.free_factor(L, c)
    CH.free_sparse(A, c)
