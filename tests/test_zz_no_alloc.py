"""gb300_backward_error_noalloc: the backward error of device-resident
solutions with the reduction scratch in a fixed device array of the library
(no allocation in the call), checked against the backward error that
gb300_solve_refined reports and against a float64 numpy evaluation."""
import ctypes as C

import numpy as np
import pytest

from conftest import make_case
from suitesparse_gb300 import cholmod as CH
from suitesparse_gb300 import matrices as M

pytestmark = pytest.mark.gpu

MAX_RHS = 64
# The residual rows are summed in the same order as the refined solve's own
# residual, but berr of a converged solution is a difference of nearly equal
# sums, so allow the rounding of a few row terms relative to |A||x| + |b|.
ABS_TOL = 1e-14
REL_TOL = 1e-10     # against numpy when berr is far above rounding level


def _fn(lib):
    f = lib.gb300_backward_error_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                  C.c_int64, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]
    return f


def _device(torch, n, Ap, Ai, Ax, X, B):
    dev = torch.device("cuda:0")
    t = dict(
        Ap=torch.from_numpy(np.ascontiguousarray(Ap, dtype=np.int64)).to(dev),
        Ai=torch.from_numpy(np.ascontiguousarray(Ai, dtype=np.int64)).to(dev),
        Ax=torch.from_numpy(np.ascontiguousarray(Ax, dtype=np.float64)).to(dev),
        # column-major n x k with leading dimension n == row-major k x n
        X=torch.from_numpy(np.ascontiguousarray(X.T, dtype=np.float64)).to(dev),
        B=torch.from_numpy(np.ascontiguousarray(B.T, dtype=np.float64)).to(dev),
        berr=torch.full((max(X.shape[1], 1),), -1.0, dtype=torch.float64, device=dev),
    )
    return t


def _call(f, torch, n, t, nrhs):
    stream = torch.cuda.current_stream().cuda_stream
    rc = f(n, t["Ap"].data_ptr(), t["Ai"].data_ptr(), t["Ax"].data_ptr(), nrhs,
           t["X"].data_ptr(), n, t["B"].data_ptr(), n, t["berr"].data_ptr(), C.c_void_p(stream))
    torch.cuda.synchronize()
    return rc, t["berr"].cpu().numpy()[:nrhs].copy()


def _numpy_berr(n, Ap, Ai, Ax, X, B):
    import scipy.sparse as sp
    A = sp.csc_matrix((Ax, Ai, Ap), shape=(n, n))
    R = B - A @ X
    anorm = np.abs(A).sum(axis=1).max()
    den = anorm * np.abs(X).max(axis=0) + np.abs(B).max(axis=0)
    return np.abs(R).max(axis=0) / den


def _solved(meta, arrays, name, nrhs, seed):
    c = CH.Common()
    n, Ap, Ai, Ax = make_case(meta, name)
    A = CH.sparse(n, Ap, Ai, Ax, c)
    L = CH.analyze_perm(A, arrays[name + "_Perm"].astype(np.int64), c)
    assert CH.factorize_mixed(A, L, c) == 1
    B = M.rhs(n, nrhs, seed)
    X, info = CH.solve_refined(A, L, B, c, tol=1e-12)
    CH.free_factor(L, c)
    CH.free_sparse(A, c)
    Fp, Fi, Fx = M.full_from_lower(n, Ap, Ai, Ax)
    return n, (Fp, Fi, Fx), np.asarray(X, dtype=np.float64), np.asarray(B, dtype=np.float64), info


@pytest.mark.parametrize("name,nrhs", [("g3", 1), ("c1", 8)])
def test_matches_refined_solve_twice(golden, lib, name, nrhs):
    torch = pytest.importorskip("torch")
    meta, arrays = golden
    f = _fn(lib)
    n, (Fp, Fi, Fx), X, B, info = _solved(meta, arrays, name, nrhs, 7 + nrhs)
    t = _device(torch, n, Fp, Fi, Fx, X, B)
    rc1, be1 = _call(f, torch, n, t, nrhs)
    rc2, be2 = _call(f, torch, n, t, nrhs)
    assert rc1 == 0 and rc2 == 0
    # two calls in a row: the scratch was left zero by the first
    assert np.array_equal(be1, be2), (be1, be2)
    assert abs(be1.max() - info["berr"]) <= ABS_TOL, (be1.max(), info)
    ref = _numpy_berr(n, Fp, Fi, Fx, X, B)
    assert np.all(np.abs(be1 - ref) <= ABS_TOL), (be1, ref)


def test_max_columns_then_one(golden, lib):
    """64 columns (the scratch limit) of unconverged solutions, then one."""
    torch = pytest.importorskip("torch")
    meta, arrays = golden
    f = _fn(lib)
    n, Ap, Ai, Ax = make_case(meta, "g3")
    Fp, Fi, Fx = M.full_from_lower(n, Ap, Ai, Ax)
    rng = np.random.default_rng(3)
    X = rng.standard_normal((n, MAX_RHS))
    B = rng.standard_normal((n, MAX_RHS))
    ref = _numpy_berr(n, Fp, Fi, Fx, X, B)
    t = _device(torch, n, Fp, Fi, Fx, X, B)
    for _ in range(2):
        rc, be = _call(f, torch, n, t, MAX_RHS)
        assert rc == 0
        np.testing.assert_allclose(be, ref, rtol=REL_TOL, atol=0)
    # a one-column call afterwards sees none of the 64-column maxima
    t1 = _device(torch, n, Fp, Fi, Fx, X[:, 5:6] * 1e-3, B[:, 5:6])
    rc, be = _call(f, torch, n, t1, 1)
    assert rc == 0
    ref1 = _numpy_berr(n, Fp, Fi, Fx, X[:, 5:6] * 1e-3, B[:, 5:6])
    np.testing.assert_allclose(be, ref1, rtol=REL_TOL, atol=0)


def test_rejects_sizes_beyond_the_scratch(golden, lib):
    torch = pytest.importorskip("torch")
    meta, arrays = golden
    f = _fn(lib)
    n, Ap, Ai, Ax = make_case(meta, "g3")
    Fp, Fi, Fx = M.full_from_lower(n, Ap, Ai, Ax)
    rng = np.random.default_rng(4)
    X = rng.standard_normal((n, MAX_RHS + 1))
    B = rng.standard_normal((n, MAX_RHS + 1))
    t = _device(torch, n, Fp, Fi, Fx, X, B)
    rc, be = _call(f, torch, n, t, MAX_RHS + 1)
    assert rc == -2                      # GB300_NOALLOC_TOO_LARGE: nothing queued
    assert np.all(be == -1.0)
    rc, _ = _call(f, torch, -1, t, 1)
    assert rc == -1                      # GB300_NOALLOC_INVALID
    # the library still works after the rejections
    rc, be = _call(f, torch, n, t, 3)
    assert rc == 0
    np.testing.assert_allclose(be, _numpy_berr(n, Fp, Fi, Fx, X[:, :3], B[:, :3]), rtol=REL_TOL)


def test_non_finite_solutions_give_nan(golden, lib):
    """A NaN or an infinity in x or b must not vanish from the maxima (a plain
    fmax drops NaN and would report such a column as converged)."""
    torch = pytest.importorskip("torch")
    meta, arrays = golden
    f = _fn(lib)
    n, Ap, Ai, Ax = make_case(meta, "g3")
    Fp, Fi, Fx = M.full_from_lower(n, Ap, Ai, Ax)
    rng = np.random.default_rng(5)
    X = rng.standard_normal((n, 5))
    B = rng.standard_normal((n, 5))
    X[:, 0] = np.nan                 # all of x NaN
    X[n // 2, 1] = np.nan            # one entry of x NaN
    X[3, 2] = np.inf                 # one entry of x infinite
    B[n - 1, 3] = np.nan             # one entry of b NaN; column 4 clean
    t = _device(torch, n, Fp, Fi, Fx, X, B)
    for _ in range(2):
        rc, be = _call(f, torch, n, t, 5)
        assert rc == 0
        assert np.all(np.isnan(be[:4])), be
        np.testing.assert_allclose(be[4], _numpy_berr(n, Fp, Fi, Fx, X[:, 4:], B[:, 4:])[0],
                                   rtol=REL_TOL)
    # the NaN maxima were cleared: a clean call afterwards is exact again
    t1 = _device(torch, n, Fp, Fi, Fx, X[:, 4:], B[:, 4:])
    rc, be = _call(f, torch, n, t1, 1)
    assert rc == 0 and np.isfinite(be[0])
    np.testing.assert_allclose(be, _numpy_berr(n, Fp, Fi, Fx, X[:, 4:], B[:, 4:]), rtol=REL_TOL)
