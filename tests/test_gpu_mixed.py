"""FP32 factor + FP64 iterative refinement reaches the FP64 accuracy target."""
import numpy as np
import pytest

from conftest import make_case
from suitesparse_gb300 import cholmod as CH
from suitesparse_gb300 import matrices as M

pytestmark = pytest.mark.gpu
TOL = 1e-12     # backward error |b-Ax|_inf / (|A|_inf |x|_inf + |b|_inf)


def setup(meta, arrays, name, c):
    n, Ap, Ai, Ax = make_case(meta, name)
    A = CH.sparse(n, Ap, Ai, Ax, c)
    L = CH.analyze_perm(A, arrays[name + "_Perm"].astype(np.int64), c)
    return (n, Ap, Ai, Ax), A, L


@pytest.mark.parametrize("name", ["g2v", "g3", "e27", "c1"])
@pytest.mark.parametrize("nrhs", [1, 8])
def test_refined_reaches_tolerance(golden, lib, oracle_mod, name, nrhs):
    meta, arrays = golden
    c = CH.Common()
    mat, A, L = setup(meta, arrays, name, c)
    assert CH.factorize_mixed(A, L, c) == 1 and c.status == CH.CHOLMOD_OK
    B = M.rhs(mat[0], nrhs, 21)
    X, info = CH.solve_refined(A, L, B, c, tol=TOL)
    be = oracle_mod.backward_error(*mat, X, B)
    assert be.max() <= TOL, (be, info)
    assert info["berr"] <= TOL and info["iterations"] >= 1
    # the FP32 factor is not written to L->x
    assert L.contents.xtype == CH.CHOLMOD_PATTERN
    CH.free_factor(L, c)
    CH.free_sparse(A, c)


@pytest.mark.parametrize("name", ["c2", "c3"])
def test_refined_full_size(golden, lib, oracle_mod, name):
    """Full size: c2 (64^3 variable-coefficient Laplacian, condition ~1e8)
    and c3 (27-point 40^3 x 3-dof elasticity), 1, 8 and 64 right-hand
    sides, each column to 1e-12 against the oracle's FP64 evaluation."""
    meta, arrays = golden
    c = CH.Common()
    mat, A, L = setup(meta, arrays, name, c)
    assert CH.factorize_mixed(A, L, c) == 1
    for nrhs in (1, 8, 64):
        B = M.rhs(mat[0], nrhs, 5 + nrhs)
        X, info = CH.solve_refined(A, L, B, c, tol=TOL)
        be = oracle_mod.backward_error(*mat, X, B)
        assert be.max() <= TOL, (nrhs, be.max(), info)
    CH.free_factor(L, c)
    CH.free_sparse(A, c)


def test_mixed_matches_fp64_solution(golden, lib, oracle_mod):
    meta, arrays = golden
    c = CH.Common()
    mat, A, L = setup(meta, arrays, "g3", c)
    B = M.rhs(mat[0], 3, 2)
    assert CH.factorize(A, L, c) == 1
    X64 = CH.solve(L, B, c)
    assert CH.factorize_mixed(A, L, c) == 1
    X, info = CH.solve_refined(A, L, B, c, tol=1e-14)
    assert np.abs(X - X64).max() <= 1e-11 * np.abs(X64).max()
    CH.free_factor(L, c)
    CH.free_sparse(A, c)


def test_mixed_not_positive_definite(golden, lib):
    meta, arrays = golden
    c = CH.Common()
    mat, A, L = setup(meta, arrays, "npd", c)
    assert CH.factorize_mixed(A, L, c) == 1
    assert c.status == CH.CHOLMOD_NOT_POSDEF
    assert L.contents.minor == meta["npd"]["minor"]
    CH.free_factor(L, c)
    CH.free_sparse(A, c)


def test_refined_tensor_core_tiles(golden, lib, oracle_mod):
    """The FP32 factorization with its tile products on the tensor cores
    (GB300_OPT_TENSOR: tcgen05, 3xTF32) still refines to the FP64 target."""
    meta, arrays = golden
    for name in ("g3", "c1"):
        c = CH.Common()
        c.set_option(CH.GB300_OPT_TENSOR, 1)
        mat, A, L = setup(meta, arrays, name, c)
        assert CH.factorize_mixed(A, L, c) == 1
        B = M.rhs(mat[0], 4, 31)
        X, info = CH.solve_refined(A, L, B, c, tol=TOL)
        be = oracle_mod.backward_error(*mat, X, B)
        assert be.max() <= TOL and not info["fp64_fallback"], (name, be.max(), info)
        CH.free_factor(L, c)
        CH.free_sparse(A, c)


def test_refinement_graph_replay_same_result(golden, lib, oracle_mod):
    """A refinement step replayed from the pattern's CUDA graph
    (GB300_OPT_GRAPH) gives the same solution bit for bit as the step
    launched kernel by kernel, for repeated solves and a change of the
    right-hand-side count (the graph is captured again)."""
    meta, arrays = golden
    res = {}
    for graph in (0, 1):
        c = CH.Common()
        c.set_option(CH.GB300_OPT_GRAPH, graph)
        mat, A, L = setup(meta, arrays, "c1", c)
        assert CH.factorize_mixed(A, L, c) == 1
        out = []
        for k, seed in ((2, 5), (2, 6), (5, 7), (2, 8)):
            B = M.rhs(mat[0], k, seed)
            X, info = CH.solve_refined(A, L, B, c, tol=TOL)
            assert oracle_mod.backward_error(*mat, X, B).max() <= TOL
            out.append((np.array(X, copy=True), info["iterations"]))
        res[graph] = out
        CH.free_factor(L, c)
        CH.free_sparse(A, c)
    for (x0, i0), (x1, i1) in zip(res[0], res[1]):
        assert i0 == i1
        assert np.array_equal(x0, x1)


def test_value_maps_follow_a_pattern_change(golden, lib, oracle_mod):
    """Refactorizations gather A's values on the device through maps built
    for A's pattern; a packed A with as many entries is compared with that
    pattern while the device factorizes.  Two entries of a column swapped in
    place (the same matrix, another pattern) must be detected: the maps are
    rebuilt and the result equals the first one bit for bit (stale maps
    would swap the two values)."""
    meta, arrays = golden
    c = CH.Common()
    mat, A, L = setup(meta, arrays, "g3", c)
    n = mat[0]
    B = M.rhs(n, 2, 4)
    assert CH.factorize_mixed(A, L, c) == 1
    X1, _ = CH.solve_refined(A, L, B, c, tol=TOL)
    a = A.contents
    nz = int(mat[1][-1])
    Ap = CH._arr(a.p, np.int64, n + 1)
    Ai = CH._arr(a.i, np.int64, nz)
    Ax = CH._arr(a.x, np.float64, nz)
    j = next(j for j in range(n) if Ap[j + 1] - Ap[j] >= 3)
    p, q = int(Ap[j]) + 1, int(Ap[j]) + 2          # two off-diagonal entries
    assert Ax[p] != Ax[q]
    Ai[p], Ai[q] = Ai[q], Ai[p]
    Ax[p], Ax[q] = Ax[q], Ax[p]
    a.sorted = 0
    assert CH.factorize_mixed(A, L, c) == 1 and c.status == CH.CHOLMOD_OK
    X2, _ = CH.solve_refined(A, L, B, c, tol=TOL)
    np.testing.assert_array_equal(X1, X2)
    # and the values of the new positions are used from now on
    Ax[p] *= 0.5                                  # still diagonally dominant
    assert CH.factorize_mixed(A, L, c) == 1
    X3, _ = CH.solve_refined(A, L, B, c, tol=TOL)
    Ai2, Ax2 = np.array(Ai), np.array(Ax)
    be = oracle_mod.backward_error(n, np.array(Ap), Ai2, Ax2, X3, B)
    assert be.max() <= TOL
    CH.free_factor(L, c)
    CH.free_sparse(A, c)


def test_solve_refined2_reuses_x(golden, lib, oracle_mod):
    """gb300_solve_refined2: a caller's X of the right shape is written in
    place (the same pointer, the same result as gb300_solve_refined); a
    NULL handle gets a new X, one of the wrong shape is replaced."""
    import ctypes as C
    meta, arrays = golden
    c = CH.Common()
    mat, A, L = setup(meta, arrays, "g3", c)
    n = mat[0]
    B = M.rhs(n, 3, 8)
    assert CH.factorize_mixed(A, L, c) == 1
    X0, _ = CH.solve_refined(A, L, B, c, tol=TOL)
    Bd = CH.dense(B, c)
    info = (C.c_double * 4)()
    Xd = CH.dense(np.zeros((n, 3)), c)
    addr = C.addressof(Xd.contents)
    h = C.pointer(Xd)
    assert lib.gb300_solve_refined2(A, L, Bd, TOL, info, h, c.ptr) == 1
    assert C.addressof(h.contents.contents) == addr
    np.testing.assert_array_equal(CH.dense_array(h.contents), X0)
    assert info[1] <= TOL
    wrong = CH.dense(np.zeros((n, 2)), c)
    h2 = C.pointer(wrong)
    assert lib.gb300_solve_refined2(A, L, Bd, TOL, info, h2, c.ptr) == 1
    assert h2.contents.contents.ncol == 3
    np.testing.assert_array_equal(CH.dense_array(h2.contents), X0)
    h3 = C.pointer(CH.DP())
    assert lib.gb300_solve_refined2(A, L, Bd, TOL, info, h3, c.ptr) == 1
    np.testing.assert_array_equal(CH.dense_array(h3.contents), X0)
    for hh in (h, h2, h3):
        CH.free_dense(hh.contents, c)
    CH.free_dense(Bd, c)
    CH.free_factor(L, c)
    CH.free_sparse(A, c)


def test_concurrent_sweep_passes(golden, lib, oracle_mod):
    """More than 16 right-hand sides: passes of 16 columns run at once on
    their own streams, each with its own dependency words and update
    vectors.  Each pass computes what a 16-column solve computes (bit for
    bit); the refined solve with 70 columns (5 passes on 4 streams) meets
    the tolerance, directly and replayed from the pattern's graph."""
    meta, arrays = golden
    c = CH.Common()
    mat, A, L = setup(meta, arrays, "c1", c)
    n = mat[0]
    B = M.rhs(n, 70, 12)
    assert CH.factorize(A, L, c) == 1
    X = CH.solve(L, B, c)
    for k0 in range(0, 70, 16):
        Xk = CH.solve(L, B[:, k0:k0 + 16], c)
        np.testing.assert_array_equal(X[:, k0:k0 + 16], Xk)
    assert oracle_mod.backward_error(*mat, X, B).max() <= 1e-14
    for k in (1, 2):                                  # passes one after another
        c.set_option(CH.GB300_OPT_SWEEP_STREAMS, k)
        np.testing.assert_array_equal(CH.solve(L, B, c), X)
    c.set_option(CH.GB300_OPT_SWEEP_STREAMS, 4)
    assert CH.factorize_mixed(A, L, c) == 1
    X1, i1 = CH.solve_refined(A, L, B, c, tol=TOL)
    X2, i2 = CH.solve_refined(A, L, B, c, tol=TOL)
    np.testing.assert_array_equal(X1, X2)
    assert oracle_mod.backward_error(*mat, X2, B).max() <= TOL
    CH.free_factor(L, c)
    CH.free_sparse(A, c)
