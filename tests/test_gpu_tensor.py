"""FP32 factorization with the tile products on the tensor cores
(GB300_OPT_TENSOR: tcgen05 kind::tf32 on operand images split into TF32 hi
and FP32 lo parts, staged by bulk asynchronous copies) against the same
factorization on the CUDA cores and against the oracle's single-precision
factor, and the mixed form refined to the FP64 target with it."""
import numpy as np
import pytest

from conftest import make_case
from suitesparse_gb300 import cholmod as CH
from suitesparse_gb300 import matrices as M

pytestmark = pytest.mark.gpu
TOL = 1e-12
L_TOL_SINGLE = 1e-4     # as for the CUDA-core FP32 factor against the oracle's
TC_VS_SIMT = 1e-5       # two FP32 factors with different summation orders


def _case(meta, arrays, name):
    if name == "p40":
        # 40^3 variable-coefficient Laplacian, nested dissection: supernodes
        # up to ~1,600 wide, update blocks with depths up to ~1,500
        return M.laplace3d(40, seed=1), M.grid_nd_perm((40, 40, 40))
    return make_case(meta, name), arrays[name + "_Perm"].astype(np.int64)


def _single_factor(mat, perm, tensor):
    n, Ap, Ai, Ax = mat
    c = CH.Common()
    c.set_option(CH.GB300_OPT_TENSOR, tensor)
    A = CH.sparse(n, Ap, Ai, Ax.astype(np.float32), c, dtype="s")
    L = CH.analyze_perm(A, perm, c)
    assert CH.factorize(A, L, c) == 1 and c.status == CH.CHOLMOD_OK
    f = CH.factor_arrays(L)
    CH.free_factor(L, c)
    CH.free_sparse(A, c)
    c.finish()
    return f


def _relerr(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("name", ["g3", "e27", "c1", "p40"])
def test_tensor_factor_matches_cuda_cores_and_oracle(golden, lib, oracle_mod, name):
    meta, arrays = golden
    mat, perm = _case(meta, arrays, name)
    f0 = _single_factor(mat, perm, 0)
    f1 = _single_factor(mat, perm, 1)
    assert np.array_equal(f0["Px"], f1["Px"])
    n, Ap, Ai, Ax = mat
    sym = {k: f1[k] for k in ("Super", "Pi", "Px", "Ls")}
    sym["n"] = n
    Sp, Si, Sx = oracle_mod.permute_lower(n, Ap, Ai, Ax, perm)
    st, minor, Lref = oracle_mod.factor(sym, Sp, Si, Sx.astype(np.float32), dtype="s")
    assert st == 0
    e_tc, e_simt = _relerr(f1["Lx"], Lref), _relerr(f0["Lx"], Lref)
    assert e_tc < L_TOL_SINGLE, (e_tc, e_simt)
    assert _relerr(f1["Lx"], f0["Lx"]) < TC_VS_SIMT, (e_tc, e_simt)


@pytest.mark.parametrize("name", ["c2", "c3"])
def test_tensor_refined_full_size(golden, lib, oracle_mod, name):
    """c2 and c3 with the tensor-core factor: every column of 1, 8 and 64
    right-hand sides to 1e-12 against the oracle's FP64 evaluation, without
    the FP64 fallback."""
    meta, arrays = golden
    n, Ap, Ai, Ax = make_case(meta, name)
    c = CH.Common()
    c.set_option(CH.GB300_OPT_TENSOR, 1)
    A = CH.sparse(n, Ap, Ai, Ax, c)
    L = CH.analyze_perm(A, arrays[name + "_Perm"].astype(np.int64), c)
    assert CH.factorize_mixed(A, L, c) == 1
    for nrhs in (1, 8, 64):
        B = M.rhs(n, nrhs, 40 + nrhs)
        X, info = CH.solve_refined(A, L, B, c, tol=TOL)
        be = oracle_mod.backward_error(n, Ap, Ai, Ax, X, B)
        assert be.max() <= TOL and not info["fp64_fallback"], (nrhs, be.max(), info)
        assert info["iterations"] <= 3, info
    CH.free_factor(L, c)
    CH.free_sparse(A, c)


def test_tensor_not_positive_definite(golden, lib):
    """A failing pivot with the tensor-core tiles: the same L->minor as the
    reference (the images of the failing panel are never read)."""
    meta, arrays = golden
    n, Ap, Ai, Ax = make_case(meta, "npd")
    c = CH.Common()
    c.set_option(CH.GB300_OPT_TENSOR, 1)
    c.set_option(CH.GB300_OPT_SMALL_COLS, 1)      # every supernode on the tile path
    A = CH.sparse(n, Ap, Ai, Ax, c)
    L = CH.analyze_perm(A, arrays["npd_Perm"].astype(np.int64), c)
    assert CH.factorize_mixed(A, L, c) == 1
    assert c.status == CH.CHOLMOD_NOT_POSDEF
    assert L.contents.minor == meta["npd"]["minor"]
    CH.free_factor(L, c)
    CH.free_sparse(A, c)
