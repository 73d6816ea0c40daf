"""Input validation and error reporting of the boundary follow CHOLMOD
(checks run before any device work, so no GPU is needed here)."""
import ctypes as C

import numpy as np

from suitesparse_gb300 import cholmod as CH
from suitesparse_gb300 import matrices as M


def setup_case(c):
    n, Ap, Ai, Ax = M.laplace2d(6, seed=3)
    A = CH.sparse(n, Ap, Ai, Ax, c)
    L = CH.analyze_perm(A, np.arange(n), c)
    return n, A, L


def test_super_numeric_rejects_bad_inputs(lib):
    c = CH.Common()
    n, A, L = setup_case(c)
    beta = (C.c_double * 2)(0, 0)
    # missing arguments
    assert lib.cholmod_l_super_numeric(None, None, beta, L, c.ptr) == 0
    assert c.status == CH.CHOLMOD_INVALID
    # unsymmetric A*F' form and upper storage are not supported
    for st in (0, 1):
        A.contents.stype = st
        assert lib.cholmod_l_super_numeric(A, None, beta, L, c.ptr) == 0
        assert c.status == CH.CHOLMOD_INVALID
    A.contents.stype = -1
    # factor that is not supernodal
    L.contents.is_super = 0
    assert lib.cholmod_l_super_numeric(A, None, beta, L, c.ptr) == 0
    assert c.status == CH.CHOLMOD_INVALID
    L.contents.is_super = 1
    # dimension mismatch
    A.contents.nrow = n - 1
    assert lib.cholmod_l_super_numeric(A, None, beta, L, c.ptr) == 0
    assert c.status == CH.CHOLMOD_INVALID
    A.contents.nrow = n
    # complex A with a real numeric L: the reference's complex type mismatch
    A.contents.xtype = CH.CHOLMOD_COMPLEX
    L.contents.xtype = CH.CHOLMOD_REAL
    assert lib.cholmod_l_super_numeric(A, None, beta, L, c.ptr) == 0
    assert c.status == CH.CHOLMOD_INVALID
    A.contents.xtype = CH.CHOLMOD_REAL
    L.contents.xtype = CH.CHOLMOD_PATTERN
    # numeric L of another dtype
    L.contents.xtype = CH.CHOLMOD_REAL
    L.contents.dtype = CH.CHOLMOD_SINGLE
    assert lib.cholmod_l_super_numeric(A, None, beta, L, c.ptr) == 0
    assert c.status == CH.CHOLMOD_INVALID
    L.contents.xtype = CH.CHOLMOD_PATTERN
    L.contents.dtype = CH.CHOLMOD_DOUBLE
    CH.free_factor(L, c)
    CH.free_sparse(A, c)


def test_super_solve_rejects_bad_inputs(lib):
    c = CH.Common()
    n, A, L = setup_case(c)
    X = CH.dense(np.zeros((n, 2)), c)
    E = CH.dense(np.zeros((1, 1)), c)
    # symbolic factor: no values
    assert lib.cholmod_l_super_lsolve(L, X, E, c.ptr) == 0
    assert c.status == CH.CHOLMOD_INVALID
    L.contents.xtype = CH.CHOLMOD_REAL
    # workspace E smaller than nrhs * maxesize
    assert L.contents.maxesize * 2 > 1
    assert lib.cholmod_l_super_ltsolve(L, X, E, c.ptr) == 0
    assert c.status == CH.CHOLMOD_INVALID
    L.contents.xtype = CH.CHOLMOD_PATTERN
    CH.free_dense(X, c)
    CH.free_dense(E, c)
    CH.free_factor(L, c)
    CH.free_sparse(A, c)


def test_error_handler_is_called(lib):
    c = CH.Common()
    seen = []
    HANDLER = C.CFUNCTYPE(None, C.c_int, C.c_char_p, C.c_int, C.c_char_p)

    def handler(status, file, line, msg):
        seen.append((status, msg))

    h = HANDLER(handler)
    off = lib.gb300_abi_offset(0, b"error_handler")
    C.c_void_p.from_address(c.ptr.value + off).value = C.cast(h, C.c_void_p).value
    n, A, L = setup_case(c)
    A.contents.stype = 1
    beta = (C.c_double * 2)(0, 0)
    assert lib.cholmod_l_super_numeric(A, None, beta, L, c.ptr) == 0
    assert seen and seen[-1][0] == CH.CHOLMOD_INVALID
    # try_catch suppresses the handler
    seen.clear()
    c["try_catch"] = 1
    assert lib.cholmod_l_super_numeric(A, None, beta, L, c.ptr) == 0
    assert not seen and c.status == CH.CHOLMOD_INVALID
    C.c_void_p.from_address(c.ptr.value + off).value = None
    A.contents.stype = -1
    CH.free_factor(L, c)
    CH.free_sparse(A, c)
