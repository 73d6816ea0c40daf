"""Failure detection without a GPU fault: a device-side wait on a flag that
nothing sets gives up after its poll limit, sets the error word the host
reads, and the CUDA context stays usable."""
import ctypes as C

import numpy as np
import pytest

from conftest import make_case
from suitesparse_gb300 import cholmod as CH
from suitesparse_gb300 import matrices as M

pytestmark = pytest.mark.gpu


def test_wait_gives_up_and_context_survives(golden, lib, oracle_mod):
    f = lib.gb300_wait_probe
    f.restype = C.c_int
    f.argtypes = [C.c_int64, C.POINTER(C.c_int32)]
    out = (C.c_int32 * 2)(-1, -1)
    assert f(2000, out) == 1
    assert out[0] == 0 and out[1] == 1          # the wait gave up and said so
    # the context still works: a factorization and solve right after
    meta, arrays = golden
    c = CH.Common()
    n, Ap, Ai, Ax = make_case(meta, "g3")
    A = CH.sparse(n, Ap, Ai, Ax, c)
    L = CH.analyze_perm(A, arrays["g3_Perm"].astype(np.int64), c)
    assert CH.factorize(A, L, c) == 1 and c.status == CH.CHOLMOD_OK
    B = M.rhs(n, 2, 4)
    X = CH.solve(L, B, c)
    assert oracle_mod.backward_error(n, Ap, Ai, Ax, X, B).max() <= 1e-14
    CH.free_factor(L, c)
    CH.free_sparse(A, c)
