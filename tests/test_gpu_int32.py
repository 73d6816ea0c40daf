"""The int32 entry points cholmod_super_numeric / cholmod_super_lsolve /
cholmod_super_ltsolve (cholmod.h:4016, 4037, 4058) give the same factor
and solutions, bit for bit, as the int64 ones on the same pattern; the
int32 Common check and a refactorization through the kept shadow."""
import ctypes as C

import numpy as np
import pytest

from conftest import make_case
from suitesparse_gb300 import cholmod as CH
from suitesparse_gb300 import matrices as M

pytestmark = pytest.mark.gpu
CHOLMOD_INT, CHOLMOD_LONG, CHOLMOD_PATTERN = 0, 2, 0


class Int32Objects:
    """int32 copies (numpy-owned index arrays) of an int64 sparse matrix
    and of an int64 supernodal symbolic factor."""

    def __init__(self, A64, L64):
        a, f = A64.contents, L64.contents
        n = f.n
        self.keep = []
        ap = CH._arr(a.p, np.int64, a.ncol + 1).astype(np.int32)
        ai = CH._arr(a.i, np.int64, int(ap[-1])).astype(np.int32)
        self.keep += [ap, ai]
        self.A = CH.cholmod_sparse()
        C.memmove(C.byref(self.A), C.addressof(a), C.sizeof(CH.cholmod_sparse))
        self.A.p, self.A.i, self.A.itype = ap.ctypes.data, ai.ctypes.data, CHOLMOD_INT
        self.L = CH.cholmod_factor()
        C.memmove(C.byref(self.L), C.addressof(f), C.sizeof(CH.cholmod_factor))
        for name, cnt in (("Perm", n), ("ColCount", n), ("super", f.nsuper + 1),
                          ("pi", f.nsuper + 1), ("px", f.nsuper + 1), ("s", f.ssize)):
            ptr = getattr(f, name)
            if ptr:
                arr = CH._arr(ptr, np.int64, cnt).astype(np.int32)
                self.keep.append(arr)
                setattr(self.L, name, arr.ctypes.data)
        self.L.IPerm = None
        self.L.x = None
        self.L.xtype = CHOLMOD_PATTERN
        self.L.itype = CHOLMOD_INT

    def lx(self):
        return np.ctypeslib.as_array(C.cast(self.L.x, C.POINTER(C.c_double)),
                                     shape=(self.L.xsize,)).copy()


def _dense(B, c):
    return CH.dense(np.asfortranarray(B), c)


@pytest.mark.parametrize("name", ["g3", "c1"])
def test_int32_entry_points_equal_int64(golden, lib, name):
    meta, arrays = golden
    n, Ap, Ai, Ax = make_case(meta, name)
    c = CH.Common()
    A = CH.sparse(n, Ap, Ai, Ax, c)
    L = CH.analyze_perm(A, arrays[name + "_Perm"].astype(np.int64), c)
    f = CH.factor_arrays(L, with_x=False)
    # int64 path: S = tril(PAP'), cholmod_l_super_numeric, both sweeps
    from oracle import oracle as O
    Sp, Si, Sx = O.permute_lower(n, Ap, Ai, Ax, f["Perm"])
    S = CH.sparse(n, Sp, Si, Sx, c)
    beta = (C.c_double * 2)(0.0, 0.0)
    o32 = Int32Objects(S, L)
    assert lib.cholmod_l_super_numeric(S, None, beta, L, c.ptr) == 1
    Lx64 = CH.factor_arrays(L)["Lx"]
    # int32 path on the int32 copies, with an int32 Common
    c32 = CH.Common()
    c32["itype"] = CHOLMOD_INT
    L32 = C.pointer(o32.L)
    A32 = C.pointer(o32.A)
    assert lib.cholmod_super_numeric(A32, None, beta, L32, c32.ptr) == 1, c32.status
    assert c32.status == CH.CHOLMOD_OK and o32.L.minor == n and o32.L.is_ll == 1
    assert np.array_equal(o32.lx(), Lx64)
    # refactorization of the same int32 factor (kept shadow and plan)
    assert lib.cholmod_super_numeric(A32, None, beta, L32, c32.ptr) == 1
    assert np.array_equal(o32.lx(), Lx64)
    # sweeps
    B = M.rhs(n, 3, 4)
    res = {}
    for tag, LL, cc in (("64", L, c), ("32", L32, c32)):
        X = _dense(B, cc)
        E = CH.dense(np.zeros((f["maxesize"] * 3 + 1, 1)), cc)
        fw = lib.cholmod_l_super_lsolve if tag == "64" else lib.cholmod_super_lsolve
        bw = lib.cholmod_l_super_ltsolve if tag == "64" else lib.cholmod_super_ltsolve
        assert fw(LL, X, E, cc.ptr) == 1 and bw(LL, X, E, cc.ptr) == 1
        res[tag] = CH.dense_array(X)
        CH.free_dense(X, cc)
        CH.free_dense(E, cc)
    assert np.array_equal(res["32"], res["64"])
    # the int32 entry points refuse an int64 Common, as the reference does
    assert lib.cholmod_super_numeric(A32, None, beta, L32, c.ptr) == 0
    assert c.status == CH.CHOLMOD_INVALID
    assert lib.gb300_release_factor(L32, c32.ptr) == 1
    libc = C.CDLL(None)
    libc.free(C.c_void_p(o32.L.x))
    CH.free_sparse(S, c)
    CH.free_factor(L, c)
    CH.free_sparse(A, c)
