"""cholmod_l_rcond: on the CPU, the host path on a factor whose diagonal is
set by the test; on the GPU, the factors of the golden cases against the
reference CHOLMOD's own cholmod_l_rcond (tests/golden/rcond.json, made by
tests/golden/make_rcond.py), through the host copy of L and through the
device-resident factor (the same value bit for bit)."""
import ctypes as C
import json
import os

import numpy as np
import pytest

from conftest import make_case
from suitesparse_gb300 import cholmod as CH
from suitesparse_gb300 import matrices as M

HERE = os.path.dirname(os.path.abspath(__file__))


def test_host_path_matches_definition(lib):
    n, Ap, Ai, Ax = M.laplace2d(12, seed=3)
    c = CH.Common()
    A = CH.sparse(n, Ap, Ai, Ax, c)
    L = CH.analyze_perm(A, np.arange(n, dtype=np.int64), c)
    f = L.contents
    # give the symbolic factor values: the diagonal entries of every
    # supernode, the rest zero (an LL' factor whose factorization succeeded)
    xsize = int(f.xsize)
    buf = (C.c_double * xsize)()
    fa = CH.factor_arrays(L, with_x=False)
    rng = np.random.default_rng(1)
    diag = rng.uniform(0.5, 4.0, n)
    for s in range(int(fa["nsuper"])):
        k1, k2 = fa["Super"][s], fa["Super"][s + 1]
        nsrow = fa["Pi"][s + 1] - fa["Pi"][s]
        for j in range(k2 - k1):
            buf[int(fa["Px"][s] + j + j * nsrow)] = diag[k1 + j]
    f.x = C.cast(buf, C.c_void_p)
    f.xtype = CH.CHOLMOD_REAL
    f.minor = n
    r = CH.rcond(L, c)
    assert r == (diag.min() / diag.max()) ** 2
    f.minor = n - 1                       # a failed factorization
    assert CH.rcond(L, c) == 0.0
    f.minor = n
    buf[int(fa["Px"][0])] = float("nan")
    assert CH.rcond(L, c) == 0.0
    f.x = None
    f.xtype = CH.CHOLMOD_PATTERN
    CH.free_factor(L, c)
    CH.free_sparse(A, c)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["g2c", "g2v", "g3", "g3a", "e27", "c1", "npd"])
def test_matches_reference_rcond(golden, lib, name):
    meta, arrays = golden
    ref = json.load(open(os.path.join(HERE, "golden", "rcond.json")))[name]
    n, Ap, Ai, Ax = make_case(meta, name)
    perm = arrays[name + "_Perm"].astype(np.int64)
    vals = []
    for keep in (0, 1):
        c = CH.Common()
        c.set_option(CH.GB300_OPT_KEEP_ON_DEVICE, keep)
        A = CH.sparse(n, Ap, Ai, Ax, c)
        L = CH.analyze_perm(A, perm, c)
        assert CH.factorize(A, L, c) == 1
        vals.append(CH.rcond(L, c))
        assert c.status in (CH.CHOLMOD_OK, CH.CHOLMOD_NOT_POSDEF)
        CH.free_factor(L, c)
        CH.free_sparse(A, c)
    assert vals[0] == vals[1]             # host copy and device-resident factor
    if ref["rcond"] == 0.0:
        assert vals[0] == 0.0
    else:
        assert abs(vals[0] - ref["rcond"]) <= 1e-12 * ref["rcond"]
