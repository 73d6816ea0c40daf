"""cholmod_l_rowfac on the GPU (the simplicial LL' and LDL' factorization
that cholmod_l_factorize runs for the simplicial method) against the
reference's own simplicial factor of the same matrix: the layout (Lp, Lnz,
Li) equal, the values within the FP64 tolerance, L->minor and the status as
the reference's."""
import ctypes as C
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, make_case
from suitesparse_gb300 import cholmod as CH

pytestmark = pytest.mark.gpu
L_TOL = 1e-10
L_TOL_SINGLE = 1e-4
CHOLMOD_PATTERN, CHOLMOD_LONG = 0, 2


@pytest.fixture(scope="module")
def simp():
    meta = json.load(open(os.path.join(GOLDEN, "simplicial.json")))
    return meta, dict(np.load(os.path.join(GOLDEN, "simplicial.npz")))


def _upper(n, Ap, Ai, Ax, perm):
    """S = triu(A(p,p)) in column form (the form factorize_p passes)."""
    from oracle import oracle as O
    Sp, Si, Sx = O.permute_lower(n, Ap, Ai, Ax, perm)
    cols = np.repeat(np.arange(n), np.diff(Sp))
    order = np.lexsort((cols, Si))            # upper: column = row of lower
    r, c, v = cols[order], Si[order], Sx[order]
    Up = np.zeros(n + 1, np.int64)
    np.add.at(Up, c + 1, 1)
    return np.cumsum(Up), r.astype(np.int64), v


class Symbolic:
    """A simplicial symbolic factor (Perm, ColCount) owned by numpy; the
    numeric arrays the call allocates are released with free()."""

    def __init__(self, n, perm, colcount, is_ll, dtype):
        self.perm = np.ascontiguousarray(perm, np.int64)
        self.cc = np.ascontiguousarray(colcount, np.int64)
        L = CH.cholmod_factor()
        L.n, L.minor = n, n
        L.Perm, L.ColCount = self.perm.ctypes.data, self.cc.ctypes.data
        L.is_ll, L.is_super, L.is_monotonic = is_ll, 0, 1
        L.itype, L.xtype, L.dtype = CHOLMOD_LONG, CHOLMOD_PATTERN, dtype
        self.L = L
        self.ptr = C.pointer(L)

    def arrays(self, single=False):
        L, n = self.L, self.L.n
        lp = CH._arr(L.p, np.int64, n + 1).copy()
        dt = np.float32 if single else np.float64
        return dict(Lp=lp, Lnz=CH._arr(L.nz, np.int64, n).copy(),
                    Li=CH._arr(L.i, np.int64, L.nzmax).copy(),
                    Lx=CH._arr(L.x, dt, L.nzmax).copy().astype(np.float64))

    def free(self):
        libc = C.CDLL(None)
        for f in ("p", "i", "x", "nz", "next", "prev"):
            v = getattr(self.L, f)
            if v:
                libc.free(C.c_void_p(v))
            setattr(self.L, f, None)


def _run(golden, simp, name, form, single=False):
    meta, arrays = golden
    smeta, sarr = simp
    key = f"{name}_{form}"
    n, Ap, Ai, Ax = make_case(meta, name)
    perm = sarr[key + "_Perm"].astype(np.int64)
    Up, Ui, Ux = _upper(n, Ap, Ai, Ax, perm)
    c = CH.Common()
    c["grow2"] = 0                    # as cholmod_factorize with final_pack
    S = CH.sparse(n, Up, Ui, Ux.astype(np.float32) if single else Ux, c, stype=1,
                  dtype="s" if single else "d")
    sym = Symbolic(n, perm, sarr[key + "_ColCount"], 1 if form == "ll" else 0,
                   1 if single else 0)
    beta = (C.c_double * 2)(0.0, 0.0)
    rc = CH.lib().cholmod_l_rowfac(S, None, beta, 0, n, sym.ptr, c.ptr)
    out = sym.arrays(single)
    res = dict(rc=rc, status=c.status, minor=sym.L.minor, nzmax=sym.L.nzmax,
               is_ll=sym.L.is_ll, rowfacfl=c["rowfacfl"], **out)
    sym.free()
    CH.free_sparse(S, c)
    return res, smeta[key], {k: sarr[key + "_" + k] for k in ("Lp", "Lnz", "Li", "Lx")}


@pytest.mark.parametrize("name", ["g2c", "g2v", "g3", "e27", "c4_21"])
@pytest.mark.parametrize("form", ["ll", "ldl"])
def test_simplicial_matches_reference(golden, lib, simp, name, form):
    r, m, ref = _run(golden, simp, name, form)
    assert r["rc"] == 1 and r["status"] == CH.CHOLMOD_OK and r["minor"] == m["minor"]
    assert r["is_ll"] == m["is_ll"] and r["nzmax"] == m["nzmax"]
    nnz = int(ref["Lp"][-1])
    assert np.array_equal(r["Lp"], ref["Lp"]) and np.array_equal(r["Lnz"], ref["Lnz"])
    assert np.array_equal(r["Li"][:nnz], ref["Li"])
    err = np.linalg.norm(r["Lx"][:nnz] - ref["Lx"]) / np.linalg.norm(ref["Lx"])
    assert err <= L_TOL, err
    # the reference's flop count: sum of (count^2 - 1), plus n square roots for LL'
    cc = np.diff(ref["Lp"]).astype(np.float64)
    assert r["rowfacfl"] == np.sum(cc * cc - 1) + (m["n"] if form == "ll" else 0)


@pytest.mark.parametrize("form", ["ll", "ldl"])
def test_simplicial_single(golden, lib, simp, form):
    r, m, ref = _run(golden, simp, "g3", form, single=True)
    assert r["rc"] == 1 and r["status"] == CH.CHOLMOD_OK
    nnz = int(ref["Lp"][-1])
    assert np.array_equal(r["Li"][:nnz], ref["Li"])
    err = np.linalg.norm(r["Lx"][:nnz] - ref["Lx"]) / np.linalg.norm(ref["Lx"])
    assert err <= L_TOL_SINGLE, err


def test_simplicial_not_positive_definite(golden, lib, simp):
    """LL': the reference's minor and status, its values before the failing
    column and zeros from it on.  LDL' of the same indefinite matrix: the
    reference goes on through negative pivots (minor = n); this library
    forms LDL' from LL' and stops at the same first non-positive pivot."""
    r, m, ref = _run(golden, simp, "npd", "ll")
    assert r["rc"] == 1 and r["status"] == CH.CHOLMOD_NOT_POSDEF and r["minor"] == m["minor"]
    nnz = int(ref["Lp"][-1])
    assert np.array_equal(r["Li"][:nnz], ref["Li"])
    err = np.linalg.norm(r["Lx"][:nnz] - ref["Lx"]) / np.linalg.norm(ref["Lx"])
    assert err <= L_TOL, err
    r2, m2, _ = _run(golden, simp, "npd", "ldl")
    assert m2["minor"] == m2["n"]
    assert r2["rc"] == 1 and r2["status"] == CH.CHOLMOD_NOT_POSDEF and r2["minor"] == m["minor"]
