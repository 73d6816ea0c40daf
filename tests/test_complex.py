"""Complex supernodal LL' (cholmod_l_super_numeric with a complex or zomplex
A, complex L) and the complex sweeps (cholmod_l_super_lsolve / _ltsolve with
a complex L and X).

CPU: the oracle's complex restatement against the reference's own complex
factors and solutions (tests/golden/make_complex.py), and the symbolic
pattern of the complex cases.  GPU: the library's factor of every golden
case against the reference's L->x, its sweeps against the reference's X,
zomplex input, the imaginary parts the reference ignores (of the diagonal,
of beta), not-positive-definite semantics, a factor computed elsewhere, the
A F form, and single precision."""
import json
import os

import numpy as np
import pytest

from suitesparse_gb300 import cholmod as CH
from suitesparse_gb300 import matrices as M

HERE = os.path.dirname(os.path.abspath(__file__))
L_TOL = 1e-10


@pytest.fixture(scope="module")
def cgold():
    with open(os.path.join(HERE, "golden", "complex.json")) as f:
        meta = json.load(f)
    return meta, dict(np.load(os.path.join(HERE, "golden", "complex.npz")))


def _case(meta, name):
    m = meta[name]
    return M.magnetic_laplacian(tuple(m["dims"]), **m["kwargs"])


def _rhs(meta, name, n):
    m = meta[name]
    return M.rhs(n, m["nrhs"], m["seed"]) + 1j * M.rhs(n, m["nrhs"], m["seed"] + 1)


def _sym(arrays, name):
    return {k: arrays[f"{name}_{k}"] for k in ("Super", "Pi", "Px", "Ls")}


def _relerr(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b))


@pytest.mark.parametrize("name", ["cx2", "cx3", "cxdiag", "cxnpd", "cx2s"])
def test_oracle_matches_reference(cgold, oracle_mod, name):
    meta, arrays = cgold
    n, Ap, Ai, Ax = _case(meta, name)
    H = oracle_mod.complex_hermitian(n, Ap, Ai, Ax, arrays[name + "_Perm"])
    st, minor, Lx = oracle_mod.complex_factor(_sym(arrays, name), H)
    assert minor == meta[name]["minor"] and st == meta[name]["factor_status"]
    tol = 1e-6 if meta[name]["dtype"] == "s" else 1e-13
    assert _relerr(Lx, arrays[name + "_Lx"]) <= tol
    if meta[name]["nrhs"]:
        B = _rhs(meta, name, n)
        Hf = oracle_mod.complex_hermitian(n, Ap, Ai, Ax)
        X = oracle_mod.complex_solve(Hf, B)
        assert _relerr(X, arrays[name + "_X"]) <= 100 * tol
        assert oracle_mod.complex_backward_error(Hf, X, B).max() <= 1e-14


@pytest.mark.parametrize("name", ["cx2", "cx3", "cxnpd"])
def test_symbolic_pattern_of_complex_cases(cgold, lib, name):
    """The library's analysis of the complex matrix's pattern, with the
    reference's permutation, is the reference's supernodal pattern."""
    meta, arrays = cgold
    n, Ap, Ai, Ax = _case(meta, name)
    c = CH.Common()
    A = CH.sparse(n, Ap, Ai, np.abs(Ax), c)
    L = CH.analyze_perm(A, arrays[name + "_Perm"], c)
    f = CH.factor_arrays(L, with_x=False)
    for k in ("Super", "Pi", "Px", "Ls"):
        assert np.array_equal(f[k], arrays[f"{name}_{k}"]), k
    CH.free_factor(L, c)
    CH.free_sparse(A, c)
    c.finish()


# ---- GPU ------------------------------------------------------------------

def _permuted_lower(n, Ap, Ai, Ax, perm):
    """tril(P A P^H) in sorted CSC of the Hermitian A given by its lower
    triangle, with the diagonal's imaginary parts kept as given."""
    cols = np.repeat(np.arange(n, dtype=np.int64), np.diff(Ap))
    H = np.zeros((n, n), dtype=np.complex128)
    H[Ai, cols] = Ax
    off = Ai != cols
    H[cols[off], Ai[off]] = np.conj(Ax[off])
    p = np.asarray(perm, np.int64)
    T = np.tril(H[np.ix_(p, p)])
    mask = np.tril(np.ones((n, n), bool)) & ((T != 0) | np.eye(n, dtype=bool))
    jj, ii = np.nonzero(mask.T)                  # column-major: by column, rows ascending
    Sp = np.zeros(n + 1, np.int64)
    np.add.at(Sp, jj + 1, 1)
    return n, np.cumsum(Sp), ii.astype(np.int64), T[ii, jj]


def _factor(meta, arrays, name, zomplex=False, beta=0.0, beta_im=0.0, quick_return=False,
            dtype=None):
    n, Ap, Ai, Ax = _case(meta, name)
    perm = arrays[name + "_Perm"]
    dtype = dtype or meta[name]["dtype"]
    c = CH.Common()
    if quick_return:
        c["quick_return_if_not_posdef"] = 1
    A = CH.sparse(n, Ap, Ai, np.abs(Ax), c)
    L = CH.analyze_perm(A, perm, c)
    CH.free_sparse(A, c)
    S = CH.csparse(*_permuted_lower(n, Ap, Ai, Ax, perm), c, dtype=dtype, zomplex=zomplex)
    ok = CH.super_numeric(S, L, c, beta=beta, beta_im=beta_im)
    CH.free_sparse(S, c)
    return c, L, ok


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["cx2", "cx3", "cxdiag", "cx2s"])
def test_factor_and_sweeps_match_reference(cgold, lib, oracle_mod, name):
    meta, arrays = cgold
    c, L, ok = _factor(meta, arrays, name)
    single = meta[name]["dtype"] == "s"
    assert ok == 1 and c.status == CH.CHOLMOD_OK
    f = CH.factor_arrays(L)
    assert f["xtype"] == CH.CHOLMOD_COMPLEX and f["minor"] == f["n"]
    e = _relerr(f["Lx"], arrays[name + "_Lx"])
    assert e <= (1e-4 if single else L_TOL), e
    # x = P' L^-H L^-1 P b through cholmod_l_super_lsolve / _ltsolve
    n, Ap, Ai, Ax = _case(meta, name)
    perm = arrays[name + "_Perm"]
    B = _rhs(meta, name, n)
    dt = "s" if single else "d"
    ok1, Y = CH.super_solve(L, B[perm], c, True, dtype=dt)
    ok2, Z = CH.super_solve(L, Y, c, False, dtype=dt)
    assert ok1 == 1 and ok2 == 1
    X = np.empty_like(Z)
    X[perm] = Z
    assert _relerr(X, arrays[name + "_X"]) <= (1e-3 if single else 1e-9)
    if not single:
        Hf = oracle_mod.complex_hermitian(n, Ap, Ai, Ax)
        assert oracle_mod.complex_backward_error(Hf, X, B).max() <= 1e-14
    CH.free_factor(L, c)
    c.finish()


@pytest.mark.gpu
def test_zomplex_input_and_ignored_imaginary_parts(cgold, lib):
    """A zomplex A gives the complex A's factor bit for bit; the imaginary
    part of beta is not used (only beta[0] is added to the real diagonal)."""
    meta, arrays = cgold
    c0, L0, _ = _factor(meta, arrays, "cxdiag")
    c1, L1, _ = _factor(meta, arrays, "cxdiag", zomplex=True)
    assert np.array_equal(CH.factor_arrays(L0)["Lx"], CH.factor_arrays(L1)["Lx"])
    c2, L2, _ = _factor(meta, arrays, "cxdiag", beta=0.25, beta_im=5.0)
    c3, L3, _ = _factor(meta, arrays, "cxdiag", beta=0.25)
    a, b = CH.factor_arrays(L2)["Lx"], CH.factor_arrays(L3)["Lx"]
    assert np.array_equal(a, b) and not np.array_equal(a, CH.factor_arrays(L0)["Lx"])
    for cc, LL in ((c0, L0), (c1, L1), (c2, L2), (c3, L3)):
        CH.free_factor(LL, cc)
        cc.finish()


@pytest.mark.gpu
@pytest.mark.parametrize("quick_return", [False, True])
def test_not_positive_definite(cgold, lib, oracle_mod, quick_return):
    meta, arrays = cgold
    c, L, ok = _factor(meta, arrays, "cxnpd", quick_return=quick_return)
    assert ok == 1 and c.status == CH.CHOLMOD_NOT_POSDEF
    f = CH.factor_arrays(L)
    assert f["minor"] == meta["cxnpd"]["minor"]
    n, Ap, Ai, Ax = _case(meta, "cxnpd")
    H = oracle_mod.complex_hermitian(n, Ap, Ai, Ax, arrays["cxnpd_Perm"])
    st, minor, Lref = oracle_mod.complex_factor(_sym(arrays, "cxnpd"), H, quick_return)
    assert minor == f["minor"]
    tail = int(np.nonzero(Lref)[0][-1]) + 1        # the zeroed rest of the factor
    assert tail < len(Lref) and not np.any(f["Lx"][tail:])
    assert _relerr(f["Lx"], Lref) <= L_TOL
    if not quick_return:
        assert _relerr(f["Lx"], arrays["cxnpd_Lx"]) <= L_TOL
    CH.free_factor(L, c)
    c.finish()


@pytest.mark.gpu
def test_sweeps_with_a_factor_from_elsewhere(cgold, lib, oracle_mod):
    """L->x replaced by the reference's own complex factor (and the device
    state dropped): the sweeps read L's values, not a device copy."""
    meta, arrays = cgold
    c, L, _ = _factor(meta, arrays, "cx3")
    f = L.contents
    v = CH._arr(f.x, np.float64, 2 * f.xsize)
    ref = arrays["cx3_Lx"]
    v[0::2] = ref.real
    v[1::2] = ref.imag
    CH.lib().gb300_release_factor(L, c.ptr)
    n, Ap, Ai, Ax = _case(meta, "cx3")
    perm = arrays["cx3_Perm"]
    B = _rhs(meta, "cx3", n)
    _, Y = CH.super_solve(L, B[perm], c, True)
    _, Z = CH.super_solve(L, Y, c, False)
    X = np.empty_like(Z)
    X[perm] = Z
    assert _relerr(X, arrays["cx3_X"]) <= 1e-12
    CH.free_factor(L, c)
    c.finish()


@pytest.mark.gpu
def test_a_times_f_form(lib, oracle_mod):
    """beta I + A F with F = A^H (stype 0, the form cholmod_factorize uses
    for an unsymmetric A): the factor of the Hermitian product, as the
    oracle computes it densely; the imaginary parts of the product's
    diagonal are ignored."""
    rng = np.random.default_rng(3)
    n, m = 120, 300
    dens = 0.03
    Ad = (rng.random((n, m)) < dens) * (rng.standard_normal((n, m)) + 1j * rng.standard_normal((n, m)))
    Ad[np.arange(n), np.arange(n)] += 3.0
    # a full column makes the product dense: its elimination tree is a
    # path, so the natural order is a postorder
    Ad[:, n] = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    beta = 0.5
    Hd = Ad @ Ad.conj().T + beta * np.eye(n)

    def csc(D):
        jj, ii = np.nonzero(D.T)
        p = np.zeros(D.shape[1] + 1, np.int64)
        np.add.at(p, jj + 1, 1)
        return np.cumsum(p), ii.astype(np.int64), D[ii, jj]

    c = CH.Common()
    # the symbolic factor of the product's pattern, natural order
    T = np.tril(Hd)
    Tp, Ti, Tx = csc(T)
    Areal = CH.sparse(n, Tp, Ti, np.abs(Tx) + 1.0, c)
    L = CH.analyze_perm(Areal, np.arange(n, dtype=np.int64), c)
    CH.free_sparse(Areal, c)
    Ap_, Ai_, Ax_ = csc(Ad)
    Fp_, Fi_, Fx_ = csc(Ad.conj().T)
    A = CH.csparse(n, Ap_, Ai_, Ax_, c, stype=0, ncol=m)
    F = CH.csparse(m, Fp_, Fi_, Fx_, c, stype=0, ncol=n)
    assert CH.super_numeric(A, L, c, beta=beta, F=F) == 1 and c.status == CH.CHOLMOD_OK
    f = CH.factor_arrays(L)
    st, minor, Lref = oracle_mod.complex_factor({k: f[k] for k in ("Super", "Pi", "Px", "Ls")}, Hd)
    assert st == 0 and _relerr(f["Lx"], Lref) <= L_TOL
    CH.free_sparse(A, c)
    CH.free_sparse(F, c)
    CH.free_factor(L, c)
    c.finish()


@pytest.mark.gpu
def test_int32_entry_points_take_complex_factors(cgold, lib):
    """cholmod_super_numeric / cholmod_super_lsolve on int32 copies of a
    complex problem give the int64 path's factor and solution bit for bit."""
    import ctypes as C
    from test_gpu_int32 import CHOLMOD_INT, Int32Objects
    meta, arrays = cgold
    n, Ap, Ai, Ax = _case(meta, "cx2")
    perm = arrays["cx2_Perm"]
    c = CH.Common()
    A = CH.sparse(n, Ap, Ai, np.abs(Ax), c)
    L = CH.analyze_perm(A, perm, c)
    CH.free_sparse(A, c)
    S = CH.csparse(*_permuted_lower(n, Ap, Ai, Ax, perm), c)
    o32 = Int32Objects(S, L)
    assert CH.super_numeric(S, L, c) == 1
    Lx64 = CH.factor_arrays(L)["Lx"]
    B = _rhs(meta, "cx2", n)[perm]
    _, Y64 = CH.super_solve(L, B, c, True)
    c32 = CH.Common()
    c32["itype"] = CHOLMOD_INT
    L32, A32 = C.pointer(o32.L), C.pointer(o32.A)
    beta = (C.c_double * 2)(0.0, 0.0)
    assert lib.cholmod_super_numeric(A32, None, beta, L32, c32.ptr) == 1, c32.status
    assert o32.L.xtype == CH.CHOLMOD_COMPLEX and o32.L.minor == n
    v = np.ctypeslib.as_array(C.cast(o32.L.x, C.POINTER(C.c_double)), shape=(2 * o32.L.xsize,))
    assert np.array_equal(v[0::2] + 1j * v[1::2], Lx64)
    X = CH.cdense(B, c32)
    me = max(int(o32.L.maxesize), 1)
    E = lib.gb300_allocate_dense(me, B.shape[1], me, CH.CHOLMOD_COMPLEX + CH.CHOLMOD_DOUBLE, c32.ptr)
    assert lib.cholmod_super_lsolve(L32, X, E, c32.ptr) == 1
    assert np.array_equal(CH.cdense_array(X), Y64)
    CH.free_dense(X, c32)
    CH.free_dense(E, c32)
    lib.gb300_release_factor(L32, c32.ptr)
    CH.free_sparse(S, c)
    CH.free_factor(L, c)
