"""Python side of the CPU oracle (oracle/oracle.c).

TEST INFRASTRUCTURE: the checker for tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py.  Never imported by the product.

``build()`` compiles oracle.c with gcc into oracle/liboracle.so.  When the
OpenBLAS bundled with scipy is present (both here and on the GPU host), its
Fortran-ABI routines are installed as the oracle's dense kernels, as the
reference CHOLMOD uses an external BLAS; otherwise the oracle's own loops run.
"""
import ctypes as C
import glob
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
_lib = None
_blas = None


def build():
    src = [os.path.join(HERE, "oracle.c")]
    hdr = os.path.join(HERE, "oracle_body.h")
    newest = max(os.path.getmtime(p) for p in src + [hdr])
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    subprocess.run(["gcc", "-O2", "-fPIC", "-shared", "-o", LIB + ".tmp"] + src + ["-lm"],
                   check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


def openblas():
    """ctypes handle of scipy's bundled OpenBLAS, or None."""
    global _blas
    if _blas is not None:
        return _blas or None
    try:
        import scipy
        d = os.path.join(os.path.dirname(scipy.__file__), "..", "scipy.libs")
        libs = sorted(glob.glob(os.path.join(d, "libscipy_openblas*.so")))
        _blas = C.CDLL(libs[0]) if libs else False
    except Exception:
        _blas = False
    return _blas or None


def lib(use_blas=True):
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        _lib = C.CDLL(LIB)
        _lib.oracle_super_numeric.restype = C.c_int
        _lib.oracle_super_solve.restype = C.c_int
        _lib.oracle_has_blas.restype = C.c_int
        _lib.oracle_super_pattern.restype = C.c_int
        _lib.oracle_free.argtypes = [C.c_void_p]
    set_blas(use_blas)
    return _lib


def set_blas(on=True):
    L = _lib
    b = openblas() if on else None
    if b is None:
        L.oracle_set_blas(*([None] * 8))
        return False
    names = ["scipy_dgemm_", "scipy_dsyrk_", "scipy_dtrsm_", "scipy_dpotrf_",
             "scipy_sgemm_", "scipy_ssyrk_", "scipy_strsm_", "scipy_spotrf_"]
    ptrs = [C.cast(getattr(b, nm), C.c_void_p) for nm in names]
    L.oracle_set_blas(*ptrs)
    return True


def blas_threads(n):
    """Set the OpenBLAS thread count (returns False without OpenBLAS)."""
    b = openblas()
    if b is None:
        return False
    for nm in ("scipy_openblas_set_num_threads", "openblas_set_num_threads"):
        if hasattr(b, nm):
            getattr(b, nm)(int(n))
            return True
    return False


def _p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


def factor(sym, Sp, Si, Sx, beta=0.0, dtype="d", quick_return=False, use_blas=True):
    """Supernodal LL' of S = tril(PAP') (sorted lower CSC) on the pattern
    ``sym`` (dict with n, Super, Pi, Px, Ls).  Returns (status, minor, Lx)."""
    L = lib(use_blas)
    Super, Pi, Px, Ls = (np.ascontiguousarray(sym[k], np.int64) for k in ("Super", "Pi", "Px", "Ls"))
    n, nsuper = int(sym["n"]), len(Super) - 1
    rt = np.float32 if dtype == "s" else np.float64
    Sp = np.ascontiguousarray(Sp, np.int64)
    Si = np.ascontiguousarray(Si, np.int64)
    Sx = np.ascontiguousarray(Sx, rt)
    Lx = np.zeros(max(int(Px[-1]), 1), rt)
    minor = C.c_int64(0)
    st = L.oracle_super_numeric(4 if dtype == "s" else 0, C.c_int64(n), C.c_int64(nsuper),
                                _p(Super, C.c_int64), _p(Pi, C.c_int64), _p(Px, C.c_int64),
                                _p(Ls, C.c_int64), _p(Sp, C.c_int64), _p(Si, C.c_int64),
                                Sx.ctypes.data_as(C.c_void_p), C.c_double(beta),
                                C.c_int(1 if quick_return else 0),
                                Lx.ctypes.data_as(C.c_void_p), C.byref(minor))
    return st, minor.value, Lx[:int(Px[-1])]


def sweep(sym, Lx, X, lower, dtype="d", use_blas=True):
    """Forward (lower=True: X = L\\X) or backward (X = L'\\X) sweep, in place
    on a copy of X (n x nrhs, permuted order); returns the result."""
    L = lib(use_blas)
    Super, Pi, Px, Ls = (np.ascontiguousarray(sym[k], np.int64) for k in ("Super", "Pi", "Px", "Ls"))
    rt = np.float32 if dtype == "s" else np.float64
    X = np.array(X, dtype=rt, order="F", copy=True)
    if X.ndim == 1:
        X = X[:, None].copy(order="F")
    n, nrhs = X.shape
    Lx = np.ascontiguousarray(Lx, rt)
    st = L.oracle_super_solve(4 if dtype == "s" else 0, C.c_int(1 if lower else 0),
                              C.c_int64(n), C.c_int64(len(Super) - 1), _p(Super, C.c_int64),
                              _p(Pi, C.c_int64), _p(Px, C.c_int64), _p(Ls, C.c_int64),
                              Lx.ctypes.data_as(C.c_void_p), C.c_int64(nrhs),
                              X.ctypes.data_as(C.c_void_p), C.c_int64(n))
    if st != 0:
        raise RuntimeError("oracle sweep failed")
    return X


def symbolic(n, Sp, Si, Super):
    """The reference's supernodal symbolic factor (dict with n, Super, Pi, Px,
    Ls) rebuilt from S = tril(PAP')'s pattern and the reference's supernode
    partition Super (a fixture), without the product library."""
    L = _lib if _lib is not None else lib()
    Sp = np.ascontiguousarray(Sp, np.int64)
    Si = np.ascontiguousarray(Si, np.int64)
    Super = np.ascontiguousarray(Super, np.int64)
    nsuper = len(Super) - 1
    Pi = np.zeros(nsuper + 1, np.int64)
    Px = np.zeros(nsuper + 1, np.int64)
    ls = C.POINTER(C.c_int64)()
    ssize = C.c_int64(0)
    st = L.oracle_super_pattern(C.c_int64(n), _p(Sp, C.c_int64), _p(Si, C.c_int64),
                                C.c_int64(nsuper), _p(Super, C.c_int64), _p(Pi, C.c_int64),
                                _p(Px, C.c_int64), C.byref(ls), C.byref(ssize))
    if st != 0:
        raise RuntimeError("oracle symbolic failed")
    Ls = np.ctypeslib.as_array(ls, shape=(ssize.value,)).copy() if ssize.value else \
        np.zeros(0, np.int64)
    L.oracle_free(ls)
    return {"n": n, "Super": Super, "Pi": Pi, "Px": Px, "Ls": Ls}


def permute_lower(n, Ap, Ai, Ax, perm):
    """S = tril(A(p,p)) in sorted CSC (numpy), A given by its lower part."""
    pinv = np.empty(n, np.int64)
    pinv[np.asarray(perm, np.int64)] = np.arange(n, dtype=np.int64)
    cols = np.repeat(np.arange(n, dtype=np.int64), np.diff(Ap))
    keep = Ai >= cols
    i, j, x = pinv[Ai[keep]], pinv[cols[keep]], Ax[keep]
    r, c = np.maximum(i, j), np.minimum(i, j)
    order = np.lexsort((r, c))
    r, c, x = r[order], c[order], x[order]
    Sp = np.zeros(n + 1, np.int64)
    np.add.at(Sp, c + 1, 1)
    return np.cumsum(Sp).astype(np.int64), r.astype(np.int64), x


def solve(sym, Lx, perm, B, dtype="d", use_blas=True):
    """X = A\\B through the oracle factor: P, forward, backward, P'."""
    B = np.asarray(B)
    if B.ndim == 1:
        B = B[:, None]
    perm = np.asarray(perm, np.int64)
    Y = B[perm, :]
    Y = sweep(sym, Lx, Y, True, dtype, use_blas)
    Y = sweep(sym, Lx, Y, False, dtype, use_blas)
    X = np.empty_like(Y)
    X[perm, :] = Y
    return X


def solve_sys(sym, Lx, perm, B, sys, natural=False, dtype="d", use_blas=True):
    """cholmod_l_solve's sys values for a supernodal LL' factor
    (CHOLMOD/Cholesky/cholmod_solve.c): the permutation only for sys = A (0),
    P (7), Pt (8) and an ordering other than natural (:262-267); P: X = P*B,
    Pt: X = P'*B (:616-650); otherwise Y = P*B, the lower sweep for A, LDLt,
    LD, L (0, 1, 2, 4), the upper for A, LDLt, DLt, Lt (0, 1, 3, 5), and
    X = P'*Y (:689-722); D (6) is the identity for LL'."""
    B = np.asarray(B)
    if B.ndim == 1:
        B = B[:, None]
    perm = np.asarray(perm, np.int64)
    use = sys in (0, 7, 8) and not natural
    Y = B[perm, :] if use and sys in (0, 7) else np.array(B, copy=True)
    if sys in (0, 1, 2, 4):
        Y = sweep(sym, Lx, Y, True, dtype, use_blas)
    if sys in (0, 1, 3, 5):
        Y = sweep(sym, Lx, Y, False, dtype, use_blas)
    if use and sys in (0, 8):
        X = np.empty_like(Y)
        X[perm, :] = Y
        return X
    return Y


def spsolve(sym, Lx, perm, n, Bp, Bi, Bx, sys=0, natural=False, dtype="d", use_blas=True):
    """cholmod_l_spsolve (CHOLMOD/Cholesky/cholmod_spsolve.c:56-278): B is
    scattered into a dense block (for a repeated row the last entry counts,
    the scatter worker of t_cholmod_spsolve_worker.c), solved with
    solve_sys, and each column's entries x != 0 (a NaN kept) appended in
    row order; returns (Xp, Xi, Xx) with nnz(X) = Xp[-1]."""
    ncol = len(Bp) - 1
    rt = np.float32 if dtype == "s" else np.float64
    Bd = np.zeros((n, ncol), rt)
    for j in range(ncol):
        for p in range(int(Bp[j]), int(Bp[j + 1])):
            Bd[int(Bi[p]), j] = Bx[p]
    X = solve_sys(sym, Lx, perm, Bd, sys, natural, dtype, use_blas)
    Xp = np.zeros(ncol + 1, np.int64)
    Xi, Xx = [], []
    for j in range(ncol):
        rows = np.nonzero(X[:, j] != 0)[0]
        Xi.append(rows)
        Xx.append(X[rows, j])
        Xp[j + 1] = Xp[j] + len(rows)
    cat = (lambda a, t: np.concatenate(a).astype(t) if a else np.zeros(0, t))
    return Xp, cat(Xi, np.int64), cat(Xx, rt)


def backward_error(n, Ap, Ai, Ax, X, B):
    """|b - A x|_inf / (|A|_inf |x|_inf + |b|_inf) per column (A lower-stored
    symmetric), the measure of CHOLMOD/Demo/cholmod_di_demo.c:614-617."""
    X = np.asarray(X, np.float64)
    B = np.asarray(B, np.float64)
    if X.ndim == 1:
        X, B = X[:, None], B[:, None]
    cols = np.repeat(np.arange(n, dtype=np.int64), np.diff(Ap))
    off = Ai != cols
    AX = np.zeros_like(X)
    np.add.at(AX, Ai, Ax[:, None] * X[cols])
    np.add.at(AX, cols[off], Ax[off][:, None] * X[Ai[off]])
    rowsum = np.zeros(n)
    np.add.at(rowsum, Ai, np.abs(Ax))
    np.add.at(rowsum, cols[off], np.abs(Ax[off]))
    anorm = rowsum.max() if n else 0.0
    R = B - AX
    return np.abs(R).max(axis=0) / (anorm * np.abs(X).max(axis=0) + np.abs(B).max(axis=0))


def complex_hermitian(n, Ap, Ai, Ax, perm=None):
    """Dense P A P^H of a Hermitian A given by its lower triangle (complex
    Ax); the imaginary part of the diagonal is dropped, as the reference's
    complex factorization ignores it (LAPACK's zpotrf reads the real part of
    a diagonal entry only)."""
    cols = np.repeat(np.arange(n, dtype=np.int64), np.diff(Ap))
    low = Ai >= cols
    i, j, v = Ai[low], cols[low], np.asarray(Ax)[low]
    H = np.zeros((n, n), dtype=np.complex128)
    d = i == j
    H[i[d], j[d]] = v[d].real
    H[i[~d], j[~d]] = v[~d]
    H[j[~d], i[~d]] = np.conj(v[~d])
    if perm is not None:
        p = np.asarray(perm, np.int64)
        H = H[np.ix_(p, p)]
    return H


def complex_factor(sym, H, quick_return=False):
    """Complex supernodal LL^H of the dense Hermitian H (already permuted) on
    the supernodal pattern sym (Super, Pi, Px, Ls), restated for small
    orders: column-by-column left-looking Cholesky, L(j,j) = sqrt(H(j,j) -
    sum |L(j,k)|^2) real, L(i,j) = (H(i,j) - sum L(i,k) conj(L(j,k))) /
    L(j,j) -- the factor the reference's complex workers compute with
    zherk / zgemm / zpotrf / ztrsm (Supernodal/t_cholmod_super_numeric_worker.c
    with L_ENTRY 2).  A non-positive pivot in column f stops it: L->minor =
    f and the failing supernode is cleaned up as in the real worker (its
    columns from f on, the whole supernode with quick_return, and every
    later entry zero).  Returns (status 0/1, minor, Lx complex)."""
    n = H.shape[0]
    L = np.zeros((n, n), dtype=np.complex128)
    minor = n
    for j in range(n):
        dj = H[j, j].real - np.sum(np.abs(L[j, :j]) ** 2)
        if not dj > 0:
            minor = j
            break
        ljj = np.sqrt(dj)
        L[j, j] = ljj
        L[j + 1:, j] = (H[j + 1:, j] - L[j + 1:, :j] @ np.conj(L[j, :j])) / ljj
    Super, Pi, Px, Ls = (np.asarray(sym[k], np.int64) for k in ("Super", "Pi", "Px", "Ls"))
    ns = len(Super) - 1
    Lx = np.zeros(int(Px[ns]), dtype=np.complex128)
    zero_from = len(Lx)
    for s in range(ns):
        k1, k2 = int(Super[s]), int(Super[s + 1])
        rows = Ls[Pi[s]:Pi[s + 1]]
        blk = L[np.ix_(rows, np.arange(k1, k2))]
        Lx[Px[s]:Px[s] + blk.size] = blk.ravel(order="F")
        if k1 <= minor < k2:
            info = minor - k1 + 1
            keep = 0 if (info == 1 or quick_return) else info - 1
            zero_from = int(Px[s]) + keep * len(rows)
    Lx[zero_from:] = 0
    return (0 if minor == n else 1), minor, Lx


def complex_solve(H, B):
    """x = H \\ b for the dense Hermitian positive definite H (numpy)."""
    return np.linalg.solve(H, np.asarray(B, np.complex128))


def complex_backward_error(H, X, B):
    """|b - H x|_inf / (|H|_inf |x|_inf + |b|_inf) per column, complex
    moduli (the measure of backward_error for a dense Hermitian H)."""
    X = np.asarray(X, np.complex128)
    B = np.asarray(B, np.complex128)
    if X.ndim == 1:
        X, B = X[:, None], B[:, None]
    R = B - H @ X
    an = np.abs(H).sum(axis=1).max()
    return np.abs(R).max(axis=0) / (an * np.abs(X).max(axis=0) + np.abs(B).max(axis=0))
