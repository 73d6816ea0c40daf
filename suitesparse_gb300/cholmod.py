"""ctypes bindings of libcholmod_gb300.so, mirroring the CHOLMOD calling style.

The library is the product: a C ABI whose entry points are the CHOLMOD ones
(``cholmod_l_super_numeric``, ``cholmod_l_super_lsolve``,
``cholmod_l_super_ltsolve``) plus ``gb300_*`` drivers.  This module only
marshals numpy arrays into CHOLMOD objects allocated by the library and calls
through the C ABI; it does no numerical work itself.  Loading fails loudly if
the shared library has not been built.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libcholmod_gb300.so")

CHOLMOD_PATTERN, CHOLMOD_REAL, CHOLMOD_COMPLEX, CHOLMOD_ZOMPLEX = 0, 1, 2, 3
CHOLMOD_DOUBLE, CHOLMOD_SINGLE = 0, 4
CHOLMOD_OK, CHOLMOD_NOT_INSTALLED, CHOLMOD_OUT_OF_MEMORY = 0, -1, -2
CHOLMOD_TOO_LARGE, CHOLMOD_INVALID, CHOLMOD_GPU_PROBLEM = -3, -4, -5
CHOLMOD_NOT_POSDEF, CHOLMOD_DSMALL = 1, 2
CHOLMOD_A, CHOLMOD_LDLt, CHOLMOD_LD, CHOLMOD_DLt, CHOLMOD_L = 0, 1, 2, 3, 4
CHOLMOD_Lt, CHOLMOD_D, CHOLMOD_P, CHOLMOD_Pt = 5, 6, 7, 8
GB300_OPT_KEEP_ON_DEVICE, GB300_OPT_SMALL_COLS, GB300_OPT_PROFILE, GB300_OPT_SWEEP = 1, 2, 3, 4
GB300_OPT_TRACE, GB300_OPT_FACTOR, GB300_OPT_TENSOR = 5, 6, 7
GB300_OPT_SUBTREE_WORK = 8
GB300_OPT_WARP_ROWS = 9
GB300_OPT_GRAPH = 10
GB300_OPT_SWEEP_STREAMS = 11
GB300_OPT_PIVOT_LOG2 = 12
GB300_OPT_UPD_GROUP = 13
GB300_OPT_AUTOTUNE = 14
TUNE_TIMER = C.CFUNCTYPE(C.c_double, C.c_void_p, C.c_void_p)
GB300_REASON_NONE, GB300_REASON_FP32_FAILED = 0, 1
GB300_REASON_SMALL_PIVOT, GB300_REASON_STALLED = 2, 3
KIND_NAMES = {1: "assemble", 2: "factor_small", 3: "potrf_diag", 4: "trsm_rows", 5: "gemm_tile",
              6: "task_graph", 15: "whole_graph"}


class cholmod_sparse(C.Structure):
    _fields_ = [("nrow", C.c_size_t), ("ncol", C.c_size_t), ("nzmax", C.c_size_t),
                ("p", C.c_void_p), ("i", C.c_void_p), ("nz", C.c_void_p),
                ("x", C.c_void_p), ("z", C.c_void_p), ("stype", C.c_int),
                ("itype", C.c_int), ("xtype", C.c_int), ("dtype", C.c_int),
                ("sorted", C.c_int), ("packed", C.c_int)]


class cholmod_factor(C.Structure):
    _fields_ = [("n", C.c_size_t), ("minor", C.c_size_t), ("Perm", C.c_void_p),
                ("ColCount", C.c_void_p), ("IPerm", C.c_void_p), ("nzmax", C.c_size_t),
                ("p", C.c_void_p), ("i", C.c_void_p), ("x", C.c_void_p),
                ("z", C.c_void_p), ("nz", C.c_void_p), ("next", C.c_void_p),
                ("prev", C.c_void_p), ("nsuper", C.c_size_t), ("ssize", C.c_size_t),
                ("xsize", C.c_size_t), ("maxcsize", C.c_size_t), ("maxesize", C.c_size_t),
                ("super", C.c_void_p), ("pi", C.c_void_p), ("px", C.c_void_p),
                ("s", C.c_void_p), ("ordering", C.c_int), ("is_ll", C.c_int),
                ("is_super", C.c_int), ("is_monotonic", C.c_int), ("itype", C.c_int),
                ("xtype", C.c_int), ("dtype", C.c_int), ("useGPU", C.c_int)]


class cholmod_dense(C.Structure):
    _fields_ = [("nrow", C.c_size_t), ("ncol", C.c_size_t), ("nzmax", C.c_size_t),
                ("d", C.c_size_t), ("x", C.c_void_p), ("z", C.c_void_p),
                ("xtype", C.c_int), ("dtype", C.c_int)]


SP = C.POINTER(cholmod_sparse)
FP = C.POINTER(cholmod_factor)
DP = C.POINTER(cholmod_dense)

_lib = None


def lib():
    """Load the C-ABI library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with "
                           "python -c 'import __graft_entry__ as g; g.build()'")
    L = C.CDLL(LIB_PATH)
    vp = C.c_void_p
    sig = {
        "gb300_start": (C.c_int, [vp]),
        "gb300_finish": (C.c_int, [vp]),
        "gb300_set_option": (C.c_int, [vp, C.c_int, C.c_int64]),
        "gb300_get_option": (C.c_int64, [vp, C.c_int]),
        "gb300_autotune": (C.c_int, [vp, vp, C.c_int, C.c_int, C.POINTER(C.c_int64), C.c_int,
                                     C.POINTER(C.c_double), vp]),
        "gb300_autotune_candidates": (C.c_int, [C.POINTER(C.c_int64), C.c_int]),
        "gb300_autotune_with": (C.c_int, [C.POINTER(C.c_int64), C.c_int, C.c_int,
                                          C.POINTER(C.c_double), TUNE_TIMER, vp, vp]),
        "gb300_get_stats": (C.c_int, [vp, C.POINTER(C.c_double), C.c_int]),
        "gb300_abi_offset": (C.c_long, [C.c_int, C.c_char_p]),
        "gb300_abi_sizeof": (C.c_long, [C.c_int]),
        "gb300_allocate_sparse": (SP, [C.c_size_t, C.c_size_t, C.c_size_t, C.c_int,
                                       C.c_int, C.c_int, C.c_int, vp]),
        "gb300_allocate_dense": (DP, [C.c_size_t, C.c_size_t, C.c_size_t, C.c_int, vp]),
        "gb300_free_sparse": (C.c_int, [C.POINTER(SP), vp]),
        "gb300_free_dense": (C.c_int, [C.POINTER(DP), vp]),
        "gb300_free_factor": (C.c_int, [C.POINTER(FP), vp]),
        "gb300_analyze_perm": (FP, [SP, C.POINTER(C.c_int64), vp]),
        "gb300_factorize": (C.c_int, [SP, C.POINTER(C.c_double), FP, vp]),
        "gb300_solve": (DP, [C.c_int, FP, DP, vp]),
        "gb300_factorize_mixed": (C.c_int, [SP, FP, vp]),
        "gb300_solve_refined": (DP, [SP, FP, DP, C.c_double, C.POINTER(C.c_double), vp]),
        "gb300_solve_refined2": (C.c_int, [SP, FP, DP, C.c_double, C.POINTER(C.c_double),
                                           C.POINTER(DP), vp]),
        "gb300_release_factor": (C.c_int, [FP, vp]),
        "gb300_mixed_reason": (C.c_int, [FP, vp]),
        "gb300_get_profile": (C.c_int, [vp, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int]),
        "gb300_factor_info": (C.c_int, [FP, vp, C.POINTER(C.c_double), C.c_int]),
        "gb300_fma_peak": (C.c_int, [C.c_int, C.POINTER(C.c_double)]),
        "gb300_get_trace": (C.c_int, [vp, C.c_int, C.POINTER(C.c_ulonglong), C.c_int64]),
        "gb300_get_factor_trace": (C.c_int, [vp, C.POINTER(C.c_ulonglong), C.c_int64]),
        "gb300_plan_tasks": (C.c_int, [FP, vp, C.POINTER(C.c_int32), C.c_int64]),
        "gb300_plan_sweep_tasks": (C.c_int, [FP, vp, C.c_int, C.POINTER(C.c_int32), C.c_int64]),
        "cholmod_l_rcond": (C.c_double, [FP, vp]),
        "cholmod_l_spsolve": (SP, [C.c_int, FP, SP, vp]),
        "gb300_batch_analyze": (FP, [C.c_int, C.POINTER(FP), C.c_int64, C.POINTER(C.c_int32), vp]),
        "cholmod_l_super_numeric": (C.c_int, [SP, SP, C.POINTER(C.c_double), FP, vp]),
        "cholmod_l_super_lsolve": (C.c_int, [FP, DP, DP, vp]),
        "cholmod_l_super_ltsolve": (C.c_int, [FP, DP, DP, vp]),
        "cholmod_super_numeric": (C.c_int, [SP, SP, C.POINTER(C.c_double), FP, vp]),
        "cholmod_l_rowfac": (C.c_int, [SP, SP, C.POINTER(C.c_double), C.c_size_t, C.c_size_t,
                                       FP, vp]),
        "cholmod_super_lsolve": (C.c_int, [FP, DP, DP, vp]),
        "cholmod_super_ltsolve": (C.c_int, [FP, DP, DP, vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


_COMMON_FIELDS = {
    "status": C.c_int, "print": C.c_int, "try_catch": C.c_int,
    "quick_return_if_not_posdef": C.c_int, "fl": C.c_double, "lnz": C.c_double,
    "anz": C.c_double, "malloc_count": C.c_size_t, "memory_inuse": C.c_size_t,
    "supernodal": C.c_int, "useGPU": C.c_int, "itype": C.c_int, "grow2": C.c_size_t,
    "final_ll": C.c_int, "rowfacfl": C.c_double,
}


class Common:
    """A cholmod_common owned by Python, initialised with gb300_start."""

    def __init__(self, print_level=0):
        L = lib()
        self._buf = C.create_string_buffer(L.gb300_abi_sizeof(0))
        self.ptr = C.cast(self._buf, C.c_void_p)
        L.gb300_start(self.ptr)
        self["print"] = print_level

    def _field(self, name):
        off = lib().gb300_abi_offset(0, name.encode())
        if off < 0:
            raise KeyError(name)
        return _COMMON_FIELDS[name].from_address(self.ptr.value + off)

    def __getitem__(self, name):
        return self._field(name).value

    def __setitem__(self, name, value):
        self._field(name).value = value

    @property
    def status(self):
        return self["status"]

    def set_option(self, option, value):
        return lib().gb300_set_option(self.ptr, option, int(value))

    def get_option(self, option):
        return lib().gb300_get_option(self.ptr, option)

    def stats(self):
        out = (C.c_double * 8)()
        lib().gb300_get_stats(self.ptr, out, 8)
        return list(out)

    def profile(self):
        ms = (C.c_double * 16)()
        cnt = (C.c_double * 16)()
        lib().gb300_get_profile(self.ptr, ms, cnt, 16)
        return {KIND_NAMES.get(k, str(k)): (ms[k], cnt[k]) for k in range(16) if cnt[k]}

    def trace(self, forward, nmax=1 << 22):
        out = (C.c_ulonglong * (3 * nmax))()
        nt = lib().gb300_get_trace(self.ptr, 1 if forward else 0, out, nmax)
        if nt < 0:
            return None
        return np.frombuffer(out, dtype=np.uint64, count=3 * nt).reshape(nt, 3).copy()

    def factor_trace(self, nmax=1 << 22):
        out = (C.c_ulonglong * (3 * nmax))()
        nt = lib().gb300_get_factor_trace(self.ptr, out, nmax)
        if nt < 0:
            return None
        return np.frombuffer(out, dtype=np.uint64, count=3 * nt).reshape(nt, 3).copy()

    def finish(self):
        if self.ptr:
            lib().gb300_finish(self.ptr)

    def __del__(self):
        try:
            self.finish()
        except Exception:
            pass


def _arr(ptr, dtype, count):
    if not ptr or count == 0:
        return np.zeros(0, dtype=dtype)
    ct = {np.int64: C.c_int64, np.float64: C.c_double, np.float32: C.c_float}[dtype]
    return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(ct)), shape=(count,))


def sparse(n, Ap, Ai, Ax, common, stype=-1, dtype="d", ncol=None):
    """Allocate a cholmod_sparse in the library and copy the CSC arrays in."""
    ncol = n if ncol is None else ncol
    nz = int(Ap[-1])
    dt = CHOLMOD_SINGLE if dtype == "s" else CHOLMOD_DOUBLE
    A = lib().gb300_allocate_sparse(n, ncol, nz, 1, 1, stype, CHOLMOD_REAL + dt, common.ptr)
    if not A:
        raise RuntimeError(f"allocate_sparse failed, status {common.status}")
    a = A.contents
    _arr(a.p, np.int64, ncol + 1)[:] = Ap
    _arr(a.i, np.int64, max(nz, 1))[:nz] = Ai
    _arr(a.x, np.float32 if dtype == "s" else np.float64, max(nz, 1))[:nz] = Ax
    return A


def csparse(n, Ap, Ai, Ax, common, stype=-1, dtype="d", ncol=None, zomplex=False):
    """A complex cholmod_sparse ((re, im) pairs; separate re and im arrays
    when zomplex) from CSC arrays with complex values."""
    ncol = n if ncol is None else ncol
    nz = int(Ap[-1])
    dt = CHOLMOD_SINGLE if dtype == "s" else CHOLMOD_DOUBLE
    xt = CHOLMOD_ZOMPLEX if zomplex else CHOLMOD_COMPLEX
    A = lib().gb300_allocate_sparse(n, ncol, nz, 1, 1, stype, xt + dt, common.ptr)
    if not A:
        raise RuntimeError(f"allocate_sparse failed, status {common.status}")
    a = A.contents
    _arr(a.p, np.int64, ncol + 1)[:] = Ap
    _arr(a.i, np.int64, max(nz, 1))[:nz] = Ai
    rdt = np.float32 if dtype == "s" else np.float64
    Ax = np.asarray(Ax)
    if zomplex:
        _arr(a.x, rdt, max(nz, 1))[:nz] = Ax.real
        _arr(a.z, rdt, max(nz, 1))[:nz] = Ax.imag
    else:
        v = _arr(a.x, rdt, 2 * max(nz, 1))
        v[0:2 * nz:2] = Ax.real
        v[1:2 * nz:2] = Ax.imag
    return A


def cdense(X, common, dtype="d"):
    """A complex cholmod_dense ((re, im) pairs) holding X (n x k)."""
    X = np.asarray(X)
    if X.ndim == 1:
        X = X[:, None]
    n, k = X.shape
    dt = CHOLMOD_SINGLE if dtype == "s" else CHOLMOD_DOUBLE
    D = lib().gb300_allocate_dense(n, k, n, CHOLMOD_COMPLEX + dt, common.ptr)
    if not D:
        raise RuntimeError(f"allocate_dense failed, status {common.status}")
    v = _arr(D.contents.x, np.float32 if dtype == "s" else np.float64, 2 * max(n * k, 1))
    flat = X.T.ravel()
    v[0:2 * n * k:2] = flat.real
    v[1:2 * n * k:2] = flat.imag
    return D


def cdense_array(D):
    d = D.contents
    dt = np.float32 if d.dtype == CHOLMOD_SINGLE else np.float64
    v = _arr(d.x, dt, 2 * d.d * d.ncol)
    z = (v[0::2] + 1j * v[1::2]).reshape(d.ncol, d.d)[:, :d.nrow].T.copy()
    return z


def super_solve(L, X, common, forward, dtype="d"):
    """cholmod_l_super_lsolve (forward) or _ltsolve on a copy of X (real or
    complex, n x k); returns (ok, solution)."""
    X = np.asarray(X)
    cx = np.iscomplexobj(X)
    k = 1 if X.ndim == 1 else X.shape[1]
    D = cdense(X, common, dtype) if cx else dense(X, common, dtype)
    dt = CHOLMOD_SINGLE if dtype == "s" else CHOLMOD_DOUBLE
    me = max(int(L.contents.maxesize), 1)
    E = lib().gb300_allocate_dense(me, k, me, (CHOLMOD_COMPLEX if cx else CHOLMOD_REAL) + dt,
                                   common.ptr)
    fn = lib().cholmod_l_super_lsolve if forward else lib().cholmod_l_super_ltsolve
    ok = fn(L, D, E, common.ptr)
    out = cdense_array(D) if cx else dense_array(D)
    free_dense(D, common)
    free_dense(E, common)
    return ok, out


def free_sparse(A, common):
    lib().gb300_free_sparse(C.byref(A), common.ptr)


def dense(X, common, dtype="d"):
    X = np.asarray(X)
    if X.ndim == 1:
        X = X[:, None]
    n, k = X.shape
    dt = CHOLMOD_SINGLE if dtype == "s" else CHOLMOD_DOUBLE
    D = lib().gb300_allocate_dense(n, k, n, CHOLMOD_REAL + dt, common.ptr)
    if not D:
        raise RuntimeError(f"allocate_dense failed, status {common.status}")
    _arr(D.contents.x, np.float32 if dtype == "s" else np.float64, max(n * k, 1))[:n * k] = \
        X.T.ravel()
    return D


def dense_array(D):
    d = D.contents
    dt = np.float32 if d.dtype == CHOLMOD_SINGLE else np.float64
    a = _arr(d.x, dt, d.d * d.ncol).reshape(d.ncol, d.d)[:, :d.nrow].T.copy()
    return a


def free_dense(D, common):
    lib().gb300_free_dense(C.byref(D), common.ptr)


def analyze_perm(A, perm, common):
    perm = np.ascontiguousarray(perm, dtype=np.int64)
    L = lib().gb300_analyze_perm(A, perm.ctypes.data_as(C.POINTER(C.c_int64)), common.ptr)
    if not L:
        raise RuntimeError(f"analyze failed, status {common.status}")
    return L


def factor_arrays(L, with_x=True):
    """numpy copies of the supernodal fields of a cholmod_factor."""
    f = L.contents
    ns = f.nsuper
    out = {
        "n": f.n, "minor": f.minor, "nsuper": ns, "ssize": f.ssize, "xsize": f.xsize,
        "maxcsize": f.maxcsize, "maxesize": f.maxesize, "is_super": f.is_super,
        "xtype": f.xtype, "dtype": f.dtype,
        "Perm": _arr(f.Perm, np.int64, f.n).copy(),
        "ColCount": _arr(f.ColCount, np.int64, f.n).copy(),
        "Super": _arr(f.super, np.int64, ns + 1).copy(),
        "Pi": _arr(f.pi, np.int64, ns + 1).copy(),
        "Px": _arr(f.px, np.int64, ns + 1).copy(),
        "Ls": _arr(f.s, np.int64, f.ssize).copy(),
    }
    if with_x and f.x:
        dt = np.float32 if f.dtype == CHOLMOD_SINGLE else np.float64
        if f.xtype == CHOLMOD_COMPLEX:
            v = _arr(f.x, dt, 2 * f.xsize)
            out["Lx"] = (v[0::2] + 1j * v[1::2]).astype(np.complex64 if dt == np.float32
                                                        else np.complex128)
        else:
            out["Lx"] = _arr(f.x, dt, f.xsize).copy()
    return out


def rcond(L, common):
    """cholmod_l_rcond: (min L(j,j) / max L(j,j))^2 of an LL' factor."""
    return lib().cholmod_l_rcond(L, common.ptr)


def free_factor(L, common):
    lib().gb300_free_factor(C.byref(L), common.ptr)


def super_numeric(S, L, common, beta=0.0, F=None, beta_im=0.0):
    b = (C.c_double * 2)(beta, beta_im)
    return lib().cholmod_l_super_numeric(S, F, b, L, common.ptr)


def factorize(A, L, common, beta=0.0):
    b = (C.c_double * 2)(beta, 0.0)
    return lib().gb300_factorize(A, b, L, common.ptr)


def sparse_arrays(A):
    """numpy copies (p, i, x) of a packed cholmod_sparse."""
    a = A.contents
    nz = int(_arr(a.p, np.int64, a.ncol + 1)[a.ncol]) if a.ncol >= 0 else 0
    dt = np.float32 if a.dtype == CHOLMOD_SINGLE else np.float64
    return (_arr(a.p, np.int64, a.ncol + 1).copy(), _arr(a.i, np.int64, nz).copy(),
            _arr(a.x, dt, nz).copy())


def spsolve(L, n, Bp, Bi, Bx, common, sys=None, dtype="d"):
    """cholmod_l_spsolve: X = A\\B for a sparse B given in CSC form; returns
    (Xp, Xi, Xx, nzmax) of the sparse solution."""
    sys = CHOLMOD_A if sys is None else sys
    ncol = len(Bp) - 1
    B = sparse(n, Bp, Bi, Bx, common, stype=0, dtype=dtype, ncol=ncol)
    X = lib().cholmod_l_spsolve(sys, L, B, common.ptr)
    free_sparse(B, common)
    if not X:
        raise RuntimeError(f"spsolve failed, status {common.status}")
    out = sparse_arrays(X) + (int(X.contents.nzmax),)
    free_sparse(X, common)
    return out


def solve(L, B, common, dtype="d", sys=None):
    sys = CHOLMOD_A if sys is None else sys
    Bd = dense(B, common, dtype)
    X = lib().gb300_solve(sys, L, Bd, common.ptr)
    free_dense(Bd, common)
    if not X:
        raise RuntimeError(f"solve failed, status {common.status}")
    out = dense_array(X)
    free_dense(X, common)
    return out


def factor_info(L, common):
    out = (C.c_double * 10)()
    if not lib().gb300_factor_info(L, common.ptr, out, 10):
        raise RuntimeError(f"factor_info failed, status {common.status}")
    keys = ["fl_taskgraph", "nlevels", "launches_factor", "cb_entries", "gemm_tasks", "nsuper",
            "launches_fwd", "launches_bwd", "cbv_entries", "mixed"]
    return dict(zip(keys, list(out)))


def fma_peak(dtype="d"):
    out = C.c_double(0)
    ok = lib().gb300_fma_peak(4 if dtype == "s" else 0, C.byref(out))
    return out.value if ok else None


def batch_analyze(Lpats, sys_pat, common):
    """Symbolic factor of the block-diagonal batch whose system i has the
    pattern Lpats[sys_pat[i]] (gb300_batch_analyze)."""
    arr = (FP * len(Lpats))(*Lpats)
    sp = np.ascontiguousarray(sys_pat, dtype=np.int32)
    L = lib().gb300_batch_analyze(len(Lpats), arr, len(sp),
                                   sp.ctypes.data_as(C.POINTER(C.c_int32)), common.ptr)
    if not L:
        raise RuntimeError(f"batch analyze failed, status {common.status}")
    return L


def factorize_mixed(A, L, common):
    return lib().gb300_factorize_mixed(A, L, common.ptr)


def solve_refined(A, L, B, common, tol=1e-12):
    Bd = dense(B, common)
    info = (C.c_double * 4)()
    X = lib().gb300_solve_refined(A, L, Bd, tol, info, common.ptr)
    free_dense(Bd, common)
    if not X:
        raise RuntimeError(f"refined solve failed, status {common.status}")
    out = dense_array(X)
    free_dense(X, common)
    return out, {"iterations": int(info[0]), "berr": info[1], "fp64_fallback": bool(info[2]),
                 "status": common.status}


def mixed_reason(L, common):
    """Why the mixed factor is in FP64 (GB300_REASON_*), -1 without one."""
    return lib().gb300_mixed_reason(L, common.ptr)
