"""The CPU oracle is pinned to the reference CHOLMOD's own outputs."""
import numpy as np
import pytest

from conftest import make_case

FULL = ["g2c", "g2v", "g3", "g3a", "e27"]


def sym_of(meta, arrays, name):
    """The reference's symbolic factor, rebuilt by the oracle from the
    reference's Perm and Super (fixtures): no product code involved."""
    from oracle import oracle as O
    n, Ap, Ai, Ax = make_case(meta, name)
    perm = arrays[name + "_Perm"].astype(np.int64)
    Sp, Si, _ = O.permute_lower(n, Ap, Ai, Ax, perm)
    return O.symbolic(n, Sp, Si, arrays[name + "_Super"]), (n, Ap, Ai, Ax)


ALL = ["g2c", "g2v", "g3", "g3a", "e27", "npd", "c1", "c2", "c3", "c4_21", "c4_25", "c4_26",
       "c4_33", "c4_65", "c4_67", "c4_72", "c4_87"]


@pytest.mark.parametrize("name", ALL)
def test_oracle_symbolic_is_the_references(golden, oracle_mod, name):
    """Pattern of L from S's pattern and the reference's supernode partition:
    the SHA-256 of (super, pi, px, s) equals the reference's own."""
    from suitesparse_gb300 import matrices as M
    meta, arrays = golden
    sym, _ = sym_of(meta, arrays, name)
    rec = meta[name]
    assert len(sym["Super"]) - 1 == rec["nsuper"] and len(sym["Ls"]) == rec["ssize"]
    assert int(sym["Px"][-1]) == rec["xsize"]
    assert M.digest(sym["Super"], sym["Pi"], sym["Px"], sym["Ls"]) == rec["pattern_sha256"]


@pytest.mark.parametrize("name", FULL)
@pytest.mark.parametrize("use_blas", [True, False])
def test_oracle_factor_matches_reference(golden, oracle_mod, name, use_blas):
    meta, arrays = golden
    sym, (n, Ap, Ai, Ax) = sym_of(meta, arrays, name)
    perm = arrays[name + "_Perm"].astype(np.int64)
    Sp, Si, Sx = oracle_mod.permute_lower(n, Ap, Ai, Ax, perm)
    st, minor, Lx = oracle_mod.factor(sym, Sp, Si, Sx, use_blas=use_blas)
    ref = arrays[name + "_Lx"]
    assert st == 0 and minor == n
    assert np.linalg.norm(Lx - ref) / np.linalg.norm(ref) < 1e-13
    # single precision restatement against the reference's single factor
    st, minor, Lxs = oracle_mod.factor(sym, Sp, Si, Sx.astype(np.float32), dtype="s",
                                       use_blas=use_blas)
    refs = arrays[name + "_Lxs"].astype(np.float64)
    assert np.linalg.norm(Lxs - refs) / np.linalg.norm(refs) < 1e-5


@pytest.mark.parametrize("name", FULL)
def test_oracle_solve_matches_reference(golden, oracle_mod, name):
    meta, arrays = golden
    from suitesparse_gb300 import matrices as M
    rec = meta[name]
    sym, (n, Ap, Ai, Ax) = sym_of(meta, arrays, name)
    perm = arrays[name + "_Perm"].astype(np.int64)
    B = M.rhs(n, rec["nrhs"], rec["rhs_seed"])
    X = oracle_mod.solve(sym, arrays[name + "_Lx"], perm, B)
    Xr = arrays[name + "_X"]
    assert np.abs(X - Xr).max() <= 1e-12 * np.abs(Xr).max()
    assert oracle_mod.backward_error(n, Ap, Ai, Ax, X, B).max() < 1e-14


def test_oracle_not_posdef(golden, oracle_mod):
    meta, arrays = golden
    rec = meta["npd"]
    sym, (n, Ap, Ai, Ax) = sym_of(meta, arrays, "npd")
    perm = arrays["npd_Perm"].astype(np.int64)
    Sp, Si, Sx = oracle_mod.permute_lower(n, Ap, Ai, Ax, perm)
    st, minor, Lx = oracle_mod.factor(sym, Sp, Si, Sx)
    ref = arrays["npd_Lx"]
    assert st == 1 and minor == rec["minor"] and rec["factor_status"] == 1
    assert np.linalg.norm(Lx - ref) <= 1e-13 * np.linalg.norm(ref)
    assert np.array_equal(Lx == 0, ref == 0)
    # quick return: the failing supernode is left all zero
    st, minor_q, Lxq = oracle_mod.factor(sym, Sp, Si, Sx, quick_return=True)
    s0 = np.searchsorted(sym["Super"], minor, side="right") - 1
    assert st == 1 and minor_q == minor
    assert np.all(Lxq[sym["Px"][s0]:] == 0)
    assert np.array_equal(Lxq[:sym["Px"][s0]], Lx[:sym["Px"][s0]])


def test_oracle_c1_solution(golden, oracle_mod):
    meta, arrays = golden
    from suitesparse_gb300 import matrices as M
    rec = meta["c1"]
    sym, (n, Ap, Ai, Ax) = sym_of(meta, arrays, "c1")
    perm = arrays["c1_Perm"].astype(np.int64)
    Sp, Si, Sx = oracle_mod.permute_lower(n, Ap, Ai, Ax, perm)
    st, minor, Lx = oracle_mod.factor(sym, Sp, Si, Sx)
    assert abs(np.linalg.norm(Lx) - rec["L_fro"]) <= 1e-12 * rec["L_fro"]
    B = M.rhs(n, 1, rec["rhs_seed"])
    X = oracle_mod.solve(sym, Lx, perm, B)
    assert np.abs(X - arrays["c1_X"]).max() <= 1e-12 * np.abs(arrays["c1_X"]).max()
