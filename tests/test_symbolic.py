"""Host supernodal symbolic analysis reproduces the reference's L pattern
bit-exactly (given the reference's final permutation)."""
import numpy as np
import pytest

from conftest import make_case
from suitesparse_gb300 import cholmod as CH
from suitesparse_gb300 import matrices as M

CASES = ["g2c", "g2v", "g3", "g3a", "e27", "npd", "c1", "c2"]


def analyze(meta, arrays, name, common):
    n, Ap, Ai, Ax = make_case(meta, name)
    A = CH.sparse(n, Ap, Ai, Ax, common)
    L = CH.analyze_perm(A, arrays[name + "_Perm"].astype(np.int64), common)
    return A, L


@pytest.mark.parametrize("name", CASES)
def test_pattern_matches_reference(golden, lib, name):
    meta, arrays = golden
    rec = meta[name]
    c = CH.Common()
    A, L = analyze(meta, arrays, name, c)
    f = CH.factor_arrays(L, with_x=False)
    assert M.digest(f["Super"], f["Pi"], f["Px"], f["Ls"]) == rec["pattern_sha256"]
    assert M.digest(f["ColCount"]) == rec["colcount_sha256"]
    for k in ("nsuper", "ssize", "xsize", "maxcsize", "maxesize"):
        assert f[k] == rec[k], k
    assert c["fl"] == rec["fl"] and c["lnz"] == rec["lnz"] and c["anz"] == rec["anz"]
    assert np.array_equal(f["Perm"], arrays[name + "_Perm"])
    assert f["is_super"] == 1 and f["xtype"] == CH.CHOLMOD_PATTERN
    CH.free_factor(L, c)
    CH.free_sparse(A, c)
    assert c["malloc_count"] == 0 and c["memory_inuse"] == 0


def test_batch_patterns(golden, lib):
    meta, arrays = golden
    c = CH.Common()
    for name in [k for k in meta if k.startswith("c4_")]:
        A, L = analyze(meta, arrays, name, c)
        f = CH.factor_arrays(L, with_x=False)
        assert M.digest(f["Super"], f["Pi"], f["Px"], f["Ls"]) == meta[name]["pattern_sha256"]
        assert c["fl"] == meta[name]["fl"]
        CH.free_factor(L, c)
        CH.free_sparse(A, c)


def test_c3_pattern(golden, lib):
    meta, arrays = golden
    c = CH.Common()
    A, L = analyze(meta, arrays, "c3", c)
    f = CH.factor_arrays(L, with_x=False)
    assert M.digest(f["Super"], f["Pi"], f["Px"], f["Ls"]) == meta["c3"]["pattern_sha256"]
    assert c["fl"] == meta["c3"]["fl"]
    CH.free_factor(L, c)
    CH.free_sparse(A, c)


def test_identity_and_trivial(lib):
    c = CH.Common()
    # 1x1 and diagonal matrices
    for n in (1, 7):
        Ap = np.arange(n + 1, dtype=np.int64)
        Ai = np.arange(n, dtype=np.int64)
        A = CH.sparse(n, Ap, Ai, np.full(n, 2.0), c)
        L = CH.analyze_perm(A, np.arange(n), c)
        f = CH.factor_arrays(L, with_x=False)
        assert f["nsuper"] >= 1 and f["Super"][-1] == n and f["Pi"][-1] == n
        CH.free_factor(L, c)
        CH.free_sparse(A, c)


def test_invalid_permutation(lib):
    c = CH.Common()
    n, Ap, Ai, Ax = M.laplace2d(5)
    A = CH.sparse(n, Ap, Ai, Ax, c)
    bad = np.arange(n)
    bad[3] = 4
    with pytest.raises(RuntimeError):
        CH.analyze_perm(A, bad, c)
    assert c.status == CH.CHOLMOD_INVALID
    CH.free_sparse(A, c)
