"""Edge shapes for the one-launch factorization and the sweeps, against the
oracle: a 1 x 1 system, a diagonal matrix (every supernode alone, no
children), dense matrices whose single front has exactly 32, 64 and 65 rows
(one-warp fronts of both sizes with no rows below the diagonal block, and
the whole-block path) and 200 rows (the tile path), and an arrow matrix
(one wide last column)."""
import numpy as np
import pytest

from suitesparse_gb300 import cholmod as CH
from suitesparse_gb300 import matrices as M

pytestmark = pytest.mark.gpu


def _lower_csc(D):
    n = D.shape[0]
    Ap, Ai, Ax = [0], [], []
    for j in range(n):
        rows = np.nonzero(D[j:, j])[0] + j
        Ai.extend(rows.tolist())
        Ax.extend(D[rows, j].tolist())
        Ap.append(len(Ai))
    return n, np.array(Ap, np.int64), np.array(Ai, np.int64), np.array(Ax, np.float64)


def _spd(kind, n, seed):
    rng = np.random.default_rng(seed)
    if kind == "diag":
        return np.diag(rng.uniform(1, 10, n))
    if kind == "arrow":
        D = np.diag(rng.uniform(n, 2 * n, n))
        D[-1, :-1] = D[:-1, -1] = rng.uniform(-1, 1, n - 1)
        return D
    G = rng.standard_normal((n, n))
    return G @ G.T + n * np.eye(n)


@pytest.mark.parametrize("kind,n", [("dense", 1), ("diag", 50), ("dense", 32), ("dense", 64),
                                    ("dense", 65), ("dense", 200), ("arrow", 300)])
def test_edge_shapes_match_oracle(lib, oracle_mod, kind, n):
    D = _spd(kind, n, n)
    n, Ap, Ai, Ax = _lower_csc(D)
    perm = np.arange(n, dtype=np.int64)
    c = CH.Common()
    A = CH.sparse(n, Ap, Ai, Ax, c)
    L = CH.analyze_perm(A, perm, c)
    assert CH.factorize(A, L, c) == 1 and c.status == CH.CHOLMOD_OK
    f = CH.factor_arrays(L)
    sym = {k: f[k] for k in ("Super", "Pi", "Px", "Ls")}
    sym["n"] = n
    Sp, Si, Sx = oracle_mod.permute_lower(n, Ap, Ai, Ax, perm)
    st, minor, Lref = oracle_mod.factor(sym, Sp, Si, Sx)
    assert st == 0
    assert np.linalg.norm(f["Lx"] - Lref) <= 1e-12 * np.linalg.norm(Lref)
    B = M.rhs(n, 2, 3)
    X = CH.solve(L, B, c)
    assert oracle_mod.backward_error(n, Ap, Ai, Ax, X, B).max() <= 1e-14
    assert CH.factorize_mixed(A, L, c) == 1
    Xm, info = CH.solve_refined(A, L, B, c, tol=1e-12)
    assert oracle_mod.backward_error(n, Ap, Ai, Ax, Xm, B).max() <= 1e-12
    CH.free_factor(L, c)
    CH.free_sparse(A, c)
