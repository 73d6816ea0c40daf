"""The selectable execution paths give the oracle's factor and solutions:
the per-level factorization (GB300_OPT_FACTOR = 0: one assembly launch, one
narrow-supernode launch and one tile task-graph launch per etree level) and
the per-level sweeps (GB300_OPT_SWEEP = 0), in FP64 and in the mixed form,
against the default single-launch paths."""
import numpy as np
import pytest

from conftest import make_case
from suitesparse_gb300 import cholmod as CH
from suitesparse_gb300 import matrices as M

pytestmark = pytest.mark.gpu
L_TOL = 1e-10


def _factor(meta, arrays, name, opts):
    n, Ap, Ai, Ax = make_case(meta, name)
    c = CH.Common()
    for k, v in opts.items():
        assert c.set_option(k, v)
    A = CH.sparse(n, Ap, Ai, Ax, c)
    L = CH.analyze_perm(A, arrays[name + "_Perm"].astype(np.int64), c)
    assert CH.factorize(A, L, c) == 1 and c.status == CH.CHOLMOD_OK
    f = CH.factor_arrays(L)
    B = M.rhs(n, 3, 17)
    X = CH.solve(L, B, c)
    assert CH.factorize_mixed(A, L, c) == 1
    Xm, info = CH.solve_refined(A, L, B, c, tol=1e-12)
    CH.free_factor(L, c)
    CH.free_sparse(A, c)
    return (n, Ap, Ai, Ax), f, B, X, Xm, info


@pytest.mark.parametrize("name", ["g3", "e27", "c1"])
@pytest.mark.parametrize("factor_mode,sweep_mode", [(0, 1), (1, 0), (0, 0)])
def test_per_level_paths_match(golden, lib, oracle_mod, name, factor_mode, sweep_mode):
    meta, arrays = golden
    mat, f, B, X, Xm, info = _factor(meta, arrays, name, {CH.GB300_OPT_FACTOR: factor_mode,
                                                           CH.GB300_OPT_SWEEP: sweep_mode})
    _, f1, _, X1, _, _ = _factor(meta, arrays, name, {})
    err = np.linalg.norm(f["Lx"] - f1["Lx"]) / np.linalg.norm(f1["Lx"])
    assert err <= L_TOL, err
    assert oracle_mod.backward_error(*mat, X, B).max() <= 1e-14
    assert np.abs(X - X1).max() <= 1e-10 * np.abs(X1).max()
    assert info["berr"] <= 1e-12
    assert oracle_mod.backward_error(*mat, Xm, B).max() <= 1e-12
