"""The seeded matrices are the ones the golden fixtures were made from
(bit-identical bytes on every machine)."""
import pytest

from conftest import make_case
from suitesparse_gb300 import matrices as M

SMALL = ["g2c", "g2v", "g3", "g3a", "e27", "npd", "c1", "c2"]


@pytest.mark.parametrize("name", SMALL)
def test_matrix_digest(golden, name):
    meta, _ = golden
    n, Ap, Ai, Ax = make_case(meta, name)
    assert n == meta[name]["n"]
    assert int(Ap[-1]) == meta[name]["nnz_lower"]
    assert M.digest(Ap, Ai, Ax) == meta[name]["matrix_sha256"]


def test_batch_digests(golden):
    meta, _ = golden
    for name in [k for k in meta if k.startswith("c4_")]:
        n, Ap, Ai, Ax = make_case(meta, name)
        assert M.digest(Ap, Ai, Ax) == meta[name]["matrix_sha256"], name


def test_c3_sizes(golden):
    meta, _ = golden
    n, Ap, Ai, Ax = make_case(meta, "c3")
    assert n == 192000 and 2 * int(Ap[-1]) - n == 14787288
    assert M.digest(Ap, Ai, Ax) == meta["c3"]["matrix_sha256"]


def test_det_exp_log():
    import numpy as np
    x = np.linspace(-30, 30, 2001)
    assert np.max(np.abs(M.det_exp(x) / np.exp(x) - 1)) < 4e-16
    for v in (1e-2, 0.1, 3.0, 10.0, 1e2):
        assert abs(M.det_log(v) - np.log(v)) <= 2e-15 * max(1, abs(np.log(v)))
