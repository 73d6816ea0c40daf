"""Fixture: the reference CHOLMOD's cholmod_l_spsolve, for every sys value,
on sparse right-hand sides of three golden cases (tests/golden/spsolve.npz),
produced by running the reference (oracle/refrun.py, built from the reference
sources by oracle/build_ref.py) with the golden orderings.  Each B has an
empty column, a column with a row index given twice (the last entry counts)
and an explicit zero, a column on the last row only, and a fuller column.
Run here, where the reference sources are; the fixture travels with the
tests."""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import numpy as np  # noqa: E402

from oracle import refrun  # noqa: E402
from conftest import make_case  # noqa: E402

CASES = ("g3a", "e27", "g2c")


def sparse_rhs(n, seed):
    """Columns: one entry; empty; rows {a, b, a} with the second a-entry and
    an explicit zero; the last row; five entries; about n/10 entries."""
    rng = np.random.default_rng(seed)
    cols = []
    cols.append(([int(rng.integers(n))], [1.0]))
    cols.append(([], []))
    a, b = (int(v) for v in rng.choice(n, 2, replace=False))
    cols.append(([a, b, a, (a + 1) % n], [2.0, -1.5, 3.25, 0.0]))
    cols.append(([n - 1], [-4.0]))
    r = rng.choice(n, 5, replace=False)
    cols.append((list(r), list(rng.standard_normal(5))))
    r = np.sort(rng.choice(n, max(n // 10, 1), replace=False))
    cols.append((list(r), list(rng.uniform(-1, 1, len(r)))))
    Bp = np.zeros(len(cols) + 1, np.int64)
    Bi, Bx = [], []
    for j, (ri, rx) in enumerate(cols):
        Bi += [int(v) for v in ri]
        Bx += [float(v) for v in rx]
        Bp[j + 1] = len(Bi)
    return Bp, np.array(Bi, np.int64), np.array(Bx, np.float64)


def main():
    if not refrun.available():
        raise SystemExit("the reference runner is not built (oracle/build_ref.py)")
    here = os.path.dirname(os.path.abspath(__file__))
    meta = json.load(open(os.path.join(here, "golden.json")))
    arrays = np.load(os.path.join(here, "golden_arrays.npz"))
    out = {}
    for k, name in enumerate(CASES):
        n, Ap, Ai, Ax = make_case(meta, name)
        perm = arrays[name + "_Perm"].astype(np.int64)
        Bp, Bi, Bx = sparse_rhs(n, 100 + k)
        r = refrun.run(n, Ap, Ai, Ax, "given", "d", perm=perm, SB=(Bp, Bi, Bx))
        out[f"{name}_Bp"], out[f"{name}_Bi"], out[f"{name}_Bx"] = Bp, Bi, Bx
        for sys_, (xp, xi, xx, nzmax) in sorted(r["SX"].items()):
            out[f"{name}_{sys_}_Xp"] = xp
            out[f"{name}_{sys_}_Xi"] = xi.astype(np.int32)
            out[f"{name}_{sys_}_Xx"] = xx
            out[f"{name}_{sys_}_nzmax"] = np.array([nzmax], np.int64)
            print(name, sys_, "nnz(X) =", int(xp[-1]), "nzmax =", nzmax, flush=True)
    np.savez_compressed(os.path.join(here, "spsolve.npz"), **out)


if __name__ == "__main__":
    main()
