"""Fixture: the reference CHOLMOD's cholmod_l_rcond of the factors of the
golden cases (tests/golden/rcond.json), produced by running the reference
(oracle/refrun.py, built from the reference sources by oracle/build_ref.py)
on the same matrices and orderings as the golden fixtures.  Run here, where
the reference sources are; the fixture travels with the tests."""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import numpy as np  # noqa: E402

from oracle import refrun  # noqa: E402
from conftest import make_case  # noqa: E402

CASES = ("g2c", "g2v", "g3", "g3a", "e27", "c1", "npd")


def main():
    if not refrun.available():
        raise SystemExit("the reference runner is not built (oracle/build_ref.py)")
    here = os.path.dirname(os.path.abspath(__file__))
    meta = json.load(open(os.path.join(here, "golden.json")))
    arrays = np.load(os.path.join(here, "golden_arrays.npz"))
    out = {}
    for name in CASES:
        n, Ap, Ai, Ax = make_case(meta, name)
        perm = arrays[name + "_Perm"].astype(np.int64)
        r = refrun.run(n, Ap, Ai, Ax, "given", "d", perm=perm)
        out[name] = {"rcond": float(r["rcond"]), "minor": int(r["minor"])}
        print(name, out[name], flush=True)
    with open(os.path.join(here, "rcond.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
