"""Generate the golden fixtures from the reference CHOLMOD (run here only).

Needs oracle/_ref (python oracle/build_ref.py, which compiles the reference
sources found by oracle/build_ref.py reference_root()).  For every case it
records what the
reference's cholmod_l_analyze / cholmod_l_factorize / cholmod_l_solve
produce on the seeded matrix of suitesparse_gb300.matrices:

  golden.json        per case: generator spec, SHA-256 of the generated
                     matrix (cross-machine determinism check), fl, lnz, anz,
                     nsuper, xsize, maxcsize, maxesize, minor, status,
                     SHA-256 of the supernodal pattern (super, pi, px, s),
                     Frobenius norm of L, backward error of the solve
  golden_arrays.npz  the final permutation and the supernode partition
                     L->super of every case (int32); for the small cases
                     also L->x (double and single) and X

Usage: python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from suitesparse_gb300 import matrices as M  # noqa: E402
from oracle import refrun  # noqa: E402

# name: (generator, kwargs, ordering, store full L/X, nrhs)
CASES = {
    "g2c": ("laplace2d", dict(nx=30, shift=1e-3), "amd", True, 2),
    "g2v": ("laplace2d", dict(nx=40, ny=33, seed=7), "amd", True, 3),
    "g3": ("laplace3d", dict(nx=12, seed=5), "metis", True, 3),
    "g3a": ("laplace3d", dict(nx=9, ny=7, nz=5, seed=6), "amd", True, 1),
    "e27": ("elastic27", dict(m=6, seed=2), "metis", True, 2),
    "npd": ("laplace2d", dict(nx=20, seed=7, shift=-0.35), "amd", True, 0),
    "c1": ("laplace2d", dict(nx=100, shift=1e-3), "amd", False, 1),
    "c2": ("laplace3d", dict(nx=64, seed=1), "metis", False, 1),
    "c3": ("elastic27", dict(m=40, seed=2), "metis", False, 1),
}
for _i, _side in enumerate(M.batch_sides()):
    CASES[f"c4_{_side}"] = ("batch", dict(index=_i, side=_side), "amd", False, 4)


def generate(kind, kw):
    if kind == "batch":
        return M.batch_system(kw["index"], kw["side"])
    return getattr(M, kind)(**kw)


def main(only=None):
    if not refrun.available():
        print("oracle/_ref/ref_dump missing: run python oracle/build_ref.py first")
        return 1
    meta_path = os.path.join(HERE, "golden.json")
    arr_path = os.path.join(HERE, "golden_arrays.npz")
    meta = json.load(open(meta_path)) if (only and os.path.exists(meta_path)) else {}
    arrays = dict(np.load(arr_path)) if (only and os.path.exists(arr_path)) else {}
    for name, (kind, kw, ordering, full, nrhs) in CASES.items():
        if only and name not in only:
            continue
        n, Ap, Ai, Ax = generate(kind, kw)
        B = M.rhs(n, nrhs, 100 + len(name)) if nrhs else None
        r = refrun.run(n, Ap, Ai, Ax, ordering, "d", B=B)
        rec = {
            "kind": kind, "kwargs": kw, "ordering": ordering, "nrhs": nrhs,
            "rhs_seed": 100 + len(name), "n": n, "nnz_lower": int(Ap[-1]),
            "matrix_sha256": M.digest(Ap, Ai, Ax),
            "pattern_sha256": M.digest(r["Super"], r["Pi"], r["Px"], r["Ls"]),
            "colcount_sha256": M.digest(r["ColCount"]),
        }
        for k in ("nsuper", "ssize", "xsize", "maxcsize", "maxesize", "minor", "status",
                  "factor_status"):
            rec[k] = int(r[k])
        for k in ("fl", "lnz", "anz", "resid", "t_factor", "t_analyze"):
            rec[k] = float(r[k])
        rec["L_fro"] = float(np.linalg.norm(r["Lx"]))
        arrays[name + "_Perm"] = r["Perm"].astype(np.int32)
        arrays[name + "_Super"] = r["Super"].astype(np.int32)
        if full:
            arrays[name + "_Lx"] = r["Lx"]
            rs = refrun.run(n, Ap, Ai, Ax, ordering, "s", B=B)
            arrays[name + "_Lxs"] = rs["Lx"].astype(np.float32)
            rec["minor_single"] = int(rs["minor"])
            if B is not None and "X" in r:
                arrays[name + "_X"] = r["X"]
                if "X" in rs:
                    arrays[name + "_Xs"] = rs["X"].astype(np.float32)
        elif name == "c1":
            arrays[name + "_X"] = r["X"]
        meta[name] = rec
        print(name, n, rec["nsuper"], rec["fl"], rec["minor"], rec["resid"], flush=True)
    with open(meta_path, "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)
    np.savez_compressed(arr_path, **arrays)
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:] or None))
