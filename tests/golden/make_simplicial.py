"""Golden simplicial factors from the reference CHOLMOD (run here only).

Runs the reference's cholmod_l_analyze + cholmod_l_factorize with the
simplicial method (Common->supernodal = CHOLMOD_SIMPLICIAL, final_ll 1 and
0: LL' and LDL') through oracle/_ref/ref_dump (REF_SIMPLICIAL=ll|ldl), for
a few cases of golden.json, and records the factor exactly as the
reference lays it out: Perm, ColCount, Lp, Lnz, Li (first Lp[n] entries),
the values Lx, L->minor and the status.

  simplicial.npz    <case>_<ll|ldl>_{Perm,ColCount,Lp,Lnz,Li,Lx}
  simplicial.json   <case>_<ll|ldl>: n, nzmax, minor, factor_status

Usage: python tests/golden/make_simplicial.py
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

CASES = ["g2c", "g2v", "g3", "e27", "npd", "c4_21"]


def main():
    if not refrun.available():
        print("oracle/_ref/ref_dump missing: run python oracle/build_ref.py first")
        return 1
    meta = json.load(open(os.path.join(HERE, "golden.json")))
    arrays, out = {}, {}
    for name in CASES:
        rec = meta[name]
        kw = rec["kwargs"]
        if rec["kind"] == "batch":
            n, Ap, Ai, Ax = M.batch_system(kw["index"], kw["side"])
        else:
            n, Ap, Ai, Ax = getattr(M, rec["kind"])(**kw)
        for form in ("ll", "ldl"):
            env = dict(os.environ, REF_SIMPLICIAL=form)
            r = refrun.run(n, Ap, Ai, Ax, rec["ordering"], "d", env=env)
            key = f"{name}_{form}"
            lp = r["Lp"]
            nnz = int(lp[-1])
            arrays[key + "_Perm"] = r["Perm"].astype(np.int32)
            arrays[key + "_ColCount"] = r["ColCount"].astype(np.int32)
            arrays[key + "_Lp"] = lp.astype(np.int64)
            arrays[key + "_Lnz"] = r["Lnz"].astype(np.int32)
            arrays[key + "_Li"] = r["Li"][:nnz].astype(np.int32)
            arrays[key + "_Lx"] = r["SLx"][:nnz]
            out[key] = {"n": n, "nzmax": int(r["nzmax"]), "minor": int(r["minor"]),
                        "factor_status": int(r["factor_status"]), "is_ll": int(r["is_ll"])}
            print(key, n, nnz, out[key], flush=True)
    with open(os.path.join(HERE, "simplicial.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    np.savez_compressed(os.path.join(HERE, "simplicial.npz"), **arrays)
    return 0


if __name__ == "__main__":
    sys.exit(main())
