"""Golden complex supernodal factors from the reference CHOLMOD (run here only).

Runs the reference's cholmod_l_analyze + cholmod_l_factorize + cholmod_l_solve
(supernodal, Common->supernodal = CHOLMOD_SUPERNODAL) on complex Hermitian
matrices through oracle/_ref/ref_dump (REF_COMPLEX=1), and records the
supernodal pattern, the complex values L->x, the solution X of a complex
right-hand side, L->minor and the status.  Matrices are
matrices.magnetic_laplacian grids (regenerated from their parameters by the
tests); the right-hand sides are matrices.rhs(n, k, seed) + i
matrices.rhs(n, k, seed + 1).

  complex.npz    <case>_{Perm,Super,Pi,Px,Ls,Lx,X}
  complex.json   <case>: dims, kwargs, ordering, dtype, nrhs, seed, n, minor,
                 factor_status, fl, lnz

Usage: python tests/golden/make_complex.py
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

# name: (dims, kwargs of magnetic_laplacian, ordering, dtype, nrhs)
CASES = {
    "cx2": ((30, 30), {"seed": 11}, "amd", "d", 3),
    "cx3": ((10, 10, 10), {"seed": 12}, "metis", "d", 2),
    "cxdiag": ((20, 24), {"seed": 13, "diag_imag": 0.37}, "amd", "d", 2),
    "cxnpd": ((16, 16), {"seed": 14, "shift": -0.6}, "amd", "d", 0),
    "cx2s": ((30, 30), {"seed": 11}, "amd", "s", 2),
}


def rhs(n, k, seed):
    return M.rhs(n, k, seed) + 1j * M.rhs(n, k, seed + 1)


def main():
    if not refrun.available():
        print("oracle/_ref/ref_dump missing: run python oracle/build_ref.py first")
        return 1
    arrays, out = {}, {}
    for name, (dims, kw, ordering, dtype, nrhs) in CASES.items():
        n, Ap, Ai, Ax = M.magnetic_laplacian(dims, **kw)
        seed = 50 + len(out)
        B = rhs(n, nrhs, seed) if nrhs else None
        r = refrun.run(n, Ap, Ai, Ax, ordering, dtype, B=B)
        for k in ("Perm", "Super", "Pi", "Px", "Ls"):
            arrays[f"{name}_{k}"] = r[k].astype(np.int64)
        arrays[f"{name}_Lx"] = r["Lx"]
        if nrhs:
            arrays[f"{name}_X"] = r["X"]
        out[name] = {"dims": list(dims), "kwargs": kw, "ordering": ordering, "dtype": dtype,
                     "nrhs": nrhs, "seed": seed, "n": n, "minor": int(r["minor"]),
                     "factor_status": int(r["factor_status"]), "fl": r["fl"], "lnz": r["lnz"],
                     "nsuper": int(r["nsuper"])}
        print(name, out[name], flush=True)
    with open(os.path.join(HERE, "complex.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    np.savez_compressed(os.path.join(HERE, "complex.npz"), **arrays)
    return 0


if __name__ == "__main__":
    sys.exit(main())
