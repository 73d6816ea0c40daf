"""Run the reference CHOLMOD (oracle/_ref/ref_dump) on a matrix, here only.

Test infrastructure: used by tests/golden/make_golden.py to produce fixtures
and by the reference-parity tests when oracle/_ref has been built.  Never
imported by the product.
"""
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DUMP = os.path.join(HERE, "_ref", "ref_dump")


def available():
    return os.path.exists(REF_DUMP) and os.access(REF_DUMP, os.X_OK)


def run(n, Ap, Ai, Ax, ordering="amd", dtype="d", B=None, perm=None, trials=1,
        env=None):
    """Analyze + factorize (+ solve if B) with the reference; returns a dict."""
    with tempfile.TemporaryDirectory() as d:
        nrhs = 0 if B is None else (1 if B.ndim == 1 else B.shape[1])
        with open(os.path.join(d, "meta.txt"), "w") as f:
            f.write(f"{n} {len(Ai)} {nrhs}\n")
        np.asarray(Ap, np.int64).tofile(os.path.join(d, "Ap.bin"))
        np.asarray(Ai, np.int64).tofile(os.path.join(d, "Ai.bin"))
        np.asarray(Ax, np.float64).tofile(os.path.join(d, "Ax.bin"))
        if B is not None:
            np.asarray(B, np.float64).reshape(n, -1).T.copy().tofile(
                os.path.join(d, "B.bin"))
        if perm is not None:
            np.asarray(perm, np.int64).tofile(os.path.join(d, "UserPerm.bin"))
        subprocess.run([REF_DUMP, d, ordering, dtype, str(trials)], check=True,
                       env=env)
        out = {}
        with open(os.path.join(d, "out_meta.txt")) as f:
            for line in f:
                k, v = line.split()
                out[k] = float(v) if any(c in v for c in ".e") else int(v)

        def rd(name, dt):
            p = os.path.join(d, name)
            return np.fromfile(p, dtype=dt) if os.path.exists(p) else None

        for name in ("Perm", "ColCount", "Super", "Pi", "Px", "Ls"):
            out[name] = rd(name + ".bin", np.int64)
        out["Lx"] = rd("Lx.bin", np.float64)
        X = rd("X.bin", np.float64)
        if X is not None:
            out["X"] = X.reshape(-1, n).T.copy()
        return out
