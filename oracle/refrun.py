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
        env=None, SB=None):
    """Analyze + factorize (+ solve if B) with the reference; returns a dict.
    SB = (Bp, Bi, Bx) of a sparse right-hand side: out["SX"][sys] =
    (Xp, Xi, Xx, nzmax) of cholmod_l_spsolve(sys) for sys = 0..8.  A complex
    Ax (and B) runs the complex factorization: out["Lx"] and out["X"] are
    complex then."""
    cx = np.iscomplexobj(Ax)
    if cx:
        env = dict(env if env is not None else os.environ, REF_COMPLEX="1")
    with tempfile.TemporaryDirectory() as d:
        nrhs = 0 if B is None else (1 if B.ndim == 1 else B.shape[1])
        sncol = 0 if SB is None else len(SB[0]) - 1
        with open(os.path.join(d, "meta.txt"), "w") as f:
            f.write(f"{n} {len(Ai)} {nrhs} {sncol}\n")
        if SB is not None:
            for name, a, dt in zip(("SBp", "SBi", "SBx"), SB, (np.int64, np.int64, np.float64)):
                np.asarray(a, dt).tofile(os.path.join(d, name + ".bin"))
        np.asarray(Ap, np.int64).tofile(os.path.join(d, "Ap.bin"))
        np.asarray(Ai, np.int64).tofile(os.path.join(d, "Ai.bin"))
        np.asarray(np.real(Ax), np.float64).tofile(os.path.join(d, "Ax.bin"))
        if cx:
            np.asarray(np.imag(Ax), np.float64).tofile(os.path.join(d, "Az.bin"))
        if B is not None:
            Bm = np.asarray(B).reshape(n, -1)
            np.asarray(np.real(Bm), np.float64).T.copy().tofile(os.path.join(d, "B.bin"))
            if cx:
                np.asarray(np.imag(Bm), np.float64).T.copy().tofile(os.path.join(d, "Bz.bin"))
        if perm is not None:
            np.asarray(perm, np.int64).tofile(os.path.join(d, "UserPerm.bin"))
        subprocess.run([REF_DUMP, d, ordering, dtype, str(trials)], check=True,
                       env=env)
        out = {}
        with open(os.path.join(d, "out_meta.txt")) as f:
            for line in f:
                k, v = line.split()
                if "," in v:
                    out[k] = [int(t) for t in v.split(",")]
                else:
                    out[k] = float(v) if any(c in v for c in ".e") else int(v)

        def rd(name, dt):
            p = os.path.join(d, name)
            return np.fromfile(p, dtype=dt) if os.path.exists(p) else None

        for name in ("Perm", "ColCount", "Super", "Pi", "Px", "Ls", "Lp", "Lnz", "Li"):
            out[name] = rd(name + ".bin", np.int64)
        out["SLx"] = rd("SLx.bin", np.float64)
        out["Lx"] = rd("Lx.bin", np.float64)
        if sncol:
            out["SX"] = {}
            for sys in range(9):
                xp = rd(f"SX{sys}p.bin", np.int64)
                if xp is not None:
                    out["SX"][sys] = (xp, rd(f"SX{sys}i.bin", np.int64),
                                      rd(f"SX{sys}x.bin", np.float64), out["spnzmax"][sys])
        X = rd("X.bin", np.float64)
        if cx:
            if out["Lx"] is not None:
                out["Lx"] = out["Lx"][0::2] + 1j * out["Lx"][1::2]
            if X is not None:
                X = X[0::2] + 1j * X[1::2]
        if X is not None:
            out["X"] = X.reshape(-1, n).T.copy()
        return out
