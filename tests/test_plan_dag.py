"""The factorization's tile task graph (csrc/gb_plan.c) on the host: for
update groups 1-4 it is acyclic, and random topological executions of every
wide supernode's tile tasks (POTRF, TRSM, UPD, DIAG, update-block tiles) on
a dense SPD front reproduce the front's blocked Cholesky to rounding
(tests/plan_dag_check.c, compiled here with the library's host sources)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from suitesparse_gb300 import build as B
from suitesparse_gb300 import matrices as M

HERE = os.path.dirname(os.path.abspath(__file__))


def test_task_graph_executes_in_any_order(tmp_path):
    if not shutil.which("gcc"):
        pytest.skip("gcc not available")
    dims = (24, 24, 24)
    n, Ap, Ai, _ = M.laplace3d(*dims)
    perm = M.grid_nd_perm(dims)
    for name, a in (("Ap", Ap), ("Ai", Ai), ("perm", perm)):
        np.asarray(a, np.int64).tofile(str(tmp_path / f"{name}.bin"))
    csrc = B.CSRC
    exe = str(tmp_path / "plan_dag_check")
    cmd = ["gcc", "-O2", "-std=c11", "-D_GNU_SOURCE", "-w", "-I" + B.INCLUDE, "-I" + csrc,
           "-I" + os.path.join(B.cuda_home(), "include"), os.path.join(HERE, "plan_dag_check.c"),
           os.path.join(csrc, "gb_plan.c"), os.path.join(csrc, "gb_symbolic.c"),
           os.path.join(csrc, "gb_util.c"), "-L" + os.path.join(B.cuda_home(), "lib64"),
           "-Wl,-rpath," + os.path.join(B.cuda_home(), "lib64"), "-lcudart", "-lm", "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True)
    r = subprocess.run([exe] + [str(tmp_path / f"{k}.bin") for k in ("Ap", "Ai", "perm")],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout
    assert "DIAG" in r.stdout and " 0 DIAG" not in r.stdout
