"""The drop-in binding: a program written against the reference CHOLMOD API,
linked against the reference library built from its sources, picks up this
library's cholmod_l_super_numeric by link order or LD_PRELOAD.

Runs where the reference sources and oracle/_ref exist (the machine that
builds the checker).  That machine has no GPU, so the interposed
cholmod_l_super_numeric answers CHOLMOD_GPU_PROBLEM: the status proves that
the reference's cholmod_l_factorize (CHOLMOD/Cholesky/cholmod_factorize.c:260)
called this library's entry point and not its own, which succeeds on the
CPU (the control run without this library)."""
import os
import subprocess
import tempfile

import pytest

from conftest import ROOT
from oracle.build_ref import reference_root

REF = reference_root()
REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libcholmod_ref.so")
GB_DIR = os.path.join(ROOT, "suitesparse_gb300")

pytestmark = pytest.mark.skipif(
    not (os.path.isdir(os.path.join(REF, "CHOLMOD")) and os.path.exists(REF_LIB)),
    reason="reference sources or oracle/_ref not present")


def _no_gpu():
    try:
        import torch
        return not torch.cuda.is_available()
    except ImportError:
        return True


def _build(d, libs):
    exe = os.path.join(d, "drv")
    subprocess.run(["gcc", "-O1", "-o", exe, os.path.join(ROOT, "tests", "interpose_driver.c"),
                    "-I" + os.path.join(REF, "CHOLMOD", "Include"),
                    "-I" + os.path.join(REF, "SuiteSparse_config")] + libs +
                   ["-Wl,-rpath," + GB_DIR, "-Wl,-rpath," + os.path.dirname(REF_LIB)],
                   check=True)
    return exe


def _run(exe, env=None, width="64", method="supernodal"):
    out = subprocess.run([exe, "20", width, method], capture_output=True, text=True, check=True,
                         env=env, timeout=120).stdout.split()
    return {out[i]: float(out[i + 1]) for i in range(0, len(out), 2)}


@pytest.mark.parametrize("width", ["64", "32"])
def test_reference_alone_factors_on_the_cpu(lib, width):
    with tempfile.TemporaryDirectory() as d:
        r = _run(_build(d, ["-L" + os.path.dirname(REF_LIB), "-lcholmod_ref"]), width=width)
    assert r["factorize_ok"] == 1 and r["status"] == 0 and r["is_super"] == 1
    assert r["minor"] == r["n"] and 0 <= r["resid"] < 1e-14


@pytest.mark.skipif(not _no_gpu(), reason="the proof by status needs a machine without a GPU")
@pytest.mark.parametrize("width", ["64", "32"])
def test_link_order_interposes_super_numeric(lib, width):
    with tempfile.TemporaryDirectory() as d:
        # --no-as-needed: the program names no symbol of this library itself,
        # and an as-needed link would drop it from the needed list
        exe = _build(d, ["-Wl,--no-as-needed", "-L" + GB_DIR, "-lcholmod_gb300",
                         "-L" + os.path.dirname(REF_LIB), "-lcholmod_ref"])
        r = _run(exe, width=width)
    assert r["status"] == -5 and r["factorize_ok"] == 0, r     # CHOLMOD_GPU_PROBLEM


@pytest.mark.skipif(not _no_gpu(), reason="the proof by status needs a machine without a GPU")
@pytest.mark.parametrize("width", ["64", "32"])
def test_ld_preload_interposes_super_numeric(lib, width):
    from suitesparse_gb300 import cholmod as CH
    with tempfile.TemporaryDirectory() as d:
        exe = _build(d, ["-L" + os.path.dirname(REF_LIB), "-lcholmod_ref"])
        env = dict(os.environ, LD_PRELOAD=CH.LIB_PATH)
        r = _run(exe, env=env, width=width)
    assert r["status"] == -5 and r["factorize_ok"] == 0, r


@pytest.mark.skipif(not _no_gpu(), reason="the proof by status needs a machine without a GPU")
def test_link_order_interposes_rowfac(lib):
    """The simplicial method: the reference's cholmod_l_factorize reaches
    cholmod_l_rowfac (Cholesky/cholmod_factorize.c:393) through its PLT."""
    with tempfile.TemporaryDirectory() as d:
        ref_alone = _run(_build(d, ["-L" + os.path.dirname(REF_LIB), "-lcholmod_ref"]),
                         method="simplicial")
        exe = _build(d, ["-Wl,--no-as-needed", "-L" + GB_DIR, "-lcholmod_gb300",
                         "-L" + os.path.dirname(REF_LIB), "-lcholmod_ref"])
        r = _run(exe, method="simplicial")
    assert ref_alone["status"] == 0 and ref_alone["is_super"] == 0 and ref_alone["resid"] < 1e-14
    assert r["status"] == -5 and r["factorize_ok"] == 0 and r["is_super"] == 0, r
