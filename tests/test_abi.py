"""The C ABI: every declared entry point is exported, and the CHOLMOD object
layouts are byte-identical to the reference's cholmod.h."""
import ctypes
import os
import re
import subprocess
import tempfile

import pytest

from conftest import ROOT

from oracle.build_ref import reference_root

REF_ROOT = reference_root()
REF_INC = os.path.join(REF_ROOT, "CHOLMOD", "Include")
OBJ = {"cholmod_common": 0, "cholmod_sparse": 1, "cholmod_factor": 2, "cholmod_dense": 3}


def declared_functions():
    names = []
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if not fn.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", fn)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"typedef struct.*?\}\s*\w+\s*;", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:int|long|size_t|void|cholmod_\w+\s*\*|int64_t)\s*\**\s*(\w+)\s*\(",
                             src, flags=re.M):
            names.append(m.group(1))
    return sorted(set(names))


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert "cholmod_l_super_numeric" in names and "cholmod_l_super_lsolve" in names
    assert "cholmod_l_super_ltsolve" in names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_boundary_symbols_are_dynamic(lib):
    from suitesparse_gb300 import cholmod as CH
    out = subprocess.run(["nm", "-D", "--defined-only", CH.LIB_PATH], capture_output=True,
                         text=True).stdout
    for name in ("cholmod_l_super_numeric", "cholmod_l_super_lsolve", "cholmod_l_super_ltsolve"):
        assert re.search(r"\bT " + name + r"\b", out), name


@pytest.mark.skipif(not os.path.isdir(REF_INC), reason="reference sources not present")
def test_layout_matches_reference_header(lib):
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "probe")
        subprocess.run(["gcc", "-o", exe, os.path.join(ROOT, "tests", "abi_probe.c"),
                        "-I" + REF_INC, "-I" + os.path.join(REF_ROOT, "SuiteSparse_config"),
                        "-I" + os.path.join(ROOT, "suitesparse_gb300", "csrc")], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    checked = 0
    for line in out.splitlines():
        parts = line.split()
        if parts[0] == "sizeof":
            assert lib.gb300_abi_sizeof(OBJ[parts[1]]) == int(parts[2]), line
        else:
            off = lib.gb300_abi_offset(OBJ[parts[0]], parts[1].encode())
            assert off == int(parts[2]), line
        checked += 1
    assert checked > 150
