"""In-tree build of libcholmod_gb300.so (the C-ABI library) for sm_103a.

CUDA sources are compiled by nvcc with ``-gencode arch=compute_103a,code=sm_103a``,
host C sources by gcc; everything is linked against the CUDA runtime into
``suitesparse_gb300/libcholmod_gb300.so``.  Translation units are compiled in
parallel and only when their sources or headers changed.
"""
import glob
import hashlib
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG, "libcholmod_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    raise RuntimeError("nvcc not found")


def _digest(paths, flags):
    h = hashlib.sha256(" ".join(flags).encode())
    for p in sorted(paths):
        with open(p, "rb") as f:
            h.update(f.read())
    return h.hexdigest()[:16]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(verbose=False):
    """Compile every CUDA and C source of the package; returns the .so path."""
    cuda = cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(BUILD, exist_ok=True)
    headers = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) \
        + glob.glob(os.path.join(INCLUDE, "*.h"))
    inc = ["-I" + INCLUDE, "-I" + CSRC, "-I" + os.path.join(cuda, "include")]
    cu_flags = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC"] + ARCH
    c_flags = ["-O2", "-fPIC", "-std=c11", "-Wall", "-Wno-unused-function",
               "-D_GNU_SOURCE"]
    jobs = []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu"))):
        jobs.append(([nvcc, "-c"] + cu_flags + inc, src))
    for src in sorted(glob.glob(os.path.join(CSRC, "*.c"))):
        jobs.append((["gcc", "-c"] + c_flags + inc, src))

    def one(job):
        base, src = job
        d = _digest([src] + headers, base)
        obj = os.path.join(BUILD, os.path.basename(src) + "." + d + ".o")
        if not os.path.exists(obj):
            out = _run(base + [src, "-o", obj + ".tmp"])
            os.replace(obj + ".tmp", obj)
            if verbose and out.strip():
                print(out)
        return obj

    with ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        objs = list(ex.map(one, jobs))
    tmp = LIB + ".tmp"
    _run([nvcc, "-shared"] + ARCH + ["-o", tmp] + objs +
         ["-Xlinker", "-rpath," + os.path.join(cuda, "lib64"),
          "-Xlinker", "--version-script=" + os.path.join(CSRC, "exports.map"),
          "-lcudart", "-lpthread"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
