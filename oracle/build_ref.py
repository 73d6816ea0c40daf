"""Build the reference CHOLMOD (CPU only) from its sources into oracle/_ref/.

Test infrastructure only: the reference library is the checker that pins the
C restatement in oracle/ (golden fixtures under tests/golden/ are generated
with it).  It is never linked into, loaded by, or timed as the product.

Recipe (no CMake, no generated code): gcc compiles, directly where they lie,
  SuiteSparse_config/SuiteSparse_config.c
  AMD/Source, CAMD/Source, COLAMD/Source, CCOLAMD/Source
  CHOLMOD/{Check,Cholesky,Utility,MatrixOps,Modify,Partition,Supernodal}/cholmod_*.c
(the file set CHOLMOD/CMakeLists.txt:372-374 globs; METIS is pulled in by
CHOLMOD/Partition/cholmod_metis_wrapper.c), with CUDA off.  The reference finds
"a" Fortran-ABI BLAS/LAPACK; the only one in this image is the OpenBLAS inside
the scipy wheel, whose exported names carry a ``scipy_`` prefix, so every
undefined BLAS/LAPACK symbol ``xyz_`` of the compiled objects is renamed to
``scipy_xyz_`` with objcopy before linking against that library.

Usage: python oracle/build_ref.py [REFERENCE_ROOT]
(default: $CHOLMOD_REFERENCE_ROOT, else /root/reference)
Outputs: oracle/_ref/libcholmod_ref.so, oracle/_ref/ref_dump (driver).
"""
import glob
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")


def reference_root():
    """Where the reference sources are read from (only this recipe, the
    fixture generators and the header-layout test read them)."""
    return os.environ.get("CHOLMOD_REFERENCE_ROOT", "/root/reference")


def openblas_path():
    import scipy
    d = os.path.join(os.path.dirname(scipy.__file__), "..", "scipy.libs")
    libs = sorted(glob.glob(os.path.join(d, "libscipy_openblas*.so")))
    if not libs:
        raise RuntimeError("scipy OpenBLAS not found in " + d)
    return os.path.realpath(libs[0])


def sources(ref):
    src = [os.path.join(ref, "SuiteSparse_config", "SuiteSparse_config.c")]
    for pkg in ("AMD", "CAMD", "COLAMD", "CCOLAMD"):
        src += sorted(glob.glob(os.path.join(ref, pkg, "Source", "*.c")))
    for sub in ("Check", "Cholesky", "Utility", "MatrixOps", "Modify",
                "Partition", "Supernodal"):
        src += sorted(glob.glob(os.path.join(ref, "CHOLMOD", sub, "cholmod_*.c")))
    return src


def includes(ref):
    inc = [os.path.join(ref, "SuiteSparse_config")]
    for pkg in ("AMD", "CAMD", "COLAMD", "CCOLAMD"):
        inc.append(os.path.join(ref, pkg, "Include"))
    ch = os.path.join(ref, "CHOLMOD")
    for sub in ("Include", "Check", "Cholesky", "Utility", "MatrixOps", "Modify",
                "Partition", "Supernodal", "SuiteSparse_metis/GKlib",
                "SuiteSparse_metis/libmetis", "SuiteSparse_metis/include"):
        inc.append(os.path.join(ch, sub))
    inc.append(ch)
    return inc


def run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(" ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else reference_root()
    if not os.path.isdir(os.path.join(ref, "CHOLMOD")):
        print("reference sources not present; oracle/_ref not built")
        return 1
    os.makedirs(os.path.join(OUT, "obj"), exist_ok=True)
    blas = openblas_path()
    inc = ["-I" + d for d in includes(ref)]
    flags = ["-O2", "-fPIC", "-fopenmp", "-DNDEBUG", "-DBLAS32",
             "-w"]
    srcs = sources(ref)

    def compile_one(s):
        rel = os.path.relpath(s, ref).replace("/", "__")
        o = os.path.join(OUT, "obj", rel[:-2] + ".o")
        if not os.path.exists(o) or os.path.getmtime(o) < os.path.getmtime(s):
            run(["gcc", "-c", s, "-o", o] + flags + inc)
        return o

    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        objs = list(ex.map(compile_one, srcs))

    # rename the Fortran BLAS/LAPACK references to the scipy_ prefixed exports
    exported = set(run(["nm", "-D", "--defined-only", blas]).split())
    undef = set()
    for o in objs:
        for line in run(["nm", "-u", o]).splitlines():
            name = line.split()[-1]
            if name.endswith("_") and ("scipy_" + name) in exported:
                undef.add(name)
    symfile = os.path.join(OUT, "blas_rename.txt")
    with open(symfile, "w") as f:
        for name in sorted(undef):
            f.write(f"{name} scipy_{name}\n")
    for o in objs:
        run(["objcopy", "--redefine-syms=" + symfile, o])

    lib = os.path.join(OUT, "libcholmod_ref.so")
    run(["gcc", "-shared", "-o", lib] + objs +
        ["-fopenmp", blas, "-Wl,-rpath," + os.path.dirname(blas), "-lm"])

    drv = os.path.join(HERE, "ref_dump.c")
    if os.path.exists(drv):
        run(["gcc", "-O2", "-o", os.path.join(OUT, "ref_dump"), drv] + flags + inc +
            [lib, "-Wl,-rpath," + OUT, blas, "-Wl,-rpath," + os.path.dirname(blas),
             "-lm"])
    print("built", lib)
    return 0


if __name__ == "__main__":
    sys.exit(main())
