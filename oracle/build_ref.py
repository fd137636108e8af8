"""Compile the reference's own EOS, flux and exact-Riemann sources into
oracle/_ref/libm2cref.so (test infrastructure only).

Where the reference tree is absent (the GPU machine) this step is skipped.
Sources compiled straight from the reference tree with g++: IoData.cpp,
parser/AssignerCore.C, parser/Dictionary.C, ExactRiemannSolverBase.cpp (with
-DWITHOUT_BOOST, the reference's own Boost-free Hugoniot root finder) plus the
header-only VarFcn*/FluxFcn* classes, against a single-rank mpi.h stand-in and
stubs for the parser / Utils symbols IoData.cpp references.  The reference's
CMake build is not used.  Usage: python oracle/build_ref.py
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# The reference checkout: $M2C_REFERENCE_DIR, else a directory named
# "reference" beside this repository's root.
REF = os.environ.get("M2C_REFERENCE_DIR") or os.path.normpath(os.path.join(HERE, "..", "..", "reference"))
OUT = os.path.join(HERE, "_ref")
SHIM = os.path.join(HERE, "ref_shim")
FLAGS = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-DWITHOUT_BOOST", "-include", "cfloat",
         "-include", "iomanip", "-w", "-I", SHIM, "-I", REF]
SOURCES = [os.path.join(REF, "IoData.cpp"), os.path.join(REF, "parser", "AssignerCore.C"),
           os.path.join(REF, "parser", "Dictionary.C"), os.path.join(REF, "ExactRiemannSolverBase.cpp"),
           os.path.join(SHIM, "ref_driver.cpp"), os.path.join(SHIM, "stubs.cpp")]


def available():
    return all(os.path.exists(s) for s in SOURCES)


def build():
    if not available():
        return None
    os.makedirs(OUT, exist_ok=True)

    def cc(src):
        obj = os.path.join(OUT, os.path.basename(src) + ".o")
        if os.path.exists(obj) and os.path.getmtime(obj) > os.path.getmtime(src):
            return obj
        r = subprocess.run(["g++"] + FLAGS + ["-x", "c++", "-c", src, "-o", obj], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"g++ failed on {src}:\n{r.stderr[-4000:]}")
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(cc, SOURCES))
    lib = os.path.join(OUT, "libm2cref.so")
    r = subprocess.run(["g++", "-shared", "-o", lib] + objs, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stderr)
    return lib


if __name__ == "__main__":
    print(build())
