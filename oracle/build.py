"""Build the oracle (test infrastructure only): oracle/lib/liboracle.so from
m2c_oracle.cpp with -ffp-contract=off and OpenMP.

build(fma=True) builds the same source with floating-point contraction into
fused multiply-adds (oracle/lib/liboracle_fma.so): the reference's numerics
as a compiler that contracts -- GCC's default on AArch64, where the reference
also builds -- would run them.  Comparing the two measures how far the
reference's own result moves with the rounding of a contracting compiler,
the yardstick for the product's FMA-contracting kernels.
Usage: python oracle/build.py"""
import os
import platform
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "lib")


def build(fma=False):
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(HERE, "m2c_oracle.cpp")
    lib = os.path.join(OUT, "liboracle_fma.so" if fma else "liboracle.so")
    deps = [src, __file__] + [os.path.join(HERE, h) for h in ("oracle_eos_flux.h", "oracle_riemann.h")]
    if os.path.exists(lib) and os.path.getmtime(lib) > max(os.path.getmtime(d) for d in deps):
        return lib
    if fma:
        contract = ["-ffp-contract=fast"] + (["-mfma"] if platform.machine() in ("x86_64", "AMD64") else [])
    else:
        contract = ["-ffp-contract=off"]
    cmd = ["g++", "-std=c++17", "-O2", "-Werror=return-type"] + contract + ["-fopenmp", "-fPIC", "-shared", "-o",
                                                                           lib + ".tmp", src]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stderr[-4000:]}")
    os.replace(lib + ".tmp", lib)
    return lib


if __name__ == "__main__":
    print(build())
    print(build(fma=True))
