"""Build the oracle (test infrastructure only): oracle/lib/liboracle.so from
m2c_oracle.cpp with -ffp-contract=off and OpenMP.  Usage: python oracle/build.py"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "lib")


def build():
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(HERE, "m2c_oracle.cpp")
    lib = os.path.join(OUT, "liboracle.so")
    deps = [src] + [os.path.join(HERE, h) for h in ("oracle_eos_flux.h", "oracle_riemann.h")]
    if os.path.exists(lib) and os.path.getmtime(lib) > max(os.path.getmtime(d) for d in deps):
        return lib
    cmd = ["g++", "-std=c++17", "-O2", "-Werror=return-type", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-o", lib + ".tmp", src]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stderr[-4000:]}")
    os.replace(lib + ".tmp", lib)
    return lib


if __name__ == "__main__":
    print(build())
