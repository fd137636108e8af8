"""Build libm2cg.so in-tree with nvcc for sm_103a (GB300).

Each translation unit compiles in parallel; the interface-Riemann unit is
compiled without floating-point contraction so its iterative decisions follow
plain binary64 rounding.  Usage: python -m m2c_gb300.build
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "lib")
BUILD = os.path.join(HERE, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
          "-Xcompiler", "-Werror=return-type",
          "-I", os.path.join(HERE, "..", "include")]
UNITS = {
    "m2cg_kernels.cu": [],
    "m2cg_tile.cu": [],
    "m2cg_riemann_kernels.cu": ["-fmad=false"],
    "m2cg_api.cu": [],
    "m2cg_noalloc.cu": ["-fmad=false"],
    "m2cg_mlp.cu": [],
    "m2cg_reinit.cu": ["-fmad=false"],
    "m2cg_peak.cu": [],
    "m2cg_probe.cu": ["-fmad=false"],
}


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _compile(src, extra, verbose_ptxas=False):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc()] + ARCH + COMMON + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
    if verbose_ptxas:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    return obj, r.stderr


def build(verbose_ptxas=False, quiet=True):
    os.makedirs(OUT, exist_ok=True)
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        futs = {ex.submit(_compile, s, e, verbose_ptxas): s for s, e in UNITS.items()}
        objs, logs = [], []
        for f in cf.as_completed(futs):
            o, log = f.result()
            objs.append(o)
            logs.append((futs[f], log))
    lib = os.path.join(OUT, "libm2cg.so")
    tmp = lib + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + sorted(objs)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, lib)
    if not quiet or verbose_ptxas:
        for s, log in logs:
            if log.strip():
                print(f"== {s}\n{log}", file=sys.stderr)
    return lib


if __name__ == "__main__":
    print(build(verbose_ptxas="-v" in sys.argv, quiet=False))
