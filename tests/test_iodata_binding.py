"""The reference-side binding (include/m2cg_iodata.hpp) compiled against the
reference's own IoData.h and parser objects (oracle/_ref, built from the
reference sources by oracle/build_ref.py): the configuration it builds from
an IoData equals, field by field, the library's defaults
(m2cg_config_default) and the product's own input reader
(m2c_gb300.inputfile) on the reference's Tests/RiemannProblems inputs.  The
statements of an input file reach IoData through the reference's assigner
objects the way its grammar applies them (tests/cpp/iodata_check.cpp).  CPU
only; skipped where the reference tree is absent."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from m2c_gb300 import abi
from m2c_gb300 import inputfile as inf
from oracle import build_ref

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "m2c_gb300", "lib")


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None or not build_ref.available() or not os.path.exists(os.path.join(LIBDIR, "libm2cg.so")):
        pytest.skip("g++, the reference sources or libm2cg.so missing")
    ref_lib = build_ref.build()
    out = str(tmp_path_factory.mktemp("iodata") / "iodata_check")
    cmd = [gxx, "-std=c++17", "-O1", "-w", "-include", "cfloat", "-include", "iomanip",
           "-I", build_ref.SHIM, "-I", build_ref.REF, "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "iodata_check.cpp"),
           "-L", os.path.dirname(ref_lib), "-lm2cref", "-L", LIBDIR, "-lm2cg",
           "-Wl,-rpath," + os.path.dirname(ref_lib), "-Wl,-rpath," + LIBDIR, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return out


def statements(text):
    """The input file as U / E / A lines for iodata_check (numbers evaluated)."""
    p = inf._Parser(text)
    lines = []

    def path():
        parts = [p.take("sym")]
        while p.peek() in (("p", "."), ("p", "[")):
            if p.take("p") == ".":
                parts.append("." + p.take("sym"))
            else:
                parts.append("[%d" % int(p.expr()))
                p.take("p", "]")
        return " ".join(parts)

    while p.peek()[0] != "eof":
        t = p.peek()
        if t[0] == "under":
            p.i += 1
            lines.append("U " + path())
            p.take("p", "{")
        elif t == ("p", "}"):
            p.i += 1
            lines.append("E")
        else:
            target = path()
            p.take("p", "=")
            v = p.peek()
            if v[0] == "sym":
                p.i += 1
                lines.append("A %s = sym %s" % (target, v[1]))
            elif v[0] == "str":
                p.i += 1
                lines.append("A %s = str %s" % (target, v[1]))
            else:
                x = p.expr()
                lines.append("A %s = %s %r" % (target, "int" if isinstance(x, int) else "dbl", x))
            p.take("p", ";")
    return "\n".join(lines) + "\n"


def run(exe, tmp_path, text):
    src = tmp_path / "stmts.txt"
    src.write_text(statements(text) if text is not None else "")
    out = tmp_path / "cfg.bin"
    r = subprocess.run([exe, str(src), str(out)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    return abi.Config.from_buffer_copy(out.read_bytes())


def fields(cfg, n_mat):
    """(name, value) of every configuration field, materials up to n_mat."""
    out = []
    for name, ty in abi.Config._fields_:
        if name.startswith("pad"):
            continue
        v = getattr(cfg, name)
        if name == "mat":
            for m in range(n_mat):
                for fn, _ in type(v[m])._fields_:
                    if not fn.startswith("pad"):
                        out.append(("mat[%d].%s" % (m, fn), getattr(v[m], fn)))
        elif hasattr(v, "__len__"):
            out.append((name, tuple(v)))
        else:
            out.append((name, v))
    return out


# the smallest input the reference accepts: one material, a mesh size and its
# boundary conditions (the reference has no default for either)
ONE_MATERIAL = ("under Equations { under Material[0] { EquationOfState = StiffenedGas; } }\n"
                "under Mesh { NumberOfCellsX = 1; NumberOfCellsY = 1; NumberOfCellsZ = 1;\n"
                "  X0 = 0.0; Xmax = 1.0; Y0 = 0.0; Ymax = 1.0; Z0 = 0.0; Zmax = 1.0;\n"
                "  BoundaryConditionX0 = Outlet; BoundaryConditionXmax = Outlet; BoundaryConditionY0 = Outlet;\n"
                "  BoundaryConditionYmax = Outlet; BoundaryConditionZ0 = Outlet; BoundaryConditionZmax = Outlet; }\n")


def test_binding_on_default_iodata_gives_the_library_defaults(exe, tmp_path):
    got = run(exe, tmp_path, ONE_MATERIAL)
    ref = abi.default_config()
    diff = [(n, a, b) for (n, a), (_, b) in zip(fields(got, 1), fields(ref, 1)) if a != b]
    assert not diff, diff


@pytest.mark.parametrize("test", ["Test%d" % i for i in (1, 2, 3, 4, 5, 6, 8, 9, 10, 11, 12)])
def test_binding_matches_the_input_reader_on_reference_inputs(exe, tmp_path, test):
    text = open(os.path.join(build_ref.REF, "Tests", "RiemannProblems", test, "input.st")).read()
    got = run(exe, tmp_path, text)
    case = inf.Case.from_text(text)
    want = case.cfg
    diff = [(n, a, b) for (n, a), (_, b) in zip(fields(got, want.n_materials), fields(want, want.n_materials))
            if a != b]
    assert not diff, diff
