"""The C-ABI library builds, loads without a GPU, exports every entry point
include/m2cg.h declares, and its structs match the ctypes mirror."""
import ctypes as C
import os
import re

import pytest

from m2c_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "m2cg.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(m2cg_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(abi.LIB_PATH):
        from m2c_gb300 import build
        build.build()
    return abi.load()


def test_header_declares_entry_points():
    syms = header_symbols()
    for must in ("m2cg_create", "m2cg_destroy", "m2cg_compute_residual", "m2cg_compute_dt", "m2cg_advance",
                 "m2cg_run", "m2cg_riemann_batch", "m2cg_flux_batch", "m2cg_levelset_residual"):
        assert must in syms


def test_library_exports_every_declared_symbol(lib):
    missing = [s for s in header_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_struct_layout_matches(lib):
    assert lib.m2cg_abi_version() == 1
    assert lib.m2cg_config_size() == C.sizeof(abi.Config)
    assert lib.m2cg_counters_size() == C.sizeof(abi.Counters)


def test_config_default_matches_python_mirror(lib):
    c = abi.Config()
    assert lib.m2cg_config_default(C.byref(c)) == 0
    p = abi.default_config()
    for name, _ in abi.Config._fields_:
        if name.startswith("pad") or name == "mat":
            continue
        a, b = getattr(c, name), getattr(p, name)
        if hasattr(a, "__len__"):
            assert list(a) == list(b), name
        else:
            assert a == b, name
    for m in range(abi.MAX_MATERIALS):
        for name, _ in abi.Material._fields_:
            if name != "pad_":
                assert getattr(c.mat[m], name) == getattr(p.mat[m], name), (m, name)


def test_create_without_device_fails_cleanly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    c = abi.default_config()
    h = C.c_void_p()
    st = lib.m2cg_create(C.byref(c), C.byref(h))
    assert st == 5  # M2CG_ERR_NO_DEVICE
    assert not h.value
