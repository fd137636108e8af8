"""Batched ensemble of independent multi-material domains (m2cg_ensemble_*).

Each member is an ordinary context -- `member(i)` returns a Solver view of it
for uploads, downloads and counters -- and `run` advances all members with one
launch per kernel and RK stage inside a CUDA graph; `run_sequential` advances
them one after another with per-domain launches, the baseline."""
import ctypes as C

from . import abi
from .solver import Solver


class Ensemble:
    def __init__(self, cfgs, lib=None):
        self.lib = lib or abi.load()
        self.cfgs = list(cfgs)
        arr = (abi.Config * len(self.cfgs))(*self.cfgs)
        h = C.c_void_p()
        abi.check(self.lib, self.lib.m2cg_ensemble_create(arr, len(self.cfgs), C.byref(h)), "m2cg_ensemble_create")
        self.h = h
        self.members = [Solver.member(self.lib, c, self.lib.m2cg_ensemble_member(h, i))
                        for i, c in enumerate(self.cfgs)]

    def __len__(self):
        return len(self.cfgs)

    def member(self, i):
        return self.members[i]

    def run(self, nsteps):
        """Batched steps; returns device milliseconds."""
        ms = C.c_float()
        abi.check(self.lib, self.lib.m2cg_ensemble_run(self.h, int(nsteps), C.byref(ms)), "m2cg_ensemble_run")
        return ms.value

    def run_sequential(self, nsteps):
        """Per-domain launches, one member after another; returns wall milliseconds."""
        ms = C.c_float()
        abi.check(self.lib, self.lib.m2cg_ensemble_run_sequential(self.h, int(nsteps), C.byref(ms)),
                  "m2cg_ensemble_run_sequential")
        return ms.value

    def autotune(self, steps=2, budgets=(4, 8, 16, 32, 64, 1 << 20)):
        """Pick the interface solves' first-pass evaluation budget by timing
        `steps` real steps per candidate (the states advance); returns
        (budget, ms per step)."""
        import numpy as np
        cand = np.ascontiguousarray(budgets, np.int32)
        best, ms = C.c_int32(), C.c_float()
        abi.check(self.lib, self.lib.m2cg_ensemble_autotune(self.h, int(steps), len(cand), abi.iptr(cand),
                                                            C.byref(best), C.byref(ms)), "m2cg_ensemble_autotune")
        return best.value, ms.value

    # block shapes tried by autotune_tiles: 128 consecutive cells, or tiles of
    # 128 cells over (x, y, z)
    TILE_SHAPES = ((0, 0, 0), (32, 4, 1), (32, 2, 2), (16, 8, 1), (16, 4, 2), (8, 4, 4))

    def autotune_tiles(self, steps=1, shapes=TILE_SHAPES):
        """Pick the cell / face kernels' block shape per size class (members
        with the same cell count along x) by timing `steps` real batched steps
        per class and shape (the states advance); returns ({nx: shape},
        ms per step of the last class's choice)."""
        import numpy as np
        sh = np.ascontiguousarray(np.asarray(shapes, np.int32).reshape(-1, 3))
        mshape = np.zeros(len(self.cfgs), np.int32)
        ms = C.c_float()
        abi.check(self.lib, self.lib.m2cg_ensemble_autotune_tiles(self.h, int(steps), len(sh), abi.iptr(sh),
                                                                  abi.iptr(mshape), C.byref(ms)),
                  "m2cg_ensemble_autotune_tiles")
        return {int(c.nx): tuple(int(v) for v in sh[mshape[i]]) for i, c in enumerate(self.cfgs)}, ms.value

    def kernel_launches(self):
        return self.lib.m2cg_ensemble_kernel_launches(self.h)

    def close(self):
        if getattr(self, "h", None):
            for m in self.members:
                m.ctx = None
            self.lib.m2cg_ensemble_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()
