#!/usr/bin/env python3
"""Benchmark: FP64 cell-stage updates per second of the multi-material
finite-volume step (3D shock-bubble, 256^3 cells, RK2) on GB300.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--size 256]

`value`: whole-job cell-stage updates/s with the state resident in HBM,
device-timed with CUDA events on the library stream over K steps (the step
loop runs as a replayed CUDA graph; dt never leaves the device).
`e2e`: the same metric through the C ABI with host buffers -- every step
uploads {V, ID, phi} from pinned host memory, computes dt, advances one step
and downloads the new state.
`--impl reference`: the reference arm -- the oracle's CPU restatement of the
reference numerics (the reference itself needs MPI and PETSc, absent on the
box) on the same workload with every host thread.
`parity` (the CPU-baseline leg): the oracle advances the same workload from
the same initial state as a fresh GPU context to each checkpoint of
--parity-steps; both states, counters and conserved totals are compared
there, beside the oracle compiled with FMA contraction (the reference's own
rounding sensitivity).  Its wall time gives `cpu_baseline`.
N > 1 (torchrun): replicas only -- every rank advances its own copy of the
workload; no data-path collective (the reference's halo exchange has no
counterpart on one GPU per replica); value = all ranks' cell-stages / max time.
"""
import argparse
import ctypes as C
import json
import os
import shutil
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "FP64 cell-stage updates/s (1 GB300) + Newton iters/interface, MLP vs cold start @1e-10"
UNIT = "cell-stage/s"
MEASURED_PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
# FP64-pipe instructions per cell of each stage kernel (warp instructions x 32 /
# cells), binary64 FLOPs per cell (2 DFMA + DMUL + DADD, active lanes), and DRAM
# bytes per cell, from the ncu capture of the 128^3 case in
# profiles/fp64_stage_kernels_shock_bubble_128.txt; the counts per cell do not
# depend on the grid size (the same code path runs on every cell or face).
FP64_PROFILE = {
    "reconstruct": {"fp64_pipe_inst_per_cell": 279.7, "fp64_flop_per_cell": 131.1, "dram_bytes_per_cell": 269.0},
    "face_flux": {"fp64_pipe_inst_per_cell": 617.5, "fp64_flop_per_cell": 706.8, "dram_bytes_per_cell": 363.0},
    "update": {"fp64_pipe_inst_per_cell": 104.5, "fp64_flop_per_cell": 122.6, "dram_bytes_per_cell": 293.9},
}
# The fused reconstruction + face-flux kernel (k_recon_flux_tile, the default
# path) and the stage update: FP64-pipe slots, binary64 FLOPs (2 DFMA + DMUL +
# DADD, thread level) and DRAM bytes per cell and launch, ncu on the 128^3 case
# (profiles/k_recon_flux_tile_shock_bubble_128.txt; mean of the two stages).
FP64_PROFILE_FUSED = {
    "face_flux": {"fp64_pipe_inst_per_cell": 610.7, "fp64_flop_per_cell": 645.7, "dram_bytes_per_cell": 150.8},
    "update": {"fp64_pipe_inst_per_cell": 104.0, "fp64_flop_per_cell": 117.5, "dram_bytes_per_cell": 295.3},
}
# DRAM bytes of one whole step graph of the 128^3 case (read + write, ncu
# --graph-profiling graph) per cell-stage: split kernels
# (profiles/reinit_graph_shock_bubble_128.txt) and fused
# (profiles/step_graph_shock_bubble_128.txt).
STEP_DRAM_BYTES_PER_CELL_STAGE = (2388.8e6 + 1971.9e6) / (128 ** 3 * 2)
STEP_DRAM_BYTES_PER_CELL_STAGE_FUSED = (1305.2e6 + 956.4e6) / (128 ** 3 * 2)
# Algorithmic bytes per cell-stage of the fused ideal (binary64 V and phi, int32
# ID, ideal halo reuse): a first stage reads W = (V, phi) 48 B + ID 4 B and
# writes 48 B = 100 B; a later stage also reads W^n = 148 B.  Mean over the
# integrator's stages: forward Euler 100, RK2 124, RK3 132.
ALG_BYTES_PER_CELL_STAGE = {1: 100.0, 2: 124.0, 3: 132.0}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--e2e-steps", type=int, default=None)
    # reference arm: cells per axis of its sample (0: the workload's own size)
    ap.add_argument("--cpu-size", type=int, default=0)
    ap.add_argument("--no-cpu", action="store_true")
    # parity leg (the oracle on the same workload from the same initial state):
    # checkpoints, and the last checkpoint the FMA-contracted oracle runs to
    ap.add_argument("--parity-steps", default="1,10,50")
    ap.add_argument("--parity-fma-steps", type=int, default=10)
    # level-set reinitialization every F steps in the main workload (0: off, as the 256^3 workload runs)
    ap.add_argument("--reinit", type=int, default=0)
    # learned warm start: training / test problems of the study (0 disables it)
    ap.add_argument("--ws-train", type=int, default=1 << 20)
    ap.add_argument("--ws-test", type=int, default=1 << 16)
    ap.add_argument("--ws-epochs", type=int, default=60)
    # batched ensemble of uneven bubble-collapse domains (0 disables it): batched
    # steps, and steps of the per-domain-launch baseline
    ap.add_argument("--ens-domains", type=int, default=512)
    ap.add_argument("--ens-steps", type=int, default=100)
    ap.add_argument("--ens-seq-steps", type=int, default=10)
    # large production-shaped run (8 gas bubbles in NASG water, 5e8 Pa shock, RK3,
    # reinitialization every 10 steps; 0 disables it)
    ap.add_argument("--large", type=int, default=512, help="cells per axis of the large run")
    ap.add_argument("--large-steps", type=int, default=10)
    return ap.parse_args()


def dist_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    def __init__(self, gpu_index):
        self.proc = None
        self.path = None
        smi = shutil.which("nvidia-smi")
        if not smi:
            return
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        self.proc = subprocess.Popen([smi, "-i", str(gpu_index), f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                      "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    try:
        return json.load(open(MEASURED_PEAKS)), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def cpu_model():
    """The host CPU's model name and logical core count (lscpu / /proc/cpuinfo)."""
    name = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.split(":")[0].strip() == "Model name":
                name = line.split(":", 1)[1].strip()
                break
    except Exception:
        pass
    if not name:
        try:
            for line in open("/proc/cpuinfo"):
                if line.lower().startswith(("model name", "cpu part")):
                    name = line.split(":", 1)[1].strip()
                    break
        except Exception:
            pass
    return {"model": name or "unknown", "logical_cpus": os.cpu_count()}


class OracleLeg:
    """The CPU-baseline leg: the oracle (the CPU restatement of the reference
    numerics) advances the benchmarked workload itself from the initial state
    to each parity checkpoint, in a background thread (ctypes releases the
    GIL) while the device-timed GPU legs run; it leaves one host core to the
    GPU's host thread.  Its wall time over all checkpoints is the all-core CPU
    rate; one step of a 64^3 sample on one thread, run before the thread
    starts, gives the single-thread rate.  Up to --parity-fma-steps the oracle
    compiled with fused multiply-add contraction runs too: how far the
    reference's own numerics move under a contracting compiler, the yardstick
    for the GPU's FMA-contracting kernels.  finish() then advances a fresh GPU
    context to the same checkpoints and compares state, IDs, counters and
    conserved totals."""

    def __init__(self, args, cfg, V, ID, phi, stages):
        import threading
        from m2c_gb300 import problems
        from oracle import binding as ob
        self.args, self.cfg, self.V, self.ID, self.phi, self.stages = args, cfg, V, ID, phi, stages
        self.cps = sorted({int(x) for x in str(args.parity_steps).split(",") if x.strip()})
        self.threads = max(1, (os.cpu_count() or 1) - 1)
        # one thread, one step of a 64^3 sample of the same problem
        ob.lib().orc_set_threads(1)
        c1, V1, I1, p1 = problems.shock_bubble(n=64)
        o1 = ob.OracleSim(c1)
        o1.upload(V1, I1, p1)
        t = time.perf_counter()
        o1.run(1)
        self.t1 = time.perf_counter() - t
        del o1
        for fma in (False, True):
            ob.lib(fma).orc_set_threads(self.threads)
        self.used = ob.lib().orc_max_threads()
        self.snap, self.snap_fma, self.error = {}, {}, None
        self.t_orc = 0.0
        self.thread = threading.Thread(target=self._run, daemon=True)
        self.thread.start()

    def _run(self):
        from oracle import binding as ob
        try:
            for fma, store, last in ((False, self.snap, self.cps[-1]), (True, self.snap_fma, self.args.parity_fma_steps)):
                if last <= 0:
                    continue
                o = ob.OracleSim(self.cfg, fma=fma)
                o.upload(self.V, self.ID, self.phi)
                store[0] = {"totals": o.conserved_totals()}
                done = 0
                for c in self.cps:
                    if c > last:
                        break
                    t = time.perf_counter()
                    o.run(c - done)
                    if not fma:
                        self.t_orc += time.perf_counter() - t
                    done = c
                    Vo, IDo, pho = o.download()
                    store[c] = {"state": (Vo, IDo, pho), "counters": o.counters(), "totals": o.conserved_totals()}
                del o
        except Exception as e:   # reported in the bench line, never hidden
            self.error = repr(e)

    def finish(self):
        from m2c_gb300.solver import FluidState, Solver
        from oracle import parity
        self.thread.join()
        if self.error:
            return {"error": self.error}, {"error": self.error}
        cfg = self.cfg
        cells = cfg.nx * cfg.ny * cfg.nz
        shape = (cfg.nz, cfg.ny, cfg.nx)
        g = Solver(cfg, FluidState(self.V, self.ID, self.phi))
        t0g, t0o = g.conserved_totals(), self.snap[0]["totals"]
        out = {"workload": "the benchmarked workload, GPU (fresh context, graph-replayed steps) and oracle from the "
                           "same initial state", "checkpoints": []}
        done = 0
        for c in self.cps:
            g.run(c - done)
            done = c
            gs = g.get_state()
            Vo, IDo, pho = self.snap[c]["state"]
            cp = {"step": c}
            cp.update(parity.compare(gs.V, gs.ID, gs.Phi, Vo, IDo, pho, shape))
            cp["counters"] = parity.counters_pair(g.counters(), self.snap[c]["counters"])
            tg, to = g.conserved_totals(), self.snap[c]["totals"]
            cp["conserved_gpu"] = parity.totals_dict(t0g, tg, ref=to)
            cp["conserved_oracle"] = parity.totals_dict(t0o, to)
            if c in self.snap_fma:
                Vf, IDf, phf = self.snap_fma[c]["state"]
                y = parity.compare(Vf, IDf, phf, Vo, IDo, pho, shape)
                y["riemann_errors"] = int(self.snap_fma[c]["counters"]["riemann_errors"])
                y["riemann_iterations"] = int(self.snap_fma[c]["counters"]["riemann_iterations"])
                cp["oracle_fma_vs_oracle"] = y
            out["checkpoints"].append(cp)
        g.close()
        rate = cells * self.stages * done / self.t_orc
        cpu = {"value": rate, "unit": UNIT, "cores": self.used, "kind": "port",
               "sample": f"oracle CPU restatement on the benchmarked workload itself ({cfg.nx}^3), {done} RK2 steps "
                         f"from the initial state, {self.t_orc:.1f} s on {self.used} threads (beside the "
                         f"device-timed GPU legs, one core left to their host thread)",
               "single_thread": {"value": 64 ** 3 * self.stages / self.t1, "unit": UNIT, "cores": 1,
                                 "sample": f"shock-bubble 64^3, 1 RK2 step, {self.t1:.2f} s"},
               "cpu": cpu_model()}
        return cpu, out


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return 0
    # each step: one RK2 step of the oracle on the benchmarked workload (or a
    # smaller sample of it when --cpu-size says so)
    threads = os.cpu_count()
    from oracle import binding as ob
    from m2c_gb300 import problems
    ob.lib().orc_set_threads(threads)
    size = args.cpu_size or args.size
    cfg, V, ID, phi = problems.shock_bubble(n=size)
    sim = ob.OracleSim(cfg)
    sim.upload(V, ID, phi)
    for _ in range(args.warmup):
        sim.run(1)
    t0 = time.perf_counter()
    sim.run(args.steps)
    t = time.perf_counter() - t0
    cells = size ** 3
    value = cells * 2 * args.steps / t
    c = sim.counters()
    sample = (f"shock-bubble {size}^3 cells (the workload's physics, initial state and numerics), "
              f"{args.steps} RK2 steps after {args.warmup} warm-up")
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": f"shock-bubble {args.size}^3, SG/SG, MUSCL-van Albada, HLLC, exact interface "
                                  f"Riemann @1e-10, RK2, CFL 0.4", "cells": cells, "sample": sample,
                      "parallelism": "replicas" if args.gpus > 1 else "single"},
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
                            "cpu": cpu_model()},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "riemann": {"mean_iters_per_solve": c["riemann_iterations"] / max(c["riemann_solves"], 1),
                       "solves": c["riemann_solves"]},
           "note": "CPU restatement of the reference numerics (oracle/), OpenMP on all host threads; "
                   "the m2c binary needs MPI + PETSc, absent on the box"}
    print(json.dumps(out))
    return 0


def ensemble_bench(n_domains, steps, seq_steps):
    """Batched ensemble (edges per axis from {32,48,64,96,128}, bubble radius
    [0.1,0.3] of the box, water 1e6..1e8 Pa, gas 1e4 Pa, RK2): the same steps
    from the same initial states, batched (one launch per kernel and stage for
    all members, persistent cell and face kernels; device-timed) and with
    per-domain launches one member after another (wall-timed, each member's own
    CUDA graph).  Before timing, the interface-solve budget and the block shape
    per size class are tuned on real steps."""
    from m2c_gb300 import problems
    from m2c_gb300.ensemble import Ensemble
    from m2c_gb300.solver import FluidState
    doms = problems.bubble_collapse_ensemble(n_domains, seed=4096)
    cells = sum(c.nx * c.ny * c.nz for c, *_ in doms)
    ens = Ensemble([d[0] for d in doms])
    out = {"workload": f"{n_domains} bubble-collapse domains, edges per axis from {{32,48,64,96,128}}, "
                       f"SG gas / SG water, MUSCL-van Albada, HLLC, exact interface Riemann @1e-10, RK2, CFL 0.4",
           "domains": n_domains, "cells": cells}
    def reset():
        for i, (c, V, ID, phi) in enumerate(doms):
            ens.member(i).set_state(FluidState(V, ID, phi))

    reset()
    t0 = time.perf_counter()
    budget, tuned_ms = ens.autotune(steps=1, budgets=(16, 24, 32, 64))
    shapes = ((0, 0, 0), (32, 4, 1), (16, 8, 1), (16, 4, 2))
    chosen, tile_ms = ens.autotune_tiles(steps=1, shapes=shapes)
    out["autotune"] = {"first_pass_eval_budget": budget, "budget_ms_per_step": tuned_ms,
                       "budget_candidates": [16, 24, 32, 64],
                       "block_shape_by_nx": {str(k): list(v) for k, v in sorted(chosen.items())},
                       "shape_candidates": [list(x) for x in shapes], "tuning_s": time.perf_counter() - t0}
    for mode, n in (("batched", steps), ("sequential", seq_steps)):
        run = ens.run if mode == "batched" else ens.run_sequential
        reset()
        run(1)  # graph capture
        reset()
        l0 = ens.kernel_launches()
        ms = run(n)
        out[mode] = {"steps": n, "ms": ms, "ms_per_step": ms / n, "value": cells * 2 * n / (ms * 1e-3), "unit": UNIT}
        if mode == "batched":
            out[mode]["gpu_launches_per_step"] = (ens.kernel_launches() - l0) / max(n, 1)
    out["speedup"] = out["sequential"]["ms_per_step"] / out["batched"]["ms_per_step"]
    ens.close()
    return out


def large_bench(n, steps, warmup=2, ws_train=1 << 20, net=None):
    """n^3 bubble cluster in NASG water hit by a 5e8 Pa shock, RK3, level set
    reinitialized every 10 steps: device-timed cell-stage updates/s (the
    reinitializations inside the timed steps included) and the interface-solve
    share of the step, cold and with the learned warm start, the same steps
    from the same initial state; plus one reinitialization timed alone."""
    from m2c_gb300 import abi, problems
    from m2c_gb300 import warmstart as ws
    from m2c_gb300.solver import FluidState, Solver
    lib = abi.load()
    cfg, V, ID, phi = problems.bubble_cluster_shock(n=n)
    cells = n ** 3
    s = Solver(cfg, FluidState(V, ID, phi))
    out = {"workload": f"{n}^3 cluster of 8 SG gas bubbles in NASG water, 5e8 Pa planar shock, MUSCL-van Albada, "
                       f"HLLC, exact interface Riemann @1e-10, RK3, CFL 0.4, level-set reinitialization every 10 steps",
           "cells": cells, "steps": steps, "stages_per_step": 3}
    own = net is None
    for mode in ("cold", "warm"):
        if mode == "warm":
            if net is None:
                _, net = ws.study(n_train=ws_train, n_test=1 << 12, epochs=60, keep_net=True)
            s.set_warm_start(net)
        s.set_state(FluidState(V, ID, phi))
        s.run(warmup)
        c0 = s.counters()
        r0 = s.reinit_stats()
        lib.m2cg_event_record(s.ctx, 0)
        s.run(steps)
        lib.m2cg_event_record(s.ctx, 1)
        lib.m2cg_sync(s.ctx)
        ms = C.c_float()
        abi.check(lib, lib.m2cg_event_elapsed(s.ctx, 0, 1, C.byref(ms)), "elapsed")
        c1 = s.counters()
        r1 = s.reinit_stats()
        ph = np.zeros(9)
        abi.check(lib, lib.m2cg_phase_times(s.ctx, 1, abi.dptr(ph)), "phase_times")
        solves = c1["riemann_solves"] - c0["riemann_solves"]
        out[mode] = {"value": cells * 3 * steps / (ms.value * 1e-3), "unit": UNIT, "ms_per_step": ms.value / steps,
                     "riemann_solves": solves,
                     "mean_iters_per_solve": (c1["riemann_iterations"] - c0["riemann_iterations"]) / max(solves, 1),
                     "riemann_first_pass_ms_per_step": float(ph[4]),
                     "riemann_stragglers_ms_per_step": float(ph[8]),
                     "interface_faces_per_stage": (c1["interface_faces"] - c0["interface_faces"]) / (3 * steps),
                     "swept_cells": c1["swept_cells"] - c0["swept_cells"],
                     "unresolved_cells": c1["unresolved_cells"] - c0["unresolved_cells"],
                     "clipped_cells": c1["clipped_cells"] - c0["clipped_cells"],
                     "reinit_calls": r1["calls"] - r0["calls"],
                     "reinit_iterations": r1["iterations"] - r0["iterations"],
                     "reinit_retries": r1["retries"] - r0["retries"]}
    # one reinitialization of the final level set, timed alone
    r0 = s.reinit_stats()
    lib.m2cg_event_record(s.ctx, 0)
    s.Reinitialize()
    lib.m2cg_event_record(s.ctx, 1)
    lib.m2cg_sync(s.ctx)
    abi.check(lib, lib.m2cg_event_elapsed(s.ctx, 0, 1, C.byref(ms)), "elapsed")
    r1 = s.reinit_stats()
    it = r1["iterations"] - r0["iterations"]
    out["reinit_alone"] = {"ms": ms.value, "iterations": it, "retries": r1["retries"] - r0["retries"],
                           "ms_per_iteration": ms.value / max(it, 1)}
    s.set_warm_start(None)
    s.close()
    if own and net is not None:
        net.close()
    return out


def max_over_ranks(pg, x):
    """The largest x over all ranks (the job's time is its slowest rank's);
    x itself without a process group.  NCCL reduces device tensors, gloo host
    tensors."""
    if pg is None:
        return x
    import torch
    dev = "cuda" if pg.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def job_rate(world, cells, stages, steps, seconds):
    """Whole-job cell-stage updates per second: every rank advances its own
    replica of `cells` cells, timed by the slowest rank."""
    return world * cells * stages * steps / seconds


def run_gb300(args):
    rank, world, local = dist_info()
    pg = None
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        pg = dist
    from m2c_gb300 import abi, problems
    from m2c_gb300.solver import FluidState, Solver
    lib = abi.load()
    cfg, V, ID, phi = problems.shock_bubble(n=args.size)
    if args.reinit > 0:
        cfg.reinit_frequency = args.reinit
    cells = cfg.nx * cfg.ny * cfg.nz
    stages = 2
    s = Solver(cfg, FluidState(V, ID, phi))
    ctx = s.ctx

    def barrier():
        if pg:
            pg.barrier()

    # warm-up (the first run captures the step into a CUDA graph)
    s.run(args.warmup)
    c0 = s.counters()
    l0 = lib.m2cg_kernel_launches(ctx)
    barrier()
    lib.m2cg_sync(ctx)
    clocks = Clocks(local)
    lib.m2cg_event_record(ctx, 0)
    s.run(args.steps)
    lib.m2cg_event_record(ctx, 1)
    lib.m2cg_sync(ctx)
    barrier()
    ms = C.c_float()
    abi.check(lib, lib.m2cg_event_elapsed(ctx, 0, 1, C.byref(ms)), "elapsed")
    launches = lib.m2cg_kernel_launches(ctx) - l0
    c1 = s.counters()
    clk = clocks.stop()
    t_ms = max_over_ranks(pg, ms.value)
    value = job_rate(world, cells, stages, args.steps, t_ms * 1e-3)
    solves = c1["riemann_solves"] - c0["riemann_solves"]
    iters = c1["riemann_iterations"] - c0["riemann_iterations"]

    # per-phase device times (CUDA events around every kernel; the straggler
    # Riemann solves overlap reconstruction and face fluxes on a second stream)
    ph = np.zeros(9)
    nph = 2
    abi.check(lib, lib.m2cg_phase_times(ctx, nph, abi.dptr(ph)), "phase_times")
    names = ["dt", "compact", "reconstruct", "face_flux", "riemann", "update", "bc", "end_of_step",
             "riemann_stragglers"]
    phase = {n: float(v) / nph for n, v in zip(names, ph)}
    dom = max(("reconstruct", "face_flux", "update"), key=lambda n: phase[n])
    fused = phase["reconstruct"] == 0.0   # the fused reconstruction + face-flux kernel ran
    profile = FP64_PROFILE_FUSED if fused else FP64_PROFILE
    pk, pk_kind = peaks()
    per_launch_ms = phase[dom] / stages
    prof = profile.get(dom)
    # achieved = algorithmic bytes of the cell-stages one launch advances (the
    # fused ideal's bytes per cell-stage x cells) / the launch's event-timed
    # duration; traffic = the kernel's own DRAM bytes per launch (ncu, 128^3
    # case, scaled by cells)
    alg = ALG_BYTES_PER_CELL_STAGE[stages]
    achieved_gbs = alg * cells / (per_launch_ms * 1e-3) / 1e9
    # the kernels' own (unfused) bytes per cell: what each reads and writes
    #   reconstruct: V 40 + ID 4 in, 6 face states 240 out                     = 284
    #   face_flux:   2 face states per face (3 faces: 240) + IDs 8 in, 3 fluxes 120 out = 368
    #   update:      6 fluxes 240 + Un/Us 80 + ID 4 + phi 8 + V 40 in, V 40 + phi 8 + U 40 out = 460
    #   fused reconstruction + face flux: V 40 + ID 4 in, 3 fluxes 120 out          = 164
    own_bytes = {"reconstruct": 284, "face_flux": 164 if fused else 368, "update": 460}
    step_ms = t_ms / args.steps
    step_dram = (STEP_DRAM_BYTES_PER_CELL_STAGE_FUSED if fused else STEP_DRAM_BYTES_PER_CELL_STAGE)
    roof = {"bound": "hbm", "kernel": "recon_flux_tile (fused)" if fused and dom == "face_flux" else dom,
            "achieved": achieved_gbs, "peak": pk["hbm_gbs"], "unit": "GB/s",
            "frac": achieved_gbs / pk["hbm_gbs"],
            "traffic": prof["dram_bytes_per_cell"] * cells if prof else None, "peak_source": pk_kind,
            "alg_bytes_per_cell_stage": alg, "launch_ms": per_launch_ms,
            "kernel_own_bytes_per_cell": own_bytes[dom],
            "step": {"alg_bytes_per_cell_stage": alg,
                     "dram_bytes_per_cell_stage": step_dram,
                     "dram_over_alg": step_dram / alg if step_dram else None,
                     "achieved_gbs": alg * cells * stages / (step_ms * 1e-3) / 1e9,
                     "frac": alg * cells * stages / (step_ms * 1e-3) / 1e9 / pk["hbm_gbs"],
                     "dram_source": "ncu whole-graph capture of the 128^3 step (profiles/" +
                                    ("step_graph_shock_bubble_128.txt)" if fused else "reinit_graph_shock_bubble_128.txt)")}}
    # the binding bound of the stage kernels: GB300's FP64 pipe.  Peak = binary64
    # FMAs/s of this GPU measured now (m2cg_fp64_peak); achieved = the kernel's
    # FP64-pipe instructions per launch (per-cell count from the ncu profile x
    # cells) / its event-timed duration.  The ceiling: the measured peak / the
    # FP64-pipe instructions of one cell-stage summed over the stage kernels.
    dfma = C.c_double()
    fp64 = None
    slots = sum(v["fp64_pipe_inst_per_cell"] for v in profile.values())
    if lib.m2cg_fp64_peak(1 << 15, C.byref(dfma), None) == 0 and prof:
        inst = prof["fp64_pipe_inst_per_cell"] * cells / (per_launch_ms * 1e-3)
        flops = prof["fp64_flop_per_cell"] * cells / (per_launch_ms * 1e-3)
        fp64 = {"bound": "fp64", "kernel": dom, "achieved": inst / 1e9, "peak": dfma.value / 1e9,
                "unit": "G FP64-pipe inst/s", "frac": inst / dfma.value,
                "flop_rate_tflops": flops / 1e12, "flop_peak_tflops": 2 * dfma.value / 1e12,
                "fp64_pipe_inst_per_cell": prof["fp64_pipe_inst_per_cell"],
                "fp64_flop_per_cell": prof["fp64_flop_per_cell"],
                "peak_source": "measured now: m2cg_fp64_peak (independent binary64 FMA chains)",
                "counts_source": "ncu, profiles/" + ("k_recon_flux_tile_shock_bubble_128.txt" if fused
                                                     else "fp64_stage_kernels_shock_bubble_128.txt"),
                "step_fp64_pipe_inst_per_cell_stage": {k: v["fp64_pipe_inst_per_cell"] for k, v in profile.items()},
                "ceiling_cell_stage_per_s": dfma.value / slots,
                "value_over_ceiling": value / (dfma.value / slots)}
    elif dfma.value > 0:
        fp64 = {"bound": "fp64", "peak": dfma.value / 1e9, "unit": "G FP64-pipe inst/s", "achieved": None,
                "frac": None, "peak_source": "measured now: m2cg_fp64_peak",
                "ceiling_cell_stage_per_s": dfma.value / slots}

    # e2e through the C ABI with host buffers
    # as many end-to-end steps as timed steps (the steps right after them): the
    # per-step cost moves with the state, so a short window is not comparable
    e2e_steps = args.e2e_steps or max(2, args.steps)
    nb_v, nb_i, nb_p = cells * 5 * 8, cells * 4, cells * 8
    hv = lib.m2cg_host_alloc(nb_v)
    hi = lib.m2cg_host_alloc(nb_i)
    hp = lib.m2cg_host_alloc(nb_p)
    Vh = np.ctypeslib.as_array(C.cast(hv, C.POINTER(C.c_double)), shape=(cells * 5,))
    Ih = np.ctypeslib.as_array(C.cast(hi, C.POINTER(C.c_int32)), shape=(cells,))
    Ph = np.ctypeslib.as_array(C.cast(hp, C.POINTER(C.c_double)), shape=(cells,))
    abi.check(lib, lib.m2cg_download_state(ctx, abi.dptr(Vh), abi.iptr(Ih), abi.dptr(Ph)), "download")
    dt, cfl = C.c_double(), C.c_double()

    def e2e_step():
        abi.check(lib, lib.m2cg_upload_state(ctx, abi.dptr(Vh), abi.iptr(Ih), abi.dptr(Ph)), "upload")
        abi.check(lib, lib.m2cg_compute_dt(ctx, C.byref(dt), C.byref(cfl)), "dt")
        abi.check(lib, lib.m2cg_advance(ctx, dt.value), "advance")
        abi.check(lib, lib.m2cg_download_state(ctx, abi.dptr(Vh), abi.iptr(Ih), abi.dptr(Ph)), "download")

    e2e_step()
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    te = time.perf_counter() - t0
    barrier()
    te = max_over_ranks(pg, te)
    e2e_value = job_rate(world, cells, stages, e2e_steps, te)
    for p in (hv, hi, hp):
        lib.m2cg_host_free(p)

    # batched ensemble (its per-domain baseline is wall-timed: it runs before
    # the oracle leg starts on the host cores)
    ensres = None
    if args.ens_domains > 0 and rank == 0:
        ensres = ensemble_bench(args.ens_domains, args.ens_steps, args.ens_seq_steps)
    # the oracle leg runs on the host cores from here on, beside the
    # device-timed legs below
    oleg = OracleLeg(args, cfg, V, ID, phi, stages) if (not args.no_cpu and rank == 0) else None

    # learned warm start: batch study (interface problems drawn from the
    # warm-start distribution) and the same step with the network in the loop
    wsres = None
    ws_net = None
    if args.ws_train > 0 and rank == 0:
        from m2c_gb300 import warmstart as ws
        res, net = ws.study(n_train=args.ws_train, n_test=args.ws_test, epochs=args.ws_epochs, keep_net=True)
        # the same steps from the same initial state, with the network in the loop
        s2 = Solver(cfg, FluidState(V, ID, phi))
        s2.set_warm_start(net)
        s2.run(args.warmup)
        w0 = s2.counters()
        lib.m2cg_event_record(s2.ctx, 0)
        s2.run(args.steps)
        lib.m2cg_event_record(s2.ctx, 1)
        lib.m2cg_sync(s2.ctx)
        wms = C.c_float()
        abi.check(lib, lib.m2cg_event_elapsed(s2.ctx, 0, 1, C.byref(wms)), "elapsed")
        w1 = s2.counters()
        s2.set_warm_start(None)
        s2.close()
        wsolves = w1["riemann_solves"] - w0["riemann_solves"]
        res["fv_step"] = {"value_warm": cells * stages * args.steps / (wms.value * 1e-3), "unit": UNIT,
                          "value_cold": value,
                          "mean_iters_per_solve_warm": (w1["riemann_iterations"] - w0["riemann_iterations"]) /
                                                       max(wsolves, 1),
                          "mean_iters_per_solve_cold": iters / max(solves, 1),
                          "warm_solves": wsolves, "cold_solves": solves,
                          "note": "the same steps from the same initial state, cold and with the network"}
        wsres = res
        ws_net = net

    largeres = None
    if args.large > 0 and rank == 0:
        s.close()  # the large run needs the device memory of the 256^3 context
        largeres = large_bench(args.large, args.large_steps, net=ws_net)
    if ws_net is not None:
        ws_net.close()

    if rank != 0:
        return 0
    cpu, parity = None, None
    if oleg is not None:
        if largeres is None:
            s.close()   # the parity leg runs its own context from the initial state
        cpu, parity = oleg.finish()
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": f"shock-bubble {args.size}^3, SG/SG, MUSCL-van Albada, HLLC, exact interface "
                                  f"Riemann @1e-10, RK2, CFL 0.4", "cells": cells, "stages_per_step": stages,
                      "l2": "inputs %s than L2 (state 52 B/cell x %.1fM cells = %.2f GB per copy)" %
                            ("larger" if 52 * cells > 129e6 else "smaller", cells / 1e6, 52 * cells / 1e9),
                      "reinit_frequency": args.reinit if args.reinit > 0 else None,
                      "parallelism": "replicas" if world > 1 else "single"},
           "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": nb_v + nb_i + nb_p,
                   "d2h_bytes_per_step": nb_v + nb_i + nb_p, "steps": e2e_steps},
           "roofline": roof,
           "roofline_fp64": fp64,
           "cpu_baseline": cpu,
           "gpu_launches": int(launches),
           "clocks": clk,
           "riemann": {"solves": solves, "mean_iters_per_solve": iters / max(solves, 1),
                       "interface_faces_per_stage": (c1["interface_faces"] - c0["interface_faces"]) /
                                                     max(stages * args.steps, 1),
                       "errors": c1["riemann_errors"] - c0["riemann_errors"], "warm_start": "cold"},
           "warm_start": wsres,
           "ensemble": ensres,
           "large": largeres,
           "phase_ms_per_step": phase,
           "parity": parity,
           "counters": {k: c1[k] for k in ("clipped_cells", "nonphysical", "swept_cells", "unresolved_cells")}}
    print(json.dumps(out))
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
