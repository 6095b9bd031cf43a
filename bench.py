"""Benchmark: SWE cell-updates/s of the batched GPU form on 50k uneven patches.

Workload (the batching configuration): 224 x 224 = 50,176 patches with
subdivision drawn uniformly from {8, 16, 32, 64}^2 (67.8 M cells, FP64), sum of
32 Gaussians bathymetry with ~20% dry area, h = max(0, 1-b) + 0.1 U[-1,1],
reflecting walls, g = 9.81, CFL 0.5.  A step is one synchronous timestep of
every patch (ghost fill + f-wave sweep with CFL reduction + update), replayed
from a captured CUDA graph.  The 4.1 GB of patch state is far larger than L2,
so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--grid G] [--plain-steps P] [--no-e2e]

`--impl reference` times the CPU restatement of the reference path (the
reference's own SWE path cannot be built: Peano 3 and the TUM SWE sources are
absent) with all host threads on a bounded sample of the same workload.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "SWE cell-updates/s batched vs per-patch on 1 GB300; p50/p99 scenario latency"
UNIT = "cell-updates/s"

# Algorithmic FP64 work of one cell update (wet cell, subsonic edges), counted
# from the f-wave operation list of pcg_device.cuh (FMA = 2 flops, divide,
# reciprocal and square root = 1 flop each): per cell 8 ops (sqrt, 1/s, p, q,
# p^2, q^2, h + b, g/2 h); per edge 16 plain ops (9 adds, 3 multiplies,
# 2 cbar, sqrt, divide, reciprocal) + 2 FMA (2 edges per cell); accumulation
# 8 FMA; update 3 FMA.
FLOP_PER_CELL = 8 + 2 * (16 + 2 * 2) + 2 * 8 + 2 * 3
# the sweep's share (everything but the update's 3 FMA)
FLOP_PER_CELL_SWEEP = FLOP_PER_CELL - 2 * 3
# Algorithmic bytes per patch step: read h, hu, hv, b with halo, write h, hu, hv.
def bytes_per_patch(n):
    return 8 * (4 * (n + 2) ** 2 + 3 * n * n)


def profile_figure(name, key):
    """A figure recorded in a committed ncu summary under profiles/ as
    `key: value` (None when absent)."""
    try:
        for line in open(os.path.join(ROOT, "profiles", name)):
            if line.startswith(key + ":"):
                return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


# FP64 instructions per cell update of the strip sweep (ncu count, see
# profiles/k_sweep_strips_uneven_patches_4k.md) and the FP64 pipe width of
# GB300 (FP64 lanes per clock per SM; the DFMA probe reaches it).
FP64_INST_PER_CELL = profile_figure("k_sweep_strips_uneven_patches_4k.md", "fp64_inst_per_cell_update") or 46.2
FP64_LANES_PER_SM_CLK = 2


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--grid", type=int, default=224)
    ap.add_argument("--plain-steps", type=int, default=2)
    ap.add_argument("--cpu-sample-grid", type=int, default=48)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default batched schedule instead of autotuning it")
    ap.add_argument("--schedule", default="",
                    help="fix the schedule instead of autotuning: tiles/VARIANT or "
                         "strips/VARIANT/CHUNK[/fused|unfused|pipelined]")
    ap.add_argument("--form", default="auto", choices=["auto", "fused", "unfused", "pipelined"],
                    help="step form: the autotuner's pick, or the fused / unfused form on the default "
                         "strip schedule (no autotuning)")
    ap.add_argument("--config-legs", default="",
                    help="comma-separated subset of the configuration legs to run (default: all)")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the secondary configurations (dam break, AMR, serving)")
    ap.add_argument("--amr-steps", type=int, default=500)
    ap.add_argument("--remesh-steps", type=int, default=300)
    ap.add_argument("--remesh-every", type=int, default=10)
    ap.add_argument("--lts-t-end", type=float, default=0.02)
    ap.add_argument("--serve-requests", type=int, default=128)
    ap.add_argument("--serve-rate", type=float, default=8.0)
    ap.add_argument("--serve-batch", type=int, default=32,
                    help="batched steps per replay of the step graph in the serving loop")
    return ap.parse_args()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def dist_init(ws):
    if ws <= 1:
        return None
    import torch
    import torch.distributed as dist
    backend = "nccl" if torch.cuda.is_available() else "gloo"
    dist.init_process_group(backend=backend)
    return dist


def dist_max(dist, v):
    if dist is None:
        return v
    import torch
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_barrier(dist):
    if dist is not None:
        dist.barrier()


def build_context(ps, prm):
    from peanoclaw_gb300 import pcg as P
    slab = int(sum(P.vector_size(n) + 32 for n in ps.n)) + 4096
    ctx = P.Context(slab_doubles=slab, max_patches=len(ps) + 16, max_groups=1, params=prm)
    ids = []
    for p in range(len(ps)):
        pid = ctx.alloc(ps.n[p], pos=ps.pos[p], size=ps.size[p], level=ps.level[p])
        if ps.wall[p]:
            ctx.set_boundary(pid, ps.wall[p])
        ids.append(pid)
    from peanoclaw_gb300.scenarios import remap_items
    ctx.set_ghost_items(remap_items(ps.items, ids))
    return ctx, ids


# Arm CPU part numbers (MIDR part field) of the host CPUs this runs on
ARM_PARTS = {"0xd4f": "Arm Neoverse-V2 (NVIDIA Grace)", "0xd40": "Arm Neoverse-V1",
             "0xd0c": "Arm Neoverse-N1", "0xd49": "Arm Neoverse-N2", "0xd8e": "Arm Neoverse-N3",
             "0xd84": "Arm Neoverse-V3"}


def cpu_model():
    """Model name of the host CPU: lscpu's, else /proc/cpuinfo's model name or
    Arm part number."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name:"):
                name = line.split(":", 1)[1].strip()
                if name and name != "-":
                    return name
    except Exception:
        pass
    try:
        for line in open("/proc/cpuinfo"):
            low = line.lower()
            if low.startswith("model name"):
                return line.split(":", 1)[1].strip()
            if low.startswith("cpu part"):
                part = line.split(":", 1)[1].strip()
                return ARM_PARTS.get(part, "Arm CPU part " + part)
    except OSError:
        pass
    return ""


def parity_check(ps, prm, steps=3):
    """In-run comparison of the batched GPU step with the FP64 oracle on a
    patch set: both advance `steps` steps from the same state; returns the
    largest absolute and relative differences over every patch vector (ghost
    layers included) and whether all bits agree."""
    from oracle import oracle as O
    from peanoclaw_gb300 import pcg as P
    oprm = O.swe_params(prm.g, prm.cfl, prm.dry_tol, prm.dry_tol_update, prm.s_min, prm.dt_inf)
    pats = []
    for p in range(len(ps)):
        op = O.Patch(ps.n[p], pos=ps.pos[p], size=ps.size[p])
        op.u[:] = ps.vector(p)
        pats.append(op)
    odts = [float(O.grid_step(pats, ps.items, ps.wall, oprm, 1e9)[0]) for _ in range(steps)]
    ref = np.concatenate([p.u for p in pats])
    ctx, ids = build_context(ps, prm)
    try:
        ctx.upload_many(ids, ps.packed)
        ctx.set_group_max_dt(0, 1e9)
        dts = [float(d) for d in ctx.run(steps, P.PCG_MODE_BATCHED)[:, 0]]
        got = ctx.download_many(ids, int(ps.packed.size))
    finally:
        ctx.close()
    diff = np.abs(got - ref)
    scale = np.maximum(np.abs(ref), 1e-300)
    return {"vs": "FP64 CPU oracle (oracle/pcoracle.c), measured in this run",
            "sample": "%d patches, %d cells, %d steps" % (len(ps), ps.cells(), steps),
            "max_abs_error": float(diff.max()), "max_rel_error": float((diff / scale).max()),
            "dt_equal": dts == odts,
            "bit_exact": bool(np.array_equal(got.view(np.int64), ref.view(np.int64)))}


def cpu_baseline(args, prm, seconds_target=15.0, fp32_seconds=6.0):
    """The oracle (CPU restatement, OpenMP over patches, all host threads) on a
    bounded sample of the same generator: a G x G slot mosaic.  Timed twice:
    the FP64 restatement (the arithmetic of the GPU path) and its FP32 twin
    (the reference's float storage and arithmetic), each with all threads and
    with one."""
    from oracle import oracle as O
    from peanoclaw_gb300 import scenarios as S
    ps = S.uneven_patches(grid=args.cpu_sample_grid)

    def patches():
        out = []
        for p in range(len(ps)):
            op = O.Patch(ps.n[p], pos=ps.pos[p], size=ps.size[p])
            op.u[:] = ps.vector(p)
            out.append(op)
        return out

    oprm = O.swe_params(prm.g, prm.cfl, prm.dry_tol, prm.dry_tol_update, prm.s_min, prm.dt_inf)
    threads = os.cpu_count() or 1
    cells = ps.cells()

    def timed(step, target, n_threads, max_steps):
        step(n_threads)  # warm-up
        steps = 0
        t0 = time.perf_counter()
        while True:
            step(n_threads)
            steps += 1
            el = time.perf_counter() - t0
            if el > target or steps >= max_steps:
                return steps, el

    pats = patches()
    f64 = lambda n: O.grid_step(pats, ps.items, ps.wall, oprm, 1e9, n_threads=n)
    steps, el = timed(f64, seconds_target, threads, 200)
    s1, el1 = timed(f64, max(2.0, seconds_target / 5), 1, 3)
    pats32 = patches()
    u32 = [np.ascontiguousarray(p.u.astype(np.float32)) for p in pats32]
    f32 = lambda n: O.grid_step_f32(pats32, u32, ps.items, ps.wall, oprm, 1e9, n_threads=n)
    steps32, el32 = timed(f32, fp32_seconds, threads, 400)
    s132, el132 = timed(f32, max(1.0, fp32_seconds / 4), 1, 3)
    return {"value": cells * steps / el, "unit": UNIT, "cores": threads, "kind": "port",
            "dtype": "f64", "single_core_value": cells * s1 / el1,
            "fp32_value": cells * steps32 / el32, "fp32_single_core_value": cells * s132 / el132,
            "cpu": cpu_model(),
            "sample": "%dx%d-slot mosaic of the same generator (%d patches, %d cells), "
                      "FP64 %d steps in %.1f s, FP32 twin %d steps in %.1f s"
                      % (args.cpu_sample_grid, args.cpu_sample_grid, len(ps), cells, steps, el,
                         steps32, el32)}


def cpu_configs(prm):
    """The oracle on the other configurations, FP64 with all host threads and
    with one, and the FP32 twin (the reference's float precision) with all
    threads: the 9x9x16^2 radial dam break (all 100 steps), the 3-level
    breaking dam (27^2 cells per patch, flux correction and restriction in
    the FP64 step) and the coastal tsunami (base 27, 27^2 cells per patch,
    3 levels, the same), each over a bounded number of steps."""
    from oracle import oracle as O
    from peanoclaw_gb300 import scenarios as S
    oprm = O.swe_params(prm.g, prm.cfl, prm.dry_tol, prm.dry_tol_update, prm.s_min, prm.dt_inf)
    threads = os.cpu_count() or 1
    out = {"cores": threads, "cpu": cpu_model(), "kind": "port"}

    def oracle_set(ps):
        pats = []
        for p in range(len(ps)):
            leaf = bool(ps.leaf[p]) if hasattr(ps, "leaf") else True
            op = O.Patch(ps.n[p], pos=ps.pos[p], size=ps.size[p], level=ps.level[p], is_leaf=leaf,
                         is_virtual=not leaf)
            op.u[:] = ps.vector(p)
            if not leaf:
                op.s.restr_lower[0], op.s.restr_lower[1] = ps.restr_lower[p]
                op.s.restr_upper[0], op.s.restr_upper[1] = ps.restr_upper[p]
            pats.append(op)
        return pats

    def timed(step, n_steps):
        step()
        t0 = time.perf_counter()
        for _ in range(n_steps):
            step()
        return time.perf_counter() - t0

    cases = (("radial_dam_break_9x9x16", lambda: S.radial_dam_break(npx=9, n=16), 100, 100, 100),
             ("adaptive_breaking_dam_3_levels", lambda: S.breaking_dam_amr(base=9, n=27, levels=3), 20, 3, 20),
             ("coastal_tsunami_3_levels", lambda: S.coastal_tsunami(), 6, 2, 6))
    for name, make, k_all, k_one, k32 in cases:
        ps = make()
        amr = hasattr(ps, "leaf")
        cells = ps.meta.get("leaf_cells", ps.cells())
        pats = oracle_set(ps)
        if amr:
            O.restrict_list(pats, ps.restrict_items)

        def f64(n):
            if amr:
                return O.amr_step(pats, ps.items, ps.wall, ps.leaf, ps.flux_items, ps.restrict_items, oprm,
                                  1e9, n_threads=n)
            return O.grid_step(pats, ps.items, ps.wall, oprm, 1e9, n_threads=n)

        el = timed(lambda: f64(threads), k_all)
        el1 = timed(lambda: f64(1), k_one)
        pats32 = oracle_set(ps)
        u32 = [np.ascontiguousarray(p.u.astype(np.float32)) for p in pats32]
        el32 = timed(lambda: O.grid_step_f32(pats32, u32, ps.items, ps.wall, oprm, 1e9, n_threads=threads), k32)
        out[name] = {"cells": cells, "fp64": cells * k_all / el, "fp64_single_core": cells * k_one / el1,
                     "fp32": cells * k32 / el32,
                     "sample": "%d / %d / %d steps (FP64 all threads / FP64 one thread / FP32 twin)"
                               % (k_all, k_one, k32),
                     "note": ("FP64 steps include flux correction and restriction; the FP32 twin "
                              "times ghost fill, sweep and update" if amr else "")}
    return out


def bench_radial(prm):
    """9 x 9 patches of 16 x 16 cells, radial dam break, 100 steps: batched and plain."""
    from peanoclaw_gb300 import pcg as P
    from peanoclaw_gb300 import scenarios as S
    out = {}
    for mode, name in ((P.PCG_MODE_BATCHED, "batched"), (P.PCG_MODE_PLAIN, "plain")):
        ps = S.radial_dam_break(npx=9, n=16)
        ctx, ids = build_context(ps, prm)
        ctx.upload_many(ids, ps.packed)
        ctx.set_group_max_dt(0, 1e9)
        if mode == P.PCG_MODE_BATCHED:
            # the schedule autotuner, then the initial state again (it advanced it)
            tuned = ctx.autotune(reps=3)
            out["schedule"] = "%d/%d/%d/%d" % ctx.get_schedule()
            out["autotune"] = {"%d/%d/%d/%d" % k: m for k, m in tuned}
            ctx.upload_many(ids, ps.packed)
            for p in ids:
                ctx.set_time(p, time=0.0, dt=0.0, est_next=0.0)
            ctx.set_group_end_time(0, 0.0, np.inf)
        c0, m0 = ctx.stats()
        ctx.run(100, mode)
        c1, m1 = ctx.stats()
        ctx.close()
        out[name] = ps.cells() * 100 / ((m1 - m0) / 1e3)
    out["cells"] = 81 * 256
    out["steps"] = 100
    return out


def bench_amr(prm, steps):
    """Adaptive breaking dam: 3 levels of 3x refinement, 27 x 27 cells per patch,
    ghost interpolation, flux correction and restriction in every step."""
    from peanoclaw_gb300 import pcg as P
    from peanoclaw_gb300 import scenarios as S
    ps = S.breaking_dam_amr(base=9, n=27, levels=3)
    slab = int(sum(P.vector_size(n) + 32 for n in ps.n)) + 4096
    res = {"patches": len(ps), "leaves": int(sum(ps.leaf)), "leaf_cells": ps.meta["leaf_cells"]}
    for mode, name, k in ((P.PCG_MODE_BATCHED, "batched", steps), (P.PCG_MODE_PLAIN, "plain", 5)):
        ctx = P.Context(slab_doubles=slab, max_patches=len(ps) + 16, max_groups=1, params=prm)
        S.install_amr(ctx, ps)
        ctx.restrict_all()
        ctx.set_group_max_dt(0, 1e9)
        if mode == P.PCG_MODE_BATCHED:
            # the schedule autotuner (untimed; it advances the simulation)
            res["autotune"] = {"%s/%d/%d%s" % ("tiles" if k[0] == 0 else "strips", k[1], k[2],
                                               ("", "/unfused", "/pipelined")[k[3]]): m
                               for k, m in ctx.autotune(reps=2)}
            res["schedule"] = "%d/%d/%d" % ctx.get_schedule()[:3]
        ctx.run(3, mode)
        c0, m0 = ctx.stats()
        ctx.run(k, mode)
        c1, m1 = ctx.stats()
        ctx.close()
        res[name] = ps.meta["leaf_cells"] * k / ((m1 - m0) / 1e3)
        res[name + "_ms_per_step"] = (m1 - m0) / k
    return res


def bench_lts(prm, t_end):
    """Local time stepping against the synchronous step on the adaptive
    breaking dam (3 levels of 3x refinement, 27 x 27 cells per patch, ghost
    interpolation and restriction, no flux correction in either run): both
    advance every leaf to the same end time; reported are the cell updates
    spent, the device time to solution and the iterations / steps."""
    from peanoclaw_gb300 import pcg as P
    from peanoclaw_gb300 import scenarios as S
    ps = S.breaking_dam_amr(base=9, n=27, levels=3)
    slab = int(sum(P.vector_size(n) + 32 for n in ps.n)) + 4096
    res = {"patches": len(ps), "leaves": int(sum(ps.leaf)), "leaf_cells": ps.meta["leaf_cells"], "t_end": t_end}
    for ts, name in ((P.TS_LOCAL, "local"), (P.TS_GLOBAL, "global")):
        ctx = P.Context(slab_doubles=slab, max_patches=len(ps) + 16, max_groups=1, params=prm)
        try:
            S.install_amr(ctx, ps, flux=False)
            ctx.restrict_all()
            ctx.set_group_max_dt(0, np.inf)
            ctx.set_group_end_time(0, 0.0, t_end)
            ctx.set_time_stepping(ts)
            if ts == P.TS_LOCAL:
                # one iteration advances few leaves: 16x16 tiles (many short
                # work items) beat the warp strips' long column marches here
                ctx.set_schedule(P.SCHED_TILES)
            ctx.synchronize()
            c0, m0 = ctx.stats()
            t0 = time.perf_counter()
            iters = 0
            while float(ctx.group_times()[0]) < t_end and iters < 100000:
                hist = ctx.run(64, P.PCG_MODE_BATCHED)
                iters += int(np.count_nonzero(hist[:, 0] > 0.0))
            ctx.synchronize()
            wall = time.perf_counter() - t0
            c1, m1 = ctx.stats()
            res[name] = {"iterations": iters, "cell_updates": int(c1 - c0), "device_ms": m1 - m0,
                         "wall_ms": wall * 1e3, "cell_updates_per_s": (c1 - c0) / ((m1 - m0) / 1e3),
                         "reached": float(ctx.group_times()[0])}
        finally:
            ctx.close()
    return res


def bench_remesh(prm, steps, every):
    """The large adaptive batched run: coastal tsunami with dynamic
    remeshing, 3 levels of 3x refinement, 27 x 27 cells per patch, base
    27 x 27 patches (an effective 6561^2 grid), Gaussian surface hump over the
    sum-of-Gaussians seafloor (seed 2000) with a coastline along x = 1; the
    device surface criterion is evaluated and the grid remeshed every `every`
    steps (new patches interpolated, coarsened ones restricted, lists
    rebuilt)."""
    from peanoclaw_gb300 import pcg as P
    from peanoclaw_gb300 import scenarios as S
    from peanoclaw_gb300.amr import DeviceAmr
    ps = S.coastal_tsunami()
    full = 729 + 6561 + 59049
    ctx = P.Context(slab_doubles=int(full * (P.vector_size(27) + 32)) + (1 << 20), max_patches=full + 64,
                    max_groups=1, params=prm)
    try:
        ids = S.install_amr(ctx, ps)
        ctx.restrict_all()
        ctx.set_group_max_dt(0, 1e9)
        dev = DeviceAmr(ctx, ps.grid, ps.b_of, criterion=ps.criterion)
        dev.pid = dict(zip(ps.grid.order(), (int(i) for i in ids)))
        ctx.run(2, P.PCG_MODE_BATCHED)
        ctx.synchronize()
        cu = 0
        leaf_cells, patches, remesh_s = [], [], []
        _, ms0 = ctx.stats()
        t0 = time.perf_counter()
        for r in range(max(1, steps // every)):
            lc = sum(ps.grid.n ** 2 for _ in ps.grid.leaves())
            leaf_cells.append(lc)
            patches.append(len(dev.pid))
            ctx.run(every, P.PCG_MODE_BATCHED)
            cu += lc * every
            t1 = time.perf_counter()
            dev.remesh()
            remesh_s.append(time.perf_counter() - t1)
        ctx.synchronize()
        wall = time.perf_counter() - t0
        _, ms1 = ctx.stats()
    finally:
        ctx.close()
    dev_s = (ms1 - ms0) / 1e3
    return {"steps": steps, "remesh_every": every, "patches_min": min(patches), "patches_max": max(patches),
            "leaf_cells_min": min(leaf_cells), "leaf_cells_max": max(leaf_cells),
            "device_cell_updates_per_s": cu / dev_s, "wall_cell_updates_per_s": cu / wall,
            "remesh_s_mean": float(np.mean(remesh_s)), "wall_s": wall}


def bench_serving(args, prm, batched_value=None):
    """Scenario stream with Poisson arrivals (seed 42): radial dam breaks and
    Gaussian-hump tsunamis, 1e4..4e6 cells (the finest level's effective
    resolution), 1-3 levels of adaptive 3x refinement (adaptive requests keep
    their hierarchy on the device and remesh every 32 of their steps), end
    time U[0.05, 0.5]."""
    from peanoclaw_gb300 import serving as SV
    reqs = SV.make_requests(args.serve_requests, rate=args.serve_rate, seed=42, n=32, levels=(1, 3))
    need = sum(int(r.cells * 1.4) for r in reqs)
    srv = SV.Server(slab_doubles=int(need * 8) + (1 << 24), max_groups=32, max_patches=400000, params=prm,
                    steps_per_batch=args.serve_batch, remesh_every=max(32, args.serve_batch))
    try:
        _, ms0 = srv.ctx.stats()
        done, wall = srv.serve(reqs, max_wall=300.0)
        _, ms1 = srv.ctx.stats()
        remesh_s, relist_s, remeshes = srv.remesh_s, srv.relist_s, srv.remeshes
    finally:
        srv.close()
    lat = np.array([r.finished - r.arrival for r in done])
    cu = sum(r.cell_updates for r in done)
    value = cu / wall
    return {"requests": len(reqs), "completed": len(done), "rate_per_s": args.serve_rate,
            "adaptive_requests": int(sum(r.levels > 1 for r in reqs)),
            "levels": {str(k): int(sum(r.levels == k for r in reqs)) for k in (1, 2, 3)},
            "p50_s": float(np.percentile(lat, 50)) if len(lat) else None,
            "p99_s": float(np.percentile(lat, 99)) if len(lat) else None,
            "cell_updates_per_s": value, "wall_s": wall,
            "device_busy": (ms1 - ms0) / 1e3 / wall, "remesh_s": remesh_s, "remeshes": remeshes,
            "remesh_relist_s": relist_s,
            "vs_batched_50k": (value / batched_value) if batched_value else None,
            "max_concurrent_groups": 32, "steps_per_batch": args.serve_batch}


def run_reference(args):
    ws, rank, _ = dist_info()
    if rank != 0:
        return 0
    from peanoclaw_gb300 import pcg as P
    prm = P.swe_params(g=9.81, cfl=0.5)
    t = max(5.0, min(60.0, 2.0 * args.steps))
    cb = cpu_baseline(args, prm, seconds_target=t / 2, fp32_seconds=t)
    # the reference stores and computes the SWE block in float: its arm is
    # the FP32 twin; the FP64 restatement's figure rides along
    ref = dict(cb, value=cb["fp32_value"], single_core_value=cb["fp32_single_core_value"],
               dtype="f32", fp64_value=cb["value"], fp64_single_core_value=cb["single_core_value"])
    for k in ("fp32_value", "fp32_single_core_value"):
        ref.pop(k)
    cb = ref
    line = {"metric": METRIC, "value": cb["value"], "unit": UNIT, "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": "uneven patches, sample of the 224x224-slot mosaic",
                       "sample_grid": args.cpu_sample_grid},
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    ws, rank, local = dist_info()
    dist = dist_init(ws)
    from peanoclaw_gb300 import pcg as P
    from peanoclaw_gb300 import scenarios as S
    prm = P.swe_params(g=9.81, cfl=0.5)
    ps = S.uneven_patches(grid=args.grid)
    cells = ps.cells()
    ctx, ids = build_context(ps, prm)
    ctx.upload_many(ids, ps.packed)
    ctx.set_group_max_dt(0, 1e9)

    # warm-up, the schedule autotuner (untimed; it advances the simulation by
    # one or two steps per candidate) and the graph instantiation
    if args.form in ("fused", "unfused"):
        ctx.set_step_form(P.FORM_UNFUSED if args.form == "unfused" else P.FORM_AUTO)
    forms = {"fused": P.STRIPS_FUSED, "unfused": P.STRIPS_UNFUSED, "pipelined": P.STRIPS_PIPELINED}
    if args.schedule:
        f = args.schedule.split("/")
        kind = P.SCHED_TILES if f[0] == "tiles" else P.SCHED_STRIPS
        ctx.set_schedule(kind, int(f[1]) if len(f) > 1 else 0, int(f[2]) if len(f) > 2 else 32,
                         forms[f[3]] if len(f) > 3 else 0)
    elif args.form == "pipelined":
        ctx.set_schedule(P.SCHED_STRIPS, 2, 32, P.STRIPS_PIPELINED)
    ctx.run(max(1, args.warmup), P.PCG_MODE_BATCHED)
    tuned = None
    if not args.no_autotune and args.form == "auto" and not args.schedule:
        tuned = ctx.autotune(reps=2)
        ctx.run(2, P.PCG_MODE_BATCHED)
    sched = ctx.get_schedule()
    fused = ctx.step_is_fused(P.PCG_MODE_BATCHED)
    pipelined = sched[0] == P.SCHED_STRIPS and sched[3] == P.STRIPS_PIPELINED
    form = "pipelined" if pipelined else "fused" if fused else "unfused"
    step_launches = ctx.step_launches()
    dist_barrier(dist)
    ctx.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    cu0, ms0 = ctx.stats()
    t0 = time.perf_counter()
    ctx.run(args.steps, P.PCG_MODE_BATCHED)
    ctx.synchronize()
    wall = time.perf_counter() - t0
    cu1, ms1 = ctx.stats()
    dev_ms = ms1 - ms0
    clk = clocks.stop()
    dist_barrier(dist)
    dev_s = dist_max(dist, dev_ms / 1e3)
    value = ws * cells * args.steps / dev_s
    ms_per_step = dev_s * 1e3 / args.steps

    # per-phase device time of the batched step (CUDA events on the launch stream)
    phases = np.array([ctx.profile_step() for _ in range(5)])
    ph = phases.mean(axis=0)
    sweep_ms = float(ph[3])
    update_ms = float(ph[4])
    fp64_peak = ctx.fp64_peak_tflops()
    import torch
    sm_count = torch.cuda.get_device_properties(local).multi_processor_count
    # dominant kernel: the sweep (unfused form: k_sweep_strips / k_sweep_tiles,
    # the sweep's flops), the fused sweep (k_fused_strips: ghost fill,
    # deferred update and sweep, all flops of a cell update) or the pipelined
    # step (k_pipeline_step: update of one step with fill, walls and sweep of
    # the next, all flops of a cell update); its average launch duration from
    # CUDA events on the launch stream
    dom_flop = FLOP_PER_CELL if (fused or pipelined) else FLOP_PER_CELL_SWEEP
    achieved = (dom_flop * cells / 1e12) / (sweep_ms / 1e3)
    step_achieved = FLOP_PER_CELL * cells / 1e12 / (ms_per_step / 1e3)
    if pipelined:
        dom_kernel = "k_pipeline_step"
    elif fused:
        dom_kernel = "k_fused_strips"
    else:
        dom_kernel = "k_sweep_tiles" if sched[0] == P.SCHED_TILES else "k_sweep_strips"
    alg_bytes = sum(bytes_per_patch(n) for n in ps.n)
    hbm_peak = None
    try:
        mp = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        hbm_peak = mp.get("hbm_gbs")
    except Exception:
        pass
    step_ms_phase = float(ph.sum())
    # DRAM traffic of the dominant kernel (sweep): bytes per cell update from
    # the ncu capture of the small case, scaled to this launch's cells
    prof = {"k_fused_strips": "k_fused_strips_uneven_patches_4k.md",
            "k_sweep_strips": "k_sweep_strips_uneven_patches_4k.md",
            "k_pipeline_step": "k_pipeline_step_uneven_patches_4k.md"}.get(dom_kernel)
    tpc = profile_figure(prof, "traffic_bytes_per_cell_update") if prof else None
    traffic = tpc * cells if tpc is not None else None
    fp64_ipc = (profile_figure(prof, "fp64_inst_per_cell_update") if prof else None) or FP64_INST_PER_CELL

    # plain per-patch form (one launch per patch per phase), same workload
    plain = None
    if args.plain_steps > 0:
        ctx.run(1, P.PCG_MODE_PLAIN)
        ctx.synchronize()
        c0, m0 = ctx.stats()
        ctx.run(args.plain_steps, P.PCG_MODE_PLAIN)
        c1, m1 = ctx.stats()
        plain = cells * args.plain_steps / ((m1 - m0) / 1e3)

    # end to end through the C ABI with host buffers: pinned upload of the
    # state, `steps` timesteps (the dt of every step read back), download.
    e2e = None
    if not args.no_e2e:
        import torch
        pinned = torch.empty(ps.packed.size, dtype=torch.float64, pin_memory=True).numpy()
        pinned[:] = ps.packed
        out = torch.empty(ps.packed.size, dtype=torch.float64, pin_memory=True).numpy()
        import ctypes as C
        idarr = np.ascontiguousarray(ids, dtype=np.int32)

        def job():
            P.check(P.lib().pcg_patches_upload(ctx.h, len(ids), idarr.ctypes.data_as(C.POINTER(C.c_int32)),
                                               pinned.ctypes.data_as(C.POINTER(C.c_double))))
            h = ctx.run(args.steps, P.PCG_MODE_BATCHED)
            P.check(P.lib().pcg_patches_download(ctx.h, len(ids), idarr.ctypes.data_as(C.POINTER(C.c_int32)),
                                                 out.ctypes.data_as(C.POINTER(C.c_double))))
            return h

        job()  # warm-up job (untimed): first-touch costs of the host buffers and copy paths
        jobs_s = []
        for _ in range(3):
            ctx.synchronize()
            t0 = time.perf_counter()
            hist = job()
            jobs_s.append(dist_max(dist, time.perf_counter() - t0))
        e2e_s = float(np.median(jobs_s))
        nbytes = int(ps.packed.nbytes)
        e2e = {"value": ws * cells * args.steps / e2e_s, "unit": UNIT,
               "h2d_bytes_per_step": nbytes // args.steps,
               "d2h_bytes_per_step": nbytes // args.steps + 8,
               "jobs_s": jobs_s,
               "note": "one job = pinned upload of all patch vectors + %d timesteps (dt read back "
                       "each step) + download; median of 3 timed jobs after one untimed job (the host "
                       "link's rate varies from run to run); bytes are per timestep" % args.steps}
        assert np.isfinite(hist).all()

    ctx.close()
    cpu = cpu_cfg = parity = None
    if rank == 0 and not args.no_cpu and ws == 1:
        cpu = cpu_baseline(args, prm)
        parity = parity_check(S.uneven_patches(grid=args.cpu_sample_grid), prm)
        cpu_cfg = cpu_configs(prm)
    configs = None
    if rank == 0 and not args.no_configs:
        legs = {"radial_dam_break_9x9x16": lambda: bench_radial(prm),
                "adaptive_breaking_dam_3_levels": lambda: bench_amr(prm, args.amr_steps),
                "adaptive_tsunami_remesh": lambda: bench_remesh(prm, args.remesh_steps, args.remesh_every),
                "serving_stream": lambda: bench_serving(args, prm, value / ws),
                "local_time_stepping_breaking_dam": lambda: bench_lts(prm, args.lts_t_end)}
        only = set(args.config_legs.split(",")) if args.config_legs else set(legs)
        configs = {k: f() for k, f in legs.items() if k in only}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "batched step (%s form, CUDA graph), 50k uneven patches "
                                   "(%d patches, {8,16,32,64}^2 cells, %d cells, %.1f%% dry), "
                                   "radial-free random Gaussian bathymetry, 200-step config "
                                   "timed over %d steps" % (form, len(ps), cells,
                                                            100 * ps.meta["dry_fraction"], args.steps),
                       "patches": len(ps), "cells": cells, "grid_slots": args.grid,
                       "l2": "inputs (%.1f GB) larger than L2, no flush" % (ps.packed.nbytes / 1e9),
                       "parallelism": "replicas x%d" % ws if ws > 1 else "1 GPU"},
            "roofline": {"bound": "fp64", "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                         "frac": achieved / fp64_peak, "traffic": traffic,
                         "kernel": dom_kernel,
                         "achieved_note": "%d algorithmic flops per cell x %d cells / the kernel's mean "
                                          "CUDA-event time (%.3f ms)" % (dom_flop, cells, sweep_ms),
                         "step_frac": step_achieved / fp64_peak,
                         "step_note": "%d flops per cell update x cells / ms_per_step, the whole step"
                                      % FLOP_PER_CELL,
                         "traffic_note": ("constant from a profile: DRAM bytes per cell of the ncu capture "
                                          "on the 4k-patch case (profiles/%s) x cells" % prof) if prof else None,
                         "fp64_pipe_frac": (fp64_ipc * cells / (sweep_ms / 1e3) /
                                            (FP64_LANES_PER_SM_CLK * sm_count * (clk.get("sm_mhz") or 2070.0) * 1e6)),
                         "fp64_pipe_note": "FP64 instructions per cell from the same profile (a constant) x cells "
                                           "/ kernel time / (2 FP64 lanes x SMs x median SM clock)",
                         "peak_source": "measured live (DFMA chain probe, FMA = 2 flops)",
                         "flop_per_cell": FLOP_PER_CELL,
                         "hbm": {"achieved_gbs": alg_bytes / (step_ms_phase / 1e3) / 1e9,
                                 "peak_gbs": hbm_peak, "peak_source": "MEASURED_PEAKS.json",
                                 "alg_bytes_per_step": alg_bytes}},
            "phase_ms": ({"pre": ph[0], "pipelined_step": ph[3], "first_launch_fill_sweep": ph[1],
                          "last_launch_update": ph[2]} if pipelined else
                         {"reset": ph[0], "fused_sweep": ph[3], "advance": ph[4]} if fused else
                         {"reset": ph[0], "ghost_items": ph[1], "walls": ph[2], "sweep": ph[3],
                          "update": ph[4]}),
            "schedule": {"kind": "tiles" if sched[0] == P.SCHED_TILES else "strips",
                         "variant": sched[1], "chunk": sched[2],
                         "form": form,
                         "autotune_ms_per_step": ({"%s/%d/%d%s" % ("tiles" if k[0] == 0 else "strips", k[1], k[2],
                                                                 ("", "/unfused", "/pipelined")[k[3]]): m
                                                   for k, m in tuned} if tuned else None)},
            "parity": parity,
            "plain_per_patch_value": plain,
            "batched_over_plain": (value / ws) / plain if plain else None,
            "e2e": e2e,
            "cpu_baseline": cpu,
            "cpu_configs": cpu_cfg,
            "configs": configs,
            "clocks": clk,
            "gpu_launches": step_launches * (args.steps + (1 if pipelined else 0)),
            "gpu_launches_note": ("kernel nodes of the captured step graph (pcg_get_step_launches, "
                                  "%d) x %s" % (step_launches, "(timed steps + 1): a pipelined run of K steps "
                                                "replays it K + 1 times" if pipelined else "timed steps")),
            "wall_s": wall,
        }
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
