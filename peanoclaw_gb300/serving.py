"""Continuous-batching scenario server on one GPU.

Independent SWE scenario solves (radial dam breaks and Gaussian-hump
tsunamis of different sizes and end times) are admitted while others are
running, as soon as a group slot and enough free HBM in the context's slab
are available.  Every resident scenario is one *group* of patches: all groups
advance together in the same batched launches (ghost fill, sweep, update), each
with its own CFL timestep (dt reduced per group on the device) and its own end
time, so a scenario's result does not depend on what else is in the batch.
A finished scenario's state is read back and its patches are freed, which
admits the next waiting requests.
"""
import time
from dataclasses import dataclass, field

import numpy as np

from . import pcg as P
from .scenarios import PatchSet, _build_grid_items, _centers, remap_items


@dataclass
class Request:
    rid: int
    kind: str            # "dam_break" | "tsunami"
    cells: int           # requested total cells
    t_end: float
    arrival: float       # seconds after the server start
    n: int = 16          # cells per patch edge
    npx: int = 0         # patches per domain edge (derived)
    seed: int = 0
    # filled by the server
    admitted: float = None
    finished: float = None
    steps: int = 0
    cell_updates: int = 0
    result: np.ndarray = None
    group: int = -1
    ids: list = field(default_factory=list)


def scenario_patchset(req):
    """Uniform grid of npx x npx patches of n x n cells on [0,1]^2 with walls."""
    n = req.n
    npx = max(1, int(round(np.sqrt(req.cells) / n)))
    req.npx = npx
    ps = PatchSet()
    L = 1.0 / npx
    grid = np.zeros((npx, npx), dtype=np.int64)
    for i in range(npx):
        for j in range(npx):
            grid[i, j] = len(ps.n)
            ps.n.append(n)
            ps.pos.append((i * L, j * L))
            ps.size.append((L, L))
            ps.level.append(0)
            m = 0
            if i == 0: m |= 1
            if i == npx - 1: m |= 2
            if j == 0: m |= 4
            if j == npx - 1: m |= 8
            ps.wall.append(m)
    ps.finalize_layout()
    rng = np.random.default_rng(req.seed)
    cx, cy = rng.uniform(0.3, 0.7, 2)
    for p in range(len(ps)):
        unew, uold, b = ps.views(p)
        X, Y = _centers(ps.pos[p], ps.size[p], n, ghost=True)
        if req.kind == "dam_break":
            r = np.sqrt((X - cx) ** 2 + (Y - cy) ** 2)
            b[:] = 0.0
            unew[0] = np.where(r[1:-1, 1:-1] <= 0.15, 2.0, 1.0)
        else:
            # Gaussian surface hump (amplitude 0.5, sigma 0.05) over a small
            # Gaussian seafloor bump
            bb = 0.1 * np.exp(-((X - 0.5) ** 2 + (Y - 0.5) ** 2) / (2 * 0.2 ** 2))
            b[:] = bb
            eta = 1.0 + 0.5 * np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2 * 0.05 ** 2))
            unew[0] = (eta - bb)[1:-1, 1:-1]
    ps.items = _build_grid_items(ps, grid, npx, npx)
    return ps


def make_requests(count, rate, seed=42, cells=(1e4, 4e6), t_end=(0.05, 0.5), n=16):
    """Poisson arrivals (rate per second), log-uniform sizes, uniform end times."""
    rng = np.random.default_rng(seed)
    t = 0.0
    reqs = []
    for k in range(count):
        t += rng.exponential(1.0 / rate)
        c = float(np.exp(rng.uniform(np.log(cells[0]), np.log(cells[1]))))
        reqs.append(Request(rid=k, kind="dam_break" if rng.uniform() < 0.5 else "tsunami",
                            cells=int(c), t_end=float(rng.uniform(*t_end)), arrival=t, n=n,
                            seed=int(rng.integers(1 << 30))))
    return reqs


class Server:
    """Admits requests by free HBM and group slots, steps all resident groups
    together, `steps_per_batch` batched steps per replay of the step graph.

    Each scenario's end time lives on the device (pcg_set_group_end_time):
    its dt is capped at the time left and a finished scenario's group goes
    inactive (its state stays untouched) until the host retires it after the
    batch."""

    def __init__(self, slab_doubles, max_groups=32, max_patches=200_000, params=None,
                 steps_per_batch=8):
        self.prm = params if params is not None else P.swe_params(g=9.81, cfl=0.5)
        self.ctx = P.Context(slab_doubles=slab_doubles, max_patches=max_patches,
                             max_groups=max_groups, params=self.prm)
        self.max_groups = max_groups
        self.steps_per_batch = max(1, int(steps_per_batch))
        self.free_groups = list(range(max_groups))
        self.resident = {}      # group -> (Request, PatchSet)
        self.items = {}         # group -> remapped items
        for g in range(max_groups):
            self.ctx.set_group_max_dt(g, np.inf)
            self.ctx.set_group_end_time(g, 0.0, 0.0)   # free slots: inactive

    def close(self):
        self.ctx.close()

    def _fits(self, ps):
        free, _ = self.ctx.slab_info()
        need = sum(P.vector_size(n) + 32 for n in ps.n)
        return need <= free

    def admit(self, req, now, ps=None):
        if ps is None:
            ps = scenario_patchset(req)
        if not self.free_groups or not self._fits(ps):
            return False
        g = self.free_groups.pop(0)
        ids = []
        try:
            for p in range(len(ps)):
                pid = self.ctx.alloc(ps.n[p], pos=ps.pos[p], size=ps.size[p])
                ids.append(pid)
                self.ctx.set_group(pid, g)
                if ps.wall[p]:
                    self.ctx.set_boundary(pid, ps.wall[p])
        except P.PcgError:
            for pid in ids:
                self.ctx.free(pid)
            self.free_groups.insert(0, g)
            return False
        self.ctx.upload_many(ids, ps.packed)
        req.group, req.ids, req.admitted = g, ids, now
        self.items[g] = remap_items(ps.items, ids)
        self.resident[g] = (req, ps)
        self.ctx.set_group_end_time(g, 0.0, req.t_end)
        self._install_items()
        return True

    def _install_items(self):
        parts = [self.items[g] for g in sorted(self.items)]
        self.ctx.set_ghost_items(np.concatenate(parts) if parts else np.zeros((0, 9), np.int32))

    def retire(self, g, now):
        req, ps = self.resident.pop(g)
        req.result = self.ctx.download_many(req.ids, int(ps.packed.size))
        for pid in req.ids:
            self.ctx.free(pid)
        req.finished = now
        del self.items[g]
        self.ctx.set_group_end_time(g, 0.0, 0.0)
        self.free_groups.append(g)
        self._install_items()
        return req

    def step(self):
        """One batch of steps of every resident group; returns the groups that
        finished (reached their end time, or took a zero step)."""
        hist = self.ctx.run(self.steps_per_batch, P.PCG_MODE_BATCHED)
        times = self.ctx.group_times()
        done = []
        for g, (req, ps) in list(self.resident.items()):
            taken = hist[:, g] > 0.0
            k = int(np.count_nonzero(taken))
            req.steps += k
            req.cell_updates += k * ps.cells()
            if times[g] >= req.t_end or k < self.steps_per_batch:
                done.append(g)
        return done

    def serve(self, requests, clock=time.perf_counter, max_wall=600.0):
        """Run the continuous-batching loop over `requests` (sorted by arrival).

        A request's patch set is built on a worker thread as soon as it
        arrives, while the device advances the resident scenarios (the
        library calls release the interpreter lock while they wait for the
        GPU); admission then only allocates and uploads."""
        from concurrent.futures import ThreadPoolExecutor
        pending = sorted(requests, key=lambda r: r.arrival)
        waiting = []
        finished = []
        built = {}
        pool = ThreadPoolExecutor(max_workers=1)
        t0 = clock()
        try:
            while pending or waiting or self.resident:
                now = clock() - t0
                if now > max_wall:
                    break
                while pending and pending[0].arrival <= now:
                    r = pending.pop(0)
                    waiting.append(r)
                    built[id(r)] = pool.submit(scenario_patchset, r)
                still = []
                for r in waiting:
                    f = built[id(r)]
                    if not self.resident or f.done():
                        if self.admit(r, now, f.result()):
                            del built[id(r)]
                            continue
                    still.append(r)
                waiting = still
                if not self.resident:
                    if pending:
                        time.sleep(max(0.0, min(0.01, pending[0].arrival - now)))
                    continue
                for g in self.step():
                    finished.append(self.retire(g, clock() - t0))
        finally:
            pool.shutdown(wait=True, cancel_futures=True)
        return finished, clock() - t0


def run_alone(req, slab_doubles, params=None, steps_per_batch=1):
    """Solve one request as the only resident scenario; returns its final state."""
    srv = Server(slab_doubles, max_groups=2, params=params, steps_per_batch=steps_per_batch)
    try:
        req2 = Request(**{k: getattr(req, k) for k in ("rid", "kind", "cells", "t_end", "arrival",
                                                     "n", "seed")})
        assert srv.admit(req2, 0.0)
        while srv.resident:
            for g in srv.step():
                srv.retire(g, 0.0)
        return req2
    finally:
        srv.close()
