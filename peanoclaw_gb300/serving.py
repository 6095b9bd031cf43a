"""Continuous-batching scenario server on one GPU.

Independent SWE scenario solves (radial dam breaks and Gaussian-hump
tsunamis of different sizes, end times and 1-3 levels of adaptive 3x
refinement) are admitted while others are running, as soon as a group slot
and enough free HBM in the context's slab are available.  Every resident
scenario is one *group* of patches: all groups advance together in the same
batched launches (ghost fill, sweep, update, flux correction and
restriction), each with its own CFL timestep (dt reduced per group on the
device) and its own end time, so a scenario's result does not depend on what
else is in the batch.  An adaptive scenario keeps its hierarchy and all its
patches (leaves and virtual patches) on the device and is remeshed every
`remesh_every` of its own steps from the device refinement criterion
(Remesh.cpp:346-423), between batches.  A finished scenario's state is read
back and its patches are freed, which admits the next waiting requests.
"""
import time
from dataclasses import dataclass, field

import numpy as np

from . import pcg as P
from .amr import DeviceAmr
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
    levels: int = 1      # levels of 3x refinement (1: uniform grid)
    # filled by the server
    admitted: float = None
    finished: float = None
    steps: int = 0
    cell_updates: int = 0
    result: np.ndarray = None
    group: int = -1
    ids: list = field(default_factory=list)


def _scenario_fields(req):
    """h_of, b_of of a request: a radial dam break (h = 2 inside radius 0.15
    of (cx, cy), 1 elsewhere, flat bottom) or a Gaussian surface hump
    (amplitude 0.5, sigma 0.05) over a Gaussian seafloor bump."""
    rng = np.random.default_rng(req.seed)
    cx, cy = rng.uniform(0.3, 0.7, 2)
    if req.kind == "dam_break":
        def b_of(X, Y):
            return np.zeros_like(X)

        def h_of(X, Y):
            r = np.sqrt((X - cx) ** 2 + (Y - cy) ** 2)
            return np.where(r <= 0.15, 2.0, 1.0)
    else:
        def b_of(X, Y):
            return 0.1 * np.exp(-((X - 0.5) ** 2 + (Y - 0.5) ** 2) / (2 * 0.2 ** 2))

        def h_of(X, Y):
            eta = 1.0 + 0.5 * np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2 * 0.05 ** 2))
            return eta - b_of(X, Y)
    return h_of, b_of


def adaptive_patchset(req, threshold=0.5):
    """A request with 2-3 levels: base x base patches of n x n cells on
    [0,1]^2, refined where the surface gradient of the initial state exceeds
    `threshold`, so the refined rim follows the dam or the hump.  The
    requested cells are the effective resolution of the finest level (base =
    sqrt(cells) / n / 3^(levels-1)): a uniform request and an adaptive one of
    the same size resolve the front alike (and take about the same steps),
    the adaptive one with fewer cells."""
    from .amr import AmrGrid
    from .pcg import PCG_CRIT_SURFACE_GRADIENT
    from .scenarios import amr_patchset
    n = req.n
    base = max(1, int(round(np.sqrt(req.cells) / n / 3 ** (req.levels - 1))))
    req.npx = base
    h_of, b_of = _scenario_fields(req)

    def needs_refine(level, i, j):
        m = base * 3 ** level
        L = 1.0 / m
        X, Y = _centers((i * L, j * L), (L, L), n, ghost=False)
        q = h_of(X, Y) + b_of(X, Y)
        dx = L / n
        gx = (q[1:, :-1] - q[:-1, :-1]) / dx
        gy = (q[:-1, 1:] - q[:-1, :-1]) / dx
        return float(np.max(np.sqrt(np.abs(gx) * np.abs(gx) + np.abs(gy) * np.abs(gy)))) > threshold

    grid = AmrGrid(base, n, req.levels, threshold=threshold)
    grid.refine_from(needs_refine)
    ps = amr_patchset(grid, h_of, b_of)
    ps.grid, ps.h_of, ps.b_of = grid, h_of, b_of
    ps.criterion = PCG_CRIT_SURFACE_GRADIENT
    return ps


def scenario_patchset(req):
    """The request's initial patch set: a uniform grid of npx x npx patches of
    n x n cells on [0,1]^2 with walls, or (levels > 1) an adaptive one."""
    if req.levels > 1:
        return adaptive_patchset(req)
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


def make_requests(count, rate, seed=42, cells=(1e4, 4e6), t_end=(0.05, 0.5), n=16, levels=(1, 1)):
    """Poisson arrivals (rate per second), log-uniform sizes, uniform end times,
    levels uniform in [levels[0], levels[1]]."""
    rng = np.random.default_rng(seed)
    t = 0.0
    reqs = []
    for k in range(count):
        t += rng.exponential(1.0 / rate)
        c = float(np.exp(rng.uniform(np.log(cells[0]), np.log(cells[1]))))
        reqs.append(Request(rid=k, kind="dam_break" if rng.uniform() < 0.5 else "tsunami",
                            cells=int(c), t_end=float(rng.uniform(*t_end)), arrival=t, n=n,
                            seed=int(rng.integers(1 << 30)),
                            levels=int(rng.integers(levels[0], levels[1] + 1))))
    return reqs


class GroupAmr(DeviceAmr):
    """The device AMR backend of one adaptive request: amr.DeviceAmr with its
    new patches in the request's group and its lists handed to the server,
    which installs the lists of every resident group together."""

    def __init__(self, server, group, ps):
        super().__init__(server.ctx, ps.grid, ps.b_of, criterion=ps.criterion)
        self.server, self.group = server, group

    def alloc(self, slot, pos, size, level):
        pid = super().alloc(slot, pos, size, level)
        self.ctx.set_group(pid, self.group)
        return pid

    def install_lists(self, lay, ids):
        self.server._set_group_lists(self.group, lay, ids)

    def restrict_all(self):
        # the server installs every group's lists and restricts once, after
        # all the groups due at this batch boundary have remeshed
        self.server.pending_restrict = True


class Server:
    """Admits requests by free HBM and group slots, steps all resident groups
    together, `steps_per_batch` batched steps per replay of the step graph.

    Each scenario's end time lives on the device (pcg_set_group_end_time):
    its dt is capped at the time left and a finished scenario's group goes
    inactive (its state stays untouched) until the host retires it after the
    batch."""

    def __init__(self, slab_doubles, max_groups=32, max_patches=200_000, params=None,
                 steps_per_batch=8, remesh_every=16):
        self.prm = params if params is not None else P.swe_params(g=9.81, cfl=0.5)
        self.ctx = P.Context(slab_doubles=slab_doubles, max_patches=max_patches,
                             max_groups=max_groups, params=self.prm)
        self.max_groups = max_groups
        self.steps_per_batch = max(1, int(steps_per_batch))
        # an adaptive group remeshes after every remesh_every of its own steps;
        # batches end on multiples of steps_per_batch of every group's steps,
        # so remesh_every must be a multiple of it
        self.remesh_every = int(remesh_every)
        if self.remesh_every % self.steps_per_batch:
            raise ValueError("remesh_every must be a multiple of steps_per_batch")
        self.free_groups = list(range(max_groups))
        self.resident = {}      # group -> (Request, PatchSet)
        self.items = {}         # group -> remapped ghost items
        self.restr = {}         # group -> (src ids, dst ids) of the restriction list
        self.flux = {}          # group -> (src, dst, dim, dir) of the flux-correction list
        self.amr = {}           # group -> device AMR backend (adaptive requests)
        self.leaf_cells = {}    # group -> leaf cells (cached)
        self.remesh_s = 0.0     # host time spent remeshing
        self.relist_s = 0.0     # of which installing the lists and restricting
        self.remeshes = 0
        self.pending_restrict = False
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
        adaptive = getattr(ps, "grid", None) is not None
        ids = []
        try:
            for p in range(len(ps)):
                leaf = bool(ps.leaf[p]) if adaptive else True
                pid = self.ctx.alloc(ps.n[p], pos=ps.pos[p], size=ps.size[p], level=ps.level[p], leaf=leaf,
                                     virtual=not leaf)
                ids.append(pid)
                self.ctx.set_group(pid, g)
                if ps.wall[p]:
                    self.ctx.set_boundary(pid, ps.wall[p])
                if not leaf:
                    self.ctx.set_time(pid, restr_lower=ps.restr_lower[p], restr_upper=ps.restr_upper[p])
        except P.PcgError:
            for pid in ids:
                self.ctx.free(pid)
            self.free_groups.insert(0, g)
            return False
        self.ctx.upload_many(ids, ps.packed)
        req.group, req.ids, req.admitted = g, ids, now
        ids = np.asarray(ids, dtype=np.int32)
        self.items[g] = remap_items(ps.items, ids)
        self.resident[g] = (req, ps)
        self.ctx.set_group_end_time(g, 0.0, req.t_end)
        if adaptive:
            r, f = ps.restrict_items, ps.flux_items
            self.restr[g] = (ids[r[:, 0]], ids[r[:, 1]])
            self.flux[g] = (ids[f[:, 0]], ids[f[:, 1]], f[:, 2], f[:, 3])
            dev = GroupAmr(self, g, ps)
            dev.pid = dict(zip(ps.grid.order(), (int(i) for i in ids)))
            self.amr[g] = dev
            self._install_lists()
            # the virtual patches receive their leaves' restriction before the
            # first ghost fill reads them
            self.ctx.restrict_all()
        else:
            self._install_lists()
        return True

    def _set_group_lists(self, g, lay, ids):
        self.items[g] = remap_items(lay["items"], ids)
        r, f = lay["restrict_items"], lay["flux_items"]
        self.restr[g] = (ids[r[:, 0]], ids[r[:, 1]])
        self.flux[g] = (ids[f[:, 0]], ids[f[:, 1]], f[:, 2], f[:, 3])

    def _install_lists(self):
        """The ghost, restriction and flux-correction lists of every resident
        group, concatenated (each group's patches are its own)."""
        gs = sorted(self.items)
        parts = [self.items[g] for g in gs]
        self.ctx.set_ghost_items(np.concatenate(parts) if parts else np.zeros((0, 9), np.int32))
        rs = [self.restr[g] for g in gs if g in self.restr]
        cat = lambda xs, k: np.concatenate([x[k] for x in xs]) if xs else np.zeros(0, np.int32)
        self.ctx.set_restriction_items(cat(rs, 0), cat(rs, 1), True)
        fs = [self.flux[g] for g in gs if g in self.flux]
        self.ctx.set_flux_correction_items(cat(fs, 0), cat(fs, 1), cat(fs, 2), cat(fs, 3), 1.0)

    def _result_ids(self, g):
        req, ps = self.resident[g]
        dev = self.amr.get(g)
        if dev is None:
            return req.ids
        return [dev.pid[s] for s in dev.grid.order()]

    def retire(self, g, now):
        ids = self._result_ids(g)
        req, ps = self.resident.pop(g)
        n = sum(P.vector_size(ps.n[0]) for _ in ids) if g in self.amr else int(ps.packed.size)
        req.result = self.ctx.download_many(ids, n)
        for pid in ids:
            self.ctx.free(pid)
        req.finished = now
        del self.items[g]
        self.restr.pop(g, None)
        self.flux.pop(g, None)
        self.amr.pop(g, None)
        self.leaf_cells.pop(g, None)
        self.ctx.set_group_end_time(g, 0.0, 0.0)
        self.free_groups.append(g)
        self._install_lists()
        return req

    def _leaf_cells(self, g):
        """Leaf cells of a resident group (cached; a remesh resets it)."""
        lc = self.leaf_cells.get(g)
        if lc is None:
            req, ps = self.resident[g]
            dev = self.amr.get(g)
            lc = ps.cells() if dev is None else len(dev.grid.leaves()) * dev.grid.n ** 2
            self.leaf_cells[g] = lc
        return lc

    def step(self):
        """One batch of steps of every resident group; returns the groups that
        finished (reached their end time, or took a zero step).  Adaptive
        groups whose step count reached a multiple of remesh_every are
        remeshed afterwards."""
        hist = self.ctx.run(self.steps_per_batch, P.PCG_MODE_BATCHED)
        times = self.ctx.group_times()
        done = []
        remesh = []
        for g, (req, ps) in list(self.resident.items()):
            taken = hist[:, g] > 0.0
            k = int(np.count_nonzero(taken))
            req.steps += k
            req.cell_updates += k * self._leaf_cells(g)
            if times[g] >= req.t_end or k < self.steps_per_batch:
                done.append(g)
            elif g in self.amr and req.steps % self.remesh_every == 0:
                remesh.append(g)
        if remesh:
            t0 = time.perf_counter()
            for g in remesh:
                self.amr[g].remesh()
                self.leaf_cells.pop(g, None)
            t1 = time.perf_counter()
            if self.pending_restrict:
                # the new lists of every remeshed group, and the virtual
                # patches (new ones included) refilled from their leaves
                # before the next ghost fill reads them
                self._install_lists()
                self.ctx.restrict_all()
                self.pending_restrict = False
            t2 = time.perf_counter()
            self.remesh_s += t2 - t0
            self.relist_s += t2 - t1
            self.remeshes += len(remesh)
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


def run_alone(req, slab_doubles, params=None, steps_per_batch=1, remesh_every=16):
    """Solve one request as the only resident scenario; returns its final state."""
    srv = Server(slab_doubles, max_groups=2, params=params, steps_per_batch=steps_per_batch,
                 remesh_every=remesh_every)
    try:
        req2 = Request(**{k: getattr(req, k) for k in ("rid", "kind", "cells", "t_end", "arrival",
                                                     "n", "seed", "levels")})
        assert srv.admit(req2, 0.0)
        while srv.resident:
            for g in srv.step():
                srv.retire(g, 0.0)
        return req2
    finally:
        srv.close()
