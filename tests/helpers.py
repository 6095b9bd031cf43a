"""Shared test helpers: identical inputs for the CUDA path and the oracle."""
import numpy as np

from oracle import oracle as O
from peanoclaw_gb300 import pcg as P


def oracle_params(prm):
    return O.swe_params(prm.g, prm.cfl, prm.dry_tol, prm.dry_tol_update, prm.s_min, prm.dt_inf)


def random_swe_vector(rng, n, dry_fraction=0.2, lake=False, ghost_b=True):
    """Patch vector (reference layout, ghost 1, 3 unknowns, b with ghost) with a
    random wet/dry state in uNew and uOld (incl. ghost ring); n is the side or
    the (nx, ny) pair."""
    nx, ny = (n, n) if np.isscalar(n) else n
    ln = P.vector_size((nx, ny))
    v = np.zeros(ln)
    a = 3 * nx * ny
    vo = (nx + 2) * (ny + 2)
    o = 3 * vo
    unew = v[:a].reshape(3, nx, ny)
    uold = v[a:a + o].reshape(3, nx + 2, ny + 2)
    b = v[a + o:a + o + vo].reshape(nx + 2, ny + 2)
    b[:] = rng.uniform(-0.3, 0.6, (nx + 2, ny + 2))
    if lake:
        # dyadic values so that h + b is exact: a lake at rest with dry cells
        b[:] = np.round(b * 64.0) / 64.0
        eta = 0.5
        h = np.maximum(0.0, eta - b)
        uold[0] = h
        unew[0] = h[1:-1, 1:-1]
        return v
    h = rng.uniform(0.0, 2.0, (nx + 2, ny + 2))
    dry = rng.uniform(0, 1, (nx + 2, ny + 2)) < dry_fraction
    h[dry] = rng.uniform(0.0, 0.02, dry.sum())
    hu = rng.normal(0.0, 0.5, (nx + 2, ny + 2))
    hv = rng.normal(0.0, 0.5, (nx + 2, ny + 2))
    uold[0], uold[1], uold[2] = h, hu, hv
    unew[0] = rng.uniform(0.0, 2.0, (nx, ny))
    unew[1] = rng.normal(0.0, 0.5, (nx, ny))
    unew[2] = rng.normal(0.0, 0.5, (nx, ny))
    v[a + o + vo:] = rng.normal(0.0, 1.0, v.size - (a + o + vo))
    return v


def oracle_patch_from(vec, n, pos=(0.0, 0.0), size=(1.0, 1.0), level=0, time=0.0, dt=0.0,
                      ghost=1, nq=3, np_wo=0, np_w=1, leaf=True, virtual=False,
                      min_neighbor_time=0.0, max_neighbor_dt=0.0):
    p = O.Patch(n, ghost=ghost, nq=nq, np_wo=np_wo, np_w=np_w, pos=pos, size=size, level=level,
                time=time, dt=dt, is_leaf=leaf, is_virtual=virtual,
                min_neighbor_time=min_neighbor_time, max_neighbor_dt=max_neighbor_dt)
    assert p.u.size == vec.size
    p.u[:] = vec
    return p


def oracle_patchset(ps):
    pats = []
    for p in range(len(ps)):
        pats.append(oracle_patch_from(ps.vector(p).copy(), ps.n[p], ps.pos[p], ps.size[p],
                                      ps.level[p]))
    return pats


def gpu_patchset(ctx, ps):
    ids = []
    for p in range(len(ps)):
        pid = ctx.alloc(ps.n[p], pos=ps.pos[p], size=ps.size[p], level=ps.level[p])
        ids.append(pid)
        ctx.set_boundary(pid, ps.wall[p])
    ctx.upload_many(ids, ps.packed)
    from peanoclaw_gb300.scenarios import remap_items
    ctx.set_ghost_items(remap_items(ps.items, ids))
    return ids


def slab_for(ps, slack=1.2):
    return int(sum(P.vector_size(n) + 32 for n in ps.n) * slack) + 4096


def oracle_amr_patchset(ps):
    pats = []
    for p in range(len(ps)):
        leaf = bool(ps.leaf[p])
        op = oracle_patch_from(ps.vector(p).copy(), ps.n[p], ps.pos[p], ps.size[p], ps.level[p],
                               leaf=leaf, virtual=not leaf)
        op.s.restr_lower[0], op.s.restr_lower[1] = ps.restr_lower[p]
        op.s.restr_upper[0], op.s.restr_upper[1] = ps.restr_upper[p]
        pats.append(op)
    return pats


def oracle_restrict_all(pats, ps):
    """Clear every destination, restrict in list order, post-process."""
    dsts = []
    for s, d in ps.restrict_items:
        if d not in dsts:
            dsts.append(int(d))
    for d in dsts:
        pats[d].unew()[:] = 0.0
        g = pats[d].s.ghost
        pats[d].uold()[:, g:-g, g:-g] = 0.0
    for s, d in ps.restrict_items:
        O.restrict(pats[s], pats[d], only_overlapped=True, swe=True)
    for d in dsts:
        O.lib().pco_swe_post_process_restriction(pats[d].ptr())


def oracle_amr_step(pats, ps, prm, max_dt, g_flux=1.0, flux=True):
    dt = O.grid_step(pats, ps.items, ps.wall, prm, max_dt)[0]
    if flux and len(ps.flux_items):
        for p in range(len(ps)):
            if ps.leaf[p]:
                O.lib().pco_compute_fluxes(pats[p].ptr(), g_flux)
        for s, d, dim, direction in ps.flux_items:
            O.lib().pco_apply_flux_correction(pats[s].ptr(), pats[d].ptr(), int(dim), int(direction))
    oracle_restrict_all(pats, ps)
    return dt


def gpu_amr_patchset(ctx, ps, flux=True, g_flux=1.0):
    from peanoclaw_gb300.scenarios import install_amr
    return install_amr(ctx, ps, flux=flux, g_flux=g_flux)


def oracle_criterion(p, kind=0):
    """Refinement criterion of an oracle patch (pcg_refinement_criterion kinds):
    0 the BreakingDam depth gradient (BreakingDam.cpp:100-116), 1 BowlOcean's
    surface differences (BowlOcean.cpp:106-122), 2 the BreakingDam stencil on
    the surface h + b."""
    h = p.unew()[0]
    if kind != 0:
        g = p.s.ghost
        h = h + p.param_w()[0][g:-g, g:-g]
    dx, dy = p.s.size[0] / p.s.nx, p.s.size[1] / p.s.ny
    gx = h[1:, :-1] - h[:-1, :-1]
    gy = h[:-1, 1:] - h[:-1, :-1]
    if kind != 1:
        gx = gx / dx
        gy = gy / dy
    g = np.sqrt(np.abs(gx) * np.abs(gx) + np.abs(gy) * np.abs(gy))
    return float(np.fmax.reduce(g.ravel(), initial=0.0))


class OracleAmr:
    """Backend of peanoclaw_gb300.amr.remesh on oracle patches (the CPU side of
    the remesh parity tests); mirrors DeviceAmr call for call."""

    def __init__(self, grid, ps, b_of, flux=True, g_flux=1.0, criterion=0):
        self.grid, self.b_of, self.flux, self.g_flux = grid, b_of, flux, g_flux
        self.criterion = criterion  # pcg_refinement_criterion kind
        pats = oracle_amr_patchset(ps)
        self.pat = dict(zip(grid.order(), pats))
        self.lay = grid.layout()
        self.walls = {}
        for s, w in zip(self.lay["order"], self.lay["wall"]):
            self.walls[s] = w

    def handle(self, slot):
        return self.pat[slot]

    def forget(self, slot):
        del self.pat[slot]

    def alloc(self, slot, pos, size, level):
        p = O.Patch(self.grid.n, pos=pos, size=size, level=level, is_leaf=True)
        self.pat[slot] = p
        return p

    def free(self, p):
        pass

    def set_leaf(self, p, leaf, wall):
        p.s.is_leaf, p.s.is_virtual = int(leaf), int(not leaf)
        p.wall = wall

    def times(self, p):
        return p.s.time, p.s.dt, p.s.est_next

    def set_times(self, p, time, dt, est):
        big = np.finfo(np.float64).max
        p.s.time, p.s.dt, p.s.est_next = time, dt, est
        p.s.min_neighbor_time = p.s.max_neighbor_dt = 0.0
        p.s.restr_lower[0] = p.s.restr_lower[1] = big
        p.s.restr_upper[0] = p.s.restr_upper[1] = -big

    def set_b(self, p, b):
        p.u[:] = 0.0
        p.param_w()[0] = b

    def interpolate_child(self, parent, child):
        n = self.grid.n
        for to_uold, current in ((0, 0), (1, 1)):
            O.interpolate((n, n), (0, 0), parent, child, to_uold=bool(to_uold),
                          to_current_time=bool(current), use_time_unew_or_uold=False, swe=True)

    def coarsen(self, parent, children):
        parent.unew()[:] = 0.0
        g = parent.s.ghost
        parent.uold()[:, g:-g, g:-g] = 0.0
        for k in children:
            O.restrict(k, parent, only_overlapped=False, swe=True)
        O.lib().pco_swe_post_process_restriction(parent.ptr())

    def switch_to_leaf(self, p):
        O.lib().pco_switch_to_leaf(p.ptr())

    def restrict_all(self):
        pats = self.patches()
        dsts = []
        for s, d in self.lay["restrict_items"]:
            if d not in dsts:
                dsts.append(int(d))
        for d in dsts:
            pats[d].unew()[:] = 0.0
            g = pats[d].s.ghost
            pats[d].uold()[:, g:-g, g:-g] = 0.0
        for s, d in self.lay["restrict_items"]:
            O.restrict(pats[s], pats[d], only_overlapped=True, swe=True)
        for d in dsts:
            O.lib().pco_swe_post_process_restriction(pats[d].ptr())

    def install(self, lay, handles):
        self.lay = lay
        for k, p in enumerate(handles):
            if not lay["leaf"][k]:
                p.s.restr_lower[0], p.s.restr_lower[1] = lay["restr_lower"][k]
                p.s.restr_upper[0], p.s.restr_upper[1] = lay["restr_upper"][k]

    # -- driver
    def patches(self):
        return [self.pat[s] for s in self.lay["order"]]

    def indicators(self):
        return {s: oracle_criterion(self.pat[s], self.criterion) for s in self.grid.leaves()}

    def step(self, prm, max_dt):
        from types import SimpleNamespace
        lay = self.lay
        ns = SimpleNamespace(items=lay["items"], wall=lay["wall"], flux_items=lay["flux_items"],
                             restrict_items=lay["restrict_items"], leaf=lay["leaf"])
        ns.__len__ = lambda: len(lay["order"])
        pats = self.patches()
        dt = O.grid_step(pats, ns.items, ns.wall, prm, max_dt)[0]
        if self.flux and len(ns.flux_items):
            for p, lf in zip(pats, ns.leaf):
                if lf:
                    O.lib().pco_compute_fluxes(p.ptr(), self.g_flux)
            for s, d, dim, direction in ns.flux_items:
                O.lib().pco_apply_flux_correction(pats[s].ptr(), pats[d].ptr(), int(dim), int(direction))
        dsts = []
        for s, d in ns.restrict_items:
            if d not in dsts:
                dsts.append(int(d))
        for d in dsts:
            pats[d].unew()[:] = 0.0
            g = pats[d].s.ghost
            pats[d].uold()[:, g:-g, g:-g] = 0.0
        for s, d in ns.restrict_items:
            O.restrict(pats[s], pats[d], only_overlapped=True, swe=True)
        for d in dsts:
            O.lib().pco_swe_post_process_restriction(pats[d].ptr())
        return dt

    def remesh(self):
        from peanoclaw_gb300.amr import remesh
        return remesh(self.grid, self, self.indicators(), self.b_of)
