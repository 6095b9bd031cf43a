"""Adaptive grids of n x n patches with Peano-style 3x refinement, and dynamic
remeshing driven by the device-side refinement criterion.

`AmrGrid` holds the hierarchy as sets of patch slots per level (level l has
(base * 3^l)^2 slots on [0,1]^2; a refined slot's patch is virtual and its 9
children exist on level l+1) and derives from it what the Peano traversal
derives per grid iteration: the ghost face-pair list (same-level copies,
coarse-to-fine interpolation; GhostlayerCompositorFunctors.cpp:23-148), the
flux-correction list (fine leaf faces against a coarser neighbour), the
neighbouring ghost-layer bounds of the virtual patches
(GhostLayerCompositor::updateLower/UpperGhostlayerBound) and the restriction
list (GridLevelTransfer::restrictToOverlappingVirtualSubgrids).

`AmrGrid.decide` turns per-leaf values of the refinement criterion
(BreakingDamSWEScenario::computeDemandedMeshWidth, BreakingDam.cpp:85-139:
refine above the threshold, coarsen below it) into the next hierarchy: a leaf
above the threshold refines (below the finest level), a refined slot
coarsens when all 9 children are leaves below the threshold, and refined
regions are grown by `buffers[l]` slots per level so that neighbouring leaves
differ by at most one level.  `remesh` applies a decision through a backend:
new patches are initialised like Remesh::createCell (Remesh.cpp:346-423:
bathymetry from the scenario, then interpolateSolution from the coarse patch
into uNew and, at the current time, into uOld; time intervals copied from the
coarse patch), a coarsening parent receives the full restriction of its
children (clear, restrictSolution with onlyOverlapped = false,
postProcessRestriction: GridLevelTransfer, Remesh::destroyCell) and becomes a
leaf with the children's time intervals (Patch::switchToLeaf re-evaluates the
restricted values, which stand for the times 0 and 1, at the leaf's time
interval).  After a remesh every virtual patch receives the restriction of
the current leaves, so the next ghost fill reads consistent data.
"""
import numpy as np

from .pcg import PCG_GHOST_COPY, PCG_GHOST_INTERP

DIRECTIONS = ((-1, 0), (1, 0), (0, -1), (0, 1), (-1, -1), (1, -1), (-1, 1), (1, 1))


class AmrGrid:
    def __init__(self, base, n, levels, buffers=(1, 2), threshold=0.1):
        self.base, self.n, self.levels = base, n, levels
        self.buffers = tuple(buffers)
        self.threshold = threshold
        self.exists = [set() for _ in range(levels)]
        self.refined = [set() for _ in range(levels)]
        self.exists[0] = {(i, j) for i in range(base) for j in range(base)}

    # -------------------------------------------------------------- geometry
    def slots_per_edge(self, l):
        return self.base * 3 ** l

    def geometry(self, l, i, j):
        L = 1.0 / self.slots_per_edge(l)
        return (i * L, j * L), (L, L)

    def is_leaf(self, l, i, j):
        return (i, j) in self.exists[l] and (i, j) not in self.refined[l]

    def wall(self, l, i, j):
        if not self.is_leaf(l, i, j):
            return 0
        m = self.slots_per_edge(l)
        w = 0
        if i == 0: w |= 1
        if i == m - 1: w |= 2
        if j == 0: w |= 4
        if j == m - 1: w |= 8
        return w

    def order(self):
        """Slots in patch order: level ascending, then (i, j)."""
        return [(l, i, j) for l in range(self.levels) for (i, j) in sorted(self.exists[l])]

    def leaves(self):
        return [s for s in self.order() if self.is_leaf(*s)]

    def buffer(self, l):
        return self.buffers[l] if l < len(self.buffers) else 1

    # ------------------------------------------------------------- hierarchy
    def _grow(self, core, l, exists_l):
        buf = self.buffer(l)
        out = set()
        for (i, j) in core:
            for di in range(-buf, buf + 1):
                for dj in range(-buf, buf + 1):
                    if (i + di, j + dj) in exists_l:
                        out.add((i + di, j + dj))
        return out

    def refine_from(self, flags):
        """Build the hierarchy top-down from refinement flags: flags(l, i, j)
        is called for every existing slot of levels 0 .. levels-2."""
        for l in range(self.levels - 1):
            core = {s for s in self.exists[l] if flags(l, *s)}
            self.refined[l] = self._grow(core, l, self.exists[l])
            self.exists[l + 1] = {(3 * i + a, 3 * j + c) for (i, j) in self.refined[l]
                                  for a in range(3) for c in range(3)}
        self.refined[self.levels - 1] = set()

    def decide(self, g):
        """Next (exists, refined) from the refinement criterion g[(l, i, j)] of
        every leaf.  Returns new lists of sets; the grid itself is unchanged."""
        thr = self.threshold
        L = self.levels
        # a refined slot stays refined unless all 9 children are leaves below
        # the threshold (a refined child, or a leaf at or above it, keeps it)
        keep = [set() for _ in range(L)]
        for l in range(L - 1):
            for (i, j) in self.refined[l]:
                kids = [(3 * i + a, 3 * j + c) for a in range(3) for c in range(3)]
                if any(not (self.is_leaf(l + 1, *ch) and g[(l + 1,) + ch] < thr) for ch in kids):
                    keep[l].add((i, j))
        exists = [set(self.exists[0])] + [set() for _ in range(L - 1)]
        refined = [set() for _ in range(L)]
        for l in range(L - 1):
            core = {s for s in keep[l] if s in exists[l]}
            core |= {s for s in exists[l] if self.is_leaf(l, *s) and g.get((l,) + s, 0.0) > thr}
            refined[l] = self._grow(core, l, exists[l])
            exists[l + 1] = {(3 * i + a, 3 * j + c) for (i, j) in refined[l]
                             for a in range(3) for c in range(3)}
        return exists, refined

    # ----------------------------------------------------------------- lists
    def layout(self):
        """Patch order and every list the batched step needs (see layout_py),
        built by the library's native builder (pcg_amr_layout)."""
        import ctypes as C
        from . import pcg as P
        order = self.order()
        npch = len(order)
        arr = np.array(order, dtype=np.int32).reshape(-1, 3)
        lvl, si, sj = (np.ascontiguousarray(arr[:, k]) for k in range(3))
        ref = np.array([0 if self.is_leaf(*s) else 1 for s in order], dtype=np.uint8)
        items = np.zeros((8 * npch + 1, 9), dtype=np.int32)
        flux = np.zeros((4 * npch + 1, 4), dtype=np.int32)
        restr = np.zeros((self.levels * npch + 1, 2), dtype=np.int32)
        lower = np.zeros((npch + 1, 2))
        upper = np.zeros((npch + 1, 2))
        walls = np.zeros(npch + 1, dtype=np.int32)
        ni, nf, nr = C.c_int32(), C.c_int32(), C.c_int32()
        i32 = lambda a: a.ctypes.data_as(C.POINTER(C.c_int32))
        P.check(P.lib().pcg_amr_layout(
            self.base, self.n, self.levels, npch, i32(lvl), i32(si), i32(sj),
            ref.ctypes.data_as(C.POINTER(C.c_uint8)), i32(items), C.byref(ni), i32(flux), C.byref(nf),
            i32(restr), C.byref(nr), lower.ctypes.data_as(C.POINTER(C.c_double)),
            upper.ctypes.data_as(C.POINTER(C.c_double)), i32(walls)))
        L = 1.0 / (self.base * np.power(3.0, lvl.astype(np.float64)))
        pos = np.stack([si * L, sj * L], axis=1)
        size = np.stack([L, L], axis=1)
        index = {s: k for k, s in enumerate(order)}
        leaf = (ref == 0).tolist()
        return {"order": order, "index": index, "pos": pos, "size": size,
                "leaf": leaf, "level": lvl.tolist(), "wall": walls[:npch].tolist(),
                "items": items[:ni.value].copy(), "flux_items": flux[:nf.value].copy(),
                "restrict_items": restr[:nr.value].copy(),
                "restr_lower": lower[:npch].copy(), "restr_upper": upper[:npch].copy(),
                "virtual_time_items": virtual_time_items(order, index, leaf)}

    def layout_py(self):
        """Patch order and every list the batched step needs, in patch-order
        indices: items (N, 9), flux_items (N, 4) (fine leaf, coarse owner,
        dim, dir), restrict_items (N, 2) (leaf, virtual ancestor),
        restr_lower / restr_upper per patch."""
        n = self.n
        order = self.order()
        index = {s: k for k, s in enumerate(order)}
        pos = [self.geometry(*s)[0] for s in order]
        size = [self.geometry(*s)[1] for s in order]
        leaf = [self.is_leaf(*s) for s in order]

        def owner(l, i, j):
            while l >= 0:
                if (l, i, j) in index:
                    return index[(l, i, j)], l
                i, j, l = i // 3, j // 3, l - 1
            return None, None

        rows, flux = [], []
        for (l, i, j) in order:
            d = index[(l, i, j)]
            if not leaf[d]:
                continue
            m = self.slots_per_edge(l)
            for dx, dy in DIRECTIONS:
                tx, ty = i + dx, j + dy
                if not (0 <= tx < m and 0 <= ty < m):
                    continue
                s, ls = owner(l, tx, ty)
                dirv = (-dx, -dy)
                sz = [n if v == 0 else 1 for v in dirv]
                dst_off = [0 if v == 0 else (-1 if v == 1 else n) for v in dirv]
                if ls == l:
                    src_off = [0 if v == 0 else (n - 1 if v == 1 else 0) for v in dirv]
                    rows.append([PCG_GHOST_COPY, s, d] + sz + src_off + dst_off)
                else:
                    rows.append([PCG_GHOST_INTERP, s, d] + sz + [0, 0] + dst_off)
                    if dx == 0 or dy == 0:
                        dim = 0 if dx != 0 else 1
                        flux.append([d, s, dim, dx if dx != 0 else dy])
        big = np.finfo(np.float64).max
        lower = [[big, big] for _ in order]
        upper = [[-big, -big] for _ in order]
        for (l, i, j), v in index.items():
            if leaf[v]:
                continue
            for dim in (0, 1):
                for step in (-1, 1):
                    key = (l, i + step, j) if dim == 0 else (l, i, j + step)
                    if key not in index or not leaf[index[key]]:
                        continue
                    nb = index[key]
                    sub = size[nb][dim] / n
                    if step < 0:
                        upper[v][dim] = max(upper[v][dim], pos[nb][dim] + size[nb][dim] + sub)
                    else:
                        lower[v][dim] = min(lower[v][dim], pos[nb][dim] - sub)
        # every leaf against its virtual ancestors; list order: virtual patch
        # index, then leaf index
        rest = []
        for (l2, i2, j2), s in index.items():
            if not leaf[s]:
                continue
            for l in range(l2 - 1, -1, -1):
                f = 3 ** (l2 - l)
                v = index[(l, i2 // f, j2 // f)]
                lo, up = lower[v], upper[v]
                overlapped = any(up[d] - pos[s][d] > 1e-8 for d in (0, 1)) or \
                    any(pos[s][d] + size[s][d] - lo[d] > 1e-8 for d in (0, 1))
                if overlapped:
                    rest.append([s, v])
        rest.sort(key=lambda sv: (sv[1], sv[0]))
        return {"order": order, "index": index, "pos": pos, "size": size, "leaf": leaf,
                "level": [s[0] for s in order], "wall": [self.wall(*s) for s in order],
                "items": np.array(rows, dtype=np.int32).reshape(-1, 9),
                "flux_items": np.array(flux, dtype=np.int32).reshape(-1, 4),
                "restrict_items": np.array(rest, dtype=np.int32).reshape(-1, 2),
                "restr_lower": lower, "restr_upper": upper,
                "virtual_time_items": virtual_time_items(order, index, leaf)}


def virtual_time_items(order, index, leaf):
    """(leaf, virtual ancestor) pairs in patch-order indices, every leaf
    against each refined slot above it, sorted by (virtual, leaf): the list
    whose intervals give the virtual patches' time intervals in local time
    stepping (the fine-grid time interval that GridLevelTransfer::stepUp
    accumulates over the children, applied transitively)."""
    rows = []
    for (l2, i2, j2) in order:
        s = index[(l2, i2, j2)]
        if not leaf[s]:
            continue
        for l in range(l2 - 1, -1, -1):
            f = 3 ** (l2 - l)
            v = index.get((l, i2 // f, j2 // f))
            if v is not None and not leaf[v]:
                rows.append((v, s))
    rows.sort()
    return np.array([(s, v) for v, s in rows], dtype=np.int32).reshape(-1, 2)


def remesh(grid, backend, g, b_of):
    """Apply grid.decide(g) through `backend` and update `grid`.

    backend provides: handle(slot), forget(slot), alloc(slot, pos, size,
    level) -> handle of a fresh zero-filled leaf, free(handle),
    set_leaf(handle, leaf, wall), times(handle) -> (time, dt, est_next),
    set_times(handle, time, dt, est), set_b(handle, b),
    interpolate_child(parent, child), coarsen(parent, children),
    switch_to_leaf(handle), install(layout, handles), restrict_all().
    Returns (#refined, #coarsened)."""
    from .scenarios import _centers
    exists, refined = grid.decide(g)
    if exists == grid.exists and refined == grid.refined:
        return 0, 0
    n = grid.n
    n_ref = n_crs = 0
    # refinement, coarse to fine: children of newly refined slots
    for l in range(grid.levels - 1):
        for (i, j) in sorted(refined[l] - grid.refined[l]):
            parent = backend.handle((l, i, j))
            t = backend.times(parent)
            for a in range(3):
                for c in range(3):
                    ch = (l + 1, 3 * i + a, 3 * j + c)
                    if (ch[1], ch[2]) in grid.exists[l + 1]:
                        continue
                    pos, size = grid.geometry(*ch)
                    h = backend.alloc(ch, pos, size, l + 1)
                    backend.set_times(h, *t)
                    X, Y = _centers(pos, size, n, ghost=True)
                    backend.set_b(h, b_of(X, Y))
                    backend.interpolate_child(parent, h)
            n_ref += 1
    # coarsening, fine to coarse: restrict the children into their parent
    for l in range(grid.levels - 2, -1, -1):
        for (i, j) in sorted(grid.refined[l] - refined[l]):
            parent = backend.handle((l, i, j))
            kids = [(l + 1, 3 * i + a, 3 * j + c) for a in range(3) for c in range(3)]
            hk = [backend.handle(k) for k in kids]
            t = backend.times(hk[0])
            backend.coarsen(parent, hk)
            backend.set_times(parent, *t)
            backend.switch_to_leaf(parent)
            for k, h in zip(kids, hk):
                backend.free(h)
                backend.forget(k)
            n_crs += 1
    old_state = {s: (grid.is_leaf(*s), grid.wall(*s)) for s in grid.order()}
    grid.exists, grid.refined = exists, refined
    lay = grid.layout()
    for s, leaf, w in zip(lay["order"], lay["leaf"], lay["wall"]):
        if old_state.get(s) != (leaf, w) or s not in old_state:
            backend.set_leaf(backend.handle(s), leaf, w)
    backend.install(lay, [backend.handle(s) for s in lay["order"]])
    # virtual patches (new ones included) receive the restriction of the
    # current leaves before the next ghost fill reads them
    backend.restrict_all()
    return n_ref, n_crs


class DeviceAmr:
    """Backend of `remesh` on a pcg.Context (and the grid's initial install)."""

    def __init__(self, ctx, grid, b_of, flux=True, g_flux=1.0):
        self.ctx, self.grid, self.b_of = ctx, grid, b_of
        self.flux, self.g_flux = flux, g_flux
        self.pid = {}
        self._bounds = {}   # restriction bounds last written per virtual patch
        self.timing = {}

    # -- remesh protocol
    def handle(self, slot):
        return self.pid[slot]

    def forget(self, slot):
        del self.pid[slot]

    def alloc(self, slot, pos, size, level):
        pid = self.ctx.alloc(self.grid.n, pos=pos, size=size, level=level, leaf=True)
        self.pid[slot] = pid
        return pid

    def free(self, pid):
        self.ctx.free(pid)

    def set_leaf(self, pid, leaf, wall):
        self.ctx.set_flags(pid, leaf=leaf, virtual=not leaf)
        self.ctx.set_boundary(pid, wall)

    def times(self, pid):
        t = self.ctx.get_time(pid)
        return t["time"], t["dt"], t["est_next"]

    def set_times(self, pid, time, dt, est):
        self.ctx.set_time(pid, time=time, dt=dt, est_next=est)

    def set_b(self, pid, b):
        from .pcg import vector_size
        n = self.grid.n
        vec = np.zeros(vector_size(n))
        off = 3 * n * n + 3 * (n + 2) * (n + 2)
        vec[off:off + (n + 2) * (n + 2)] = np.ascontiguousarray(b).ravel()
        self.ctx.upload(pid, vec)

    def interpolate_child(self, parent, child):
        from . import pcg as P
        n = self.grid.n
        for to_uold, current in ((0, 0), (1, 1)):
            P.check(P.lib().pcg_interpolate_solution(self.ctx.h, P.i2((n, n)), P.i2((0, 0)), parent,
                                                      child, to_uold, current, 0, 1))

    def coarsen(self, parent, children):
        from . import pcg as P
        self.ctx.clear_subgrid(parent)
        for k in children:
            P.check(P.lib().pcg_restrict_solution(self.ctx.h, k, parent, 0, 1))
        P.check(P.lib().pcg_post_process_restriction(self.ctx.h, parent))

    def switch_to_leaf(self, pid):
        self.ctx.switch_to_leaf(pid)

    def restrict_all(self):
        self.ctx.restrict_all()

    def install(self, lay, handles):
        ids = np.asarray(handles, dtype=np.int32)
        bounds = {}
        for k, pid in enumerate(ids):
            if not lay["leaf"][k]:
                b = (tuple(lay["restr_lower"][k]), tuple(lay["restr_upper"][k]))
                bounds[int(pid)] = b
                if self._bounds.get(int(pid)) == b:
                    continue
                t = self.ctx.get_time(int(pid))
                self.ctx.set_time(int(pid), time=t["time"], dt=t["dt"], est_next=t["est_next"],
                                  restr_lower=b[0], restr_upper=b[1])
        self._bounds = bounds
        from .scenarios import remap_items
        self.ctx.set_ghost_items(remap_items(lay["items"], ids))
        r = lay["restrict_items"]
        self.ctx.set_restriction_items(ids[r[:, 0]], ids[r[:, 1]], True)
        vt = lay["virtual_time_items"]
        self.ctx.set_virtual_time_items(ids[vt[:, 0]], ids[vt[:, 1]])
        f = lay["flux_items"]
        if self.flux and len(f):
            self.ctx.set_flux_correction_items(ids[f[:, 0]], ids[f[:, 1]], f[:, 2], f[:, 3], self.g_flux)
        else:
            self.ctx.set_flux_correction_items([], [], [], [], self.g_flux)

    # -- driver
    def indicators(self):
        leaves = self.grid.leaves()
        vals = self.ctx.refinement_indicator([self.pid[s] for s in leaves])
        return dict(zip(leaves, vals))

    def remesh(self):
        import time
        t0 = time.perf_counter()
        g = self.indicators()
        t1 = time.perf_counter()
        r = remesh(self.grid, self, g, self.b_of)
        self.ctx.synchronize()
        t2 = time.perf_counter()
        self.timing = {"indicators_s": t1 - t0, "remesh_s": t2 - t1}
        return r
