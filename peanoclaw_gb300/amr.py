"""Adaptive grids of n x n patches with Peano-style 3x refinement, and dynamic
remeshing driven by the device-side refinement criterion.

`AmrGrid` holds the hierarchy as boolean arrays over the patch slots of each
level (level l has (base * 3^l)^2 slots on [0,1]^2; a refined slot's patch is
virtual and its 9 children exist on level l+1) and derives from it what the Peano traversal
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


class _Layout(dict):
    """The lists of AmrGrid.layout; "index" (slot -> position in the patch
    order) is built on first use."""

    def __missing__(self, key):
        if key != "index":
            raise KeyError(key)
        order = self["order"]
        v = dict(zip(order, range(len(order))))
        self["index"] = v
        return v


class AmrGrid:
    """The hierarchy as one boolean array per level over its slots:
    `exists` (the slot holds a patch) and `refined` (its patch is virtual and
    its 9 children exist).  The set views `grid.exists[l]` / `grid.refined[l]`
    (sets of (i, j)) are derived on demand; assigning them (sets or arrays)
    replaces the state."""

    def __init__(self, base, n, levels, buffers=(1, 2), threshold=0.1):
        self.base, self.n, self.levels = base, n, levels
        self.buffers = tuple(buffers)
        self.threshold = threshold
        self._E = [np.zeros((m, m), dtype=bool) for m in self._sizes()]
        self._R = [np.zeros((m, m), dtype=bool) for m in self._sizes()]
        self._E[0][:] = True
        self._cache = {}

    def _sizes(self):
        return [self.slots_per_edge(l) for l in range(self.levels)]

    # ----------------------------------------------------------------- state
    def arrays(self):
        """(exists, refined): lists of per-level boolean arrays (not copies)."""
        return self._E, self._R

    def set_arrays(self, E, R):
        self._E = [np.array(e, dtype=bool) for e in E]
        self._R = [np.array(r, dtype=bool) for r in R]
        self._cache = {}

    def _to_arrays(self, sets):
        out = []
        for l, m in enumerate(self._sizes()):
            a = np.zeros((m, m), dtype=bool)
            v = sets[l]
            if isinstance(v, np.ndarray):
                a[:] = v
            elif len(v):
                ij = np.array(list(v), dtype=np.int64).reshape(-1, 2)
                a[ij[:, 0], ij[:, 1]] = True
            out.append(a)
        return out

    def _sets(self, key, arrs):
        if key not in self._cache:
            out = []
            for a in arrs:
                ii, jj = np.nonzero(a)
                out.append(set(zip(ii.tolist(), jj.tolist())))
            self._cache[key] = out
        return self._cache[key]

    @property
    def exists(self):
        return self._sets("exists", self._E)

    @exists.setter
    def exists(self, v):
        self._E = self._to_arrays(v)
        self._cache = {}

    @property
    def refined(self):
        return self._sets("refined", self._R)

    @refined.setter
    def refined(self, v):
        self._R = self._to_arrays(v)
        self._cache = {}

    # -------------------------------------------------------------- geometry
    def slots_per_edge(self, l):
        return self.base * 3 ** l

    def geometry(self, l, i, j):
        L = 1.0 / self.slots_per_edge(l)
        return (i * L, j * L), (L, L)

    def is_leaf(self, l, i, j):
        m = self.slots_per_edge(l)
        if not (0 <= l < self.levels and 0 <= i < m and 0 <= j < m):
            return False
        return bool(self._E[l][i, j] and not self._R[l][i, j])

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

    def slot_arrays(self):
        """Patch order as arrays (level, i, j, refined) (cached)."""
        if "slots" not in self._cache:
            lv, si, sj, rf = [], [], [], []
            for l in range(self.levels):
                ii, jj = np.nonzero(self._E[l])
                lv.append(np.full(len(ii), l, dtype=np.int64))
                si.append(ii)
                sj.append(jj)
                rf.append(self._R[l][ii, jj])
            self._cache["slots"] = tuple(np.concatenate(x) for x in (lv, si, sj, rf))
        return self._cache["slots"]

    def order(self):
        """Slots in patch order: level ascending, then (i, j)."""
        if "order" not in self._cache:
            lv, si, sj, _ = self.slot_arrays()
            self._cache["order"] = list(zip(lv.tolist(), si.tolist(), sj.tolist()))
        return list(self._cache["order"])

    def leaves(self):
        if "leaves" not in self._cache:
            lv, si, sj, rf = self.slot_arrays()
            k = ~rf
            self._cache["leaves"] = list(zip(lv[k].tolist(), si[k].tolist(), sj[k].tolist()))
        return list(self._cache["leaves"])

    def leaf_arrays(self):
        """Leaves as arrays (level, i, j), in the order of leaves() (cached)."""
        if "leaf_arrays" not in self._cache:
            lv, si, sj, rf = self.slot_arrays()
            k = ~rf
            self._cache["leaf_arrays"] = (lv[k], si[k], sj[k])
        return self._cache["leaf_arrays"]

    def buffer(self, l):
        return self.buffers[l] if l < len(self.buffers) else 1

    # ------------------------------------------------------------- hierarchy
    @staticmethod
    def _dilate(a, b):
        """Slots within Chebyshev distance b of a marked slot."""
        if b <= 0:
            return a.copy()
        m0, m1 = a.shape
        p = np.pad(a, b)
        out = np.zeros_like(a)
        for di in range(2 * b + 1):
            for dj in range(2 * b + 1):
                out |= p[di:di + m0, dj:dj + m1]
        return out

    @staticmethod
    def _children(a):
        return a.repeat(3, axis=0).repeat(3, axis=1)

    def refine_from(self, flags):
        """Build the hierarchy top-down from refinement flags: flags(l, i, j)
        is called for every existing slot of levels 0 .. levels-2."""
        E = [e.copy() for e in self._E]
        R = [np.zeros_like(e) for e in E]
        for l in range(self.levels - 1):
            core = np.zeros_like(E[l])
            for i, j in zip(*np.nonzero(E[l])):
                core[i, j] = bool(flags(l, int(i), int(j)))
            R[l] = self._dilate(core, self.buffer(l)) & E[l]
            E[l + 1] = self._children(R[l])
        self.set_arrays(E, R)

    def _values(self, g):
        """Per-level arrays of the criterion g (dict (l, i, j) -> value, or an
        object with an `arrays` attribute (level, i, j, value)); 0 where absent."""
        G = [np.zeros((m, m)) for m in self._sizes()]
        if hasattr(g, "arrays"):
            lv, ii, jj, vv = g.arrays
        elif len(g):
            kk = np.array(list(g.keys()), dtype=np.int64).reshape(-1, 3)
            lv, ii, jj = kk[:, 0], kk[:, 1], kk[:, 2]
            vv = np.fromiter(g.values(), dtype=np.float64, count=len(g))
        else:
            return G
        for l in range(self.levels):
            k = lv == l
            G[l][ii[k], jj[k]] = vv[k]
        return G

    def decide(self, g):
        """Next (exists, refined), as per-level boolean arrays, from the
        refinement criterion g[(l, i, j)] of every leaf; the grid itself is
        unchanged.  A refined slot stays refined unless all 9 children are
        leaves below the threshold; a leaf above the threshold refines;
        refined regions grow by buffers[l] slots within the existing ones."""
        thr = self.threshold
        L = self.levels
        G = self._values(g)
        leaf = [self._E[l] & ~self._R[l] for l in range(L)]
        keep = []
        for l in range(L - 1):
            m = self.slots_per_edge(l)
            ok = (leaf[l + 1] & (G[l + 1] < thr)).reshape(m, 3, m, 3).all(axis=(1, 3))
            keep.append(self._R[l] & ~ok)
        E = [self._E[0].copy()] + [None] * (L - 1)
        R = [None] * L
        for l in range(L - 1):
            core = (keep[l] & E[l]) | (E[l] & leaf[l] & (G[l] > thr))
            R[l] = self._dilate(core, self.buffer(l)) & E[l]
            E[l + 1] = self._children(R[l])
        R[L - 1] = np.zeros_like(E[L - 1])
        return E, R

    def decide_py(self, g):
        """decide() on the set views, slot by slot (the reference for tests).
        Returns lists of sets."""
        thr = self.threshold
        L = self.levels
        keep = [set() for _ in range(L)]
        for l in range(L - 1):
            for (i, j) in self.refined[l]:
                kids = [(3 * i + a, 3 * j + c) for a in range(3) for c in range(3)]
                if any(not (self.is_leaf(l + 1, *ch) and g.get((l + 1,) + ch, 0.0) < thr) for ch in kids):
                    keep[l].add((i, j))
        exists = [set(self.exists[0])] + [set() for _ in range(L - 1)]
        refined = [set() for _ in range(L)]
        for l in range(L - 1):
            core = {s for s in keep[l] if s in exists[l]}
            core |= {s for s in exists[l] if self.is_leaf(l, *s) and g.get((l,) + s, 0.0) > thr}
            buf = self.buffer(l)
            refined[l] = {(i + di, j + dj) for (i, j) in core for di in range(-buf, buf + 1)
                          for dj in range(-buf, buf + 1) if (i + di, j + dj) in exists[l]}
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
        lv, ii, jj, rf = self.slot_arrays()
        lvl, si, sj = (np.ascontiguousarray(a, dtype=np.int32) for a in (lv, ii, jj))
        ref = rf.astype(np.uint8)
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
        leaf = (ref == 0).tolist()
        return _Layout({"order": order, "pos": pos, "size": size,
                "leaf": leaf, "level": lvl.tolist(), "wall": walls[:npch].tolist(),
                "items": items[:ni.value].copy(), "flux_items": flux[:nf.value].copy(),
                "restrict_items": restr[:nr.value].copy(),
                "restr_lower": lower[:npch].copy(), "restr_upper": upper[:npch].copy(),
                "virtual_time_items": self._virtual_time_items(lv, ii, jj, rf)})

    def _virtual_time_items(self, lv, ii, jj, rf):
        """virtual_time_items() on the slot arrays: every leaf against each
        refined ancestor, found by binary search of the ancestors' keys in the
        patch order (which is sorted by (level, i, j))."""
        M = self.slots_per_edge(self.levels - 1)
        keys = (lv * M + ii) * M + jj
        lf = np.nonzero(~rf)[0]
        vs, ss = [], []
        for d in range(1, self.levels):
            s = lf[lv[lf] >= d]
            f = 3 ** d
            ak = ((lv[s] - d) * M + ii[s] // f) * M + jj[s] // f
            pos = np.searchsorted(keys, ak)
            ok = pos < len(keys)
            ok[ok] = keys[pos[ok]] == ak[ok]
            ok[ok] = rf[pos[ok]]
            vs.append(pos[ok])
            ss.append(s[ok])
        if not vs:
            return np.zeros((0, 2), dtype=np.int32)
        v = np.concatenate(vs)
        s = np.concatenate(ss)
        o = np.lexsort((s, v))
        return np.stack([s[o], v[o]], axis=1).astype(np.int32).reshape(-1, 2)

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


_POOL = None


def _pool():
    global _POOL
    if _POOL is None:
        import os
        from concurrent.futures import ThreadPoolExecutor
        _POOL = ThreadPoolExecutor(max_workers=max(1, min(16, os.cpu_count() or 1)))
    return _POOL


def ghost_centers_many(pos, size, n):
    """Cell centres with ghost ring of many patches at once, (K, n+2, n+2)
    each: the values of scenarios._centers(pos[k], size[k], n, ghost=True),
    element for element."""
    pos = np.asarray(pos, dtype=np.float64).reshape(-1, 2)
    size = np.asarray(size, dtype=np.float64).reshape(-1, 2)
    r = np.arange(-1, n + 1)
    h0 = (size[:, 0] / n)[:, None]
    h1 = (size[:, 1] / n)[:, None]
    xs = (pos[:, 0:1] + h0 * r) + h0 * 0.5
    ys = (pos[:, 1:2] + h1 * r) + h1 * 0.5
    K = len(pos)
    X = np.ascontiguousarray(np.broadcast_to(xs[:, :, None], (K, n + 2, n + 2)))
    Y = np.ascontiguousarray(np.broadcast_to(ys[:, None, :], (K, n + 2, n + 2)))
    return X, Y


def bathymetry_many(b_of, pos, size, n, chunk=None):
    """b_of over the ghost-ring cell centres of many new patches: one
    vectorised call per chunk of patches, the chunks spread over the host's
    cores (numpy releases the interpreter lock inside its array loops).
    b_of must be elementwise, as every scenario's is."""
    X, Y = ghost_centers_many(pos, size, n)
    return eval_many(b_of, X, Y, chunk)


def eval_many(f, X, Y, chunk=None):
    """f(X, Y) for an elementwise f over (K, ...) arrays, in chunks of patches
    spread over the host's cores."""
    K = len(X)
    if K == 0:
        return np.zeros_like(X)
    if chunk is None:
        workers = _pool()._max_workers
        chunk = max(32, -(-K // workers))
    parts = [(a, min(K, a + chunk)) for a in range(0, K, chunk)]
    if len(parts) == 1:
        return np.asarray(f(X, Y), dtype=np.float64)
    out = np.empty(X.shape, dtype=np.float64)

    def one(ab):
        a, b = ab
        out[a:b] = f(X[a:b], Y[a:b])

    list(_pool().map(one, parts))
    return out


def remesh(grid, backend, g, b_of):
    """Apply grid.decide(g) through `backend` and update `grid`.

    backend provides: handle(slot), forget(slot), alloc(slot, pos, size,
    level) -> handle of a fresh zero-filled leaf, free(handle),
    set_leaf(handle, leaf, wall), times(handle) -> (time, dt, est_next),
    set_times(handle, time, dt, est), set_b(handle, b),
    interpolate_child(parent, child), coarsen(parent, children),
    switch_to_leaf(handle), install(layout, handles), restrict_all().
    Returns (#refined, #coarsened)."""
    E1, R1 = grid.decide(g)
    E0, R0 = grid.arrays()
    if all(np.array_equal(a, b) for a, b in zip(E1 + R1, E0 + R0)):
        return 0, 0
    n = grid.n
    n_ref = n_crs = 0
    # refinement, coarse to fine: children of newly refined slots, created one
    # level at a time (a new child can be refined in the same remesh)
    for l in range(grid.levels - 1):
        kids = []
        for i, j in np.argwhere(R1[l] & ~R0[l]).tolist():
            parent = backend.handle((l, i, j))
            t = backend.times(parent)
            for a in range(3):
                for c in range(3):
                    ch = (l + 1, 3 * i + a, 3 * j + c)
                    if E0[l + 1][ch[1], ch[2]]:
                        continue
                    pos, size = grid.geometry(*ch)
                    kids.append([parent, ch, pos, size, l + 1, t, None])
            n_ref += 1
        # bathymetry of the new children (with ghost ring) in one batch
        bs = bathymetry_many(b_of, [k[2] for k in kids], [k[3] for k in kids], n)
        for k, b in zip(kids, bs):
            k[6] = b
        kids = [tuple(k) for k in kids]
        if hasattr(backend, "create_children"):
            backend.create_children(kids)
        else:
            for parent, ch, pos, size, lvl, t, b in kids:
                h = backend.alloc(ch, pos, size, lvl)
                backend.set_times(h, *t)
                backend.set_b(h, b)
                backend.interpolate_child(parent, h)
    # coarsening, fine to coarse: restrict the children into their parent
    for l in range(grid.levels - 2, -1, -1):
        for i, j in np.argwhere(R0[l] & ~R1[l]).tolist():
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
    # slots that are new or changed between leaf and refined get their flags
    changed = [E1[l] & (~E0[l] | (R1[l] != R0[l])) for l in range(grid.levels)]
    grid.set_arrays(E1, R1)
    lay = grid.layout()
    # positions in the patch order (sorted by level, i, j) by binary search
    lv, si, sj, _ = grid.slot_arrays()
    M = grid.slots_per_edge(grid.levels - 1)
    keys = (lv * M + si) * M + sj
    for l in range(grid.levels):
        ch = np.argwhere(changed[l])
        if not len(ch):
            continue
        at = np.searchsorted(keys, (l * M + ch[:, 0]) * M + ch[:, 1])
        for (i, j), k in zip(ch.tolist(), at.tolist()):
            backend.set_leaf(backend.handle((l, i, j)), lay["leaf"][k], lay["wall"][k])
    backend.install(lay, [backend.handle(s) for s in lay["order"]])
    # virtual patches (new ones included) receive the restriction of the
    # current leaves before the next ghost fill reads them
    backend.restrict_all()
    return n_ref, n_crs


class LeafValues:
    """Refinement criterion of the leaves as arrays (level, i, j, value): the
    form AmrGrid.decide reads without going through a dict."""

    def __init__(self, lv, ii, jj, vv):
        self.arrays = (lv, ii, jj, vv)


class DeviceAmr:
    """Backend of `remesh` on a pcg.Context (and the grid's initial install)."""

    def __init__(self, ctx, grid, b_of, flux=True, g_flux=1.0, criterion=0):
        self.ctx, self.grid, self.b_of = ctx, grid, b_of
        self.flux, self.g_flux = flux, g_flux
        self.criterion = criterion  # pcg_refinement_criterion kind
        self.pid = {}
        self._bounds = None   # (virtual?, lower, upper) last written, per patch id
        self._order_ids = None  # (grid slot arrays, patch ids in that order) at the last install
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

    def create_children(self, kids):
        """The per-child sequence of remesh (alloc, time interval of the coarse
        patch, bathymetry, interpolation into uNew, then into uOld at the
        current time) for all new children of one level, in batched calls."""
        if not kids:
            return
        from .pcg import vector_size
        n = self.grid.n
        pids = [self.alloc(ch, pos, size, lvl) for _, ch, pos, size, lvl, _, _ in kids]
        ts = np.array([t for _, _, _, _, _, t, _ in kids], dtype=np.float64).reshape(-1, 3)
        self.ctx.set_times_many(pids, ts[:, 0], ts[:, 1], ts[:, 2])
        ln = vector_size(n)
        off = 3 * n * n + 3 * (n + 2) * (n + 2)
        packed = np.zeros(ln * len(kids))
        for k, kid in enumerate(kids):
            packed[k * ln + off:k * ln + off + (n + 2) * (n + 2)] = np.ascontiguousarray(kid[6]).ravel()
        self.ctx.upload_many(pids, packed)
        parents = [kid[0] for kid in kids]
        sz = np.tile(np.array([n, n], dtype=np.int32), (len(kids), 1))
        of = np.zeros((len(kids), 2), dtype=np.int32)
        for to_uold, current in ((0, 0), (1, 1)):
            self.ctx.interpolate_many(parents, pids, sz, of, to_uold, current, 0, True)

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
        self._order_ids = (self.grid.slot_arrays(), ids.copy())
        # restriction bounds of the virtual patches whose bounds are new or
        # changed since the last install, in one call
        virt = ~np.asarray(lay["leaf"], dtype=bool)
        vid = ids[virt]
        lo = np.asarray(lay["restr_lower"], dtype=np.float64).reshape(-1, 2)[virt]
        up = np.asarray(lay["restr_upper"], dtype=np.float64).reshape(-1, 2)[virt]
        m = int(ids.max()) + 1 if len(ids) else 0
        if self._bounds is None or len(self._bounds[0]) < m:
            old = self._bounds
            self._bounds = (np.zeros(m, dtype=bool), np.zeros((m, 2)), np.zeros((m, 2)))
            if old is not None:
                k = len(old[0])
                self._bounds[0][:k], self._bounds[1][:k], self._bounds[2][:k] = old
        known, plo, pup = self._bounds
        changed = ~known[vid] | (plo[vid] != lo).any(axis=1) | (pup[vid] != up).any(axis=1)
        if changed.any():
            self.ctx.set_restriction_bounds(vid[changed], lo[changed], up[changed])
        known[:] = False
        known[vid] = True
        plo[vid] = lo
        pup[vid] = up
        self.install_lists(lay, ids)

    def install_lists(self, lay, ids):
        """The grid's ghost, restriction, virtual-time and flux-correction
        lists with patch ids, into the context."""
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
        """The refinement criterion of every leaf, as a dict slot -> value."""
        leaves = self.grid.leaves()
        vals = self.ctx.refinement_indicator([self.pid[s] for s in leaves], self.criterion)
        return dict(zip(leaves, vals))

    def indicator_arrays(self):
        """The same values as LeafValues (what remesh() passes to decide)."""
        lv, ii, jj = self.grid.leaf_arrays()
        slots = self.grid.slot_arrays()
        # the ids of the last install are in the patch order while the grid
        # is unchanged since (its cached slot arrays are the same object)
        if self._order_ids is not None and self._order_ids[0] is slots:
            ids = self._order_ids[1][~slots[3]]
        else:
            ids = [self.pid[s] for s in self.grid.leaves()]
        return LeafValues(lv, ii, jj, self.ctx.refinement_indicator(ids, self.criterion))

    def remesh(self):
        import time
        t0 = time.perf_counter()
        g = self.indicator_arrays()
        t1 = time.perf_counter()
        r = remesh(self.grid, self, g, self.b_of)
        self.ctx.synchronize()
        t2 = time.perf_counter()
        self.timing = {"indicators_s": t1 - t0, "remesh_s": t2 - t1}
        return r
