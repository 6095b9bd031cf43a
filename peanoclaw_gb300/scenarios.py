"""Synthetic SWE workloads (patch sets, initial states, face-pair lists).

A workload is a `PatchSet`: per patch its subdivision, position, size, level
and domain-wall mask, the initial data vector of every patch in the
reference layout (uNew holds h, hu, hv; the bathymetry b is a parameter with
ghost layer, filled on the ghost ring too so that lake-at-rest states stay
exactly still across patch faces), and the ghost-layer items a Peano
traversal would issue for it (GhostlayerCompositorFunctors.cpp:23-221):
same-size neighbours copy (transferGhostlayer), neighbours of another size
interpolate (SWE interpolateSolution, h+b wrapped).

Layout of one patch vector (src/peanoclaw/grid/LinearizationZYXQ.h:20-88):
  [uNew 3*n*n][uOld 3*(n+2)^2][b (n+2)^2][fluxes 2*3*(n+n)]
"""
import numpy as np

from .pcg import PCG_GHOST_COPY, PCG_GHOST_INTERP, vector_size

NQ = 3


class PatchSet:
    def __init__(self):
        self.n = []          # subdivision (square patches)
        self.pos = []
        self.size = []
        self.level = []
        self.wall = []
        self.offsets = None  # start of each patch vector in `packed`
        self.packed = None   # all patch vectors back to back
        self.items = np.zeros((0, 9), dtype=np.int32)
        self.meta = {}

    def __len__(self):
        return len(self.n)

    def vec_len(self, p):
        return vector_size(self.n[p])

    def vector(self, p):
        o = self.offsets[p]
        return self.packed[o: o + self.vec_len(p)]

    def finalize_layout(self):
        lens = np.array([vector_size(n) for n in self.n], dtype=np.int64)
        self.offsets = np.zeros(len(lens), dtype=np.int64)
        if len(lens) > 1:
            self.offsets[1:] = np.cumsum(lens)[:-1]
        self.packed = np.zeros(int(lens.sum()), dtype=np.float64)
        return self

    def views(self, p):
        """uNew (3,n,n), uOld (3,n+2,n+2), b (n+2,n+2) views into packed."""
        n = self.n[p]
        v = self.vector(p)
        a = NQ * n * n
        o = NQ * (n + 2) * (n + 2)
        return (v[:a].reshape(NQ, n, n), v[a:a + o].reshape(NQ, n + 2, n + 2),
                v[a + o:a + o + (n + 2) * (n + 2)].reshape(n + 2, n + 2))

    def cells(self):
        return int(sum(n * n for n in self.n))


def _centers(pos, size, n, ghost=True):
    """Cell centres (Patch::getSubcellCenter) of the patch, with ghost ring."""
    h0 = size[0] / n
    h1 = size[1] / n
    r = np.arange(-1, n + 1) if ghost else np.arange(n)
    xs = (pos[0] + h0 * r) + h0 * 0.5
    ys = (pos[1] + h1 * r) + h1 * 0.5
    return np.meshgrid(xs, ys, indexing="ij")


def face_adjacent_traversal():
    """The face transfers GhostLayerCompositor issues around one vertex in 2D
    (FaceAdjacentPatchTraversal.cpph), as (source, destination, direction)
    over the vertex's 4 adjacent patches.  Peano numbers them with bit d set
    for the patch on the negative side of the vertex in dimension d; the
    direction points from the source to the destination, i.e. bits(source) -
    bits(destination).  Sources in descending index, for each its face
    neighbours in dimension order."""
    calls = []
    for src in (3, 2, 1, 0):
        for d in (0, 1):
            dst = src ^ (1 << d)
            calls.append((src, dst, tuple(((src >> e) & 1) - ((dst >> e) & 1) for e in (0, 1))))
    return calls


def edge_adjacent_traversal():
    """The corner transfers around one vertex in 2D
    (EdgeAdjacentPatchTraversal.cpph): each patch to the diagonally opposite
    one, sources in descending index; numbering and direction as in
    face_adjacent_traversal."""
    calls = []
    for src in (3, 2, 1, 0):
        dst = 3 - src
        calls.append((src, dst, tuple(((src >> e) & 1) - ((dst >> e) & 1) for e in (0, 1))))
    return calls


def _build_grid_items(ps, grid_index, nslots_x, nslots_y):
    """Face and corner items for a regular grid of equally sized slots holding
    patches of different subdivision.  Same subdivision: copy; otherwise
    interpolation from the neighbour (its subcells are larger or smaller).
    Returns an (N, 9) int32 array: kind, src, dst, size[2], src_offset[2],
    dst_offset[2] (the pcg_ghost_item layout).  The items are the calls of
    face_adjacent_traversal and edge_adjacent_traversal over every interior
    vertex (each face once), ordered by destination; every ghost cell is
    written by one item, so the order does not change the result."""
    rows = []
    for sx in range(nslots_x):
        for sy in range(nslots_y):
            d = int(grid_index[sx, sy])
            nd = ps.n[d]
            for dx, dy in ((-1, 0), (1, 0), (0, -1), (0, 1), (-1, -1), (1, -1), (-1, 1), (1, 1)):
                tx, ty = sx + dx, sy + dy
                if not (0 <= tx < nslots_x and 0 <= ty < nslots_y):
                    continue
                s = int(grid_index[tx, ty])
                ns = ps.n[s]
                # direction from source to destination (functor convention)
                dirv = (-dx, -dy)
                size = [nd if v == 0 else 1 for v in dirv]
                dst_off = [0 if v == 0 else (-1 if v == 1 else nd) for v in dirv]
                if ns == nd:
                    src_off = [0 if v == 0 else (nd - 1 if v == 1 else 0) for v in dirv]
                    rows.append([PCG_GHOST_COPY, s, d] + size + src_off + dst_off)
                else:
                    rows.append([PCG_GHOST_INTERP, s, d] + size + [0, 0] + dst_off)
    return np.array(rows, dtype=np.int32).reshape(-1, 9)


def remap_items(items, ids):
    """Items with patch indices replaced by the ids `ids[index]`."""
    out = np.array(items, dtype=np.int32, copy=True).reshape(-1, 9)
    ids = np.asarray(ids, dtype=np.int32)
    out[:, 1] = ids[out[:, 1]]
    out[:, 2] = ids[out[:, 2]]
    return out


def radial_dam_break(npx=9, n=16, radius=0.15, h_in=2.0, h_out=1.0):
    """Regular grid of npx x npx patches of n x n cells on [0,1]^2, flat
    bathymetry, h = h_in inside `radius` around the centre, reflecting walls."""
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
    for p in range(len(ps)):
        unew, uold, b = ps.views(p)
        X, Y = _centers(ps.pos[p], ps.size[p], n, ghost=False)
        r = np.sqrt((X - 0.5) ** 2 + (Y - 0.5) ** 2)
        unew[0] = np.where(r <= radius, h_in, h_out)
        b[:] = 0.0
    ps.items = _build_grid_items(ps, grid, npx, npx)
    ps.meta = {"workload": "radial dam break, %dx%d patches of %dx%d cells" % (npx, npx, n, n)}
    return ps


def gaussian_sum_bathymetry(seed, k=32, amp=(-0.5, 0.5), sigma=(0.01, 0.1)):
    rng = np.random.default_rng(seed)
    A = rng.uniform(amp[0], amp[1], k)
    S = rng.uniform(sigma[0], sigma[1], k)
    Cc = rng.uniform(0.0, 1.0, (k, 2))
    return A, S, Cc


def eval_bathymetry(X, Y, A, S, Cc):
    b = np.zeros_like(X)
    for a, s, c in zip(A, S, Cc):
        b += a * np.exp(-((X - c[0]) ** 2 + (Y - c[1]) ** 2) / (2.0 * s * s))
    return b


def bathymetry_lift(A, S, Cc, dry_area=0.2, samples=1024):
    """Constant added to the Gaussian sum so that `dry_area` of the domain lies
    above the still-water level 1 (the amplitude range alone keeps b < 1)."""
    t = (np.arange(samples) + 0.5) / samples
    X, Y = np.meshgrid(t, t, indexing="ij")
    b = eval_bathymetry(X, Y, A, S, Cc)
    return float(1.0 - np.quantile(b, 1.0 - dry_area))


def uneven_patches(grid=224, sizes=(8, 16, 32, 64), seed_sizes=1234, seed_bathy=1235,
                   seed_perturb=1236, perturb=0.1, dry_area=0.2):
    """Mosaic of grid x grid equally sized slots on [0,1]^2, each holding one
    patch whose subdivision is drawn uniformly from `sizes`; bathymetry is a sum
    of 32 Gaussians lifted so that `dry_area` of the domain is above the still
    water level, h = max(0, 1 - b) + perturb*U[-1,1] clamped >= 0, hu = hv = 0.
    grid = 224 gives 50,176 patches (about 68 M cells)."""
    rng = np.random.default_rng(seed_sizes)
    choice = rng.integers(0, len(sizes), grid * grid)
    ps = PatchSet()
    L = 1.0 / grid
    gi = np.zeros((grid, grid), dtype=np.int64)
    k = 0
    for i in range(grid):
        for j in range(grid):
            gi[i, j] = len(ps.n)
            ps.n.append(int(sizes[choice[k]]))
            k += 1
            ps.pos.append((i * L, j * L))
            ps.size.append((L, L))
            ps.level.append(0)
            m = 0
            if i == 0: m |= 1
            if i == grid - 1: m |= 2
            if j == 0: m |= 4
            if j == grid - 1: m |= 8
            ps.wall.append(m)
    ps.finalize_layout()
    A, S, Cc = gaussian_sum_bathymetry(seed_bathy)
    lift = bathymetry_lift(A, S, Cc, dry_area) if dry_area > 0 else 0.0
    nall = np.array(ps.n)
    cell_start = np.zeros(len(ps) + 1, dtype=np.int64)
    cell_start[1:] = np.cumsum(nall * nall)
    # one perturbation draw per interior cell, in patch order
    pert = np.random.default_rng(seed_perturb).uniform(-1.0, 1.0, int(cell_start[-1]))
    posx = np.array([q[0] for q in ps.pos])
    posy = np.array([q[1] for q in ps.pos])
    dry = 0
    for n in sizes:
        idx = np.nonzero(nall == n)[0]
        h0 = L / n
        r = np.arange(-1, n + 1)
        for c0 in range(0, len(idx), 1024):
            sel = idx[c0:c0 + 1024]
            xs = (posx[sel, None] + h0 * r[None, :]) + h0 * 0.5
            ys = (posy[sel, None] + h0 * r[None, :]) + h0 * 0.5
            X = np.broadcast_to(xs[:, :, None], (len(sel), n + 2, n + 2))
            Y = np.broadcast_to(ys[:, None, :], (len(sel), n + 2, n + 2))
            bb = eval_bathymetry(X, Y, A, S, Cc) + lift
            pr = np.stack([pert[cell_start[p]:cell_start[p + 1]].reshape(n, n) for p in sel])
            h = np.maximum(np.maximum(0.0, 1.0 - bb[:, 1:-1, 1:-1]) + perturb * pr, 0.0)
            dry += int(np.count_nonzero(h <= 0.01))
            base = ps.offsets[sel]
            a = 3 * n * n
            o = 3 * (n + 2) * (n + 2)
            hi = base[:, None] + np.arange(n * n)[None, :]
            ps.packed[hi] = h.reshape(len(sel), n * n)
            bi = base[:, None] + a + o + np.arange((n + 2) * (n + 2))[None, :]
            ps.packed[bi] = bb.reshape(len(sel), (n + 2) * (n + 2))
    total = int(cell_start[-1])
    ps.items = _build_grid_items(ps, gi, grid, grid)
    ps.meta = {"workload": "uneven patches %d x {%s}^2 cells" % (len(ps), ",".join(map(str, sizes))),
               "dry_fraction": dry / max(1, total), "bathymetry_lift": lift}
    return ps


def breaking_dam_amr(base=9, n=27, levels=3, buffers=(1, 2), x_dam=0.5, h_left=1.0, h_right=0.5,
                     bump=(0.2, 0.05, 0.7, 0.5), threshold=0.1):
    """Adaptive breaking dam on [0,1]^2 with Peano-style 3x refinement.

    Level l has (base * 3^l)^2 patch slots of n x n cells.  A patch is refined
    when the BreakingDam gradient criterion (max |grad h| over forward
    differences inside the patch, BreakingDam.cpp:85-139) exceeds `threshold`
    for it or for a patch within `buffers[l]` slots, so that leaves of
    neighbouring patches differ by at most one level.  Refined patches stay as
    virtual patches (they receive the restriction of their leaves for the
    ghost layers of coarse neighbours).  h = h_left for x < x_dam else h_right,
    b = a * exp(-|x - c|^2 / (2 s^2)) with bump = (a, s, cx, cy).

    Returns a PatchSet with, in addition to the usual fields, `leaf`,
    `restr_lower`, `restr_upper`, `restrict_items` ((N,2) src, dst) and
    `flux_items` ((N,4) src, dst, dim, dir)."""
    a_b, s_b, cx_b, cy_b = bump

    def h_of(X, Y=None):
        return np.where(X < x_dam, h_left, h_right)

    def b_of(X, Y):
        return a_b * np.exp(-((X - cx_b) ** 2 + (Y - cy_b) ** 2) / (2.0 * s_b * s_b))

    def needs_refine(level, i, j):
        m = base * 3 ** level
        L = 1.0 / m
        X, Y = _centers((i * L, j * L), (L, L), n, ghost=False)
        h = h_of(X)
        dx = L / n
        gx = (h[1:, :-1] - h[:-1, :-1]) / dx
        gy = (h[:-1, 1:] - h[:-1, :-1]) / dx
        return float(np.max(np.sqrt(np.abs(gx) * np.abs(gx) + np.abs(gy) * np.abs(gy)))) > threshold

    from .amr import AmrGrid
    grid = AmrGrid(base, n, levels, buffers=buffers, threshold=threshold)
    grid.refine_from(needs_refine)
    ps = amr_patchset(grid, h_of, b_of)
    ps.grid = grid
    ps.h_of, ps.b_of = h_of, b_of
    return ps


def amr_patchset(grid, h_of, b_of):
    """PatchSet of an AmrGrid: patch order, geometry, leaf flags, walls, the
    ghost / flux / restriction lists and the restriction bounds; leaves get
    h = h_of(x, y) (at rest), every patch b = b_of(x, y) including its ghost ring."""
    lay = grid.layout()
    n = grid.n
    ps = PatchSet()
    ps.leaf = list(lay["leaf"])
    for k in range(len(lay["order"])):
        ps.n.append(n)
        ps.pos.append(lay["pos"][k])
        ps.size.append(lay["size"][k])
        ps.level.append(lay["level"][k])
        ps.wall.append(lay["wall"][k])
    ps.finalize_layout()
    # every patch's cell centres at once; b and h evaluated in batches over
    # the host's cores (the values of a per-patch evaluation, element for
    # element)
    from .amr import eval_many, ghost_centers_many
    X, Y = ghost_centers_many(ps.pos, ps.size, n)
    B = eval_many(b_of, X, Y)
    leaves = [p for p in range(len(ps)) if ps.leaf[p]]
    H = eval_many(h_of, np.ascontiguousarray(X[leaves, 1:-1, 1:-1]),
                  np.ascontiguousarray(Y[leaves, 1:-1, 1:-1])) if leaves else None
    hk = {p: k for k, p in enumerate(leaves)}
    for p in range(len(ps)):
        unew, uold, b = ps.views(p)
        b[:] = B[p]
        if ps.leaf[p]:
            unew[0] = H[hk[p]]
    ps.items = lay["items"]
    ps.flux_items = lay["flux_items"]
    ps.restrict_items = lay["restrict_items"]
    ps.restr_lower = lay["restr_lower"]
    ps.restr_upper = lay["restr_upper"]
    ps.virtual_time_items = lay["virtual_time_items"]
    ps.meta = {"workload": "adaptive grid, %d levels, %d patches (%d leaves) of %dx%d cells"
                           % (grid.levels, len(ps), sum(ps.leaf), n, n),
               "leaf_cells": int(sum(n * n for p in range(len(ps)) if ps.leaf[p]))}
    return ps


def install_amr(ctx, ps, flux=True, g_flux=1.0):
    """Allocate an adaptive PatchSet (breaking_dam_amr) in a pcg.Context:
    leaves and virtual patches with their restriction bounds, the ghost
    face-pair list, the restriction list, the virtual-time list (local time
    stepping) and (flux=True) the flux-correction list.  Returns the patch
    ids in PatchSet order."""
    ids = []
    for p in range(len(ps)):
        leaf = bool(ps.leaf[p])
        pid = ctx.alloc(ps.n[p], pos=ps.pos[p], size=ps.size[p], level=ps.level[p], leaf=leaf,
                        virtual=not leaf)
        ids.append(pid)
        if ps.wall[p]:
            ctx.set_boundary(pid, ps.wall[p])
        if not leaf:
            ctx.set_time(pid, restr_lower=ps.restr_lower[p], restr_upper=ps.restr_upper[p])
    ids = np.array(ids, dtype=np.int32)
    ctx.upload_many(ids, ps.packed)
    ctx.set_ghost_items(remap_items(ps.items, ids))
    ctx.set_restriction_items(ids[ps.restrict_items[:, 0]], ids[ps.restrict_items[:, 1]], True)
    vt = getattr(ps, "virtual_time_items", None)
    if vt is not None and len(vt):
        ctx.set_virtual_time_items(ids[vt[:, 0]], ids[vt[:, 1]])
    if flux and len(ps.flux_items):
        f = ps.flux_items
        ctx.set_flux_correction_items(ids[f[:, 0]], ids[f[:, 1]], f[:, 2], f[:, 3], g_flux)
    return ids


def adaptive_tsunami(base=27, n=27, levels=3, hump=(0.5, 0.02, 0.4, 0.5), coast=(0.9, 0.95),
                     threshold=0.1, buffers=(1, 2)):
    """Gaussian surface hump over a flat seafloor that ramps up to a coastline:
    b = 0 for x < coast[0], rising linearly to the still-water surface (1.0)
    at x = coast[1] and above it beyond (dry land).  h = max(0, 1 + A exp(-r^2 /
    (2 s^2)) - b) with hump = (A, s, cx, cy), at rest.  The hierarchy is
    refined where the BreakingDam criterion of the initial state exceeds
    `threshold` (levels of 3x refinement, n x n cells per patch; base = 27,
    n = 27, levels = 3 is a 6561^2 grid when fully refined)."""
    from .amr import AmrGrid
    A, s, cx, cy = hump
    x0, x1 = coast

    def b_of(X, Y):
        return np.where(X < x0, 0.0, (X - x0) * (1.0 / (x1 - x0)))

    def h_of(X, Y):
        eta = 1.0 + A * np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2.0 * s * s))
        return np.maximum(0.0, eta - b_of(X, Y))

    def needs_refine(level, i, j):
        m = base * 3 ** level
        L = 1.0 / m
        X, Y = _centers((i * L, j * L), (L, L), n, ghost=False)
        h = h_of(X, Y)
        dx = L / n
        gx = (h[1:, :-1] - h[:-1, :-1]) / dx
        gy = (h[:-1, 1:] - h[:-1, :-1]) / dx
        return float(np.max(np.sqrt(np.abs(gx) * np.abs(gx) + np.abs(gy) * np.abs(gy)))) > threshold

    grid = AmrGrid(base, n, levels, buffers=buffers, threshold=threshold)
    grid.refine_from(needs_refine)
    ps = amr_patchset(grid, h_of, b_of)
    ps.grid = grid
    ps.h_of, ps.b_of = h_of, b_of
    return ps


def coastal_tsunami(base=27, n=27, levels=3, hump=(0.5, 0.02, 0.5, 0.5), seed_bathy=2000,
                    coast=(0.95, 2.5), threshold=0.1, buffers=(1, 2)):
    """Large adaptive tsunami: a Gaussian surface hump of amplitude A and
    width s at (cx, cy) (hump = (A, s, cx, cy)) over a random seafloor, the
    sum of 32 Gaussians of the uneven-patch generator (amplitudes in
    [-0.5, 0.5], widths in [0.01, 0.1], seeded with `seed_bathy`), with a
    coastline along x = 1: in the last 5 % of the domain (x > coast[0]) the
    seafloor rises linearly by coast[1] at x = 1, above the still-water
    surface 1.  h = max(0, 1 + A exp(-r^2 / (2 s^2)) - b), at rest, so the
    dry land and any islands start dry.

    Refinement follows the surface elevation h + b (pcg_refinement_criterion
    kind PCG_CRIT_SURFACE_GRADIENT, the BreakingDam stencil and threshold on
    the surface that BowlOcean's wave-front criterion differences): a still
    lake over the bumpy seafloor stays coarse, the hump, the waves it sends
    out and the coastline refine.  base = 27, n = 27, levels = 3 is an
    effective 6561^2 grid (243^2 patches when fully refined)."""
    from .amr import AmrGrid
    from .pcg import PCG_CRIT_SURFACE_GRADIENT
    A, s, cx, cy = hump
    GA, GS, GC = gaussian_sum_bathymetry(seed_bathy)
    x0, rise = coast

    def b_of(X, Y):
        return eval_bathymetry(X, Y, GA, GS, GC) + np.maximum(0.0, X - x0) * (rise / (1.0 - x0))

    def h_of(X, Y):
        eta = 1.0 + A * np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2.0 * s * s))
        return np.maximum(0.0, eta - b_of(X, Y))

    def needs_refine(level, i, j):
        m = base * 3 ** level
        L = 1.0 / m
        X, Y = _centers((i * L, j * L), (L, L), n, ghost=False)
        q = h_of(X, Y) + b_of(X, Y)
        dx = L / n
        gx = (q[1:, :-1] - q[:-1, :-1]) / dx
        gy = (q[:-1, 1:] - q[:-1, :-1]) / dx
        return float(np.max(np.sqrt(np.abs(gx) * np.abs(gx) + np.abs(gy) * np.abs(gy)))) > threshold

    grid = AmrGrid(base, n, levels, buffers=buffers, threshold=threshold)
    grid.refine_from(needs_refine)
    ps = amr_patchset(grid, h_of, b_of)
    ps.grid = grid
    ps.h_of, ps.b_of = h_of, b_of
    ps.criterion = PCG_CRIT_SURFACE_GRADIENT
    ps.meta["workload"] = ("coastal tsunami over a sum-of-Gaussians seafloor, " + ps.meta["workload"])
    return ps
