"""The ghost-layer transfers around a vertex (GhostLayerCompositor's face and
corner traversals) and the face-pair lists built from them (CPU).

Known answers: GhostLayerCompositorTest::testFaceAdjacentPatchTraversal2D and
testEdgeAdjacentPatchTraversal2D (GhostLayerCompositorTest.cpp:747-843), the
calls (source, destination, direction) in order.  The lists of the mosaic
builders hold exactly the calls of both traversals over every interior
vertex, and no ghost cell is written by two items, so the order of a list
(by destination, not by vertex) cannot change what the ghost fill writes."""
import numpy as np

from peanoclaw_gb300 import scenarios as S

# GhostLayerCompositorTest.cpp:747-806
FACE_CALLS = [(3, 2, (1, 0)), (3, 1, (0, 1)), (2, 3, (-1, 0)), (2, 0, (0, 1)),
              (1, 0, (1, 0)), (1, 3, (0, -1)), (0, 1, (-1, 0)), (0, 2, (0, -1))]
# GhostLayerCompositorTest.cpp:808-843
EDGE_CALLS = [(3, 0, (1, 1)), (2, 1, (-1, 1)), (1, 2, (1, -1)), (0, 3, (-1, -1))]


def test_face_adjacent_traversal_known_answer():
    assert S.face_adjacent_traversal() == FACE_CALLS


def test_edge_adjacent_traversal_known_answer():
    assert S.edge_adjacent_traversal() == EDGE_CALLS


def _slot_grid(ps):
    """Slot (i, j) -> patch index of a mosaic of equally sized slots."""
    L = ps.size[0][0]
    m = int(round(1.0 / L))
    g = np.full((m, m), -1, dtype=np.int64)
    for p in range(len(ps)):
        g[int(round(ps.pos[p][0] / L)), int(round(ps.pos[p][1] / L))] = p
    assert (g >= 0).all()
    return g


def _direction(item, n_dst):
    """Direction (source -> destination) of an item from its destination
    offset: the ghost layer below (-1) lies towards a source on the negative
    side."""
    off = item[7:9]
    return tuple(1 if o == -1 else (-1 if o == n_dst else 0) for o in off)


def _check(ps):
    g = _slot_grid(ps)
    m = g.shape[0]
    # the traversals over every interior vertex: patch k of vertex (vx, vy)
    # sits in slot (vx - bit0(k), vy - bit1(k))
    want = set()
    for vx in range(1, m):
        for vy in range(1, m):
            slot = {k: g[vx - (k & 1), vy - ((k >> 1) & 1)] for k in range(4)}
            for src, dst, d in S.face_adjacent_traversal() + S.edge_adjacent_traversal():
                want.add((int(slot[src]), int(slot[dst]), d))
    have = set()
    for it in np.asarray(ps.items):
        t = (int(it[1]), int(it[2]), _direction(it, ps.n[int(it[2])]))
        assert t not in have, t          # every call once
        have.add(t)
    assert have == want
    # every ghost cell written once
    for d in range(len(ps)):
        n = ps.n[d]
        hits = np.zeros((n + 2, n + 2), dtype=np.int64)
        for it in np.asarray(ps.items)[np.asarray(ps.items)[:, 2] == d]:
            sx, sy = it[3], it[4]
            ox, oy = it[7] + 1, it[8] + 1
            hits[ox:ox + sx, oy:oy + sy] += 1
        assert hits.max() <= 1
        assert hits[1:-1, 1:-1].sum() == 0   # only ghost cells


def test_mosaic_lists_are_the_vertex_traversals():
    _check(S.uneven_patches(grid=6, sizes=(8, 16, 32)))


def test_regular_grid_lists_are_the_vertex_traversals():
    _check(S.radial_dam_break(npx=5, n=8))


def test_adaptive_lists_write_each_ghost_cell_once():
    """The same for the lists of the adaptive hierarchies (copies between
    leaves of one level, interpolation from coarser leaves and virtual
    patches, corners included): no ghost cell of a destination is written
    twice and no interior cell at all."""
    for ps in (S.breaking_dam_amr(base=3, n=9, levels=3), S.adaptive_tsunami(base=5, n=8, levels=3)):
        items = np.asarray(ps.items)
        for d in np.unique(items[:, 2]):
            n = ps.n[int(d)]
            hits = np.zeros((n + 2, n + 2), dtype=np.int64)
            for it in items[items[:, 2] == d]:
                ox, oy = it[7] + 1, it[8] + 1
                hits[ox:ox + it[3], oy:oy + it[4]] += 1
            assert hits.max() <= 1 and hits[1:-1, 1:-1].sum() == 0, int(d)
