"""Dynamic remeshing (AmrGrid.decide + remesh) on the oracle: the hierarchy
follows a moving breaking-dam front (refines ahead of it, coarsens behind
it) and keeps the invariants of the patch lists; refining and coarsening a
lake at rest keeps it at rest up to round-off (the d-linear interpolation
weights and the 1/9 area weights of the restriction are not exact in binary,
and the steps on the refined grid move those ulps around)."""
import copy

import numpy as np

from helpers import OracleAmr, oracle_params
from peanoclaw_gb300 import pcg as P
from peanoclaw_gb300 import scenarios as S
from peanoclaw_gb300.amr import AmrGrid, LeafValues

PRM = P.swe_params(g=9.81, cfl=0.5)


def _check_lists(grid):
    lay = grid.layout()
    idx = lay["index"]
    for (l, i, j) in lay["order"]:
        if (i, j) in grid.refined[l]:
            for a in range(3):
                for c in range(3):
                    assert (l + 1, 3 * i + a, 3 * j + c) in idx
        if l > 0:
            assert (i // 3, j // 3) in grid.refined[l - 1]
    leaf = lay["leaf"]
    for row in lay["items"]:
        assert leaf[row[2]]          # ghost fill writes leaves only
    for s, d in lay["restrict_items"]:
        assert leaf[s] and not leaf[d]
    # leaves cover the domain exactly once
    area = sum(lay["size"][k][0] * lay["size"][k][1] for k in range(len(leaf)) if leaf[k])
    assert abs(area - 1.0) < 1e-12


def test_remesh_follows_a_moving_front():
    ps = S.breaking_dam_amr(base=3, n=9, levels=3, h_left=1.0, h_right=0.2, threshold=1.0)
    grid = ps.grid
    _check_lists(grid)
    b_of = ps.b_of
    be = OracleAmr(grid, ps, b_of)
    prm = oracle_params(PRM)
    history = []
    for r in range(10):
        for _ in range(4):
            be.step(prm, 1e9)
        history.append(be.remesh())
        _check_lists(grid)
        assert set(be.pat) == set(grid.order())
    refined = sum(h[0] for h in history)
    coarsened = sum(h[1] for h in history)
    assert refined > 0 and coarsened > 0
    for p in be.patches():
        assert np.all(np.isfinite(p.u))


def test_remesh_of_a_lake_at_rest_keeps_it_at_rest():
    # flat surface over a bump: refinement forced everywhere the criterion of
    # a stepped threshold says so, then everything coarsens again
    ps = S.breaking_dam_amr(base=3, n=9, levels=2, h_left=1.0, h_right=1.0,
                            bump=(0.0, 0.05, 0.7, 0.5))
    grid = ps.grid
    b_of = ps.b_of
    be = OracleAmr(grid, ps, b_of)
    g_all = {s: 1.0 for s in grid.leaves()}   # every leaf asks to refine
    from peanoclaw_gb300.amr import remesh
    remesh(grid, be, g_all, b_of)
    assert len(grid.exists[1]) == 9 * 9
    prm = oracle_params(PRM)
    for _ in range(3):
        be.step(prm, 1e9)
    g_none = {s: 0.0 for s in grid.leaves()}
    remesh(grid, be, g_none, b_of)
    assert len(grid.exists[1]) == 0
    for p in be.patches():
        assert np.max(np.abs(p.unew()[0] - 1.0)) <= 1e-14
        assert np.max(np.abs(p.unew()[1:])) <= 1e-14


def test_native_layout_equals_the_python_builder():
    """pcg_amr_layout (library) and AmrGrid.layout_py give the same lists."""
    grids = [S.breaking_dam_amr(base=3, n=9, levels=3).grid,
             S.breaking_dam_amr(base=4, n=6, levels=3, buffers=(2, 1)).grid,
             S.adaptive_tsunami(base=5, n=8, levels=3).grid]
    # and one after a remesh of a moving front
    ps = S.breaking_dam_amr(base=3, n=9, levels=3, h_left=1.0, h_right=0.2, threshold=1.0)
    be = OracleAmr(ps.grid, ps, ps.b_of)
    prm = oracle_params(PRM)
    for _ in range(8):
        be.step(prm, 1e9)
    be.remesh()
    grids.append(ps.grid)
    for g in grids:
        a, b = g.layout(), g.layout_py()
        assert a["order"] == b["order"]
        for k in ("items", "flux_items", "restrict_items", "restr_lower", "restr_upper", "wall",
                  "leaf", "level", "pos", "size", "virtual_time_items"):
            assert np.array_equal(np.asarray(a[k]), np.asarray(b[k])), k


def test_array_decision_equals_the_slot_by_slot_decision():
    """AmrGrid.decide (per-level arrays) and AmrGrid.decide_py (sets, slot by
    slot) give the same next hierarchy for random criterion values around
    the threshold, on grids with and without refined regions."""
    rng = np.random.default_rng(7)
    grids = [S.breaking_dam_amr(base=3, n=9, levels=3, h_left=1.0, h_right=0.2, threshold=1.0).grid,
             S.breaking_dam_amr(base=4, n=6, levels=3, buffers=(2, 1)).grid,
             S.adaptive_tsunami(base=5, n=8, levels=3).grid,
             AmrGrid(3, 4, 2)]
    for grid in grids:
        leaves = grid.leaves()
        for scale in (0.5, 1.0, 2.0):
            vals = rng.uniform(0.0, 2.0 * scale * grid.threshold, len(leaves))
            g = dict(zip(leaves, vals.tolist()))
            E, R = grid.decide(g)
            e2, r2 = grid.decide_py(g)
            for l in range(grid.levels):
                assert set(map(tuple, np.argwhere(E[l]).tolist())) == e2[l]
                assert set(map(tuple, np.argwhere(R[l]).tolist())) == r2[l]
            # the same values as leaf arrays (what the device driver passes)
            lv, ii, jj = grid.leaf_arrays()
            assert list(zip(lv.tolist(), ii.tolist(), jj.tolist())) == leaves
            E3, R3 = grid.decide(LeafValues(lv, ii, jj, vals))
            for l in range(grid.levels):
                assert np.array_equal(E3[l], E[l]) and np.array_equal(R3[l], R[l])


class _FakeCtx:
    """The calls DeviceAmr.install and indicator_arrays make, recorded; the
    criterion of patch id k is k / 1000."""

    def __init__(self):
        self.calls = []

    def refinement_indicator(self, ids, kind=None):
        ids = np.asarray(ids, dtype=np.int64)
        self.calls.append(("indicator", ids.copy()))
        return ids.astype(np.float64) / 1000.0

    def __getattr__(self, name):
        def record(*a, **k):
            self.calls.append((name, a))
        return record


def test_device_indicator_arrays_follow_the_leaf_order():
    """DeviceAmr.indicator_arrays (what DeviceAmr.remesh passes to decide)
    carries, per leaf in leaves() order, the value of that leaf's patch id:
    through the ids of the last install while the grid is unchanged, through
    the slot -> id map once it changed; decide reads it like the dict form."""
    from peanoclaw_gb300.amr import DeviceAmr
    ps = S.breaking_dam_amr(base=3, n=9, levels=3, h_left=1.0, h_right=0.2, threshold=1.0)
    grid = ps.grid
    ctx = _FakeCtx()
    dev = DeviceAmr(ctx, grid, ps.b_of)
    order = grid.order()
    ids = np.arange(100, 100 + len(order))[::-1].copy()   # ids unrelated to positions
    dev.pid = dict(zip(order, ids.tolist()))
    leaves = grid.leaves()
    want = np.array([dev.pid[s] for s in leaves], dtype=np.float64) / 1000.0
    # before any install: the slot -> id map
    lv, ii, jj, vv = dev.indicator_arrays().arrays
    assert list(zip(lv.tolist(), ii.tolist(), jj.tolist())) == leaves
    assert np.array_equal(vv, want)
    # after an install: the install's ids, same values
    dev.install(grid.layout(), ids.tolist())
    assert dev._order_ids[0] is grid.slot_arrays()
    assert np.array_equal(dev.indicator_arrays().arrays[3], want)
    # the decision equals the one from the dict of the same values
    g = dict(zip(leaves, want.tolist()))
    for a, b in zip(grid.decide(dev.indicator_arrays()), grid.decide(g)):
        assert all(np.array_equal(x, y) for x, y in zip(a, b))
    # a changed grid invalidates the install's ids (its slot arrays are new)
    E, R = grid.decide({s: 1e9 for s in leaves})
    grid.set_arrays(E, R)
    assert dev._order_ids[0] is not grid.slot_arrays()
    new_leaves = grid.leaves()
    for k, s in enumerate(grid.order()):
        dev.pid.setdefault(s, 10_000 + k)
    got = dev.indicator_arrays().arrays[3]
    assert np.array_equal(got, np.array([dev.pid[s] for s in new_leaves], dtype=np.float64) / 1000.0)
