"""The oracle's local-time-stepping iteration (pco_grid_step_lts) on the CPU:
with max_dt below every CFL dt it is the synchronous step; otherwise every
leaf reaches the end time exactly, no advancing leaf lies ahead of its ghost
sources, and fewer cell updates are spent than with the synchronous step."""
import numpy as np

from helpers import oracle_params, oracle_patchset
from oracle import oracle as O
from peanoclaw_gb300 import pcg as P
from peanoclaw_gb300 import scenarios as S

PRM = P.swe_params(g=9.81, cfl=0.5)


def _tu(p):
    return p.s.time + p.s.dt


def test_small_max_dt_is_the_synchronous_step():
    ps = S.uneven_patches(grid=4, sizes=(8, 16))
    prm = oracle_params(PRM)
    a, b = oracle_patchset(ps), oracle_patchset(ps)
    for _ in range(5):
        dt = O.grid_step(a, ps.items, ps.wall, prm, 1e-5)[0]
        n, dto = O.grid_step_lts(b, ps.items, ps.wall, prm, 1e-5, np.inf)
        assert dt == 1e-5 and n == len(b) and np.all(dto == 1e-5)
    for p, q in zip(a, b):
        assert np.array_equal(p.u.view(np.int64), q.u.view(np.int64))
        assert (p.s.time, p.s.dt) == (q.s.time, q.s.dt)


def test_every_leaf_reaches_the_end_time_without_running_ahead():
    ps = S.uneven_patches(grid=5, sizes=(8, 16, 32))
    prm = oracle_params(PRM)
    pats = oracle_patchset(ps)
    t_end = 0.02
    src = {}
    for it in ps.items:
        src.setdefault(int(it[2]), set()).add(int(it[1]))
    lts_updates = 0
    for _ in range(1000):
        before = [_tu(p) for p in pats]
        n, dto = O.grid_step_lts(pats, ps.items, ps.wall, prm, np.inf, t_end)
        if n == 0:
            break
        for p in np.flatnonzero(dto > 0.0):
            # an advancing leaf was not ahead of any source (time tolerance 1e-8)
            assert all(before[p] <= before[s] + 1e-8 for s in src.get(int(p), ()))
            lts_updates += ps.n[p] ** 2
    assert all(_tu(p) == t_end for p in pats)
    glob = oracle_patchset(ps)
    t, steps = 0.0, 0
    while t < t_end:
        t += O.grid_step(glob, ps.items, ps.wall, prm, t_end - t)[0]
        steps += 1
    assert lts_updates < steps * sum(n * n for n in ps.n)


def test_virtual_patches_take_the_intersection_of_their_leaves_intervals():
    from helpers import oracle_amr_patchset, oracle_restrict_all
    ps = S.breaking_dam_amr(base=3, n=9, levels=3, h_left=1.0, h_right=0.2, threshold=1.0)
    prm = oracle_params(PRM)
    pats = oracle_amr_patchset(ps)
    oracle_restrict_all(pats, ps)
    t_end = 0.01
    vt = ps.virtual_time_items
    virtuals = sorted(set(vt[:, 1].tolist()))
    leaves_of = {v: vt[vt[:, 1] == v, 0] for v in virtuals}
    assert all(not ps.leaf[v] for v in virtuals) and all(ps.leaf[s] for s in vt[:, 0])
    # every leaf lies below its virtual ancestors on every level above it
    assert len(vt) == sum(ps.level[s] for s in range(len(ps)) if ps.leaf[s])
    iterations = 0
    for _ in range(3000):
        before = {s: (pats[s].s.time, _tu(pats[s])) for s in range(len(ps)) if ps.leaf[s]}
        n, dto = O.grid_step_lts(pats, ps.items, ps.wall, prm, np.inf, t_end, vt)
        for v in virtuals:
            start = max(before[s][0] for s in leaves_of[v])
            end = min(before[s][1] for s in leaves_of[v])
            assert pats[v].s.time == start and pats[v].s.dt == end - start
        if n == 0:
            break
        iterations += 1
        oracle_restrict_all(pats, ps)
    assert iterations > 50
    for p, lf in zip(pats, ps.leaf):
        if lf:
            assert _tu(p) == t_end


def _patch_test_intervals():
    # the nine fine intervals of PatchTest::testCoarsePatchTimeInterval
    # (src/peanoclaw/tests/PatchTest.cpp:140-215): (time, dt)
    return [(1.0, 2.0), (1.0, 2.0), (1.0, 3.0), (0.0, 3.0), (1.0, 1.7), (0.0, 4.0), (0.0, 3.0),
            (1.0, 2.0), (2.5, 1.5)]


def test_virtual_interval_known_answer():
    """PatchTest::testCoarsePatchTimeInterval: the coarse patch over nine fine
    patches takes time 2.5 and timestep 0.2 (the intersection of the fine
    intervals).  Here the fine patches are leaves under one virtual patch and
    an iteration that advances nothing (end time 0) sets the interval."""
    from helpers import oracle_patch_from
    leaves = []
    for k, (t, dt) in enumerate(_patch_test_intervals()):
        p = oracle_patch_from(np.zeros(P.vector_size(3)), 3, pos=((k // 3) / 3.0, (k % 3) / 3.0),
                              size=(1.0 / 3.0, 1.0 / 3.0), level=1, time=t, dt=dt)
        leaves.append(p)
    virt = oracle_patch_from(np.zeros(P.vector_size(3)), 3, pos=(0.0, 0.0), size=(1.0, 1.0), level=0,
                             leaf=False, virtual=True)
    pats = leaves + [virt]
    vt = np.array([[k, 9] for k in range(9)], dtype=np.int32)
    n, dto = O.grid_step_lts(pats, np.zeros((0, 9), dtype=np.int32), np.zeros(10, dtype=np.uint8),
                             oracle_params(PRM), np.inf, 0.0, vt)
    assert n == 0 and np.all(dto == 0.0)
    assert virt.s.time == 2.5
    assert abs(virt.s.dt - 0.2) <= 1e-12
