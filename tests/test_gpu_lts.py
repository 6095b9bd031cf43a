"""Local time stepping (pcg_set_time_stepping(PCG_TS_LOCAL)) on the GPU against
the oracle's two-phase iteration (pco_grid_step_lts): on a mosaic of patches
with different mesh widths every iteration advances the same leaves with the
same dts, and the patch vectors and time intervals agree bit for bit until
every leaf has reached the end time."""
import numpy as np
import pytest

from helpers import gpu_patchset, oracle_params, oracle_patchset, slab_for
from oracle import oracle as O
from peanoclaw_gb300 import pcg as P
from peanoclaw_gb300 import scenarios as S

pytestmark = pytest.mark.gpu

PRM = P.swe_params(g=9.81, cfl=0.5)


@pytest.mark.parametrize("sched", [(P.SCHED_STRIPS, 2, 32), (P.SCHED_STRIPS, 0, 16),
                                   (P.SCHED_TILES, 0, 32)])
def test_local_time_stepping_matches_the_oracle(sched):
    ps = S.uneven_patches(grid=5, sizes=(8, 16, 32))
    t_end = 0.02
    c = P.Context(slab_doubles=slab_for(ps), max_patches=len(ps) + 8, max_groups=1, params=PRM)
    try:
        ids = gpu_patchset(c, ps)
        c.set_group_max_dt(0, np.inf)
        c.set_group_end_time(0, 0.0, t_end)
        c.set_schedule(*sched)
        c.set_time_stepping(P.TS_LOCAL)
        pats = oracle_patchset(ps)
        prm = oracle_params(PRM)
        seen = set()
        iterations = 0
        advanced_cells = 0
        cu0, _ = c.stats()
        done = False
        while not done:
            # four iterations per replay of the captured graph
            hist = c.run(4)[:, 0]
            for k in range(4):
                n, dto = O.grid_step_lts(pats, ps.items, ps.wall, prm, np.inf, t_end)
                taken = dto[dto > 0.0]
                assert hist[k] == (taken.min() if n else 0.0), (iterations, k)
                seen.update(taken.tolist())
                advanced_cells += sum(ps.n[p] ** 2 for p in np.flatnonzero(dto > 0.0))
                if n == 0:
                    done = True
                else:
                    iterations += 1
            assert iterations < 400
        out = c.download_many(ids, int(ps.packed.size))
        ref = np.concatenate([p.u for p in pats])
        assert np.array_equal(out.view(np.int64), ref.view(np.int64))
        for p, pid in enumerate(ids):
            t = c.get_time(pid)
            assert (t["time"], t["dt"]) == (pats[p].s.time, pats[p].s.dt)
            assert t["time"] + t["dt"] == t_end
        assert c.group_times()[0] == t_end
        # the statistics count the cells of the leaves that advanced
        cu1, _ = c.stats()
        assert cu1 - cu0 == advanced_cells
        # more dts than one per step of a synchronous scheme
        assert len(seen) > 3 * iterations // 4
        # nothing changes once every leaf is at the end time
        assert np.all(c.run(2) == 0.0)
        again = c.download_many(ids, int(ps.packed.size))
        assert np.array_equal(again.view(np.int64), out.view(np.int64))
    finally:
        c.close()


def test_local_time_stepping_with_a_small_max_dt_is_the_synchronous_step():
    # every leaf's CFL dt exceeds max_dt: every leaf advances by max_dt in
    # every iteration, as in the global step
    ps = S.uneven_patches(grid=4, sizes=(8, 16))
    outs = []
    for ts in (P.TS_GLOBAL, P.TS_LOCAL):
        c = P.Context(slab_doubles=slab_for(ps), max_patches=len(ps) + 8, max_groups=1, params=PRM)
        try:
            ids = gpu_patchset(c, ps)
            c.set_group_max_dt(0, 1e-5)
            c.set_time_stepping(ts)
            hist = c.run(6)[:, 0]
            assert np.all(hist == 1e-5)
            outs.append(c.download_many(ids, int(ps.packed.size)))
        finally:
            c.close()
    assert np.array_equal(outs[0].view(np.int64), outs[1].view(np.int64))


def test_local_time_stepping_arguments_and_states():
    ps = S.uneven_patches(grid=3, sizes=(8, 16))
    c = P.Context(slab_doubles=slab_for(ps), max_patches=len(ps) + 8, max_groups=1, params=PRM)
    try:
        gpu_patchset(c, ps)
        c.set_group_max_dt(0, np.inf)
        for bad in (-1, 2, 7):
            with pytest.raises(P.PcgError):
                c.set_time_stepping(bad)
        c.set_time_stepping(P.TS_LOCAL)
        with pytest.raises(P.PcgError):
            c.step(P.PCG_MODE_PLAIN)
        with pytest.raises(P.PcgError):
            c.run(2, P.PCG_MODE_PLAIN)
        c.run(2)
        c.set_time_stepping(P.TS_GLOBAL)
        c.step(P.PCG_MODE_PLAIN)
    finally:
        c.close()


def test_local_time_stepping_across_levels_matches_the_oracle():
    # 3-level breaking dam (virtual patches between the levels): coarse leaves
    # next to a refined region wait for its finest leaves and read them
    # through the restricted virtual patches
    from helpers import oracle_amr_patchset, oracle_restrict_all
    ps = S.breaking_dam_amr(base=3, n=9, levels=3, h_left=1.0, h_right=0.2, threshold=1.0)
    assert len(ps.virtual_time_items) and not all(ps.leaf)
    t_end = 0.012
    c = P.Context(slab_doubles=8_000_000, max_patches=len(ps) + 8, max_groups=1, params=PRM)
    try:
        ids = S.install_amr(c, ps, flux=False)
        c.restrict_all()
        c.set_group_max_dt(0, np.inf)
        c.set_group_end_time(0, 0.0, t_end)
        c.set_time_stepping(P.TS_LOCAL)
        pats = oracle_amr_patchset(ps)
        oracle_restrict_all(pats, ps)
        prm = oracle_params(PRM)
        iterations = 0
        done = False
        while not done:
            hist = c.run(8)[:, 0]
            for k in range(8):
                n, dto = O.grid_step_lts(pats, ps.items, ps.wall, prm, np.inf, t_end,
                                         ps.virtual_time_items)
                if n:
                    oracle_restrict_all(pats, ps)
                    iterations += 1
                else:
                    done = True
                taken = dto[dto > 0.0]
                assert hist[k] == (taken.min() if n else 0.0), (iterations, k)
            assert iterations < 2000
        assert iterations > 50
        out = c.download_many(ids, int(ps.packed.size))
        ref = np.concatenate([p.u for p in pats])
        assert np.array_equal(out.view(np.int64), ref.view(np.int64))
        for p, pid in enumerate(ids):
            t = c.get_time(int(pid))
            assert (t["time"], t["dt"]) == (pats[p].s.time, pats[p].s.dt), p
        assert c.group_times()[0] == t_end
    finally:
        c.close()


def test_local_time_stepping_refuses_flux_correction_lists():
    ps = S.breaking_dam_amr(base=3, n=9, levels=3, h_left=1.0, h_right=0.2, threshold=1.0)
    c = P.Context(slab_doubles=8_000_000, max_patches=len(ps) + 8, max_groups=1, params=PRM)
    try:
        S.install_amr(c, ps, flux=True)
        c.set_group_max_dt(0, np.inf)
        c.set_time_stepping(P.TS_LOCAL)
        assert len(ps.flux_items)
        with pytest.raises(P.PcgError):
            c.run(1)
    finally:
        c.close()


def test_virtual_interval_known_answer_on_the_device():
    """PatchTest::testCoarsePatchTimeInterval (PatchTest.cpp:140-215) through
    pcg_set_virtual_time_items: nine leaves with the test's intervals under one
    virtual patch; an iteration that advances nothing sets its interval to
    time 2.5, timestep 0.2, bit-identical to the oracle."""
    from test_oracle_lts import _patch_test_intervals
    c = P.Context(slab_doubles=200_000, max_patches=16, max_groups=1, params=PRM)
    try:
        leaves = []
        for k, (t, dt) in enumerate(_patch_test_intervals()):
            pid = c.alloc(3, pos=((k // 3) / 3.0, (k % 3) / 3.0), size=(1.0 / 3.0, 1.0 / 3.0), level=1)
            c.set_time(pid, time=t, dt=dt)
            leaves.append(pid)
        virt = c.alloc(3, pos=(0.0, 0.0), size=(1.0, 1.0), level=0, leaf=False, virtual=True)
        c.set_virtual_time_items(leaves, [virt] * 9)
        c.set_group_max_dt(0, np.inf)
        c.set_group_end_time(0, 0.0, 0.0)
        c.set_time_stepping(P.TS_LOCAL)
        assert np.all(c.run(1) == 0.0)
        t = c.get_time(virt)
        assert t["time"] == 2.5
        assert t["dt"] == 1.0 + 1.7 - 2.5
    finally:
        c.close()
