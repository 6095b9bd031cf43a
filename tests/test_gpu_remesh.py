"""Dynamic remeshing on the GPU (device refinement criterion, new patches by
interpolation from the coarse patch, coarsening by full restriction and
switchToLeaf, lists rebuilt) against the same remesh on the oracle: the
criterion values, the dts, the hierarchy and every patch vector agree bit for
bit while the grid follows a moving breaking-dam front."""
import copy

import numpy as np
import pytest

from helpers import OracleAmr, oracle_params
from peanoclaw_gb300 import pcg as P
from peanoclaw_gb300 import scenarios as S
from peanoclaw_gb300.amr import DeviceAmr

pytestmark = pytest.mark.gpu

PRM = P.swe_params(g=9.81, cfl=0.5)


@pytest.mark.parametrize("mode", [P.PCG_MODE_BATCHED, P.PCG_MODE_PLAIN])
def test_remesh_matches_the_oracle(mode):
    ps = S.breaking_dam_amr(base=3, n=9, levels=3, h_left=1.0, h_right=0.2, threshold=1.0)
    ctx = P.Context(slab_doubles=8_000_000, max_patches=1024, max_groups=1, params=PRM)
    try:
        ids = S.install_amr(ctx, ps)
        ctx.restrict_all()
        ctx.set_group_max_dt(0, 1e9)
        dev = DeviceAmr(ctx, ps.grid, ps.b_of)
        dev.pid = dict(zip(ps.grid.order(), (int(i) for i in ids)))
        ora = OracleAmr(copy.deepcopy(ps.grid), ps, ps.b_of)
        ora.restrict_all()
        prm = oracle_params(PRM)
        changes = []
        for r in range(8):
            hist = ctx.run(4, mode)[:, 0]
            odts = [ora.step(prm, 1e9) for _ in range(4)]
            assert list(hist) == odts
            gd, go = dev.indicators(), ora.indicators()
            assert gd.keys() == go.keys()
            assert all(np.float64(gd[k]).view(np.int64) == np.float64(go[k]).view(np.int64) for k in gd)
            cd = dev.remesh()
            co = ora.remesh()
            assert cd == co
            changes.append(cd)
            assert dev.grid.order() == ora.grid.order()
        assert sum(c[0] for c in changes) > 0
        # forced rounds: every leaf below the threshold (everything that can
        # coarsen does), steps, then every leaf above it (refine everywhere)
        from peanoclaw_gb300.amr import remesh
        for val in (0.0, 1e9):
            cd = remesh(dev.grid, dev, {s: val for s in dev.grid.leaves()}, ps.b_of)
            co = remesh(ora.grid, ora, {s: val for s in ora.grid.leaves()}, ps.b_of)
            assert cd == co and cd[1 if val == 0.0 else 0] > 0
            hist = ctx.run(3, mode)[:, 0]
            assert list(hist) == [ora.step(prm, 1e9) for _ in range(3)]
        hist = ctx.run(3, mode)[:, 0]
        assert list(hist) == [ora.step(prm, 1e9) for _ in range(3)]
        order = dev.grid.order()
        for s in order:
            p = ora.pat[s]
            got = ctx.download(dev.pid[s], p.u.size)
            assert np.array_equal(got.view(np.int64), p.u.view(np.int64)), s
            t = ctx.get_time(dev.pid[s])
            assert (t["time"], t["dt"]) == (p.s.time, p.s.dt)
    finally:
        ctx.close()


def test_batched_restriction_bounds():
    """pcg_patches_set_restriction_bounds writes the bounds of every listed
    patch, keeps their other time fields and rejects repeated ids."""
    import ctypes as C
    ctx = P.Context(slab_doubles=1_000_000, max_patches=16, max_groups=1, params=PRM)
    try:
        ids = [ctx.alloc(8, pos=(0.1 * k, 0.0), size=(0.1, 0.1)) for k in range(6)]
        for k, pid in enumerate(ids):
            ctx.set_time(pid, time=0.5 + k, dt=0.25, est_next=0.125)
        sel = np.array(ids[1:5], dtype=np.int32)
        lo = np.arange(8, dtype=np.float64).reshape(4, 2) * 0.01
        up = 1.0 + lo
        ctx.set_restriction_bounds(sel, lo, up)
        arr = (P.PatchTime * len(ids))()
        P.check(P.lib().pcg_patches_get_time(ctx.h, len(ids), np.asarray(ids, dtype=np.int32).ctypes.data_as(
            C.POINTER(C.c_int32)), arr))
        big = np.finfo(np.float64).max
        for k, pid in enumerate(ids):
            t = arr[k]
            assert (t.time, t.dt, t.est_next) == (0.5 + k, 0.25, 0.125)
            if 1 <= k <= 4:
                assert tuple(t.restr_lower) == tuple(lo[k - 1]) and tuple(t.restr_upper) == tuple(up[k - 1])
            else:
                assert tuple(t.restr_lower) == (big, big) and tuple(t.restr_upper) == (-big, -big)
        with pytest.raises(P.PcgError):
            ctx.set_restriction_bounds([ids[0], ids[0]], np.zeros((2, 2)), np.zeros((2, 2)))
        with pytest.raises(P.PcgError):
            ctx.set_restriction_bounds([99], np.zeros((1, 2)), np.zeros((1, 2)))
    finally:
        ctx.close()


def test_batched_times_and_interpolations():
    """pcg_patches_set_time writes every listed record; pcg_interpolate_solution_many
    equals one pcg_interpolate_solution per item; both reject repeated or
    conflicting ids."""
    import ctypes as C
    rng = np.random.default_rng(3)
    ctx = P.Context(slab_doubles=2_000_000, max_patches=32, max_groups=1, params=PRM)
    try:
        coarse = [ctx.alloc(9, pos=(0.3 * k, 0.0), size=(0.3, 0.3)) for k in range(2)]
        for k, pid in enumerate(coarse):
            v = np.zeros(P.vector_size(9))
            v[:] = rng.uniform(0.5, 1.5, v.size)
            ctx.upload(pid, v)
        fine_a = [ctx.alloc(9, pos=(0.3 * (k // 3) + 0.1 * (k % 3), 0.0), size=(0.1, 0.1), level=1) for k in range(6)]
        fine_b = [ctx.alloc(9, pos=(0.3 * (k // 3) + 0.1 * (k % 3), 0.0), size=(0.1, 0.1), level=1) for k in range(6)]
        ctx.set_times_many(coarse + fine_a + fine_b, np.full(14, 0.5), np.full(14, 0.25), np.full(14, 0.125))
        for pid in coarse + fine_a:
            t = ctx.get_time(pid)
            assert (t["time"], t["dt"], t["est_next"]) == (0.5, 0.25, 0.125)
        src = [coarse[k // 3] for k in range(6)]
        for to_uold, cur in ((0, 0), (1, 1)):
            ctx.interpolate_many(src, fine_a, np.full((6, 2), 9), np.zeros((6, 2)), to_uold, cur, 0, True)
            for s, d in zip(src, fine_b):
                P.check(P.lib().pcg_interpolate_solution(ctx.h, P.i2((9, 9)), P.i2((0, 0)), s, d, to_uold, cur, 0, 1))
        a = ctx.download_many(fine_a, 6 * P.vector_size(9))
        b = ctx.download_many(fine_b, 6 * P.vector_size(9))
        assert np.array_equal(a.view(np.int64), b.view(np.int64))
        with pytest.raises(P.PcgError):
            ctx.interpolate_many(src[:2], [fine_a[0], fine_a[0]], np.full((2, 2), 9), np.zeros((2, 2)), 0, 0, 0)
        with pytest.raises(P.PcgError):
            ctx.interpolate_many([fine_a[0], coarse[0]], [fine_a[1], fine_a[0]], np.full((2, 2), 9),
                                 np.zeros((2, 2)), 0, 0, 0)
        with pytest.raises(P.PcgError):
            ctx.set_times_many([coarse[0], coarse[0]], [0, 0], [0, 0], [0, 0])
    finally:
        ctx.close()


@pytest.mark.parametrize("kind", [P.PCG_CRIT_DEPTH_GRADIENT, P.PCG_CRIT_SURFACE_DIFFERENCE,
                                  P.PCG_CRIT_SURFACE_GRADIENT])
def test_refinement_criteria_match_the_oracle(kind):
    """pcg_refinement_criterion of every kind on random wet/dry patches of
    several sizes equals the oracle backend's criterion bit for bit."""
    from helpers import oracle_criterion, oracle_patch_from, random_swe_vector
    rng = np.random.default_rng(90 + kind)
    ctx = P.Context(slab_doubles=2_000_000, max_patches=64, max_groups=1, params=PRM)
    try:
        for n, size in ((9, 1.0 / 9), (16, 0.05), (27, 1.0 / 81)):
            vec = random_swe_vector(rng, n)
            pid = ctx.alloc(n, pos=(0.0, 0.0), size=(size, size))
            ctx.upload(pid, vec)
            got = ctx.refinement_indicator([pid], kind)[0]
            want = oracle_criterion(oracle_patch_from(vec, n, size=(size, size)), kind)
            assert np.float64(got).view(np.int64) == np.float64(want).view(np.int64), (n, got, want)
            ctx.free(pid)
    finally:
        ctx.close()
