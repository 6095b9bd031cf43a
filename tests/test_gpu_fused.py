"""The fused form of the synchronous step (ghost fill, deferred update, sweep
and CFL in one kernel per step) against the oracle and against the unfused
form: every patch vector (ghost layers, signed zeros) and every dt bit for
bit, across strip variants and chunk widths, in the batched and the plain
form, with downloads (which apply the pending update) between runs, and with
groups that stop at different end times."""
import numpy as np
import pytest

from oracle import oracle as O
from peanoclaw_gb300 import pcg as P
from peanoclaw_gb300 import scenarios as S

from helpers import gpu_patchset, oracle_params, oracle_patchset, slab_for

pytestmark = pytest.mark.gpu

PRM = P.swe_params(g=9.81, cfl=0.5)


def _ctx(ps, groups=1):
    return P.Context(slab_doubles=slab_for(ps), max_patches=len(ps) + 16, max_groups=groups, params=PRM)


def _bits(a):
    return np.ascontiguousarray(a).view(np.int64)


@pytest.mark.parametrize("variant,chunk", [(2, 32), (0, 16), (4, 8), (3, 32)])
def test_fused_batched_matches_the_oracle(variant, chunk):
    ps = S.uneven_patches(grid=10)
    steps = 6
    ctx = _ctx(ps)
    try:
        ids = gpu_patchset(ctx, ps)
        ctx.set_schedule(P.SCHED_STRIPS, variant, chunk)
        ctx.set_group_max_dt(0, 1e9)
        assert ctx.step_is_fused(P.PCG_MODE_BATCHED)
        dts = list(ctx.run(steps, P.PCG_MODE_BATCHED)[:, 0])
        got = ctx.download_many(ids, int(ps.packed.size))
        times = [ctx.get_time(i) for i in ids[:5]]
    finally:
        ctx.close()
    pats = oracle_patchset(ps)
    odts = [O.grid_step(pats, ps.items, ps.wall, oracle_params(PRM), 1e9)[0] for _ in range(steps)]
    assert dts == odts
    ref = np.concatenate([p.u for p in pats])
    assert np.array_equal(_bits(got), _bits(ref))
    for t, p in zip(times, pats[:5]):
        assert (t["time"], t["dt"], t["est_next"]) == (p.s.time, p.s.dt, p.s.est_next)


def test_fused_plain_matches_the_oracle():
    ps = S.uneven_patches(grid=6)
    steps = 4
    ctx = _ctx(ps)
    try:
        ids = gpu_patchset(ctx, ps)
        ctx.set_group_max_dt(0, 1e9)
        assert ctx.step_is_fused(P.PCG_MODE_PLAIN)
        dts = list(ctx.run(steps, P.PCG_MODE_PLAIN)[:, 0])
        got = ctx.download_many(ids, int(ps.packed.size))
    finally:
        ctx.close()
    pats = oracle_patchset(ps)
    odts = [O.grid_step(pats, ps.items, ps.wall, oracle_params(PRM), 1e9)[0] for _ in range(steps)]
    assert dts == odts
    assert np.array_equal(_bits(got), _bits(np.concatenate([p.u for p in pats])))


def test_fused_equals_unfused_with_downloads_between_runs():
    """Runs of 1, 2 and 3 steps with a download (the pending update applied)
    after each, fused against unfused on the same schedule, and single steps
    through pcg_step."""
    ps = S.uneven_patches(grid=12)
    out = {}
    for form in (P.FORM_AUTO, P.FORM_UNFUSED):
        ctx = _ctx(ps)
        try:
            ids = gpu_patchset(ctx, ps)
            ctx.set_schedule(P.SCHED_STRIPS, 2, 32)
            ctx.set_step_form(form)
            ctx.set_group_max_dt(0, 1e9)
            assert ctx.step_is_fused() == (form == P.FORM_AUTO)
            rec = []
            for k in (1, 2, 3):
                rec.append(list(ctx.run(k, P.PCG_MODE_BATCHED)[:, 0]))
                # fused: sweep with ghost fill and deferred update, time
                # advance, reset; unfused: reset, ghost fill, walls, sweep,
                # update, dt history
                assert ctx.step_launches() == (3 if form == P.FORM_AUTO else 6)
                rec.append(_bits(ctx.download_many(ids, int(ps.packed.size))))
            for _ in range(2):
                rec.append(list(ctx.step(P.PCG_MODE_BATCHED)))
            rec.append(_bits(ctx.download_many(ids, int(ps.packed.size))))
            out[form] = rec
        finally:
            ctx.close()
    for a, b in zip(out[P.FORM_AUTO], out[P.FORM_UNFUSED]):
        if isinstance(a, list):
            assert a == b
        else:
            assert np.array_equal(a, b)


def test_fused_radial_dam_break_with_walls_and_corners():
    """Reflecting walls on every side (wall corners written by the flush),
    100 steps of the 9 x 9 x 16^2 radial dam break, fused against the
    oracle."""
    ps = S.radial_dam_break(npx=9, n=16)
    steps = 100
    ctx = _ctx(ps)
    try:
        ids = gpu_patchset(ctx, ps)
        ctx.set_schedule(P.SCHED_STRIPS, 2, 32)
        ctx.set_group_max_dt(0, 1e9)
        assert ctx.step_is_fused()
        dts = list(ctx.run(steps, P.PCG_MODE_BATCHED)[:, 0])
        got = ctx.download_many(ids, int(ps.packed.size))
    finally:
        ctx.close()
    pats = oracle_patchset(ps)
    odts = [O.grid_step(pats, ps.items, ps.wall, oracle_params(PRM), 1e9)[0] for _ in range(steps)]
    assert dts == odts
    assert np.array_equal(_bits(got), _bits(np.concatenate([p.u for p in pats])))


def test_fused_groups_with_end_times():
    """Two independent mosaics in two groups with different end times in one
    run: the group that reaches its end stops (its pending update applied once
    at the download), the other goes on; each equals the oracle stepped with
    max_dt = t_end - t."""
    a = S.uneven_patches(grid=5, seed_sizes=11)
    b = S.uneven_patches(grid=5, seed_sizes=12)
    t_end = (2.5e-3, 6e-3)
    ctx = P.Context(slab_doubles=slab_for(a) + slab_for(b), max_patches=len(a) + len(b) + 16, max_groups=2,
                    params=PRM)
    try:
        ids = []
        for g, ps in enumerate((a, b)):
            gi = gpu_patchset(ctx, ps)
            for i in gi:
                ctx.set_group(i, g)
            ids.append(gi)
        # the face-pair lists of both mosaics in one list
        from peanoclaw_gb300.scenarios import remap_items
        ctx.set_ghost_items(np.concatenate([remap_items(a.items, ids[0]), remap_items(b.items, ids[1])]))
        ctx.set_schedule(P.SCHED_STRIPS, 2, 16)
        for g in range(2):
            ctx.set_group_max_dt(g, np.inf)
            ctx.set_group_end_time(g, 0.0, t_end[g])
        assert ctx.step_is_fused()
        hist = ctx.run(40, P.PCG_MODE_BATCHED)
        times = ctx.group_times()
        got = [ctx.download_many(ids[g], int(ps.packed.size)) for g, ps in enumerate((a, b))]
    finally:
        ctx.close()
    for g, ps in enumerate((a, b)):
        pats = oracle_patchset(ps)
        t = 0.0
        odts = []
        while t < t_end[g]:
            dt = O.grid_step(pats, ps.items, ps.wall, oracle_params(PRM), t_end[g] - t)[0]
            odts.append(dt)
            t = t + dt
        assert times[g] == t
        steps = len(odts)
        assert list(hist[:steps, g]) == odts
        assert np.all(hist[steps:, g] == 0.0)
        assert np.array_equal(_bits(got[g]), _bits(np.concatenate([p.u for p in pats])))
