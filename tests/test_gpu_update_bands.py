"""Inside a batched run the unfused strip update writes the old state into
the uOld interior only in the bands the next ghost fill reads (every other
cell is overwritten by the next sweep before anything reads it); the run's
last step and the step at which a group reaches its end time write the whole
interior.  Whatever the run lengths, every patch vector (uOld included) and
every dt equals the oracle's bit for bit."""
import numpy as np
import pytest

from oracle import oracle as O
from peanoclaw_gb300 import pcg as P
from peanoclaw_gb300 import scenarios as S

from helpers import gpu_patchset, oracle_params, oracle_patchset, slab_for

pytestmark = pytest.mark.gpu

PRM = P.swe_params(g=9.81, cfl=0.5)


def _bits(a):
    return np.ascontiguousarray(a).view(np.int64)


@pytest.mark.parametrize("runs", [(5,), (2, 3, 1, 4)])
def test_unfused_strip_runs_match_the_oracle(runs):
    """Uneven sizes (interpolated ghost cells read bands up to several cells
    deep), runs of several steps with downloads in between."""
    ps = S.uneven_patches(grid=10)
    ctx = P.Context(slab_doubles=slab_for(ps), max_patches=len(ps) + 16, max_groups=1, params=PRM)
    pats = oracle_patchset(ps)
    try:
        ids = gpu_patchset(ctx, ps)
        ctx.set_schedule(P.SCHED_STRIPS, 2, 32, P.STRIPS_UNFUSED)
        ctx.set_group_max_dt(0, 1e9)
        for k in runs:
            dts = list(ctx.run(k, P.PCG_MODE_BATCHED)[:, 0])
            odts = [O.grid_step(pats, ps.items, ps.wall, oracle_params(PRM), 1e9)[0] for _ in range(k)]
            assert dts == odts
            got = ctx.download_many(ids, int(ps.packed.size))
            assert np.array_equal(_bits(got), _bits(np.concatenate([p.u for p in pats])))
    finally:
        ctx.close()


def test_group_that_ends_inside_a_run_keeps_the_reference_layout():
    """Two mosaics in two groups; the first reaches its end time a few steps
    into a 30-step run (its last update writes the whole interior), the
    second goes on to the end of the run."""
    a = S.uneven_patches(grid=5, seed_sizes=11)
    b = S.uneven_patches(grid=5, seed_sizes=12)
    t_end = (2.5e-3, np.inf)
    ctx = P.Context(slab_doubles=slab_for(a) + slab_for(b), max_patches=len(a) + len(b) + 16, max_groups=2,
                    params=PRM)
    try:
        ids = []
        for g, ps in enumerate((a, b)):
            gi = gpu_patchset(ctx, ps)
            for i in gi:
                ctx.set_group(i, g)
            ids.append(gi)
        from peanoclaw_gb300.scenarios import remap_items
        ctx.set_ghost_items(np.concatenate([remap_items(a.items, ids[0]), remap_items(b.items, ids[1])]))
        ctx.set_schedule(P.SCHED_STRIPS, 2, 16, P.STRIPS_UNFUSED)
        for g in range(2):
            ctx.set_group_max_dt(g, 1e9)
            ctx.set_group_end_time(g, 0.0, t_end[g])
        hist = ctx.run(30, P.PCG_MODE_BATCHED)
        got = [ctx.download_many(ids[g], int(ps.packed.size)) for g, ps in enumerate((a, b))]
    finally:
        ctx.close()
    for g, ps in enumerate((a, b)):
        pats = oracle_patchset(ps)
        t = 0.0
        odts = []
        while t < t_end[g] and len(odts) < 30:
            dt = O.grid_step(pats, ps.items, ps.wall, oracle_params(PRM), min(1e9, t_end[g] - t))[0]
            odts.append(dt)
            t = t + dt
        assert list(hist[:len(odts), g]) == odts
        assert np.array_equal(_bits(got[g]), _bits(np.concatenate([p.u for p in pats])))
    assert np.count_nonzero(hist[:, 0]) < 30
