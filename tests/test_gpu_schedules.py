"""Every batched schedule (16x16 tiles, warp strips of each CTA variant and
chunk width) and the autotuner give results bit-identical to the oracle,
on mosaics whose patch sizes do not divide into the strip/tile shapes."""
import numpy as np
import pytest

from helpers import gpu_patchset, oracle_params, oracle_patchset, slab_for
from oracle import oracle as O
from peanoclaw_gb300 import pcg as P
from peanoclaw_gb300 import scenarios as S

pytestmark = pytest.mark.gpu

PRM = P.swe_params(g=9.81, cfl=0.5)


def _oracle_run(ps, steps, max_dt=1e9):
    pats = oracle_patchset(ps)
    dts = [O.grid_step(pats, ps.items, ps.wall, oracle_params(PRM), max_dt)[0] for _ in range(steps)]
    return np.concatenate([p.u for p in pats]), dts


def _gpu_run(ps, steps, sched=None, autotune_reps=0):
    c = P.Context(slab_doubles=slab_for(ps), max_patches=len(ps) + 8, max_groups=1, params=PRM)
    try:
        ids = gpu_patchset(c, ps)
        c.set_group_max_dt(0, 1e9)
        tuned = None
        if sched is not None:
            c.set_schedule(*sched)
        if autotune_reps:
            tuned = c.autotune(autotune_reps)
        dts = list(c.run(steps, P.PCG_MODE_BATCHED)[:, 0]) if steps else []
        out = c.download_many(ids, int(ps.packed.size))
        return out, dts, tuned, c.get_schedule()
    finally:
        c.close()


SCHEDULES = [
    (P.SCHED_TILES, 0, 32),
    (P.SCHED_STRIPS, 2, 32, 1),
    (P.SCHED_STRIPS, 0, 32),
    (P.SCHED_STRIPS, 1, 16),
    (P.SCHED_STRIPS, 2, 32),
    (P.SCHED_STRIPS, 3, 7),
    (P.SCHED_STRIPS, 0, 1),
    (P.SCHED_STRIPS, 4, 32),
]


@pytest.mark.parametrize("sched", SCHEDULES)
def test_schedule_bit_exact_on_ragged_sizes(sched):
    # 5 (six 5-row groups per warp), 12, 33 (17 + 16 rows), 40 (20 + 20 rows,
    # two 20-column chunks) cells per patch edge, wet and dry
    ps = S.uneven_patches(grid=5, sizes=(5, 12, 33, 40))
    assert ps.meta["dry_fraction"] > 0.05
    out, dts, _, got = _gpu_run(ps, 12, sched=sched)
    assert got[:3] == sched[:3]
    oout, odts = _oracle_run(ps, 12)
    assert dts == odts
    assert np.all(np.isfinite(out))
    assert np.array_equal(out.view(np.int64), oout.view(np.int64))


def test_autotuner_picks_a_candidate_and_keeps_results_exact():
    ps = S.uneven_patches(grid=4, sizes=(8, 16, 32, 64))
    out, dts, tuned, got = _gpu_run(ps, 3, autotune_reps=1)
    # 16 candidates (the sizes are even: tiles with TMA staging too; strips of
    # chunk 32 and 16 in 5 variants, of chunk 10 and 8 in 2), and the best
    # strip schedule in the unfused form (where the fused one applied) and in
    # the pipelined form when a strip schedule won
    assert len(tuned) in (16, 17, 18)
    assert any(k[:2] == (P.SCHED_TILES, 1) for k, _ in tuned)
    assert all(ms > 0.0 for _, ms in tuned)
    best = min(tuned, key=lambda t: t[1])[0]
    assert got == best
    # the autotuner advanced the simulation by one step per candidate
    oout, odts = _oracle_run(ps, len(tuned) + 3)
    assert dts == odts[-3:]
    assert np.array_equal(out.view(np.int64), oout.view(np.int64))


def test_tuned_schedule_is_reused_for_the_same_patch_mix():
    ps = S.uneven_patches(grid=4, sizes=(8, 16, 32, 64))
    _, _, tuned, got = _gpu_run(ps, 0, autotune_reps=1)
    _, _, _, got2 = _gpu_run(ps, 1)
    assert got2 == got


def test_schedule_arguments_are_checked():
    ps = S.radial_dam_break(npx=2, n=8)
    c = P.Context(slab_doubles=slab_for(ps), max_patches=8, max_groups=1, params=PRM)
    try:
        for bad in [(2, 0, 32), (1, 9, 32), (1, 5, 32), (1, 0, 0), (1, 0, 33)]:
            with pytest.raises(P.PcgError):
                c.set_schedule(*bad)
    finally:
        c.close()


def test_tma_tile_staging_bit_exact_on_even_sizes():
    """Tiles staged by tensor copies (uNew, uOld and bathymetry boxes) on
    even patch sizes whose tiles are partial (18 = 16 + 2, 34, 40) and on
    8 x 8 patches (one tile smaller than the box), walls, copies and
    interpolations between sizes: 12 steps bit for bit against the oracle."""
    ps = S.uneven_patches(grid=5, sizes=(8, 18, 34, 40))
    out, dts, _, got = _gpu_run(ps, 12, sched=(P.SCHED_TILES, 1, 32))
    assert got[:2] == (P.SCHED_TILES, 1)
    oout, odts = _oracle_run(ps, 12)
    assert dts == odts
    assert np.array_equal(out.view(np.int64), oout.view(np.int64))


def test_tma_tile_staging_refuses_odd_sizes():
    ps = S.uneven_patches(grid=3, sizes=(5, 12))
    c = P.Context(slab_doubles=slab_for(ps), max_patches=len(ps) + 8, max_groups=1, params=PRM)
    try:
        gpu_patchset(c, ps)
        c.set_group_max_dt(0, 1e9)
        c.set_schedule(P.SCHED_TILES, 1, 32)
        with pytest.raises(P.PcgError):
            c.run(1, P.PCG_MODE_BATCHED)
    finally:
        c.close()
