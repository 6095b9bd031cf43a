"""Adaptive grid (3 levels, 3x refinement, 27x27 cells per patch): ghost
fill with coarse-to-fine interpolation and copies from virtual patches, flux
correction at level interfaces, restriction into virtual patches -- the whole
batched step bit for bit against the oracle."""
import numpy as np
import pytest

from peanoclaw_gb300 import pcg as P
from peanoclaw_gb300 import scenarios as S

from helpers import (gpu_amr_patchset, oracle_amr_patchset, oracle_amr_step, oracle_params,
                     oracle_restrict_all)

PRM = P.swe_params(g=9.81, cfl=0.5)


def test_amr_builder_levels_and_balance():
    ps = S.breaking_dam_amr(base=9, n=27, levels=3)
    assert np.bincount(ps.level).tolist() == [81, 243, 1215]
    assert sum(ps.leaf) == 1377
    # every interpolation item goes from a leaf exactly one level coarser
    for it in ps.items:
        if it[0] == P.PCG_GHOST_INTERP:
            s, d = it[1], it[2]
            assert ps.leaf[s] and ps.level[d] - ps.level[s] == 1
    assert len(ps.restrict_items) > 0 and len(ps.flux_items) > 0


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [P.PCG_MODE_BATCHED, P.PCG_MODE_PLAIN])
def test_amr_step_bit_exact(mode):
    ps = S.breaking_dam_amr(base=3, n=9, levels=3)
    steps = 8
    ctx = P.Context(slab_doubles=int(ps.packed.size * 1.3) + 4096, max_patches=len(ps) + 8,
                    max_groups=1, params=PRM)
    try:
        ids = gpu_amr_patchset(ctx, ps)
        ctx.restrict_all()
        ctx.set_group_max_dt(0, 1e9)
        dts = list(ctx.run(steps, mode)[:, 0])
        out = ctx.download_many(ids, int(ps.packed.size))
    finally:
        ctx.close()
    pats = oracle_amr_patchset(ps)
    oracle_restrict_all(pats, ps)
    odts = [oracle_amr_step(pats, ps, oracle_params(PRM), 1e9) for _ in range(steps)]
    ref = np.concatenate([p.u for p in pats])
    assert dts == odts
    assert np.all(np.isfinite(out))
    assert np.array_equal(out, ref)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [P.PCG_MODE_BATCHED, P.PCG_MODE_PLAIN])
def test_breaking_dam_full_size_bit_exact(mode):
    """The adaptive configuration at its own size: 3 levels of 3x refinement,
    27 x 27 cells per patch, 1,539 patches (1,377 leaves), interpolation, flux
    correction and restriction every step; 5 steps bit for bit."""
    ps = S.breaking_dam_amr(base=9, n=27, levels=3)
    assert len(ps) == 1539
    steps = 5
    ctx = P.Context(slab_doubles=int(ps.packed.size * 1.3) + 4096, max_patches=len(ps) + 8,
                    max_groups=1, params=PRM)
    try:
        ids = gpu_amr_patchset(ctx, ps)
        ctx.restrict_all()
        ctx.set_group_max_dt(0, 1e9)
        dts = list(ctx.run(steps, mode)[:, 0])
        out = ctx.download_many(ids, int(ps.packed.size))
    finally:
        ctx.close()
    pats = oracle_amr_patchset(ps)
    oracle_restrict_all(pats, ps)
    odts = [oracle_amr_step(pats, ps, oracle_params(PRM), 1e9) for _ in range(steps)]
    ref = np.concatenate([p.u for p in pats])
    assert dts == odts
    assert np.array_equal(out.view(np.int64), ref.view(np.int64))


@pytest.mark.gpu
def test_bounded_transfer_wait_reports_and_context_stays_usable():
    """The level transfer's wait between its flux and restriction phases is
    bounded: made to wait for a counter nothing sets, every wait runs out,
    the error word comes back to the host, and no patch data changed -- the
    run continued afterwards equals the oracle bit for bit."""
    ps = S.breaking_dam_amr(base=3, n=9, levels=3)
    ctx = P.Context(slab_doubles=int(ps.packed.size * 1.3) + 4096, max_patches=len(ps) + 8, max_groups=1,
                    params=PRM)
    try:
        ids = gpu_amr_patchset(ctx, ps)
        ctx.restrict_all()
        ctx.set_group_max_dt(0, 1e9)
        dts = list(ctx.run(2, P.PCG_MODE_BATCHED)[:, 0])
        ctx.selftest_transfer_wait()
        dts += list(ctx.run(2, P.PCG_MODE_BATCHED)[:, 0])
        out = ctx.download_many(ids, int(ps.packed.size))
    finally:
        ctx.close()
    pats = oracle_amr_patchset(ps)
    oracle_restrict_all(pats, ps)
    odts = [oracle_amr_step(pats, ps, oracle_params(PRM), 1e9) for _ in range(4)]
    assert dts == odts
    ref = np.concatenate([p.u for p in pats])
    assert np.array_equal(out.view(np.int64), ref.view(np.int64))
