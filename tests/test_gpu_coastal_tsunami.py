"""The large adaptive tsunami at its full size against the oracle: 3 levels of
3x refinement, 27 x 27 cells per patch (an effective 6561^2 grid), a
Gaussian surface hump over the sum-of-Gaussians seafloor (seed 2000) with a
coastline along x = 1, interpolation, flux correction and restriction every
step, and dynamic remeshing every 10 steps driven by the device's surface
criterion.  Twenty steps with two remeshes: dts, criterion values,
hierarchy changes and every patch vector bit for bit."""
import copy

import numpy as np
import pytest

from helpers import OracleAmr, oracle_params
from peanoclaw_gb300 import pcg as P
from peanoclaw_gb300 import scenarios as S
from peanoclaw_gb300.amr import DeviceAmr

pytestmark = pytest.mark.gpu

PRM = P.swe_params(g=9.81, cfl=0.5)


def test_coastal_tsunami_full_size_with_remeshing():
    ps = S.coastal_tsunami()
    assert ps.grid.base == 27 and ps.grid.n == 27 and ps.grid.levels == 3
    slab = int(ps.packed.size * 2.0) + 4096
    ctx = P.Context(slab_doubles=slab, max_patches=4 * len(ps), max_groups=1, params=PRM)
    try:
        ids = S.install_amr(ctx, ps)
        ctx.restrict_all()
        ctx.set_group_max_dt(0, 1e9)
        dev = DeviceAmr(ctx, ps.grid, ps.b_of, criterion=ps.criterion)
        dev.pid = dict(zip(ps.grid.order(), (int(i) for i in ids)))
        ora = OracleAmr(copy.deepcopy(ps.grid), ps, ps.b_of, criterion=ps.criterion)
        ora.restrict_all()
        prm = oracle_params(PRM)
        for r in range(2):
            hist = ctx.run(10, P.PCG_MODE_BATCHED)[:, 0]
            odts = [ora.step(prm, 1e9) for _ in range(10)]
            assert list(hist) == odts
            gd, go = dev.indicators(), ora.indicators()
            assert gd.keys() == go.keys()
            assert all(np.float64(gd[k]).view(np.int64) == np.float64(go[k]).view(np.int64) for k in gd)
            assert dev.remesh() == ora.remesh()
            assert dev.grid.order() == ora.grid.order()
        hist = ctx.run(2, P.PCG_MODE_BATCHED)[:, 0]
        assert list(hist) == [ora.step(prm, 1e9) for _ in range(2)]
        order = dev.grid.order()
        got = ctx.download_many([dev.pid[s] for s in order], sum(ora.pat[s].u.size for s in order))
        ref = np.concatenate([ora.pat[s].u for s in order])
        assert np.array_equal(got.view(np.int64), ref.view(np.int64))
        # the seafloor leaves dry land and wet cells; nothing went negative
        leaf_h = [ora.pat[s].unew()[0] for s in dev.grid.leaves()]
        h = np.concatenate([a.ravel() for a in leaf_h])
        assert np.all(h >= 0.0) and np.any(h == 0.0) and np.any(h > 0.5)
    finally:
        ctx.close()
