"""Full-size checks on the 50k-patch uneven mosaic (67.8 M cells) through
size-independent properties: the warp-strip and the tile schedules (two
independent work decompositions) give bit-identical states and dts, every
value stays finite and the depth non-negative, and a device-side end time
stops the run exactly."""
import numpy as np
import pytest

from peanoclaw_gb300 import pcg as P
from peanoclaw_gb300 import scenarios as S

pytestmark = pytest.mark.gpu

PRM = P.swe_params(g=9.81, cfl=0.5)


def _run(ps, sched, steps):
    slab = int(sum(P.vector_size(n) + 32 for n in ps.n)) + 4096
    c = P.Context(slab_doubles=slab, max_patches=len(ps) + 16, max_groups=1, params=PRM)
    try:
        ids = []
        for p in range(len(ps)):
            pid = c.alloc(ps.n[p], pos=ps.pos[p], size=ps.size[p])
            if ps.wall[p]:
                c.set_boundary(pid, ps.wall[p])
            ids.append(pid)
        c.upload_many(ids, ps.packed)
        c.set_ghost_items(S.remap_items(ps.items, ids))
        c.set_schedule(*sched)
        c.set_group_max_dt(0, np.inf)
        c.set_group_end_time(0, 0.0, 1e-3)
        dts = c.run(steps, P.PCG_MODE_BATCHED)[:, 0]
        t = c.group_times()[0]
        return c.download_many(ids, int(ps.packed.size)), dts, t
    finally:
        c.close()


def test_schedules_agree_at_full_size():
    ps = S.uneven_patches(grid=224)
    a, da, ta = _run(ps, (P.SCHED_STRIPS, 2, 32), 6)
    b, db, tb = _run(ps, (P.SCHED_TILES, 0, 32), 6)
    assert np.array_equal(da, db) and ta == tb
    assert np.array_equal(a.view(np.int64), b.view(np.int64))
    assert np.all(np.isfinite(a))
    n_h = [ps.offsets[p] + np.arange(ps.n[p] ** 2) for p in range(0, len(ps), 97)]
    assert np.all(a[np.concatenate(n_h)] >= 0.0)
    # the end time 1e-3 is reached within the 6 steps only if the dts add up
    if np.sum(da) >= 1e-3:
        assert ta == 1e-3
