"""Device-side end times (pcg_set_group_end_time): each group stops exactly at
its end time inside one replayed run of many steps, its result equals the
oracle stepped with max_dt = t_end - t, and further steps leave it untouched."""
import numpy as np
import pytest

from helpers import oracle_params, oracle_patchset
from oracle import oracle as O
from peanoclaw_gb300 import pcg as P
from peanoclaw_gb300 import scenarios as S

pytestmark = pytest.mark.gpu

PRM = P.swe_params(g=9.81, cfl=0.5)


def _oracle_until(ps, t_end):
    pats = oracle_patchset(ps)
    t = 0.0
    steps = 0
    while t < t_end:
        dt = O.grid_step(pats, ps.items, ps.wall, oracle_params(PRM), max(0.0, t_end - t))[0]
        if dt <= 0.0:
            break
        t += dt
        steps += 1
    return np.concatenate([p.u for p in pats]), t, steps


@pytest.mark.parametrize("mode", [P.PCG_MODE_BATCHED, P.PCG_MODE_PLAIN])
def test_groups_stop_at_their_end_times(mode):
    ps = S.radial_dam_break(npx=3, n=16)
    ends = (0.011, 0.027)
    c = P.Context(slab_doubles=4 * int(ps.packed.size) + 8192, max_patches=64, max_groups=2, params=PRM)
    try:
        ids = []
        for g in range(2):
            gi = []
            for p in range(len(ps)):
                pid = c.alloc(ps.n[p], pos=ps.pos[p], size=ps.size[p])
                c.set_group(pid, g)
                c.set_boundary(pid, ps.wall[p])
                gi.append(pid)
            c.upload_many(gi, ps.packed)
            ids.append(gi)
        c.set_ghost_items(np.concatenate([S.remap_items(ps.items, gi) for gi in ids]))
        for g in range(2):
            c.set_group_max_dt(g, np.inf)
            c.set_group_end_time(g, 0.0, ends[g])
        hist = c.run(60, mode)
        times = c.group_times()
        out = [c.download_many(gi, int(ps.packed.size)) for gi in ids]
        c.run(5, mode)   # both groups are finished: nothing may change
        again = [c.download_many(gi, int(ps.packed.size)) for gi in ids]
    finally:
        c.close()
    for g in range(2):
        ref, t, steps = _oracle_until(ps, ends[g])
        assert times[g] == t == ends[g]
        assert int(np.count_nonzero(hist[:, g] > 0.0)) == steps
        assert np.array_equal(out[g].view(np.int64), ref.view(np.int64))
        assert np.array_equal(again[g].view(np.int64), out[g].view(np.int64))
