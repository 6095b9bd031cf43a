"""Full-size checks on the 50k-patch uneven mosaic (224 x 224 slots, 67.8 M
cells): three batched steps of the fused and of the pipelined form bit for
bit against the oracle on the whole mosaic, the warp-strip, the tile and the
pipelined schedules (independent work decompositions) give bit-identical
states and dts over six steps, every value
stays finite and the depth non-negative, and a device-side end time stops the
run exactly."""
import numpy as np
import pytest

from peanoclaw_gb300 import pcg as P
from peanoclaw_gb300 import scenarios as S

from helpers import oracle_params, oracle_patchset

pytestmark = pytest.mark.gpu

PRM = P.swe_params(g=9.81, cfl=0.5)


@pytest.fixture(scope="module")
def mosaic():
    return S.uneven_patches(grid=224)


def _run(ps, sched, steps, t_end=1e-3):
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
        c.set_group_end_time(0, 0.0, t_end)
        dts = c.run(steps, P.PCG_MODE_BATCHED)[:, 0]
        t = c.group_times()[0]
        return c.download_many(ids, int(ps.packed.size)), dts, t
    finally:
        c.close()


@pytest.fixture(scope="module")
def oracle_3_steps(mosaic):
    ps = mosaic
    pats = oracle_patchset(ps)
    from oracle import oracle as O
    odts = [O.grid_step(pats, ps.items, ps.wall, oracle_params(PRM), np.inf)[0] for _ in range(3)]
    return np.concatenate([p.u for p in pats]), odts


@pytest.mark.parametrize("form", [P.STRIPS_FUSED, P.STRIPS_UNFUSED, P.STRIPS_PIPELINED])
def test_full_mosaic_matches_the_oracle(mosaic, oracle_3_steps, form):
    """The headline workload itself, three steps of the fused, the unfused
    (old state written in bands inside the run) and the pipelined form, every
    patch vector (ghost layers and signed zeros included) and every dt bit for
    bit."""
    ps = mosaic
    got, dts, _ = _run(ps, (P.SCHED_STRIPS, 2, 32, form), 3, t_end=np.inf)
    ref, odts = oracle_3_steps
    assert list(dts) == odts
    for p in range(0, len(ps), 4096):
        a, b = ps.offsets[p], ps.offsets[p] + ps.vec_len(p)
        assert np.array_equal(got[a:b].view(np.int64), ref[a:b].view(np.int64)), p
    assert np.array_equal(got.view(np.int64), ref.view(np.int64))


def test_schedules_agree_at_full_size(mosaic):
    ps = mosaic
    a, da, ta = _run(ps, (P.SCHED_STRIPS, 2, 32), 6)
    b, db, tb = _run(ps, (P.SCHED_TILES, 0, 32), 6)
    c, dc, tc = _run(ps, (P.SCHED_STRIPS, 2, 32, P.STRIPS_PIPELINED), 6)
    assert np.array_equal(da, db) and ta == tb
    assert np.array_equal(a.view(np.int64), b.view(np.int64))
    assert np.array_equal(da, dc) and ta == tc
    assert np.array_equal(a.view(np.int64), c.view(np.int64))
    assert np.all(np.isfinite(a))
    n_h = [ps.offsets[p] + np.arange(ps.n[p] ** 2) for p in range(0, len(ps), 97)]
    assert np.all(a[np.concatenate(n_h)] >= 0.0)
    # the end time 1e-3 is reached within the 6 steps only if the dts add up
    if np.sum(da) >= 1e-3:
        assert ta == 1e-3
