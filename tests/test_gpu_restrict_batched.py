"""The batched restriction (pcg_set_restriction_items + pcg_restrict_all) on
destinations that take each of its forms, in one list, against the oracle's
item-by-item restriction (clear, restrict in list order, post-process):
- 9 sources whose regions lie inside the destination: the table walk;
- 144 sources into one destination (more than the 128 items of the table):
  the item-by-item form;
- 4 unknowns per cell: the item-by-item form;
- 16 sources whose cells straddle the destination's: the table walk with
  destination cells held by two rectangles.
Whole-patch and overlapped-only restriction; sources with time intervals
(time factors other than 0 and 1) and source cells that straddle the
destination's cells (1/108 against 1/81)."""
import numpy as np
import pytest

from helpers import oracle_patch_from
from oracle import oracle as O
from peanoclaw_gb300 import pcg as P

pytestmark = pytest.mark.gpu

THIRD = 1.0 / 3.0


def _tiles(x0, y0, extent, k, n):
    """k x k source tiles of the square [x0, x0 + extent]^2, n^2 cells each."""
    s = extent / k
    return [((x0 + i * s, y0 + j * s), (s, s), n) for i in range(k) for j in range(k)]


# (destination pos, size, n, unknowns), its sources
LAYOUT = [
    (((0.0, 0.0), (THIRD, THIRD), 27, 3), _tiles(0.0, 0.0, THIRD, 12, 3)),
    (((THIRD, 0.0), (THIRD, THIRD), 9, 3), _tiles(THIRD, 0.0, THIRD, 3, 9)),
    (((2 * THIRD, 0.0), (THIRD, THIRD), 9, 4), _tiles(2 * THIRD, 0.0, THIRD, 2, 6)),
    # table walk with source cells straddling the destination's: the
    # rectangles of neighbouring sources share their boundary cells
    (((0.0, THIRD), (THIRD, THIRD), 27, 3), _tiles(0.0, THIRD, THIRD, 4, 9)),
]


@pytest.mark.parametrize("only_overlapped", [False, True])
def test_batched_restriction_all_forms(only_overlapped):
    rng = np.random.default_rng(77 + int(only_overlapped))
    n_src = sum(len(s) for _, s in LAYOUT)
    c = P.Context(slab_doubles=400_000, max_patches=n_src + 8, max_groups=1,
                  params=P.swe_params(g=9.81, cfl=0.5))
    try:
        src_ids, dst_ids, gpu_dst, ora = [], [], [], {}
        for (dpos, dsize, dn, nq), sources in LAYOUT:
            v = rng.normal(1.0, 0.3, P.vector_size(dn, 1, nq, 0, 1))
            d = c.alloc(dn, nq=nq, pos=dpos, size=dsize, level=0, leaf=False, virtual=True)
            c.upload(d, v)
            # neighbouring ghost-layer bounds: ghost layers reach 0.25 (0.2) in
            # from the lower faces and 0.3 (0.25) in from the upper faces
            rl = (dpos[0] + 0.7 * dsize[0], dpos[1] + 0.75 * dsize[1])
            ru = (dpos[0] + 0.25 * dsize[0], dpos[1] + 0.2 * dsize[1])
            c.set_time(d, time=0.0, dt=0.0, restr_lower=rl, restr_upper=ru)
            od = oracle_patch_from(v.copy(), dn, dpos, dsize, nq=nq, leaf=False, virtual=True)
            od.s.restr_lower[0], od.s.restr_lower[1] = rl
            od.s.restr_upper[0], od.s.restr_upper[1] = ru
            gpu_dst.append((d, v.size))
            ora[d] = od
            for spos, ssize, sn in sources:
                vs = rng.normal(1.0, 0.3, P.vector_size(sn, 1, nq, 0, 1))
                t, dt = float(rng.uniform(0.0, 1.0)), float(rng.uniform(0.1, 0.5))
                s = c.alloc(sn, nq=nq, pos=spos, size=ssize, level=1)
                c.upload(s, vs)
                c.set_time(s, time=t, dt=dt)
                ora[s] = oracle_patch_from(vs, sn, spos, ssize, nq=nq, level=1, time=t, dt=dt)
                src_ids.append(s)
                dst_ids.append(d)
        assert sum(1 for d in dst_ids if d == gpu_dst[0][0]) > 128
        c.set_restriction_items(src_ids, dst_ids, only_overlapped=only_overlapped)
        c.restrict_all()
        # the oracle: clear every destination, restrict in list order, post-process
        for d, _ in gpu_dst:
            od = ora[d]
            od.unew()[:] = 0.0
            od.uold()[:, 1:-1, 1:-1] = 0.0
        for s, d in zip(src_ids, dst_ids):
            O.restrict(ora[s], ora[d], only_overlapped=only_overlapped, swe=True)
        for d, _ in gpu_dst:
            O.lib().pco_swe_post_process_restriction(ora[d].ptr())
        for d, size in gpu_dst:
            got = c.download(d, size)
            assert np.array_equal(got.view(np.int64), ora[d].u.view(np.int64)), d
            # every destination received something
            assert np.count_nonzero(ora[d].unew()) > 0
    finally:
        c.close()
