"""The PyClaw-style `Peano` driver on the GPU: subgrids initialised through
the reference's callback convention give the same result as the direct
batched path, a lake at rest over bumpy bathymetry (aux field) stays exactly
at rest, and gather_solution hands out every subgrid with its new time."""
from types import SimpleNamespace

import numpy as np
import pytest

from helpers import gpu_patchset, slab_for
from peanoclaw_gb300 import pcg as P
from peanoclaw_gb300 import scenarios as S
from peanoclaw_gb300.pyclaw import Peano

pytestmark = pytest.mark.gpu

PRM = P.swe_params(g=9.81, cfl=0.5)


def _solution(n, naux):
    dim = lambda: SimpleNamespace(lower=0.0, upper=1.0, num_cells=n)
    return SimpleNamespace(state=SimpleNamespace(grid=SimpleNamespace(dimensions=[dim(), dim()]),
                                                 num_eqn=3, num_aux=naux))


def _centers(px, py, sx, sy, n):
    hx, hy = sx / n, sy / n
    r = np.arange(n)
    return np.meshgrid((px + hx * r) + hx * 0.5, (py + hy * r) + hy * 0.5, indexing="ij")


def test_dam_break_equals_the_direct_path():
    def init(q, qbc, aux, n0, n1, n2, nq, naux, sx, sy, sz, px, py, pz, skip):
        X, Y = _centers(px, py, sx, sy, n0)
        r = np.sqrt((X - 0.5) ** 2 + (Y - 0.5) ** 2)
        q[0] = np.where(r <= 0.15, 2.0, 1.0)
        q[1:] = 0.0
        return 1.0 / 9
    peano = Peano(_solution(16, 0), 1.0 / 9, 1, 1e-3, init)
    try:
        peano.evolve_to_time(0.02)
        got = []
        peano.gather_solution(lambda q, qbc, g, sx, sy, sz, px, py, pz, t: got.append((q.copy(), t)))
    finally:
        peano.teardown()
    ps = S.radial_dam_break(npx=9, n=16)
    c = P.Context(slab_doubles=slab_for(ps), max_patches=len(ps) + 8, max_groups=1, params=PRM)
    try:
        ids = gpu_patchset(c, ps)
        c.set_group_max_dt(0, np.inf)
        c.set_group_end_time(0, 0.0, 0.02)
        c.run(200, P.PCG_MODE_BATCHED)
        assert c.group_times()[0] == 0.02
        ref = c.download_many(ids, int(ps.packed.size))
    finally:
        c.close()
    assert len(got) == 81
    for p, (q, t) in enumerate(got):
        assert t == 0.02
        unew, _, _ = ps.views(p)
        o = ps.offsets[p]
        assert np.array_equal(q.ravel().view(np.int64), ref[o:o + q.size].view(np.int64))


def test_lake_at_rest_with_bathymetry_aux():
    def init(q, qbc, aux, n0, n1, n2, nq, naux, sx, sy, sz, px, py, pz, skip):
        X, Y = _centers(px, py, sx, sy, n0)
        # dyadic bathymetry so that h + b is exact
        b = np.round(0.3 * np.exp(-((X - 0.4) ** 2 + (Y - 0.6) ** 2) / 0.01) * 64.0) / 64.0
        aux[0] = b
        q[0] = 1.0 - b
        q[1:] = 0.0
        return 0.25
    peano = Peano(_solution(12, 1), 0.25, 1, 1e-3, init)
    try:
        peano.evolve_to_time(0.05)
        out = []
        peano.gather_solution(lambda q, qbc, g, sx, sy, sz, px, py, pz, t: out.append(q.copy()))
        b = [peano.ps.views(p)[2][1:-1, 1:-1] for p in range(len(peano.ps))]
    finally:
        peano.teardown()
    for q, bb in zip(out, b):
        assert np.all(q[0] + bb == 1.0)
        assert np.all(q[1:] == 0.0)
